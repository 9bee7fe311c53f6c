"""Free energy and its gradient (hand-written backward kernels behind a
torch.autograd.Function) against FP64 references.

F is checked against N times the oracle's DA quality; dF/dY, dF/dT and
dF/dbeta against the FP64 analytic gradient and against FP64 central finite
differences of the oracle's F (step 1e-6).  On a Blackwell GPU with D <= 189
the contractions run on the tensor cores in the split-BF16 form (three BF16
products per FP32 product, FP32 accumulation, FP64 reductions); elsewhere on
FP32 CUDA cores.  Relative tolerances 1e-5 on F, 1e-3 on gradients.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def sub(pkg, name):
    return importlib.import_module(pkg.__name__ + "." + name)


def oracle_F(orc, Y, T, beta, temp):
    Dm = orc.dist(Y, T)
    R, vgc, vgc2 = orc.resp(Dm, beta, 1, temp)
    N, D = T.shape
    return T.shape[0] * orc.qual(N, Y.shape[0], D, beta, vgc2, 1, temp), R, Dm


@pytest.fixture(scope="module")
def problem(pkg):
    ds = sub(pkg, "datasets")
    st = sub(pkg, "gtm_setup")
    T = ds.gaussian_mixture(2048, 16, 16, 0.2, seed=4)
    X, FI = st.setup_grid(2, 256, 16, 1.0)
    rng = np.random.default_rng(4)
    Y = T[rng.integers(0, T.shape[0], 256)] + 0.05 * rng.standard_normal((256, 16))
    # work in the FP32-rounded values so both sides see the same inputs
    return Y.astype(np.float32).astype(np.float64), T.astype(np.float32).astype(np.float64)


def run_fe(pkg, Y, T, beta, temp):
    ag = sub(pkg, "autograd")
    Yt = torch.tensor(Y, dtype=torch.float32, device="cuda", requires_grad=True)
    Tt = torch.tensor(T, dtype=torch.float32, device="cuda", requires_grad=True)
    bt = torch.tensor(beta, dtype=torch.float64, device="cuda", requires_grad=True)
    F = ag.free_energy(Yt, Tt, bt, temp)
    F.backward()
    torch.cuda.synchronize()
    return F.item(), Yt.grad.double().cpu().numpy(), Tt.grad.double().cpu().numpy(), bt.grad.item()


@pytest.mark.parametrize("beta,temp", [(6.0, 1.0), (6.0, 2.5)])
def test_free_energy_and_analytic_gradient(pkg, orc, problem, beta, temp):
    Y, T = problem
    F, dY, dT, db = run_fe(pkg, Y, T, beta, temp)
    Fo, R, Dm = oracle_F(orc, Y, T, beta, temp)
    assert F == pytest.approx(Fo, rel=1e-5)
    G = R.sum(1)
    dY_ref = -beta * (G[:, None] * Y - R @ T)
    dT_ref = -beta * (T - R.T @ Y)
    N, D = T.shape
    db_ref = N * D / (2 * beta) - 0.5 * (R * Dm).sum()
    assert np.max(np.abs(dY - dY_ref)) <= 1e-3 * np.max(np.abs(dY_ref))
    assert np.max(np.abs(dT - dT_ref)) <= 1e-3 * np.max(np.abs(dT_ref))
    assert db == pytest.approx(db_ref, rel=1e-3)


@pytest.mark.parametrize("N,K,D,binary", [(1000, 300, 37, False), (3000, 520, 166, True),
                                          (777, 64, 189, False), (129, 130, 1, False),
                                          (5000, 2100, 64, False)])
def test_shapes_against_oracle(pkg, orc, N, K, D, binary):
    """Ragged point and centre counts (tiles and chunks only partly filled),
    D from 1 to the split form's 189, binary and real-valued data; the
    centre count 2100 spans two 2048-centre accumulator segments of the data
    gradient."""
    rng = np.random.default_rng(N + K + D)
    if binary:
        T = (rng.random((N, D)) < 0.3).astype(np.float64)
        Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
        beta = 3.0
    else:
        T = rng.random((N, D))
        Y = T[rng.integers(0, N, K)] + 0.05 * rng.standard_normal((K, D))
        beta = 40.0 / max(1.0, D ** 0.5)
    Y = Y.astype(np.float32).astype(np.float64)
    T = T.astype(np.float32).astype(np.float64)
    temp = 1.6
    F, dY, dT, db = run_fe(pkg, Y, T, beta, temp)
    Fo, R, Dm = oracle_F(orc, Y, T, beta, temp)
    G = R.sum(1)
    dY_ref = -beta * (G[:, None] * Y - R @ T)
    dT_ref = -beta * (T - R.T @ Y)
    db_ref = N * D / (2 * beta) - 0.5 * (R * Dm).sum()
    print(f"N={N} K={K} D={D}: F {abs(F / Fo - 1):.1e} dY "
          f"{np.max(np.abs(dY - dY_ref)) / np.max(np.abs(dY_ref)):.1e} dT "
          f"{np.max(np.abs(dT - dT_ref)) / np.max(np.abs(dT_ref)):.1e} db {abs(db / db_ref - 1):.1e}")
    assert F == pytest.approx(Fo, rel=1e-5)
    assert np.max(np.abs(dY - dY_ref)) <= 1e-3 * np.max(np.abs(dY_ref))
    assert np.max(np.abs(dT - dT_ref)) <= 1e-3 * np.max(np.abs(dT_ref))
    assert db == pytest.approx(db_ref, rel=1e-3)


def test_gradient_against_central_differences(pkg, orc, problem):
    Y, T = problem
    beta, temp, h = 6.0, 1.7, 1e-6
    F, dY, dT, db = run_fe(pkg, Y, T, beta, temp)
    rng = np.random.default_rng(1)

    def fd(fun):
        return (fun(+h) - fun(-h)) / (2 * h)

    for _ in range(4):
        k, d = rng.integers(0, Y.shape[0]), rng.integers(0, Y.shape[1])

        def fy(e):
            Y2 = Y.copy()
            Y2[k, d] += e
            return oracle_F(orc, Y2, T, beta, temp)[0]

        g = fd(fy)
        assert dY[k, d] == pytest.approx(g, rel=2e-3, abs=2e-3 * np.max(np.abs(dY)))
        n = rng.integers(0, T.shape[0])

        def ft(e):
            T2 = T.copy()
            T2[n, d] += e
            return oracle_F(orc, Y, T2, beta, temp)[0]

        g = fd(ft)
        assert dT[n, d] == pytest.approx(g, rel=2e-3, abs=2e-3 * np.max(np.abs(dT)))
    gb = fd(lambda e: oracle_F(orc, Y, T, beta + e, temp)[0])
    assert db == pytest.approx(gb, rel=1e-3)


def test_projection_moves_points_onto_the_map(pkg, problem):
    ag = sub(pkg, "autograd")
    Y, T = problem
    Yt = torch.tensor(Y, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(8)
    Tn = torch.tensor(T[:512] + 0.3 * rng.standard_normal((512, T.shape[1])), dtype=torch.float32,
                      device="cuda")
    P = ag.project(Tn, Yt, 6.0, steps=20)

    def nearest(X):
        return torch.cdist(X.double(), Yt.double()).min(dim=1).values.mean().item()

    assert nearest(P) < 0.5 * nearest(Tn)
    assert torch.isfinite(P).all()


def test_differentiation_configuration_full_size(pkg):
    """The differentiation configuration at its full size: N = 65,536 points
    in D = 64 from a 16-component mixture (sd 0.2), K = 4096 (64 x 64).  The
    dense FP64 oracle is too slow here, so the FP32 forward/backward is
    checked against the library's FP64 form on the same inputs (itself
    parity-tested against the oracle): F = N nfree; dF/dY = -beta (G Y - R T);
    dF/dT = -beta (T - R^T Y) with R^T Y from dgtm_map in 8-column slices;
    dF/dbeta against FP64 central differences of N nfree.  Tolerances as for
    the small problem: 1e-5 on F, 1e-3 on the gradients."""
    ds = sub(pkg, "datasets")
    st = sub(pkg, "gtm_setup")
    N, D, K = 65536, 64, 4096
    T = ds.gaussian_mixture(N, D, 16, 0.2, seed=0).astype(np.float32).astype(np.float64)
    X, FI = st.setup_grid(2, K, 16, 1.0)
    rng = np.random.default_rng(0)
    Y = (T[rng.integers(0, N, K)] + 0.05 * rng.standard_normal((K, D))).astype(np.float32)
    Y = Y.astype(np.float64)
    beta, temp = 4.0, 2.0
    F, dY, dT, db = run_fe(pkg, Y, T, beta, temp)
    h = 1e-4 * beta
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        fp = N * c.estep(beta + h, 1, temp)[1]
        fm = N * c.estep(beta - h, 1, temp)[1]
        Fref = N * c.estep(beta, 1, temp)[1]
        RtY = np.concatenate([c.map(np.ascontiguousarray(Y[:, s:s + 8])) for s in range(0, D, 8)],
                             axis=1)
        c.mstep(want_W=False)
        G, RT = c.get_stats()
    assert F == pytest.approx(Fref, rel=1e-5)
    dY_ref = -beta * (G[:, None] * Y - RT)
    dT_ref = -beta * (T - RtY)
    assert np.max(np.abs(dY - dY_ref)) <= 1e-3 * np.max(np.abs(dY_ref))
    assert np.max(np.abs(dT - dT_ref)) <= 1e-3 * np.max(np.abs(dT_ref))
    assert db == pytest.approx((fp - fm) / (2 * h), rel=1e-3)
