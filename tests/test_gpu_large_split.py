"""The large split-precision configuration: K = 32,768 (32^3) latent points,
M = 512 (8^3) basis functions + bias, binary data in D = 166 (50
prototypes), split-BF16 form; then gradient projection of held-out points of
the same generator onto the fixed map through the backward kernels.

* At full size (N = 4,000,000; 1,000,000 held-out points) the dense oracle
  cannot run, so the EM step is checked by size-independent identities
  (every column of R sums to one: sum_k G_k = N and sum_k RT_k = sum_n t_n,
  2e-5 as at the headline size) and the projection against an FP64 numpy
  restatement of the same iteration on 4096 sampled held-out points: with
  step 1/beta at temp 1, one gradient step is the fixed-point update
  t <- sum_k R_kn(t) y_k (1e-4, the split form's stated error).
* At the same K and M with N = 100,000 points the oracle holds every
  quantity (its dense K x N computation over point chunks): one EM step of
  both forms against it -- qualities, G, RT, R on sampled blocks, the new
  centres Y = FI W (A W = B solved by the oracle's Cholesky at M1 = 513) and
  beta.  FP64 form: 1e-12 / 1e-13 on the E-step quantities, 1e-8 on Y and
  beta (cond(A) ~ 1e7 bounds two FP64 solvers); split form 1e-5 on the
  qualities, 1e-4 on the rest.

Basis width factor 0.5: with the reference's 2, M = 512 basis functions on
a 32^3 grid are numerically dependent (cond(FI^T FI) = 3e19, 262 eigenvalues
below 1e-12 of the largest), W is not determined and the new centres reach
+-100 where the data lie in [0, 1].  At 0.5, cond(FI^T FI) = 6e5.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

D, K, M = 166, 32768, 512


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def mods(pkg):
    return (importlib.import_module(pkg.__name__ + ".datasets"),
            importlib.import_module(pkg.__name__ + ".gtm_setup"))


def fixed_point_fp64(P, Y, beta, steps):
    """t <- sum_k R_kn(t) y_k at temp 1 (FP64, numpy): the projection's update."""
    from oracle import oracle_blas as OB
    P = np.array(P, dtype=np.float64)
    for _ in range(steps):
        R = OB.resp_columns(P, Y, beta, 1, 1.0)  # K x n
        P = R.T @ Y
    return P


def test_large_split_configuration(pkg):
    ds, st = mods(pkg)
    ag = importlib.import_module(pkg.__name__ + ".autograd")
    N = 4_000_000
    T = ds.fingerprints(N, D, 50, seed=2)
    X, FI = st.setup_grid(3, K, M, 0.5)
    assert FI.shape == (K, M + 1)
    rng = np.random.default_rng(2)
    Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
    temp = st.start_temp(T[:200_000], 0.99)
    beta = 4.0
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        b, _, Yn = c.mstep(want_W=False, want_Y=True)
        G, RT = c.get_stats()
    assert np.isfinite(llh) and np.isfinite(nfree)
    assert abs(G.sum() - N) / N <= 2e-5
    colsum = T.sum(axis=0)
    assert np.max(np.abs(RT.sum(axis=0) - colsum)) <= 2e-5 * np.max(colsum)
    assert np.isfinite(b) and b > 0 and np.all(np.isfinite(Yn))
    assert -2.0 <= Yn.min() and Yn.max() <= 3.0  # binary data: a smooth fit near [0, 1]
    del T
    # held-out points of the same generator, projected onto the fixed map
    Th = ds.fingerprints(1_000_000, D, 50, seed=3)
    Tt = torch.tensor(Th, dtype=torch.float32, device="cuda")
    Y32 = Yn.astype(np.float32)
    Yt = torch.tensor(Y32, device="cuda")
    steps = 3
    P = ag.project(Tt, Yt, b, steps=steps)
    assert torch.isfinite(P).all()
    idx = np.sort(rng.choice(1_000_000, 4096, replace=False))
    Pg = P[torch.tensor(idx, device="cuda")].double().cpu().numpy()
    Pr = fixed_point_fp64(Th[idx].astype(np.float32), Y32.astype(np.float64), b, steps)
    err = rel(Pg, Pr)
    print(f"projection of 4096 sampled points, {steps} steps: {err:.2e}")
    assert err <= 1e-4
    moved = np.abs(Pr - Th[idx]).max()
    assert moved > 0.1  # the points did move


@pytest.fixture(scope="module")
def analogue(pkg):
    ds, st = mods(pkg)
    N = 100_000
    T = ds.fingerprints(N, D, 50, seed=4)
    X, FI = st.setup_grid(3, K, M, 0.5)
    rng = np.random.default_rng(4)
    Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
    return T, FI, Y, st.start_temp(T, 0.99), 4.0


@pytest.fixture(scope="module")
def analogue_oracle(orc, analogue):
    """The oracle's EM step over point chunks: E-step quantities, then A, B,
    the Cholesky solve (M1 = 513), Y = FI W and beta = N D / sum R o D with
    sum R o D = sum_k G_k |y_k|^2 - 2 y_k . RT_k + sum_n |t_n|^2."""
    from oracle import oracle_blas as OB
    T, FI, Y, temp, beta = analogue
    N = T.shape[0]
    llh, nfree, G, RT = OB.estep_stats(T, Y, beta, 1, temp, chunk=4096)
    cols = (0, N // 2, N - 256)
    R = [OB.resp_columns(T[c:c + 256], Y, beta, 1, temp) for c in cols]
    A = FI.T @ (G[:, None] * FI)
    B = FI.T @ RT
    Yn = orc.fiw(FI, orc.solve_chol(A, B))
    s = (G * (Yn * Yn).sum(1)).sum() - 2.0 * (Yn * RT).sum() + (T * T).sum()
    return dict(llh=llh, nfree=nfree, G=G, RT=RT, R=R, cols=cols, Y=Yn, beta=N * D / s)


@pytest.mark.parametrize("form", ["fp64", "bf16x3"])
def test_large_basis_analogue_against_oracle(pkg, analogue, analogue_oracle, form):
    T, FI, Y, temp, beta = analogue
    o = analogue_oracle
    with pkg.Context(T, FI, form) as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        R = [c.R_block(0, K, n0, 256) for n0 in o["cols"]]
        b, _, Yn = c.mstep(want_W=False, want_Y=True)
        G, RT = c.get_stats()
    tq, ts, tr, ty = ((1e-12, 1e-12, 1e-13, 1e-8) if form == "fp64"
                      else (1e-5, 1e-4, 1e-4, 1e-4))
    er = max(float(np.max(np.abs(a - b_))) for a, b_ in zip(R, o["R"]))
    print(f"{form}: llh {abs(llh / o['llh'] - 1):.1e} nfree {abs(nfree / o['nfree'] - 1):.1e} "
          f"G {rel(G, o['G']):.1e} RT {rel(RT, o['RT']):.1e} R {er:.1e} "
          f"Y {rel(Yn, o['Y']):.1e} beta {abs(b / o['beta'] - 1):.1e}")
    assert llh == pytest.approx(o["llh"], rel=tq)
    assert nfree == pytest.approx(o["nfree"], rel=tq)
    assert rel(G, o["G"]) <= ts
    assert rel(RT, o["RT"]) <= ts
    assert er <= tr
    assert rel(Yn, o["Y"]) <= ty
    assert b == pytest.approx(o["beta"], rel=ty)
