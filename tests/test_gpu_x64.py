"""The exact-slice FP64 form (estep_x64.cu) on 0/1 data, against the oracle
(comm/comm.c:560-629 distances, comm/mpicomm.c:316-500 responsibilities and
qualities, the M-step of comm/comm.c:1299-1348) and against the CUDA-core
FP64 form of the same library (DGTM_X64=0).

Distances are exact integers from the tensor cores (fixed-point digit slices
of the centres on a 2^-F grid, 2^-52 of the largest centre value or |y|^2/2m),
the exponentials double-float (~2^-47), the per-point sums 128-bit fixed point
at 2^-63 and the responsibilities of R T 2^-48 fixed point.  Tolerances are the FP64 form's: 1e-12 on the qualities, G and R T,
1e-13 absolute on R, 1e-9 on beta and the new centres.

Shapes cover the three panel counts (D = 20, 100, 166, 189: 1, 2 and 3
panels of 64, and 3 columns of -|y|^2/2 pieces at D = 189), ragged N and K,
several 16384-point units and 256-point segments per centre block, both
temperatures of the E-step, the zero-column fallback and the reference's
underflow of exp(-beta d / 2).
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def problem(N, D, K, M=8, seed=0, density=0.2):
    rng = np.random.default_rng(seed)
    # 0/1 data: a few prototypes with 10 % of their bits flipped
    proto = (rng.random((12, D)) < density).astype(np.float64)
    T = proto[rng.integers(0, 12, N)]
    flip = rng.random((N, D)) < 0.1
    T = np.where(flip, 1.0 - T, T)
    FI = np.concatenate([rng.standard_normal((K, M)), np.ones((K, 1))], axis=1)
    Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
    return T, FI, Y


def oracle_step(orc, T, Y, FI, beta, isDA, temp):
    Dm = orc.dist(Y, T)
    R, vgc, vgc2 = orc.resp(Dm, beta, isDA, temp)
    N, D = T.shape
    K = Y.shape[0]
    llh = orc.qual(N, K, D, beta, vgc, 0, temp)
    nfree = orc.qual(N, K, D, beta, vgc2, 1, temp) if isDA else -llh
    G, A, B = orc.mstep_stats(R, FI, T)
    Yn = orc.fiw(FI, orc.solve_chol(A, B))
    bn, _, _ = orc.beta_update(Yn, T, R)
    return dict(R=R, llh=llh, nfree=nfree, G=G, RT=R @ T, Y=Yn, beta=bn)


def run_step(pkg, T, FI, Y, beta, isDA, temp):
    with pkg.Context(T, FI, "fp64") as c:
        path = c.path
        c.set_Y(Y)
        llh, nfree = c.estep(beta, isDA, temp)
        R = c.R_block(0, Y.shape[0], 0, T.shape[0])
        b, _, Yn = c.mstep(want_W=False, want_Y=True)
        G, RT = c.get_stats()
    return dict(path=path, R=R, llh=llh, nfree=nfree, G=G, RT=RT, Y=Yn, beta=b)


def test_path_selection(pkg, monkeypatch):
    T, FI, Y = problem(600, 30, 40)
    with pkg.Context(T, FI, "fp64") as c:
        assert c.path == "exact_slices"
    with pkg.Context(T + 0.5, FI, "fp64") as c:  # not 0/1
        assert c.path == "cuda_cores"
    with pkg.Context(T, FI, "bf16x3") as c:
        assert c.path == "split_bf16"
    with pkg.Context(T, FI, "fp32") as c:
        assert c.path == "cuda_cores"
    monkeypatch.setenv("DGTM_X64", "0")
    with pkg.Context(T, FI, "fp64") as c:
        assert c.path == "cuda_cores"


@pytest.mark.parametrize("N,D,K,isDA,temp", [
    (3000, 166, 300, 1, 2.5),   # three panels, two temperatures
    (2999, 20, 203, 0, 1.0),    # one panel, ragged N and K, no annealing
    (4100, 100, 77, 1, 1.0),    # two panels, isDA at temperature 1
    (1000, 189, 40, 1, 3.0),    # three pad columns for -|y|^2/2
])
def test_em_step_against_oracle_and_cuda_cores(pkg, orc, monkeypatch, N, D, K, isDA, temp):
    T, FI, Y = problem(N, D, K, seed=N + D)
    beta = 30.0 / D
    o = oracle_step(orc, T, Y, FI, beta, isDA, temp)
    g = run_step(pkg, T, FI, Y, beta, isDA, temp)
    monkeypatch.setenv("DGTM_X64", "0")
    s = run_step(pkg, T, FI, Y, beta, isDA, temp)
    assert g["path"] == "exact_slices" and s["path"] == "cuda_cores"
    print(f"N={N} D={D} K={K}: llh {abs(g['llh'] / o['llh'] - 1):.1e} "
          f"nfree {abs(g['nfree'] / o['nfree'] - 1):.1e} R {np.max(np.abs(g['R'] - o['R'])):.1e} "
          f"G {rel(g['G'], o['G']):.1e} RT {rel(g['RT'], o['RT']):.1e} "
          f"Y {rel(g['Y'], o['Y']):.1e} beta {abs(g['beta'] / o['beta'] - 1):.1e}")
    for ref, tq in ((o, 1e-12), (s, 1e-12)):
        assert g["llh"] == pytest.approx(ref["llh"], rel=tq)
        assert g["nfree"] == pytest.approx(ref["nfree"], rel=tq)
        assert np.max(np.abs(g["R"] - ref["R"])) <= 1e-13
        assert rel(g["G"], ref["G"]) <= 1e-12
        assert rel(g["RT"], ref["RT"]) <= 1e-12
        assert rel(g["Y"], ref["Y"]) <= 1e-9
        assert g["beta"] == pytest.approx(ref["beta"], rel=1e-9)
    # every column of R sums to one
    assert np.max(np.abs(g["R"].sum(0) - 1.0)) <= 1e-13


def test_units_segments_and_padding_centres(pkg, orc):
    """40000 points: per centre block two full 16384-point units and a ragged
    one, each of many 256-point segments; K = 50 leaves 78 padding centres
    in the last 128-centre tile and 2 in the last 16-centre block."""
    N, D, K = 40000, 166, 50
    T, FI, Y = problem(N, D, K, seed=3)
    beta, temp = 30.0 / D, 1.5
    o = oracle_step(orc, T, Y, FI, beta, 1, temp)
    g = run_step(pkg, T, FI, Y, beta, 1, temp)
    print(f"G {rel(g['G'], o['G']):.1e} RT {rel(g['RT'], o['RT']):.1e} "
          f"R {np.max(np.abs(g['R'] - o['R'])):.1e}")
    assert g["path"] == "exact_slices"
    assert g["llh"] == pytest.approx(o["llh"], rel=1e-12)
    assert g["nfree"] == pytest.approx(o["nfree"], rel=1e-12)
    assert np.max(np.abs(g["R"] - o["R"])) <= 1e-13
    assert rel(g["G"], o["G"]) <= 1e-12
    assert rel(g["RT"], o["RT"]) <= 1e-12
    assert abs(g["G"].sum() - N) <= 1e-9 * N


def test_zero_column_fallback_exact_slices(pkg, orc):
    """A point whose every exp(-beta d/2) underflows (comm/mpicomm.c:382-389):
    its responsibilities are 1/K, as in the oracle."""
    N, D, K = 500, 166, 24
    T, FI, Y = problem(N, D, K, seed=5, density=0.05)
    T[7] = 1.0                          # all ones, far from every centre
    Y = 0.02 * np.abs(np.random.default_rng(5).standard_normal((K, D)))
    beta = 10.0                         # beta/2 d > 745 for point 7 only
    for isDA, temp in ((1, 3.0), (0, 1.0)):
        o = oracle_step(orc, T, Y, FI, beta, isDA, temp)
        with pkg.Context(T, FI, "fp64") as c:
            assert c.path == "exact_slices"
            c.set_Y(Y)
            llh, nfree = c.estep(beta, isDA, temp)
            R = c.R_block(0, K, 0, N)
            c.mstep()
            G, RT = c.get_stats()
        assert np.allclose(R[:, 7], 1.0 / K, rtol=1e-15)
        assert np.max(np.abs(R - o["R"])) <= 1e-13
        assert rel(G, o["G"]) <= 1e-12
        assert rel(RT, o["RT"]) <= 1e-12
        if isDA:
            assert llh == o["llh"] == -np.inf
            assert nfree == pytest.approx(o["nfree"], rel=1e-12)
        else:
            assert llh == pytest.approx(o["llh"], rel=1e-12)


@pytest.mark.parametrize("x64", ["1", "0"])
def test_reference_underflow_rule(pkg, orc, monkeypatch, x64):
    """The reference forms exp(-beta d / 2) before tempering
    (comm/mpicomm.c:326-336): a responsibility whose beta d / 2 exceeds 745.13
    is exactly 0 there.  A centre that far from every point has R = 0, G = 0,
    and a critical temperature of HUGE_VAL; both FP64 paths follow."""
    monkeypatch.setenv("DGTM_X64", x64)
    N, D, K = 2000, 166, 24
    T, FI, Y = problem(N, D, K, seed=7)
    Y[5] = 8.0
    beta, temp = 30.0 / D, 4.0
    o = oracle_step(orc, T, Y, FI, beta, 1, temp)
    assert o["R"][5].max() == 0.0
    with pkg.Context(T, FI, "fp64") as c:
        assert c.path == ("exact_slices" if x64 == "1" else "cuda_cores")
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        R = c.R_block(0, K, 0, N)
        ct = c.next_ctemp(temp, beta, 1e-6)
        c.mstep()
        G, RT = c.get_stats()
    assert np.all(R[5] == 0.0) and G[5] == 0.0 and np.all(RT[5] == 0.0)
    assert np.max(np.abs(R - o["R"])) <= 1e-13
    assert rel(G, o["G"]) <= 1e-12 and rel(RT, o["RT"]) <= 1e-12
    assert ct == orc.next_ctemp(T, Y, o["R"], o["G"], temp, beta, 1e-6) == np.inf
