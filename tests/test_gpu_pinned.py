"""Each measurement configuration checked against the oracle at its own size.

* CPU-sized plain FP64 (N 1000, D 12, K 400, M 16, width 1, EXP alpha 0.99):
  a 100-iteration trace against the oracle's loop with the reference's SVD
  solve (``dagtm_solve2``, comm/comm.c:1299-1348) and with Cholesky: the
  nfree, llh and beta traces 1e-9; the final centres 1e-8 (the oracle's own
  SVD and Cholesky runs end 1.0e-9 apart in Y).
* Fingerprint shape (N 100,000, D 166, K 8000, M 64, width 1): one EM
  iteration of the FP64 and FP32 forms against the dense C oracle (6.4 GB per
  K x N matrix): qualities, G and RT 1e-12 and beta 1e-9 (FP64); 1e-5 and
  1e-4 (FP32).  A = FI^T diag(G) FI has cond 1.1e10 here: a 1e-15 relative
  change of G moves the solved centres by 1.4e-7 (measured with the oracle),
  so no two FP64 implementations agree on Y beyond that.  The solve is
  therefore checked by its backward error against the oracle's own A and B
  (FP64 form: 1e-10 of B), Y at 1e-6 (FP64) / 1e-4 (FP32).  Then 200 iterations of the
  FP32 form's trace against the FP64 form's (1e-4).
* The headline shape (N 1,000,000, D 166, K 8000, M 64, width 2): both forms
  against the oracle over all points (llh, nfree, G, RT summed over point
  chunks of the reference's dense computation) and on three 256-point blocks
  of R: FP64 1e-12 (R 1e-13 absolute), split form 1e-5 on the qualities,
  1e-4 on G, RT and R.

The oracle runs on the host cores (OpenMP C for the dense configurations,
numpy/BLAS over point chunks at N = 1M).  Reference path:
dagtm/dagtm.cxx:1531-1795.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def mods(pkg):
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    return ds, st


# ---------------------------------------------------------------------------
# CPU-sized configuration: 100 iterations, both solvers
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("solver,orc_solver", [("svd", 0), ("cholesky", 1)])
def test_cpu_sized_config_100_iterations(pkg, orc, solver, orc_solver):
    ds, st = mods(pkg)
    T = ds.make("gmm_n1k", seed=0)
    X, FI, W, beta = st.random_init(T, 2, 400, 16, 1.0, seed=0)
    Y0 = FI @ W
    temp0 = st.start_temp(T, 0.99)
    kw = dict(isDA=1, alpha=0.99, eps=1e-6, maxloop=100)
    ref = orc.run(T, FI, Y0, beta, temp0, solver=orc_solver, **kw)
    with pkg.Context(T, FI, "fp64", solver=solver) as c:
        c.set_Y(Y0)
        out = pkg.anneal(c, beta, temp0, **kw)
        Yg = c.get_Y()
    assert ref["n"] == 100 and len(out.nfree_trace) == 100
    assert np.array_equal(out.temp_trace, ref["temp_trace"])
    assert rel(out.nfree_trace, ref["nfree_trace"]) <= 1e-9
    assert rel(out.llh_trace, ref["llh_trace"]) <= 1e-9
    assert rel(out.beta_trace, ref["beta_trace"]) <= 1e-9
    assert out.beta == pytest.approx(ref["beta"], rel=1e-9)
    assert rel(Yg, ref["Y"]) <= 1e-8


# ---------------------------------------------------------------------------
# fingerprint shape: N = 100,000, K = 8000, M = 64
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def fingerprint(pkg):
    ds, st = mods(pkg)
    N = 100_000
    T = ds.fingerprints(N, 166, 20, seed=6)
    X, FI = st.setup_grid(3, 8000, 64, 1.0)  # width 1: A regular, no pivot dropped
    rng = np.random.default_rng(6)
    Y = T[rng.integers(0, N, 8000)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((8000, 166))
    return T, FI, Y, st.start_temp(T, 0.99), 4.0


@pytest.fixture(scope="module")
def fingerprint_oracle(orc, fingerprint):
    """One EM iteration of the dense C oracle (reference semantics, Cholesky
    solve as the GPU's default)."""
    T, FI, Y, temp, beta = fingerprint
    N, D = T.shape
    K = Y.shape[0]
    Dm = orc.dist(Y, T)
    R, vgc, vgc2 = orc.resp(Dm, beta, 1, temp)
    del Dm
    llh = orc.qual(N, K, D, beta, vgc, 0, temp)
    nfree = orc.qual(N, K, D, beta, vgc2, 1, temp)
    G, A, B = orc.mstep_stats(R, FI, T)
    RT = R @ T
    Yn = orc.fiw(FI, orc.solve_chol(A, B))
    bn, _, _ = orc.beta_update(Yn, T, R)
    return dict(llh=llh, nfree=nfree, G=G, RT=RT, Y=Yn, beta=bn, A=A, B=B)


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_fingerprint_shape_against_oracle(pkg, fingerprint, fingerprint_oracle, form):
    T, FI, Y, temp, beta = fingerprint
    o = fingerprint_oracle
    with pkg.Context(T, FI, form) as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        b, W, Yn = c.mstep(want_W=True, want_Y=True)
        G, RT = c.get_stats()
    # (the backward error is an FP64-solve property: the FP32 form's A and B
    # carry its own rounding, so only its Y is compared)
    tq, ts, tb, ty, tw = ((1e-12, 1e-12, 1e-9, 1e-6, 1e-10) if form == "fp64"
                          else (1e-5, 1e-4, 1e-4, 1e-4, np.inf))
    bwd = float(np.max(np.abs(o["A"] @ W - o["B"])) / np.max(np.abs(o["B"])))
    print(f"{form}: llh {abs(llh / o['llh'] - 1):.1e} nfree {abs(nfree / o['nfree'] - 1):.1e} "
          f"G {rel(G, o['G']):.1e} RT {rel(RT, o['RT']):.1e} Y {rel(Yn, o['Y']):.1e} "
          f"beta {abs(b / o['beta'] - 1):.1e} backward {bwd:.1e}")
    assert llh == pytest.approx(o["llh"], rel=tq)
    assert nfree == pytest.approx(o["nfree"], rel=tq)
    assert rel(G, o["G"]) <= ts
    assert rel(RT, o["RT"]) <= ts
    assert b == pytest.approx(o["beta"], rel=tb)
    assert bwd <= tw
    assert rel(Yn, o["Y"]) <= ty


def test_fingerprint_shape_200_iterations_fp32_against_fp64(pkg, fingerprint):
    """200 EM iterations (EXP cooling from the start temperature, capped by
    maxloop) of the FP32 form against the FP64 form: the traces of nfree,
    llh and beta within the FP32 form's stated 1e-4."""
    T, FI, Y, temp, beta = fingerprint
    runs = {}
    for form in ("fp64", "fp32"):
        with pkg.Context(T, FI, form) as c:
            c.set_Y(Y)
            runs[form] = pkg.anneal(c, beta, temp, isDA=1, alpha=0.99, eps=1e-6, maxloop=200)
    a, b = runs["fp32"], runs["fp64"]
    assert len(b.nfree_trace) == 200
    n = min(len(a.nfree_trace), len(b.nfree_trace))
    assert n == 200
    assert rel(a.nfree_trace[:n], b.nfree_trace[:n]) <= 1e-4
    assert rel(a.llh_trace[:n], b.llh_trace[:n]) <= 1e-4
    assert rel(a.beta_trace[:n], b.beta_trace[:n]) <= 1e-4


# ---------------------------------------------------------------------------
# the headline shape: N = 1,000,000
# ---------------------------------------------------------------------------
R_COLS = (0, 499_776, 999_744)


@pytest.fixture(scope="module")
def headline(pkg):
    ds, st = mods(pkg)
    T = ds.fingerprints(1_000_000, 166, 20, seed=1)
    X, FI = st.setup_grid(3, 8000, 64, 2.0)
    rng = np.random.default_rng(1)
    Y = T[rng.integers(0, T.shape[0], 8000)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((8000, 166))
    return T, FI, Y, st.start_temp(T[:200_000], 0.99)


@pytest.mark.parametrize("beta", [4.0, 30.0])
def test_headline_shape_against_oracle(pkg, headline, beta):
    from oracle import oracle_blas as OB
    T, FI, Y, temp = headline
    llh_o, nfree_o, G_o, RT_o = OB.estep_stats(T, Y, beta, 1, temp, chunk=16384)
    R_o = [OB.resp_columns(T[c:c + 256], Y, beta, 1, temp) for c in R_COLS]
    tol = {"fp64": (1e-12, 1e-12, 1e-13), "bf16x3": (1e-5, 1e-4, 1e-4)}
    for form in ("fp64", "bf16x3"):
        with pkg.Context(T, FI, form) as c:
            c.set_Y(Y)
            llh, nfree = c.estep(beta, 1, temp)
            R = [c.R_block(0, c.K, n0, 256) for n0 in R_COLS]
            c.mstep(want_W=False)
            G, RT = c.get_stats()
        tq, ts, tr = tol[form]
        er = max(float(np.max(np.abs(a - b))) for a, b in zip(R, R_o))
        print(f"{form} beta={beta}: llh {abs(llh / llh_o - 1):.1e} nfree "
              f"{abs(nfree / nfree_o - 1):.1e} G {rel(G, G_o):.1e} RT {rel(RT, RT_o):.1e} "
              f"R {er:.1e}")
        assert llh == pytest.approx(llh_o, rel=tq), form
        assert nfree == pytest.approx(nfree_o, rel=tq), form
        assert rel(G, G_o) <= ts, form
        assert rel(RT, RT_o) <= ts, form
        assert er <= tr, form
