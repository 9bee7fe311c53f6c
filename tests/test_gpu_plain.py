"""Parity of the plain forms (FP64, FP32) through the C ABI against the oracle.

Tolerances: FP64 form 1e-12 relative for the qualities, G and RT, and 1e-9
for beta, the centres Y = FI W and the free-energy / beta traces on a
well-conditioned basis (cond(FI^T FI) ~ 6e6).  On the reference's oil data
A = FI^T diag(G) FI has cond ~ 6e9, so two correct FP64 solvers (and two
summation orders of B) already differ in Y by ~cond x eps; there Y, beta and
the traces are compared at 1e-6.  W itself is compared through Y.  FP32 form:
1e-5 relative on the qualities, 1e-4 on beta / Y.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def oil(golden):
    return golden


def oracle_estep(orc, T, Y, beta, isDA, temp):
    Dm = orc.dist(Y, T)
    R, vgc, vgc2 = orc.resp(Dm, beta, isDA, temp)
    N, D = T.shape
    K = Y.shape[0]
    llh = orc.qual(N, K, D, beta, vgc, 0, temp)
    nfree = orc.qual(N, K, D, beta, vgc2, 1, temp) if isDA else -llh
    return R, llh, nfree


@pytest.mark.parametrize("temp,isDA", [(1.0, 1), (2.5, 1), (1.0, 0)])
def test_estep_qualities_fp64(pkg, orc, oil, temp, isDA):
    T, Y, FI, beta = oil["T"], oil["Y"], oil["FI"], oil["beta"][0]
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, isDA, temp)
    _, ollh, onfree = oracle_estep(orc, T, Y, beta, isDA, temp)
    assert llh == pytest.approx(ollh, rel=1e-12, abs=1e-13)
    assert nfree == pytest.approx(onfree, rel=1e-12, abs=1e-13)


def test_map_and_R_block_reproduce_reference_output(pkg, oil):
    T, Y, FI, beta = oil["T"], oil["Y"], oil["FI"], oil["beta"][0]
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        c.estep(beta, 1, 1.0)
        M = c.map(oil["X"])
        R = c.R_block(0, 125, 0, 1000)
    assert np.max(np.abs(M - oil["M"])) <= 1e-13
    assert np.max(np.abs(R[:, oil["R_cols"]] - oil["R_sub"])) <= 1e-13
    assert np.max(np.abs(R.sum(0) - 1.0)) <= 1e-13


def gmm_problem(pkg):
    ds = pkg_mod(pkg, "datasets")
    st = pkg_mod(pkg, "gtm_setup")
    T = ds.make("gmm_n1k", seed=0)
    X, FI, W, beta = st.random_init(T, 2, 400, 16, 1.0, seed=1)
    return T, FI, FI @ W, beta, st.start_temp(T, 0.99)


@pytest.mark.parametrize("solver", ["cholesky", "svd"])
@pytest.mark.parametrize("data", ["oil", "gmm"])
def test_mstep_fp64(pkg, orc, oil, solver, data):
    if data == "oil":
        T, Y, FI, beta = oil["T"], oil["Y"], oil["FI"], oil["beta"][0]
        temp, tol = 1.7, 1e-6
    else:
        T, FI, Y, beta, temp = gmm_problem(pkg)
        tol = 1e-9
    R, _, _ = oracle_estep(orc, T, Y, beta, 1, temp)
    G, A, B = orc.mstep_stats(R, FI, T)
    Wo = orc.solve_chol(A, B) if solver == "cholesky" else orc.solve2(A, B)
    Yo = orc.fiw(FI, Wo)
    bo, _, _ = orc.beta_update(Yo, T, R)
    with pkg.Context(T, FI, "fp64", solver=solver) as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        b, W, Yn = c.mstep(want_W=True, want_Y=True)
        Gg, RT = c.get_stats()
    assert rel(Gg, G) <= 1e-12
    assert rel(RT, R @ T) <= 1e-12
    assert rel(Yn, Yo) <= tol
    assert rel(FI @ W, Yo) <= tol
    assert b == pytest.approx(bo, rel=tol)


def test_trajectory_matches_oracle_fp64(pkg, orc, oil):
    T, FI = oil["T"], oil["FI"]
    kw = dict(isDA=1, alpha=0.9, eps=1e-6, maxloop=15)
    ref = orc.run(T, FI, oil["Y"], oil["beta"][0], 1.5, solver=1, **kw)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(oil["Y"])
        out = pkg.anneal(c, oil["beta"][0], 1.5, **kw)
        Yg = c.get_Y()
    # oil: cond(A) ~ 6e9 (see the module docstring)
    assert len(out.nfree_trace) == ref["n"]
    assert np.array_equal(out.temp_trace, ref["temp_trace"])
    assert rel(out.nfree_trace, ref["nfree_trace"]) <= 1e-6
    assert rel(out.llh_trace, ref["llh_trace"]) <= 1e-6
    assert rel(out.beta_trace, ref["beta_trace"]) <= 1e-6
    assert out.beta == pytest.approx(ref["beta"], rel=1e-6)
    assert rel(Yg, ref["Y"]) <= 1e-6


def test_gmm_config_trajectory_fp64(pkg, orc):
    T, FI, Y0, beta, temp0 = gmm_problem(pkg)
    kw = dict(isDA=1, alpha=0.95, eps=1e-6, maxloop=20)
    ref = orc.run(T, FI, Y0, beta, temp0, solver=1, **kw)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y0)
        out = pkg.anneal(c, beta, temp0, **kw)
    assert rel(out.nfree_trace, ref["nfree_trace"]) <= 1e-9
    assert rel(out.llh_trace, ref["llh_trace"]) <= 1e-9
    assert rel(out.beta_trace, ref["beta_trace"]) <= 1e-9


def pkg_mod(pkg, name):
    import importlib
    return importlib.import_module(pkg.__name__ + "." + name)


@pytest.mark.parametrize("N,D,K,M1", [(517, 37, 203, 10), (64, 16, 64, 5), (2, 3, 1, 1),
                                      (130, 256, 70, 7)])
def test_ragged_shapes_fp64(pkg, orc, N, D, K, M1):
    rng = np.random.default_rng(N + D + K)
    T = rng.random((N, D))
    Y = rng.random((K, D))
    FI = np.concatenate([rng.random((K, M1 - 1)), np.ones((K, 1))], axis=1)
    beta, temp = 3.0, 1.3
    R, ollh, onfree = oracle_estep(orc, T, Y, beta, 1, temp)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        assert llh == pytest.approx(ollh, rel=1e-12)
        assert nfree == pytest.approx(onfree, rel=1e-12)
        Rg = c.R_block(0, K, 0, N)
        assert np.max(np.abs(Rg - R)) <= 1e-13
        try:
            c.mstep()
        except pkg.DgtmError as e:  # a degenerate exact fit gives beta = inf
            assert e.code == 4
            return
        G, RT = c.get_stats()
    assert rel(G, R.sum(1)) <= 1e-12
    assert rel(RT, R @ T) <= 1e-12


def test_zero_column_fallback(pkg, orc):
    rng = np.random.default_rng(11)
    N, D, K = 40, 4, 9
    T = rng.random((N, D))
    T[7] = 60.0  # exp(-beta d / 2) underflows for every centre
    Y = rng.random((K, D))
    FI = np.concatenate([rng.random((K, 3)), np.ones((K, 1))], axis=1)
    beta = 2.0
    for isDA, temp in ((1, 3.0), (0, 1.0)):
        R, ollh, onfree = oracle_estep(orc, T, Y, beta, isDA, temp)
        with pkg.Context(T, FI, "fp64") as c:
            c.set_Y(Y)
            llh, nfree = c.estep(beta, isDA, temp)
            Rg = c.R_block(0, K, 0, N)
        assert np.allclose(Rg[:, 7], 1.0 / K, rtol=1e-15)
        assert np.max(np.abs(Rg - R)) <= 1e-13
        if isDA:
            assert llh == ollh == -np.inf
            assert nfree == pytest.approx(onfree, rel=1e-12)
        else:
            assert llh == pytest.approx(ollh, rel=1e-12)


def test_fp32_form(pkg, orc, oil):
    T, Y, FI, beta = oil["T"], oil["Y"], oil["FI"], oil["beta"][0]
    temp = 1.7
    R, ollh, onfree = oracle_estep(orc, T, Y, beta, 1, temp)
    G, A, B = orc.mstep_stats(R, FI, T)
    Yo = orc.fiw(FI, orc.solve_chol(A, B))
    bo, _, _ = orc.beta_update(Yo, T, R)
    with pkg.Context(T, FI, "fp32") as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        b, W, Yn = c.mstep(want_Y=True)
    assert llh == pytest.approx(ollh, rel=1e-5)
    assert nfree == pytest.approx(onfree, rel=1e-5)
    assert rel(Yn, Yo) <= 1e-4
    assert b == pytest.approx(bo, rel=1e-4)


def test_call_order_and_argument_errors(pkg, oil):
    T, Y, FI = oil["T"], oil["Y"], oil["FI"]
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        with pytest.raises(pkg.DgtmError) as e:
            c.mstep()
        assert e.value.code == 7
        with pytest.raises(pkg.DgtmError) as e:
            c.estep(-1.0, 1, 1.0)
        assert e.value.code == 1
        with pytest.raises(pkg.DgtmError) as e:
            c.R_block(0, 200, 0, 10)
        assert e.value.code == 7  # no E-step yet
        c.estep(oil["beta"][0], 1, 1.0)
        with pytest.raises(pkg.DgtmError) as e:
            c.R_block(0, 200, 0, 10)
        assert e.value.code == 1


def test_reruns_are_bit_identical(pkg, oil):
    T, Y, FI, beta = oil["T"], oil["Y"], oil["FI"], oil["beta"][0]
    outs = []
    for _ in range(2):
        with pkg.Context(T, FI, "fp64") as c:
            c.set_Y(Y)
            q = c.estep(beta, 1, 2.0)
            b, W, Yn = c.mstep(want_Y=True)
            outs.append((q, b, Yn))
    assert outs[0][0] == outs[1][0] and outs[0][1] == outs[1][1]
    assert np.array_equal(outs[0][2], outs[1][2])


@pytest.mark.parametrize("form,tol", [("fp64", 1e-8), ("bf16x3", 1e-4)])
def test_large_basis_cholesky(pkg, orc, form, tol):
    """M = 512 basis functions + bias (M1 = 513, the large split-precision
    configuration's basis) on a 9^3 latent grid: the Cholesky factor lives in
    global memory and the substitution uses 24 registers per lane.  Width
    factor 0.5 keeps A regular (cond 2.4e7, no pivot dropped), so two FP64
    solvers agree to cond x eps: 1e-8 on the new centres against the oracle's
    Cholesky solve of its own A and B; the split form to its stated 1e-4."""
    ds = pkg_mod(pkg, "datasets")
    st = pkg_mod(pkg, "gtm_setup")
    T = ds.gaussian_mixture(3000, 12, 6, 0.2, seed=5)
    X, FI = st.setup_grid(3, 729, 512, 0.5)
    rng = np.random.default_rng(5)
    Y = T[rng.integers(0, 3000, 729)] * 0.8 + 0.1
    beta, temp = 8.0, 1.5
    R, _, _ = oracle_estep(orc, T, Y, beta, 1, temp)
    G, A, B = orc.mstep_stats(R, FI, T)
    Yo = orc.fiw(FI, orc.solve_chol(A, B))
    with pkg.Context(T, FI, form) as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        b, W, Yn = c.mstep(want_Y=True)
    assert FI.shape[1] == 513
    assert rel(Yn, Yo) <= tol


def test_linear_schedule_trajectory_fp64(pkg, orc):
    """LINEAR cooling (temp -= delta after each temperature, -c linear,
    dagtm/dagtm.cxx:2168-2171) on the CPU-sized mixture: the trace matches the
    oracle's loop at 1e-9."""
    T, FI, Y0, beta, temp0 = gmm_problem(pkg)
    kw = dict(isDA=1, delta=0.1, eps=1e-6, maxloop=30)
    ref = orc.run(T, FI, Y0, beta, temp0, schedule=1, solver=1, **kw)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y0)
        out = pkg.anneal(c, beta, temp0, schedule="linear", **kw)
    assert len(out.nfree_trace) == ref["n"]
    assert np.array_equal(out.temp_trace, ref["temp_trace"])
    assert rel(out.nfree_trace, ref["nfree_trace"]) <= 1e-9
    assert rel(out.beta_trace, ref["beta_trace"]) <= 1e-9
