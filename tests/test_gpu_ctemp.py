"""AUTO cooling: dgtm_next_ctemp against the oracle's restatement of
dagtm_mpi_next_ctemp (comm/mpicomm.c:562-674).

The oracle builds each centre's 2D x 2D H and takes all its eigenvalues, as
the reference does; the library takes the two D x D diagonal blocks of H
after the orthogonal block transform.  The same responsibilities go into both
(the FP64 form reproduces the oracle's R to ~1e-12), so the critical
temperatures agree to FP64 eigenvalue accuracy: 1e-9 relative.  The FP32 and
split-BF16 forms form the scatter matrices and find the eigenvalue in FP32
(Householder reduction to tridiagonal form, Sturm bisection), and the split
form's R carries its stated error: 1e-4 relative.  On 0/1 data
the split form forms the scatter as a tensor-core GEMM over pair features
(R and R^2 against u_n = (t_i t_j, t_i, 1)); DGTM_CTEMP_PAIRS=0 selects the
CUDA-core scatter instead, and the two agree centre by centre to 1e-4.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def sub(pkg, name):
    return importlib.import_module(pkg.__name__ + "." + name)


def problem(pkg, kind, N, D, K, seed=5):
    ds = sub(pkg, "datasets")
    st = sub(pkg, "gtm_setup")
    if kind == "binary":
        T = ds.fingerprints(N, D, 8, seed=seed)
    else:
        T = ds.gaussian_mixture(N, D, 5, 0.2, seed=seed)
    L = 2
    X, FI = st.setup_grid(L, K, 4, 1.0)
    rng = np.random.default_rng(seed)
    Y = T[rng.integers(0, N, K)] * 0.6 + 0.2 + 0.05 * rng.standard_normal((K, D))
    return T, FI, Y


def oracle_ctemp(orc, T, Y, beta, temp, eps, gg=None):
    R, _, _ = orc.resp(orc.dist(Y, T), beta, 1, temp)
    if gg is None:
        gg = R.sum(axis=1)
    return orc.next_ctemp(T, Y, R, gg, temp, beta, eps), R


@pytest.mark.parametrize("kind,N,D,K,form,tol", [
    ("binary", 600, 20, 64, "fp64", 1e-9),
    ("real", 500, 13, 49, "fp64", 1e-9),
    ("binary", 400, 166, 9, "fp64", 1e-9),   # D x D block just inside shared memory
    ("real", 300, 170, 9, "fp64", 1e-9),     # D x D block beyond shared memory
    ("binary", 600, 20, 64, "bf16x3", 1e-4),
    ("binary", 400, 166, 9, "bf16x3", 1e-4),  # FP32 eigenvalues, 512 threads
    ("real", 500, 13, 49, "fp32", 1e-4),
    ("real", 300, 250, 4, "fp32", 1e-4),      # FP32 block beyond shared memory
    ("real", 300, 1, 9, "fp64", 1e-9),        # 1 x 1 blocks: no reduction step
    ("real", 300, 2, 9, "fp64", 1e-9),        # 2 x 2: the last pair only
    ("real", 300, 3, 9, "fp32", 1e-4),        # one reflection
])
def test_next_ctemp_matches_oracle(pkg, orc, kind, N, D, K, form, tol):
    T, FI, Y = problem(pkg, kind, N, D, K)
    beta, temp, eps = 30.0 / D, 4.0, 1e-6
    ref, R = oracle_ctemp(orc, T, Y, beta, temp, eps)
    with pkg.Context(T, FI, form) as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        got = c.next_ctemp(temp, beta, eps)
        got_w = c.next_ctemp(temp, beta, eps, gg=R.sum(axis=1))
    assert np.isfinite(ref) and ref < temp
    assert got == pytest.approx(ref, rel=tol)
    assert got_w == pytest.approx(ref, rel=tol)


@pytest.mark.parametrize("form,tol", [("fp64", 1e-9), ("bf16x3", 1e-4)])
def test_next_ctemp_in_chunks_and_batches(pkg, orc, monkeypatch, form, tol):
    """Points in chunks of 96 (5 chunks, the last one ragged) and centres in
    batches of 2 (1 MB of scratch at D = 166): the running sums over the
    chunks and the batch offsets give the single-pass result."""
    T, FI, Y = problem(pkg, "binary", 450, 166, 9)
    beta, temp, eps = 30.0 / 166, 4.0, 1e-6
    ref, R = oracle_ctemp(orc, T, Y, beta, temp, eps)
    with pkg.Context(T, FI, form) as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        whole, whole_k = c.next_ctemp(temp, beta, eps, per_centre=True)
        monkeypatch.setenv("DGTM_CTEMP_CHUNK", "96")
        monkeypatch.setenv("DGTM_CTEMP_SCRATCH_MB", "1")
        parts, parts_k = c.next_ctemp(temp, beta, eps, per_centre=True)
    assert whole == pytest.approx(ref, rel=tol)
    assert parts == pytest.approx(ref, rel=tol)
    np.testing.assert_allclose(parts_k, whole_k, rtol=1e-12 if form == "fp64" else 1e-4)


@pytest.fixture(scope="module")
def pairs_case(pkg, orc):
    """9000 binary points in D = 166, K = 16, and the oracle's answer (its
    2D x 2D eigenproblems are the expensive part: computed once)."""
    T, FI, Y = problem(pkg, "binary", 9000, 166, 16, seed=9)
    beta, temp, eps = 30.0 / 166, 4.0, 1e-6
    ref, _ = oracle_ctemp(orc, T, Y, beta, temp, eps)
    return T, FI, Y, beta, temp, eps, ref


@pytest.mark.parametrize("gemm_mb", ["8192", "64"])
def test_pair_feature_gemm_chunks_and_segments(pkg, monkeypatch, pairs_case, gemm_mb):
    """The pair-feature GEMM over 9000 binary points: with the default budget
    the points form one chunk of 9216 (three 4096-point accumulation segments,
    the last ragged); with 64 MB three chunks of 4096.  Against the oracle
    (1e-4) and, centre by centre, against the CUDA-core scatter of the same
    form (1e-4)."""
    T, FI, Y, beta, temp, eps, ref = pairs_case
    monkeypatch.setenv("DGTM_CTEMP_GEMM_MB", gemm_mb)
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        got, got_k = c.next_ctemp(temp, beta, eps, per_centre=True)
        monkeypatch.setenv("DGTM_CTEMP_PAIRS", "0")
        simt, simt_k = c.next_ctemp(temp, beta, eps, per_centre=True)
    print(f"pairs {got / ref - 1:.2e}, cuda cores {simt / ref - 1:.2e}, per centre "
          f"{np.max(np.abs(got_k / simt_k - 1)):.2e}")
    assert got == pytest.approx(ref, rel=1e-4)
    assert simt == pytest.approx(ref, rel=1e-4)
    np.testing.assert_allclose(got_k, simt_k, rtol=1e-4)


@pytest.mark.parametrize("far,finite", [(6.0, True), (8.0, False)])
def test_pair_feature_gemm_far_centres(pkg, orc, monkeypatch, far, finite):
    """A centre far from every point.  At 6 (beta d / 2 ~ 470) its
    responsibilities (~1e-52) are below the split form's FP32 planes, so the
    pair-feature GEMM sees a zero row: it is redone from FP64 responsibilities,
    scaled by a power of two into FP32's range, and its own critical
    temperature matches the FP64 one (the CUDA-core path, which does not scale,
    is compared on the other centres only).  At 8 (beta d / 2 ~ 865) the reference's
    exp(-beta d / 2) underflows, its responsibilities are exactly 0 and
    comm/mpicomm.c:574-577 makes the critical temperature HUGE_VAL: so here."""
    T, FI, Y = problem(pkg, "binary", 3000, 166, 16, seed=13)
    Y[9] = far
    beta, temp, eps = 30.0 / 166, 4.0, 1e-6
    ref, R = oracle_ctemp(orc, T, Y, beta, temp, eps)
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        got, got_k = c.next_ctemp(temp, beta, eps, per_centre=True)
        monkeypatch.setenv("DGTM_CTEMP_PAIRS", "0")
        simt, simt_k = c.next_ctemp(temp, beta, eps, per_centre=True)
    keep = np.arange(16) != 9
    if finite:
        assert 0.0 < R[9].sum() < 1e-40
        assert np.all(np.isfinite(got_k)) and np.isfinite(got)
        np.testing.assert_allclose(got_k[keep], simt_k[keep], rtol=1e-4)
        assert got == pytest.approx(ref, rel=1e-4)
        # the far centre's own critical temperature, from its FP64 responsibilities
        # (far below FP32's normal range): the spectrum of H is that of 2 S1 and
        # of 2 (S1 - S2); eigenvalues at or above (temp - eps) gg 2 / beta count
        # as 0; ctemp = beta / (2 gg) times the largest
        X = T - Y[9]
        S1 = (X * R[9][:, None]).T @ X
        S2 = (X * (R[9] ** 2)[:, None]).T @ X
        gk = R[9].sum()
        lam = np.concatenate([np.linalg.eigvalsh(2 * S1), np.linalg.eigvalsh(2 * (S1 - S2))])
        lam[lam >= (temp - eps) * gk * 2 / beta] = 0.0
        assert got_k[9] == pytest.approx(beta / (2 * gk) * lam.max(), rel=1e-4)
    else:
        assert R[9].sum() == 0.0 and ref == np.inf
        assert got == simt == np.inf and got_k[9] == simt_k[9] == np.inf
        np.testing.assert_allclose(got_k[keep], simt_k[keep], rtol=1e-4)


def test_next_ctemp_oil(pkg, orc, golden):
    T, Y, FI, beta = golden["T"], golden["Y"], golden["FI"], golden["beta"][0]
    temp, eps = 2.5, 1e-6
    R, _, _ = orc.resp(orc.dist(Y, T), beta, 1, temp)
    gg = R.sum(axis=1) * 1.01  # weights other than the current row sums
    ref = orc.next_ctemp(T, Y, R, gg, temp, beta, eps)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        got = c.next_ctemp(temp, beta, eps, gg=gg)
    assert got == pytest.approx(ref, rel=1e-9)


def test_zero_weight_gives_huge(pkg):
    T, FI, Y = problem(pkg, "binary", 256, 16, 25)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        c.estep(2.0, 1, 3.0)
        gg = np.ones(25)
        gg[3] = 0.0
        assert c.next_ctemp(3.0, 2.0, 1e-6, gg=gg) == np.inf


def test_anneal_auto_cools_monotonically(pkg, orc):
    T, FI, Y = problem(pkg, "real", 800, 8, 49)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y)
        run = pkg.anneal(c, 6.0, 3.0, schedule="auto", alpha=0.9, eps=1e-5, maxloop=80)
    temps = []
    for t in run.temp_trace:
        if not temps or t != temps[-1]:
            temps.append(t)
    assert temps[0] == 3.0 and len(temps) >= 2
    assert all(a > b for a, b in zip(temps, temps[1:]))
