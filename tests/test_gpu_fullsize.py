"""The headline problem size: N = 1,000,000 binary fingerprints, D = 166,
K = 8000 (20^3), M = 64 (4^3) + bias, width 2, at the start temperature.

The oracle's dense K x N matrices do not fit at this size, so parity rests on
(1) properties that hold at any size: every column of R sums to one, hence
sum_k G_k = N and sum_k RT_k = sum_n t_n; and (2) the FP64 form, which is
itself parity-tested against the oracle, run on the same input.  The split
form's R T is accumulated by the tensor pipe in FP32 over 4096 points at a
time (each MMA's FP32 sum is rounded down a little, so a longer run drifts
low) and then moved to FP32 slots; the identities bound what that loses.
Tolerances: identities 1e-12 (FP64 form) and 2e-5 (split form, relative);
split form against FP64 form as stated for the split form (qualities 1e-5,
G and RT 1e-4; R 1e-4 absolute on three 256-point blocks).  W and Y are not
compared: at width 2 with M = 64 the matrix
A is numerically singular, pivots are dropped, and the new centres depend on
rounding in any two implementations.  Beta is compared through the split
form's statistics with the FP64 form's new centres (beta = N D / (sum_k G_k
|y_k|^2 - 2 y_k . RT_k + sum_n |t_n|^2)): 2e-5.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def headline(pkg):
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    T = ds.fingerprints(1_000_000, 166, 20, seed=1)
    X, FI = st.setup_grid(3, 8000, 64, 2.0)
    rng = np.random.default_rng(1)
    Y = T[rng.integers(0, T.shape[0], 8000)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((8000, 166))
    temp = st.start_temp(T[:200_000], 0.99)
    return T, FI, Y, temp


R_COLS = (0, 499_776, 999_744)  # 256-point blocks at the start, middle and end


def one_step(pkg, form, T, FI, Y, beta, temp):
    with pkg.Context(T, FI, form) as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        R = [c.R_block(0, c.K, n0, 256) for n0 in R_COLS]
        b, _, Yn = c.mstep(want_W=False, want_Y=True)
        G, RT = c.get_stats()
    return dict(llh=llh, nfree=nfree, G=G, RT=RT, beta=b, Y=Yn, R=R)


def beta_from_stats(G, RT, Y, N, D, sum_t2):
    return N * D / ((G * (Y * Y).sum(axis=1)).sum() - 2.0 * (Y * RT).sum() + sum_t2)


@pytest.mark.parametrize("beta", [4.0, 30.0])
def test_headline_size_identities_and_forms(pkg, headline, beta):
    T, FI, Y, temp = headline
    N = T.shape[0]
    colsum_T = T.sum(axis=0)
    out = {f: one_step(pkg, f, T, FI, Y, beta, temp) for f in ("bf16x3", "fp64")}
    for form, tol in (("fp64", 1e-12), ("bf16x3", 2e-5)):
        o = out[form]
        eg = abs(o["G"].sum() - N) / N
        ert = rel(o["RT"].sum(axis=0), colsum_T)
        print(f"{form} beta={beta}: |sum G - N|/N = {eg:.2e}, sum_k RT vs sum_n t: {ert:.2e}")
        assert eg <= tol, form
        assert ert <= tol, form
    a, b = out["bf16x3"], out["fp64"]
    assert a["llh"] == pytest.approx(b["llh"], rel=1e-5)
    assert a["nfree"] == pytest.approx(b["nfree"], rel=1e-5)
    assert rel(a["G"], b["G"]) <= 1e-4
    assert rel(a["RT"], b["RT"]) <= 1e-4
    # responsibilities (the split form's stated 1e-4, absolute)
    for Ra, Rb in zip(a["R"], b["R"]):
        assert np.max(np.abs(Ra - Rb)) <= 1e-4
    D, t2 = T.shape[1], float((T * T).sum())
    b64 = beta_from_stats(b["G"], b["RT"], b["Y"], N, D, t2)
    assert b64 == pytest.approx(b["beta"], rel=1e-12)
    bsplit = beta_from_stats(a["G"], a["RT"], b["Y"], N, D, t2)
    print(f"beta from split statistics: {bsplit / b64 - 1:.2e}")
    assert bsplit == pytest.approx(b64, rel=2e-5)


def test_fingerprint_shape_fp64_and_fp32(pkg):
    """The FP64 / FP32 configuration at its own size: N = 100,000 binary
    vectors, D = 166, K = 8000, M = 64.  One EM step in each form: the FP64
    form's column-sum identities at 1e-12; the FP32 form against the FP64
    form at its stated tolerances (qualities 1e-5, G and RT 1e-4, beta and the
    new centres 1e-4).  Width 1 (cond(FI^T FI) = 1e10, no pivot dropped)
    keeps the new centres determined; at width 2 with M = 64 they are not."""
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    N = 100_000
    T = ds.fingerprints(N, 166, 20, seed=6)
    X, FI = st.setup_grid(3, 8000, 64, 1.0)
    rng = np.random.default_rng(6)
    Y = T[rng.integers(0, N, 8000)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((8000, 166))
    temp, beta = st.start_temp(T, 0.99), 4.0
    out = {}
    for form in ("fp64", "fp32"):
        with pkg.Context(T, FI, form) as c:
            c.set_Y(Y)
            llh, nfree = c.estep(beta, 1, temp)
            b, _, Yn = c.mstep(want_W=False, want_Y=True)
            G, RT = c.get_stats()
        out[form] = dict(llh=llh, nfree=nfree, beta=b, Y=Yn, G=G, RT=RT)
    f64, f32 = out["fp64"], out["fp32"]
    assert abs(f64["G"].sum() - N) / N <= 1e-12
    assert rel(f64["RT"].sum(axis=0), T.sum(axis=0)) <= 1e-12
    assert f32["llh"] == pytest.approx(f64["llh"], rel=1e-5)
    assert f32["nfree"] == pytest.approx(f64["nfree"], rel=1e-5)
    assert rel(f32["G"], f64["G"]) <= 1e-4
    assert rel(f32["RT"], f64["RT"]) <= 1e-4
    assert f32["beta"] == pytest.approx(f64["beta"], rel=1e-4)
    assert rel(f32["Y"], f64["Y"]) <= 1e-4
