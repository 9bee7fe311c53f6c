"""The host temperature loop (``anneal``) on the CPU.

``anneal`` reaches its context only through estep / mstep / get_stats /
next_ctemp / get_W / set_basis.  Here those calls are served by the oracle's
FP64 primitives (dense K x N, the reference's semantics), so the loop's
control flow -- the |diff| < eps test before the M-step, the 50-wide moving
average, maxloop, the EXP / LINEAR / AUTO schedules and the hierarchical
expansion -- is checked against the oracle's own loops without a GPU:
``orc.run`` (the C restatement of dagtm/dagtm.cxx:1508-1795 for EXP and
LINEAR) and ``orc.run_hda`` (dagtm/dagtm.cxx:1912-2124).  Both sides call the
same primitives in the same order, so the traces agree to rounding (1e-12).
"""
import importlib

import numpy as np
import pytest

from oracle_ctx import OracleCtx


def traces(run):
    return (np.array(run.temp_trace), np.array(run.nfree_trace), np.array(run.llh_trace),
            np.array(run.beta_trace))


@pytest.mark.parametrize("isDA,schedule,temp0,maxloop", [
    (1, "exp", 1.5, 0),      # EXP down to temp 1, both stopping tests
    (1, "linear", 1.35, 0),  # LINEAR steps of delta
    (0, "exp", 1.0, 30),     # plain EM, maxloop ends the run
    (1, "exp", 1.5, 7),      # maxloop inside the first temperature
])
def test_anneal_follows_the_oracle_loop(pkg, orc, golden, isDA, schedule, temp0, maxloop):
    T, FI, Y, beta = golden["T"], golden["FI"], golden["Y"], golden["beta"][0]
    kw = dict(alpha=0.9, delta=0.1, eps=1e-6, maxloop=maxloop)
    ref = orc.run(T, FI, Y, beta, temp0, isDA=isDA, schedule=1 if schedule == "linear" else 0,
                  solver=1, **kw)
    ctx = OracleCtx(orc, T, FI, Y)
    run = pkg.anneal(ctx, beta, temp0, isDA=isDA, schedule=schedule, **kw)
    got = traces(run)
    assert len(got[0]) == ref["n"]
    np.testing.assert_array_equal(got[0], ref["temp_trace"])
    for g, r in zip(got[1:], (ref["nfree_trace"], ref["llh_trace"], ref["beta_trace"])):
        np.testing.assert_allclose(g, r, rtol=1e-12)
    assert run.beta == pytest.approx(ref["beta"], rel=1e-12)
    np.testing.assert_allclose(run.W, ref["W"], rtol=1e-9, atol=1e-12)
    if maxloop:
        assert run.nloop == maxloop
    # the E-step precedes every M-step, and a temperature ends after an E-step
    assert ctx.calls[0] == "estep"
    assert all(not (a == "mstep" and b == "mstep") for a, b in zip(ctx.calls, ctx.calls[1:]))


def test_anneal_auto_takes_the_critical_temperature(pkg, orc, golden):
    """AUTO: at the end of each temperature the next one is the critical
    temperature from next_ctemp, weighted by the G of the last M-step, or
    temp * alpha when that is not below the current temperature
    (dagtm/dagtm.cxx:1919-1934)."""
    T, FI, Y, beta = golden["T"], golden["FI"], golden["Y"], golden["beta"][0]
    ctx = OracleCtx(orc, T, FI, Y)
    run = pkg.anneal(ctx, beta, 3.0, schedule="auto", alpha=0.9, eps=1e-5, maxloop=400)
    temps = []
    for t in run.temp_trace:
        if not temps or t != temps[-1]:
            temps.append(t)
    asks = [c for c in ctx.calls if isinstance(c, tuple) and c[0] == "ctemp"]
    assert len(temps) >= 3 and len(asks) >= len(temps) - 1
    for (_, t_in, c, w), t_next in zip(asks, temps[1:]):
        assert w is not None  # the G of the last M-step
        want = c if c < t_in else t_in * 0.9
        assert t_next == max(want, 1.0)


def test_anneal_auto_without_a_critical_temperature_cools_by_alpha(pkg, orc, golden):
    """AUTO when next_ctemp finds no eigenvalue below the limit (the
    reference's HUGE_VAL): the next temperature is temp * alpha, so the run
    is the EXP loop of the oracle."""
    class NoCritical(OracleCtx):
        def next_ctemp(self, temp, beta, eps, gg=None, per_centre=False):
            super().next_ctemp(temp, beta, eps, gg, per_centre)
            return np.inf

    T, FI, Y, beta = golden["T"], golden["FI"], golden["Y"], golden["beta"][0]
    ref = orc.run(T, FI, Y, beta, 1.5, isDA=1, schedule=0, alpha=0.9, eps=1e-6, solver=1)
    ctx = NoCritical(orc, T, FI, Y)
    run = pkg.anneal(ctx, beta, 1.5, schedule="auto", alpha=0.9, eps=1e-6)
    got = traces(run)
    np.testing.assert_array_equal(got[0], ref["temp_trace"])
    np.testing.assert_allclose(got[1], ref["nfree_trace"], rtol=1e-12)
    assert sum(isinstance(c, tuple) and c[0] == "ctemp" for c in ctx.calls) == \
        len(set(ref["temp_trace"].tolist())) - 1


def test_anneal_hda_follows_the_oracle_loop(pkg, orc):
    """HDA: the same expansions at the same iterations as orc.run_hda, K in
    the trace following them, and the traces equal to rounding."""
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    T = ds.gaussian_mixture(400, 5, 8, 0.2, seed=3)
    _, FI, W, beta = st.random_init(T, 2, 4, 4, 2.0, seed=1)
    t0 = st.first_critical_temp(T) * 0.8
    kw = dict(alpha=0.9, eps=1e-6, eps2=1e-3, Kmax=64, maxloop=600)
    ref = orc.run_hda(T, FI, FI @ W, beta, t0, 2, **kw)
    ctx = OracleCtx(orc, T, FI, FI @ W)
    run = pkg.anneal(ctx, beta, t0, hda=True, T=T, L=2, **kw)
    assert run.expansions == ref["expansions"]
    assert [c[1] for c in ctx.calls if isinstance(c, tuple) and c[0] == "basis"] == \
        [e[2] for e in ref["expansions"]]
    got = traces(run)
    assert len(got[0]) == ref["n"]
    np.testing.assert_array_equal(got[0], ref["temp_trace"])
    for g, r in zip(got[1:], (ref["nfree_trace"], ref["llh_trace"], ref["beta_trace"])):
        np.testing.assert_allclose(g, r, rtol=1e-10)
