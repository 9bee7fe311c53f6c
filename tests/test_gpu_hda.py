"""Hierarchical DA (-H): anneal(hda=True) against the oracle's restatement of
the expansion logic of dagtm/dagtm.cxx:1912-2124 (oracle.run_hda).

The case grows the grid three times (K = 4 -> 16 -> 64 -> 256, L = 2).  Its
decisions have margins far above either form's error: the critical
temperatures that set the ready flag clear temp * alpha by 4.5-11 %, and the
log-likelihood gains that confirm an expansion are 7e-3 to 0.16 against
eps2 = 1e-3.  The FP64 form follows the oracle's trajectory iteration by
iteration: 1e-9 on the traces, 1e-8 on the final centres.  The split-BF16
form carries ~1e-5 in the qualities, which is above the 1e-6 step test that
ends a temperature, so it may spend a few iterations more or fewer at a
temperature; it makes the same expansions at the same temperatures and ends
within 1e-4 of the oracle's qualities.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def case(pkg, orc):
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    T = ds.gaussian_mixture(400, 5, 8, 0.2, seed=3)
    _, FI, W, beta = st.random_init(T, 2, 4, 4, 2.0, seed=1)
    t0 = st.first_critical_temp(T) * 0.8
    kw = dict(alpha=0.9, eps=1e-6, eps2=1e-3, Kmax=256, maxloop=1500)
    ref = orc.run_hda(T, FI, FI @ W, beta, t0, 2, **kw)
    return T, FI, FI @ W, beta, t0, kw, ref


def test_hda_trajectory_matches_oracle_fp64(pkg, case):
    T, FI, Y0, beta, t0, kw, ref = case
    assert [e[1:] for e in ref["expansions"]] == [(4, 16), (16, 64), (64, 256)]
    seen = []
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y0)
        out = pkg.anneal(c, beta, t0, hda=True, T=T, L=2,
                         on_expand=lambda ctx, info: seen.append(info), **kw)
        assert c.K == 256
        Yg = c.get_Y()
    assert out.expansions == ref["expansions"]
    assert len(out.nfree_trace) == ref["n"]
    assert rel(out.nfree_trace, ref["nfree_trace"]) <= 1e-9
    assert rel(out.llh_trace, ref["llh_trace"]) <= 1e-9
    assert rel(out.beta_trace, ref["beta_trace"]) <= 1e-9
    assert rel(Yg, ref["Y"]) <= 1e-8
    assert [(i["K"], i["K_new"]) for i in seen] == [(4, 16), (16, 64), (64, 256)]
    for info, (it, K, _) in zip(seen, ref["expansions"]):
        assert info["index"] == it - 1
        assert info["ctemp"].shape == (K,) and np.all(np.isfinite(info["ctemp"]))
        assert info["W"].shape == (FI.shape[1], T.shape[1])


def test_hda_split_form_expands_at_the_same_temperatures(pkg, case):
    T, FI, Y0, beta, t0, kw, ref = case
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y0)
        out = pkg.anneal(c, beta, t0, hda=True, T=T, L=2, **kw)
        assert c.K == 256
    assert [e[1:] for e in out.expansions] == [e[1:] for e in ref["expansions"]]
    temps = [out.temp_trace[it - 1] for it, _, _ in out.expansions]
    assert temps == pytest.approx([ref["temp_trace"][it - 1] for it, _, _ in ref["expansions"]],
                                  rel=1e-12)
    assert out.temp == pytest.approx(ref["temp"], rel=1e-12)
    assert out.nfree_trace[-1] == pytest.approx(ref["nfree_trace"][-1], rel=1e-4)
    assert out.llh_trace[-1] == pytest.approx(ref["llh_trace"][-1], rel=1e-4)


def test_next_ctemp_per_centre(pkg, case):
    T, FI, Y0, beta, t0, kw, ref = case
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y0)
        c.estep(beta, 1, t0)
        cmax, ck = c.next_ctemp(t0, beta, 1e-6, per_centre=True)
        assert cmax == c.next_ctemp(t0, beta, 1e-6)
    assert ck.shape == (4,) and cmax == ck.max()


def test_set_basis_rebuilds_for_new_K(pkg, case):
    T, FI, Y0, beta, t0, kw, ref = case
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    _, FI2 = st.setup_grid(2, 16, 4, 2.0)
    with pkg.Context(T, FI, "fp64") as c:
        c.set_Y(Y0)
        c.estep(beta, 1, t0)
        _, W, _ = c.mstep()
        c.set_basis(T, FI2, FI2 @ W)
        assert c.K == 16
        assert rel(c.get_Y(), FI2 @ W) == 0.0
        llh, nfree = c.estep(beta, 1, t0)
        assert np.isfinite(llh) and np.isfinite(nfree)
        with pytest.raises(ValueError):
            c.set_basis(T[:10], FI2, FI2 @ W)
