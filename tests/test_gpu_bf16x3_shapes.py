"""Split-BF16 form across operand shapes, against the FP64 oracle.

Both tensor-core kernels are compiled once per operand shape: the number of
64-wide depth panels (D + 3 rounded up to 64, 1 to 3), the 16-deep steps
used in the last panel (1 to 4), and whether the data are exact in BF16
(one data piece) or split in two.  Each case below lands on a different
shape; odd D also takes the scalar path of the best-centre distance.
Tolerances as in test_gpu_bf16x3: qualities 1e-5 relative for exact data,
1e-4 for split data; G, R T, Y, beta 1e-4 relative.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def sub(pkg, name):
    return importlib.import_module(pkg.__name__ + "." + name)


def shape_of(D):
    """(panels, steps in the last panel) of the distance products for D."""
    ksteps = (D + 3 + 15) // 16
    npanel = (D + 3 + 63) // 64
    return npanel, ksteps - 4 * (npanel - 1)


# one D per (panels, last-panel steps): D + 3 = 16, 23, 40, 64, 65, 88, 104, 128,
# 129, 153, 169, 192
DS = [13, 20, 37, 61, 62, 85, 101, 125, 126, 150, 166, 189]


def test_cases_cover_every_shape():
    assert sorted({shape_of(D) for D in DS}) == [(p, k) for p in (1, 2, 3) for k in (1, 2, 3, 4)]


@pytest.mark.parametrize("exact", [True, False], ids=["binary", "real"])
@pytest.mark.parametrize("D", DS)
def test_em_step_shape(pkg, orc, D, exact):
    ds = sub(pkg, "datasets")
    st = sub(pkg, "gtm_setup")
    N, K, M = 700, 125, 8
    if exact:
        T = ds.fingerprints(N, D, 12, seed=D)
    else:
        T = ds.gaussian_mixture(N, D, 6, 0.15, seed=D)
    X, FI = st.setup_grid(3, K, M, 1.0)
    rng = np.random.default_rng(D)
    Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
    beta, temp = 40.0 / D, 1.7
    Dm = orc.dist(Y, T)
    R, vgc, vgc2 = orc.resp(Dm, beta, 1, temp)
    llh = orc.qual(N, K, D, beta, vgc, 0, temp)
    nfree = orc.qual(N, K, D, beta, vgc2, 1, temp)
    G, A, B = orc.mstep_stats(R, FI, T)
    Yn = orc.fiw(FI, orc.solve_chol(A, B))
    bn, _, _ = orc.beta_update(Yn, T, R)
    tol_q = 1e-5 if exact else 1e-4
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        l, f = c.estep(beta, 1, temp)
        Rg = c.R_block(0, K, 0, 200)
        b, W, Yg = c.mstep(want_Y=True)
        Gg, RTg = c.get_stats()
    assert l == pytest.approx(llh, rel=tol_q)
    assert f == pytest.approx(nfree, rel=tol_q)
    assert np.max(np.abs(Rg - R[:, :200])) <= 1e-4
    assert rel(Gg, G) <= 1e-4
    assert rel(RTg, R @ T) <= 1e-4
    assert rel(Yg, Yn) <= 1e-4
    assert b == pytest.approx(bn, rel=1e-4)


def test_wide_data_is_refused(pkg):
    """D + 3 > 192 does not fit the pass-2 tensor-memory plan: ENOTSUP."""
    ds = sub(pkg, "datasets")
    st = sub(pkg, "gtm_setup")
    T = ds.fingerprints(300, 190, 8, seed=1)
    X, FI = st.setup_grid(2, 25, 4, 1.0)
    with pytest.raises(pkg.DgtmError) as e:
        pkg.Context(T, FI, "bf16x3")
    assert e.value.code == 8


# Pass 2 moves R T out of tensor memory every 64 tiles (4096 points); a unit
# is 256 tiles.  N = 20000 gives one unit of four segments and one of a
# single segment per centre tile.  Binary D = 166 and real D = 85 sum the
# segments in shared memory; real D = 150 (two data pieces, three panels)
# adds them to the slot at L2.
@pytest.mark.parametrize("D,exact", [(166, True), (85, False), (150, False)],
                         ids=["binary166-shared", "real85-shared", "real150-l2"])
def test_multi_segment_units(pkg, orc, D, exact):
    ds = sub(pkg, "datasets")
    st = sub(pkg, "gtm_setup")
    N, K, M = 20000, 125, 8
    if exact:
        T = ds.fingerprints(N, D, 12, seed=D)
    else:
        T = ds.gaussian_mixture(N, D, 6, 0.15, seed=D)
    X, FI = st.setup_grid(3, K, M, 1.0)
    rng = np.random.default_rng(D)
    Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
    beta, temp = 40.0 / D, 1.7
    R, _, _ = orc.resp(orc.dist(Y, T), beta, 1, temp)
    G, _, _ = orc.mstep_stats(R, FI, T)
    RT = R @ T
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        c.estep(beta, 1, temp)
        c.mstep(want_W=False)
        Gg, RTg = c.get_stats()
    assert rel(Gg, G) <= 1e-4
    assert rel(RTg, RT) <= 1e-4
    assert abs(Gg.sum() - N) / N <= 2e-5
    assert rel(RTg.sum(axis=0), T.sum(axis=0)) <= 2e-5
