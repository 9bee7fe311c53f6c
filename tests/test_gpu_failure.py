"""Failure detection without a GPU fault: every wait in the tensor-core
kernels is bounded by a wall-clock limit, records a site code when it gives
up, and the host reports DGTM_ETIMEOUT.  Here one such wait runs out on a
barrier that nothing arrives at (50 ms limit); the error reaches the host
and the device keeps working."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_device_stays_usable(pkg, orc):
    code, site, ms = pkg.wait_probe(50)
    assert code == 5  # DGTM_ETIMEOUT
    assert site == 90
    assert 50.0 <= ms < 2000.0
    msg = pkg.load_library().dgtm_last_error_string().decode()
    assert "gave up" in msg and "site 90" in msg
    # the tensor-core kernels and a whole EM step still run afterwards
    assert pkg.selftest() == [0.0, 0.0, 0.0, 0.0]
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    T = ds.fingerprints(600, 40, 8, seed=4)
    X, FI = st.setup_grid(2, 64, 9, 1.0)
    rng = np.random.default_rng(4)
    Y = T[rng.integers(0, 600, 64)] * 0.7 + 0.15
    R, vgc, vgc2 = orc.resp(orc.dist(Y, T), 1.0, 1, 2.0)
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        llh, nfree = c.estep(1.0, 1, 2.0)
        c.mstep()
    assert llh == pytest.approx(orc.qual(600, 64, 40, 1.0, vgc, 0, 2.0), rel=1e-5)


def test_wait_probe_rejects_bad_limits(pkg):
    code, _, _ = pkg.wait_probe(0)
    assert code == 1  # DGTM_EINVAL
