"""The driver's -J output on the CPU: after a -j stop the MAP and the -R dump
come from R o D, the R that dagtm_mpi_beta multiplied in place by the squared
distances to the new centres (comm/mpicomm.c:288, dagtm/dagtm.cxx:2348-2414).
The driver is linked against the C ABI served by the oracle (its dgtm_map_rd
and dgtm_get_RD_block read the oracle's R after the beta update), and its
output is checked against the oracle's own loop, which leaves R o D too."""
import os
import sys

import numpy as np

from conftest import ROOT
from test_driver_loop_cpu import OIL_IN, cpu_driver, drive, start_state  # noqa: F401

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_golden import H5File  # noqa: E402


def test_driver_J_writes_R_o_D_after_a_maxloop_stop(cpu_driver, tmp_path, orc, golden):
    extra = ["-K", "125", "-L", "3", "-M", "8", "-s", "5", "-a", "0.9"]
    FI, Y, beta, temp, it = start_state(cpu_driver, tmp_path, extra)
    drive(cpu_driver, ["-i", OIL_IN, "-r", "s0.h5", "-o", "rd.h5", "-j", "9", "-n", "-J", "-R",
                       "-Q", "cholesky", "-a", "0.9", "-e", "0"], tmp_path)
    T = golden["T_in"].astype(np.float64)
    ref = orc.run(T, FI, Y, beta, temp, isDA=1, alpha=0.9, eps=0.0, iter0=it, maxloop=9,
                  solver=1, want_R=True)
    f = H5File(str(tmp_path / "rd.h5"))
    RD = ref["R"]
    assert not np.allclose(RD.sum(axis=0), 1.0)
    np.testing.assert_allclose(f.read("R"), RD, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(f.read("M"), RD.T @ f.read("X"), rtol=1e-12, atol=1e-13)
