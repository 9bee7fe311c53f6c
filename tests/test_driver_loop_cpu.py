"""The `dagtm` driver's host loop on the CPU.

The driver's sources are linked here against ``tests/fake_abi/oracle_abi.c``,
the C ABI served by the oracle's FP64 routines, instead of the CUDA library.
The driver and the package's ``anneal`` (over the same routines, through
``OracleCtx``) then start from one restart file, and their full-precision
traces (the Temp / LLH / NFree datasets of the output file) must agree:
EXP, LINEAR and AUTO cooling, and the hierarchical expansion.  Together with
the GPU tests of the driver this separates the host loop from the kernels.
"""
import glob
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from oracle_ctx import OracleCtx

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_golden import H5File  # noqa: E402

OIL_IN = os.path.join(ROOT, "tests", "golden", "oil_input.h5")


@pytest.fixture(scope="module")
def cpu_driver(tmp_path_factory, orc):
    d = tmp_path_factory.mktemp("cpu_driver")
    inc, orc_dir = os.path.join(ROOT, "include"), os.path.join(ROOT, "oracle")
    lib = str(d / "libdagtm_gb300.so")
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                           "-I" + inc, "-I" + orc_dir,
                           os.path.join(ROOT, "tests", "fake_abi", "oracle_abi.c"),
                           os.path.join(orc_dir, "dagtm_oracle.c"), "-o", lib, "-lm"])
    exe = str(d / "dagtm")
    srcs = sorted(glob.glob(os.path.join(ROOT, "da-gtm_gb300", "driver", "*.cc")))
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + inc] + srcs +
                          ["-L" + str(d), "-ldagtm_gb300", "-Wl,-rpath," + str(d), "-o", exe])
    return exe


def drive(exe, args, cwd):
    out = subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return out.stdout


def start_state(exe, tmp_path, extra):
    """One driver iteration from its own set-up: the restart file both loops start from."""
    drive(exe, ["-i", OIL_IN, "-o", "s0.h5", "-j", "1", "-n", "-Q", "cholesky"] + extra, tmp_path)
    f = H5File(str(tmp_path / "s0.h5"))
    return (f.read("FI"), f.read("Y"), float(f.read("beta")[0]), float(f.read("temp")[0]),
            int(f.read("iter")[0]))


@pytest.mark.parametrize("schedule", ["exp", "linear", "auto"])
def test_driver_loop_matches_anneal(cpu_driver, tmp_path, pkg, orc, golden, schedule):
    extra = ["-K", "125", "-L", "3", "-M", "8", "-s", "7", "-a", "0.9", "-c", schedule]
    FI, Y, beta, temp, it = start_state(cpu_driver, tmp_path, extra)
    drive(cpu_driver, ["-i", OIL_IN, "-r", "s0.h5", "-o", "s1.h5", "-j", "150", "-n", "-p",
                       "-Q", "cholesky", "-a", "0.9", "-e", "1e-6", "-c", schedule], tmp_path)
    f = H5File(str(tmp_path / "s1.h5"))
    T = golden["T_in"].astype(np.float64)
    ctx = OracleCtx(orc, T, FI, Y)
    run = pkg.anneal(ctx, beta, temp, schedule=schedule, alpha=0.9, delta=0.1, eps=1e-6,
                     iter0=it, maxloop=150)
    temps = f.read("Temp")
    # the maxloop test follows the M-step (dagtm/dagtm.cxx:1790-1795): a
    # temperature that ends on the |diff| test at iteration 150 is followed by
    # one more E-step, in both loops
    assert len(temps) == len(run.temp_trace) >= 150
    assert len(set(temps.tolist())) >= 2  # the run crosses temperatures
    np.testing.assert_allclose(temps, run.temp_trace, rtol=1e-12)
    np.testing.assert_allclose(f.read("LLH"), run.llh_trace, rtol=1e-9)
    np.testing.assert_allclose(f.read("NFree"), run.nfree_trace, rtol=1e-9)
    np.testing.assert_allclose(f.read("Y"), ctx.Y, rtol=1e-8, atol=1e-12)
    assert int(f.read("iter")[0]) == run.nloop


def test_driver_hda_matches_anneal(cpu_driver, tmp_path, pkg, orc, golden):
    st = __import__("importlib").import_module(pkg.__name__ + ".gtm_setup")
    T = golden["T_in"].astype(np.float64)
    t0 = 0.6 * st.first_critical_temp(T)
    extra = ["-K", "8", "-L", "3", "-M", "8", "-s", "3", "-H", "-S", f"{float(t0):.17g}",
             "-a", "0.9"]
    FI, Y, beta, temp, it = start_state(cpu_driver, tmp_path, extra)
    drive(cpu_driver, ["-i", OIL_IN, "-r", "s0.h5", "-o", "s1.h5", "-j", "200", "-n", "-p", "-H",
                       "-Q", "cholesky", "-a", "0.9", "-e", "1e-6"], tmp_path)
    ctx = OracleCtx(orc, T, FI, Y)
    run = pkg.anneal(ctx, beta, temp, alpha=0.9, eps=1e-6, iter0=it, maxloop=200, hda=True,
                     T=T, L=3)
    assert [e[1:] for e in run.expansions] == [(8, 64), (64, 512)]
    f = H5File(str(tmp_path / "s1.h5"))
    assert f.read("Y").shape == (512, 12)
    np.testing.assert_allclose(f.read("Temp"), run.temp_trace, rtol=1e-12)
    nf = f.read("NFree")
    first = run.expansions[0][0] - it  # trace entries before the first expansion
    np.testing.assert_allclose(nf[:first], run.nfree_trace[:first], rtol=1e-12)
    # after an expansion the two loops form Y = FI W by different host products
    # (a C++ loop, numpy), and A is ill-conditioned on the oil basis: the
    # tolerance of the GPU driver tests
    np.testing.assert_allclose(nf, run.nfree_trace, rtol=1e-5, atol=1e-5)
