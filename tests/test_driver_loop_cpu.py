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
                          ["-L" + str(d), "-ldagtm_gb300", "-lz", "-Wl,-rpath," + str(d), "-o",
                           exe])
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
    assert np.ptp(f.read("NFree")) > 1.0  # and the centres leave the trivial solution
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
    seen = []
    run = pkg.anneal(ctx, beta, temp, alpha=0.9, eps=1e-6, iter0=it, maxloop=200, hda=True,
                     T=T, L=3, on_expand=lambda c, info: seen.append(info))
    assert [e[1:] for e in run.expansions] == [(8, 64), (64, 512)]
    f = H5File(str(tmp_path / "s1.h5"))
    assert f.read("Y").shape == (512, 12)
    # the snapshots written before each expansion (dagtm/dagtm.cxx:1980-2096),
    # under the index of the temperature trace, against the package loop's
    for info, tol in zip(seen, (1e-9, 1e-4)):
        i, K = info["index"], info["K"]
        assert f.read(f"X.{i}").shape == (K, 3) and f.read(f"M.{i}").shape == (1000, 3)
        assert f.read(f"FI.{i}").shape == (K, 9) and f.read(f"Y.{i}").shape == (K, 12)
        np.testing.assert_allclose(f.read(f"W.{i}"), info["W"], rtol=tol, atol=tol)
        np.testing.assert_allclose(f.read(f"ctemp.{i}"), info["ctemp"], rtol=tol)
        assert float(f.read(f"beta.{i}")[0]) == pytest.approx(info["beta"], rel=tol)
    np.testing.assert_allclose(f.read("Temp"), run.temp_trace, rtol=1e-12)
    nf = f.read("NFree")
    first = run.expansions[0][0] - it  # trace entries before the first expansion
    np.testing.assert_allclose(nf[:first], run.nfree_trace[:first], rtol=1e-12)
    # after an expansion the two loops form Y = FI W by different host products
    # (a C++ loop, numpy), and A is ill-conditioned on the oil basis: the
    # tolerance of the GPU driver tests
    np.testing.assert_allclose(nf, run.nfree_trace, rtol=1e-5, atol=1e-5)


def test_driver_checkpoint_restart_and_outputs(cpu_driver, tmp_path, golden):
    """Checkpoints every 5 iterations, restart, -R, -I and the output layout
    (dagtm/dagtm.cxx:1609-1687, 1161-1232, 2342-2414).  A checkpoint is taken
    after an iteration's E-step, before its M-step, as the reference takes it:
    a restart from the 10th therefore repeats the E-step of iteration 10 (its
    iterations 11..16 are 10..15 of an uninterrupted run) and ends on the same
    centres as an uninterrupted run of 15.  Started below the first critical
    temperature, so that the trace moves from one iteration to the next."""
    common = ["-i", OIL_IN, "-K", "125", "-L", "3", "-M", "8", "-s", "3", "-a", "0.9",
              "-e", "0", "-S", "1.5", "-Q", "cholesky"]
    drive(cpu_driver, common + ["-j", "15", "-n", "-p", "-o", "full.h5"], tmp_path)
    drive(cpu_driver, common + ["-j", "10", "-P", "5", "-w", "ck."], tmp_path)
    assert (tmp_path / "ck.5.h5").exists() and (tmp_path / "ck.10.h5").exists()
    ck = H5File(str(tmp_path / "ck.10.h5"))
    for name in ("X", "FI", "Y", "beta", "temp", "iter", "seed", "qual"):
        assert name in ck.datasets, name
    assert int(ck.read("iter")[0]) == 10
    drive(cpu_driver, ["-i", OIL_IN, "-r", "ck.10.h5", "-j", "6", "-n", "-p", "-R",
                       "-Q", "cholesky", "-e", "0", "-o", "rest.h5"], tmp_path)
    full, rest = H5File(str(tmp_path / "full.h5")), H5File(str(tmp_path / "rest.h5"))
    nf = full.read("NFree")
    assert np.min(np.abs(np.diff(nf[9:15]))) > 1e-6 * np.max(np.abs(nf))  # the trace moves
    np.testing.assert_allclose(rest.read("NFree"), nf[9:15], rtol=1e-13)
    np.testing.assert_allclose(rest.read("LLH"), full.read("LLH")[9:15], rtol=1e-13)
    np.testing.assert_allclose(rest.read("Y"), full.read("Y"), rtol=1e-12, atol=1e-15)
    assert int(rest.read("iter")[0]) == 16
    for name in ("T", "M", "X", "FI", "Y", "W", "beta", "temp", "iter", "seed", "qual", "id", "lb",
                 "Temp", "LLH", "NFree"):
        assert name in full.datasets, name
    assert np.array_equal(full.read("T"), golden["T_in"].astype(np.float64))
    R = rest.read("R")
    assert R.shape == (125, 1000) and np.allclose(R.sum(axis=0), 1.0, atol=1e-12)
    M = full.read("M")
    assert M.shape == (1000, 3) and np.all(np.abs(M) <= 1.0 + 1e-12)
    drive(cpu_driver, ["-i", OIL_IN, "-I", "-r", "ck.10.h5", "-o", "interp.h5"], tmp_path)
    Mi = H5File(str(tmp_path / "interp.h5")).read("M")
    assert Mi.shape == (1000, 3) and np.all(np.isfinite(Mi))


def test_driver_signal_forces_a_checkpoint_and_exit(cpu_driver, tmp_path):
    """SIGCHLD makes the driver write a checkpoint at the next iteration and
    exit 0 (dagtm/dagtm.cxx:978, 1609-1687)."""
    import signal
    import time
    p = subprocess.Popen([cpu_driver, "-i", OIL_IN, "-K", "125", "-L", "3", "-M", "8", "-s", "5",
                          "-e", "0", "-j", "1000000", "-n", "-w", "sig."], cwd=tmp_path,
                         stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    time.sleep(2.0)
    p.send_signal(signal.SIGCHLD)
    try:
        out, err = p.communicate(timeout=120)
    except subprocess.TimeoutExpired:
        p.kill()  # this test's own child
        p.communicate()
        raise
    assert p.returncode == 0, err
    files = list(tmp_path.glob("sig.*.h5"))
    assert len(files) == 1
    n = int(H5File(str(files[0])).read("iter")[0])
    assert n > 1 and str(files[0]).endswith(f"sig.{n}.h5")


def test_driver_setup_matches_package_setup(cpu_driver, tmp_path, pkg, golden):
    """The driver's set-up (C++) against the package's (numpy), both restating
    the reference's (dagtm/dagtm.cxx:1104-1160; comm/comm.c:1118-1185,
    1401-1448; comm/mpicomm.c:511-559).  A checkpoint at iteration 1 holds the
    state before the first M-step: the initial centres, beta and the start
    temperature.  Both solve the least-squares fit of W through the normal
    equations FI^T FI, whose conditioning on the oil basis bounds the centres'
    agreement (1e-6); grid, basis, beta and temperature agree to rounding."""
    st = __import__("importlib").import_module(pkg.__name__ + ".gtm_setup")
    drive(cpu_driver, ["-i", OIL_IN, "-K", "125", "-L", "3", "-M", "8", "-s", "7", "-a", "0.95",
                       "-j", "1", "-P", "1", "-w", "init.", "-Q", "cholesky"], tmp_path)
    f = H5File(str(tmp_path / "init.1.h5"))
    T = golden["T_in"].astype(np.float64)
    X, FI, W0, beta0 = st.random_init(T, 3, 125, 8, 2.0, seed=7)
    assert np.array_equal(f.read("X"), X)
    np.testing.assert_allclose(f.read("FI"), FI, rtol=0, atol=1e-15)
    assert float(f.read("beta")[0]) == pytest.approx(beta0, rel=1e-13)
    assert float(f.read("temp")[0]) == pytest.approx(st.start_temp(T, 0.95), rel=1e-13)
    Y0 = FI @ W0
    assert np.max(np.abs(f.read("Y") - Y0)) <= 1e-6 * np.max(np.abs(Y0))
