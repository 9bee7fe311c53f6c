"""The `dagtm` command end to end on the reference's oil input: the options,
the `:::` trace, checkpoints, restart, interpolation and the output layout of
dagtm/dagtm.cxx, with the EM step on the GPU."""
import os
import re
import signal
import subprocess
import sys
import time

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_golden import H5File  # noqa: E402

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(ROOT, "da-gtm_gb300", "dagtm")
OIL_IN = os.path.join(ROOT, "tests", "golden", "oil_input.h5")
TRACE = re.compile(r"^:::\s+(\d+)\s+(\d+)\s+(\d+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)")


def run(args, cwd):
    out = subprocess.run([DRIVER] + args, cwd=cwd, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return out.stdout


def trace(stdout):
    rows = [TRACE.match(ln) for ln in stdout.splitlines()]
    return np.array([[float(x) for x in m.groups()] for m in rows if m])


def test_run_trace_and_output(tmp_path, pkg, golden):
    # -e 0: every iteration stays at the start temperature, so the comparison
    # below does not hinge on where |diff| first drops under eps
    out = run(["-i", OIL_IN, "-o", "out.h5", "-K", "125", "-L", "3", "-M", "8", "-s", "7",
               "-j", "40", "-n", "-p", "-a", "0.95", "-e", "0", "-F", "fp64"], tmp_path)
    tr = trace(out)
    assert len(tr) == 40 and tr[0][0] == 1 and tr[-1][0] == 40
    assert "SUMMARY" in out and "Num. of Iterations" in out
    f = H5File(str(tmp_path / "out.h5"))
    for name in ("T", "M", "X", "FI", "Y", "W", "beta", "temp", "iter", "seed", "qual", "id", "lb",
                 "Temp", "LLH", "NFree"):
        assert name in f.datasets, name
    assert np.array_equal(f.read("T"), golden["T_in"].astype(np.float64))
    assert np.array_equal(f.read("lb"), golden["lb_in"])
    X, FI, Y, W = f.read("X"), f.read("FI"), f.read("Y"), f.read("W")
    assert X.shape == (125, 3) and FI.shape == (125, 9) and W.shape == (9, 12)
    assert np.array_equal(X, golden["X"]) and np.max(np.abs(FI - golden["FI"])) < 1e-15
    assert np.max(np.abs(FI @ W - Y)) < 1e-6 * np.max(np.abs(Y))
    M = f.read("M")
    assert M.shape == (1000, 3) and np.all(np.abs(M) <= 1.0 + 1e-12)
    assert int(f.read("iter")[0]) == 40 and int(f.read("seed")[0]) == 7
    assert np.allclose(f.read("NFree"), tr[:, 4], rtol=1e-6)
    # the driver's trace agrees with the package's own loop from the same set-up
    st = __import__("importlib").import_module(pkg.__name__ + ".gtm_setup")
    T = golden["T_in"].astype(np.float64)
    _, FI0, W0, beta0 = st.random_init(T, 3, 125, 8, 2.0, seed=7)
    with pkg.Context(T, FI0, "fp64", solver="svd") as c:
        c.set_Y(FI0 @ W0)
        ref = pkg.anneal(c, beta0, st.start_temp(T, 0.95), alpha=0.95, eps=0.0, maxloop=40)
    assert np.allclose(tr[:, 4], ref.nfree_trace, rtol=1e-5, atol=1e-6)


def test_checkpoint_restart_and_interpolation(tmp_path):
    # -e 0 keeps the whole run at one temperature, where a restart resumes exactly
    common = ["-i", OIL_IN, "-K", "125", "-L", "3", "-M", "8", "-s", "3", "-a", "0.9", "-e", "0"]
    full = trace(run(common + ["-j", "16", "-n"], tmp_path))
    run(common + ["-j", "10", "-P", "5", "-w", "ck."], tmp_path)
    assert (tmp_path / "ck.5.h5").exists() and (tmp_path / "ck.10.h5").exists()
    ck = H5File(str(tmp_path / "ck.10.h5"))
    for name in ("X", "FI", "Y", "beta", "temp", "iter", "seed", "qual"):
        assert name in ck.datasets
    assert int(ck.read("iter")[0]) == 10
    rest = trace(run(common + ["-r", "ck.10.h5", "-j", "6", "-n"], tmp_path))
    assert rest[0][0] == 11 and len(rest) == 6
    # a checkpoint is taken after an iteration's E-step, before its M-step (as
    # the reference takes it), so the restart repeats the E-step of iteration
    # 10: its iterations 11..16 are 10..15 of the uninterrupted run
    assert np.allclose(rest[:, 4], full[9:15, 4], rtol=1e-12)
    assert np.allclose(rest[:, 5], full[9:15, 5], rtol=1e-12)
    run(["-i", OIL_IN, "-I", "-r", "ck.10.h5", "-o", "interp.h5"], tmp_path)
    M = H5File(str(tmp_path / "interp.h5")).read("M")
    assert M.shape == (1000, 3) and np.all(np.isfinite(M))


def test_signal_forces_a_checkpoint_and_exit(tmp_path):
    p = subprocess.Popen([DRIVER, "-i", OIL_IN, "-K", "125", "-L", "3", "-M", "8", "-s", "5",
                          "-e", "0", "-j", "1000000", "-n", "-w", "sig."], cwd=tmp_path,
                         stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    time.sleep(3.0)
    p.send_signal(signal.SIGCHLD)
    out, err = p.communicate(timeout=120)
    assert p.returncode == 0, err
    files = list(tmp_path.glob("sig.*.h5"))
    assert len(files) == 1
    n = int(H5File(str(files[0])).read("iter")[0])
    assert str(files[0]).endswith(f"sig.{n}.h5")


def test_auto_schedule_matches_package_loop(tmp_path, pkg, golden):
    # -c auto: after each temperature the next one is the critical temperature
    # of dgtm_next_ctemp (or temp * alpha when none is below the current one)
    out = run(["-i", OIL_IN, "-o", "auto.h5", "-K", "125", "-L", "3", "-M", "8", "-s", "3",
               "-j", "60", "-c", "auto", "-a", "0.9", "-e", "1e-3", "-F", "fp64"], tmp_path)
    assert "Cooling Schedule = AUTO" in " ".join(out.split())
    tr = trace(out)
    temps = []
    for t in tr[:, 3]:
        if not temps or t != temps[-1]:
            temps.append(t)
    assert len(temps) >= 2 and all(a > b for a, b in zip(temps, temps[1:]))
    st = __import__("importlib").import_module(pkg.__name__ + ".gtm_setup")
    T = golden["T_in"].astype(np.float64)
    _, FI0, W0, beta0 = st.random_init(T, 3, 125, 8, 2.0, seed=3)
    with pkg.Context(T, FI0, "fp64", solver="svd") as c:
        c.set_Y(FI0 @ W0)
        ref = pkg.anneal(c, beta0, st.start_temp(T, 0.9), schedule="auto", alpha=0.9, eps=1e-3,
                         maxloop=60)
    n = min(len(tr), len(ref.nfree_trace))
    assert n >= 10
    assert np.allclose(tr[:n, 3], ref.temp_trace[:n], rtol=1e-6)
    assert np.allclose(tr[:n, 4], ref.nfree_trace[:n], rtol=1e-5, atol=1e-6)


def test_hda_expands_and_writes_snapshots(tmp_path, pkg, golden):
    # -H on the EXP schedule from K = 8 (L = 3), started below the first
    # critical temperature: the grid doubles per dimension twice within 200
    # iterations (8 -> 64 -> 512), as the package loop does from the same set-up
    st = __import__("importlib").import_module(pkg.__name__ + ".gtm_setup")
    T = golden["T_in"].astype(np.float64)
    t0 = 0.6 * st.first_critical_temp(T)
    out = run(["-i", OIL_IN, "-o", "hda.h5", "-K", "8", "-L", "3", "-M", "8", "-s", "3", "-H",
               "-S", f"{float(t0):.17g}", "-j", "200", "-n", "-p", "-a", "0.9", "-e", "1e-6", "-F", "fp64",
               "-Q", "cholesky"], tmp_path)
    tr = trace(out)
    Ks = tr[:, 2].astype(int)
    assert Ks[0] == 8 and Ks[-1] == 512
    grow = [int(tr[i, 0]) for i in range(1, len(tr)) if Ks[i] != Ks[i - 1]]
    _, FI0, W0, beta0 = st.random_init(T, 3, 8, 8, 2.0, seed=3)
    with pkg.Context(T, FI0, "fp64") as c:
        c.set_Y(FI0 @ W0)
        ref = pkg.anneal(c, beta0, t0, alpha=0.9, eps=1e-6, maxloop=200, hda=True, T=T, L=3)
    assert [e[1:] for e in ref.expansions] == [(8, 64), (64, 512)]
    # the first iteration at the new K follows the expansion's last one
    assert grow == [e[0] + 1 for e in ref.expansions]
    n = min(len(tr), len(ref.nfree_trace))
    # the host products Y = FI W of the two loops round differently, and A is
    # ill-conditioned on the oil basis: the tolerance of the other driver tests
    assert np.allclose(tr[:n, 4], ref.nfree_trace[:n], rtol=1e-5, atol=1e-6)
    f = H5File(str(tmp_path / "hda.h5"))
    for (it, K, _), (Kx, Mx) in zip(ref.expansions, ((8, 8), (64, 8))):
        idx = it - 1  # the temperature collection holds one entry per iteration
        assert f.read(f"X.{idx}").shape == (K, 3)
        assert f.read(f"FI.{idx}").shape == (K, Mx + 1)
        assert f.read(f"Y.{idx}").shape == (K, 12)
        assert f.read(f"W.{idx}").shape == (Mx + 1, 12)
        assert f.read(f"M.{idx}").shape == (1000, 3)
        assert f.read(f"ctemp.{idx}").shape == (K,)
        assert f.read(f"beta.{idx}").shape == (1,)
    assert f.read("X").shape == (512, 3) and f.read("Y").shape == (512, 12)


def test_split_form_with_linear_cooling(tmp_path, pkg, golden):
    # -F bf16x3 -c linear: the driver's loop over the split form agrees with
    # the package's loop from the same set-up (one library, two host loops)
    out = run(["-i", OIL_IN, "-o", "lin.h5", "-K", "125", "-L", "3", "-M", "8", "-s", "4",
               "-j", "40", "-n", "-c", "linear", "-e", "1e-3", "-F", "bf16x3"], tmp_path)
    assert "Cooling Schedule = LINEAR" in " ".join(out.split())
    tr = trace(out)
    st = __import__("importlib").import_module(pkg.__name__ + ".gtm_setup")
    T = golden["T_in"].astype(np.float64)
    _, FI0, W0, beta0 = st.random_init(T, 3, 125, 8, 2.0, seed=4)
    with pkg.Context(T, FI0, "bf16x3", solver="svd") as c:
        c.set_Y(FI0 @ W0)
        ref = pkg.anneal(c, beta0, st.start_temp(T, 0.99), schedule="linear", delta=0.1,
                         eps=1e-3, maxloop=40)
    n = min(len(tr), len(ref.nfree_trace))
    assert n >= 10
    assert np.allclose(tr[:n, 3], ref.temp_trace[:n], rtol=1e-6)
    assert np.allclose(tr[:n, 4], ref.nfree_trace[:n], rtol=1e-5, atol=1e-6)
    f = H5File(str(tmp_path / "lin.h5"))
    assert f.read("Y").shape == (125, 12) and np.all(np.isfinite(f.read("Y")))
