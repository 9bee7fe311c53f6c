"""The command-line driver's HDF5 reader on the reference's own files
(written by the HDF5 library the reference links): the input data/Oil.h5
(contiguous datasets) and the output data/Oil.out.h5 (chunked datasets with
the deflate filter); no GPU needed."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

DRIVER = os.path.join(ROOT, "da-gtm_gb300", "dagtm")
OIL_IN = os.path.join(ROOT, "tests", "golden", "oil_input.h5")
OIL_OUT = os.path.join(ROOT, "tests", "golden", "oil_output.h5")


def dump(path):
    out = subprocess.run([DRIVER, "--h5dump", path], capture_output=True, text=True, check=True)
    return {ln.split()[0]: ln.split() for ln in out.stdout.splitlines()}


def test_reader_on_reference_input(built_lib, golden):
    out = subprocess.run([DRIVER, "--h5dump", OIL_IN], capture_output=True, text=True, check=True)
    rows = {ln.split()[0]: ln.split() for ln in out.stdout.splitlines()}
    assert rows["T"][1:4] == ["float", "1000", "12"]
    assert float(rows["T"][4].split("=")[1]) == golden["T_in"].astype(np.float64).sum()
    assert rows["id"][1:3] == ["int", "1000"] and float(rows["id"][3].split("=")[1]) == 500500
    assert float(rows["lb"][3].split("=")[1]) == golden["lb_in"].sum()


def test_reader_on_reference_chunked_deflate_output(built_lib, golden):
    """Every dataset of the reference's output file, decoded by the C++
    reader, against the arrays the fixture script decoded with its own
    (Python, zlib) reader: shapes and sums."""
    rows = dump(OIL_OUT)
    want = {"FI.dat": golden["FI"], "M.dat": golden["M"], "T.dat": golden["T"],
            "W.dat": golden["W"], "X.dat": golden["X"], "Y.dat": golden["Y"],
            "beta.dat": golden["beta"], "lb.dat": golden["lb"]}
    for name, arr in want.items():
        r = rows[name]
        assert [int(x) for x in r[2:2 + arr.ndim]] == list(arr.shape), name
        got = float(r[2 + arr.ndim].split("=")[1])
        assert got == pytest.approx(float(arr.astype(np.float64).sum()), rel=1e-13, abs=1e-13), name
    r = rows["R.dat"]
    assert r[1:4] == ["float", "125", "1000"]
    assert float(r[4].split("=")[1]) == pytest.approx(float(golden["R_colsum"].sum()), rel=1e-13)


@pytest.mark.parametrize("src", ["oil_input.h5", "oil_output.h5"])
def test_reader_refuses_truncated_files_without_crashing(built_lib, tmp_path, src):
    """Truncated copies of both files: the reader either reports an error or
    reads what is complete, and never reads outside the file (no signal)."""
    data = open(os.path.join(ROOT, "tests", "golden", src), "rb").read()
    cuts = sorted(set([8, 95, 96, 200, 700, 1500, 4000] + [len(data) * i // 13 for i in range(1, 13)]))
    for cut in cuts:
        p = tmp_path / f"cut{cut}.h5"
        p.write_bytes(data[:cut])
        out = subprocess.run([DRIVER, "--h5dump", str(p)], capture_output=True, text=True,
                             timeout=60)
        assert out.returncode >= 0, (cut, out.returncode)


def test_help_lists_reference_options(built_lib):
    out = subprocess.run([DRIVER, "-h"], capture_output=True, text=True)
    assert out.returncode == 0
    for flag in ("-K number", "-L number", "-M number", "-S number", "-c schedule", "-a number",
                 "-e number", "-j number", "-s number", "-r filename", "-o filename", "-H ",
                 "-k number", "-E number"):
        assert flag in out.stderr


def test_unsupported_options_are_refused(built_lib):
    for args in (["-g", "spacefilling"], ["-c", "fast"]):
        out = subprocess.run([DRIVER] + args, capture_output=True, text=True)
        assert out.returncode != 0
