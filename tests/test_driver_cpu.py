"""The command-line driver's HDF5 reader on the reference's own input file
(written by the HDF5 library the reference links); no GPU needed."""
import os
import subprocess

import numpy as np

from conftest import ROOT

DRIVER = os.path.join(ROOT, "da-gtm_gb300", "dagtm")
OIL_IN = os.path.join(ROOT, "tests", "golden", "oil_input.h5")


def test_reader_on_reference_input(built_lib, golden):
    out = subprocess.run([DRIVER, "--h5dump", OIL_IN], capture_output=True, text=True, check=True)
    rows = {ln.split()[0]: ln.split() for ln in out.stdout.splitlines()}
    assert rows["T"][1:4] == ["float", "1000", "12"]
    assert float(rows["T"][4].split("=")[1]) == golden["T_in"].astype(np.float64).sum()
    assert rows["id"][1:3] == ["int", "1000"] and float(rows["id"][3].split("=")[1]) == 500500
    assert float(rows["lb"][3].split("=")[1]) == golden["lb_in"].sum()


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
