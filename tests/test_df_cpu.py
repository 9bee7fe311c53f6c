"""The double-float arithmetic of the exact-slice FP64 form
(da-gtm_gb300/csrc/df.cuh), compiled for the host from the same header and
checked against long-double and exact integer results (tests/df_check.cc):

* exp_df on [-45, 1], table edges included: relative error below 2e-14
  (the form's exponentials; 2^-47 is 7.1e-15);
* sum4, the recombination of four exact slice partials, also under
  cancellation: relative error below 1e-14 of the exact integer;
* mul: below 2e-14;
* fixed48, round(E 2^48) for 0 <= E < 2: within one unit;
* fixed48r: 60000 terms summed as 2^-48 integers plus an FP32 sum of the
  exact rounding remainders, within 1e-16 of the long-double sum (the form's
  per-point sums over K centres).
"""
import os
import re
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def df_check(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("df") / "df_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "df_check.cc"), "-lm"])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300, check=True).stdout
    return out


def value(out, key):
    m = re.search(key + r"\s+([-+0-9.eE]+)", out)
    assert m, out
    return float(m.group(1))


def test_exp(df_check):
    assert value(df_check, "exp_df max_rel") <= 2e-14
    assert "exp_df below_cut 0 0" in df_check


def test_slice_recombination(df_check):
    assert value(df_check, "sum4 max_rel") <= 1e-14


def test_mul(df_check):
    assert value(df_check, "mul max_rel") <= 2e-14


def test_fixed_point(df_check):
    assert value(df_check, "fixed48 max_abs_units") <= 1.0


def test_fixed_point_48_with_remainders(df_check):
    assert value(df_check, "fixed48r sum_rel") <= 1e-16
