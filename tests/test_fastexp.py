"""The integer-pipe FP64 exponential and logarithm of the engine, checked on the host
against the C library: within one unit in the last place (the logarithm where |ln x| >
1/256, and within 2^-60 absolute near x = 1); products of split exponentials (how the
engine forms equilibrium constants) within a few units of exp of the summed argument."""
import os
import subprocess

from conftest import ROOT


def test_fastexp_host(tmp_path):
    exe = os.path.join(str(tmp_path), "fastexp_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "fastexp_check.cpp")])
    out = subprocess.check_output([exe, "1500000"]).decode().split()
    vals = dict(zip(out[0::2], out[1::2]))
    assert float(vals["max_ulp"]) <= 1.0
    assert float(vals["max_ulp_neg"]) <= 1.0
    assert float(vals["max_rel_product"]) < 1e-15
    assert float(vals["max_ulp_log"]) <= 1.0
    assert float(vals["max_abs_log_near1"]) < 2.0 ** -60
