"""The dense LU's panel form (four pivots per trailing update) keeps the unblocked form's
operations and their order, so its factors are the same bit for bit: both orders restated on
the host with explicit fused multiply-adds (lu_panel_order.cpp) and compared (no GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_panel_lu_order_gives_the_unblocked_factors(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "lu_panel_order")
    # no contraction: every fused multiply-add is the explicit one of the device code
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-o", exe,
                    os.path.join(HERE, "lu_panel_order.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "double mismatches 0, float mismatches 0" in r.stdout
