"""The C ABI library: it loads, exports every symbol include/gbchem.h declares, and
reports errors through GB_ERR + gb_get_error (no GPU work in these tests)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gbchem.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_\w+)\s*\(", src)))


def test_exports_every_declared_symbol():
    import cantera_gb300 as gb
    L = gb.library()
    names = _declared()
    assert "gb_net_advance" in names and "gb_kin_net_production_rates_ddCi" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_error_convention(tmp_path):
    import cantera_gb300 as gb
    L = gb.library()
    h = L.gb_mech_load(os.path.join(str(tmp_path), "nope.yaml").encode(), b"")
    assert h == gb.GB_ERR
    buf = ctypes.create_string_buffer(512)
    n = L.gb_get_error(512, buf)
    assert n > 0 and "nope.yaml" in buf.value.decode()
    assert L.gb_net_advance(12345, 1.0) == gb.GB_ERR
    L.gb_get_error(512, buf)
    assert "handle" in buf.value.decode()
    assert L.gb_mech_n_species(-1) == gb.GB_ERR
