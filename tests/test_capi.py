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


def test_error_paths_of_the_network_settings_and_data_directories():
    import cantera_gb300 as gb
    L = gb.library()
    buf = ctypes.create_string_buffer(512)
    for rc in (L.gb_net_set_tolerances(12345, 1e-8, 1e-15), L.gb_net_set_max_steps(12345, 100),
               L.gb_net_set_max_time_step(12345, 1e-3)):
        assert rc == gb.GB_ERR
        L.gb_get_error(512, buf)
        assert "handle" in buf.value.decode()
    assert L.gb_add_data_directory(None) == gb.GB_ERR
    assert L.gb_add_data_directory(gb.DATA_DIR.encode()) == 0
