"""The bounds-checked build (GBCHEM_CHECKED): every index the kernels take from the
mechanism's tables or from a queue is checked.  On the reference's mechanisms (the common
rate forms, the less common ones, the largest mechanism) the kinetics and integrator
kernels (the dense and the Krylov paths, FP64 and FP32) record no violation, and the checks
change no result: the checked library's outputs equal the normal library's bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import DATA, MECHS, ROOT, gpu_solution, random_states

pytestmark = pytest.mark.gpu

SCRIPT = r'''
import ctypes, os, sys
import numpy as np
sys.path.insert(0, {root!r})
sys.path.insert(0, os.path.join({root!r}, "tests"))
import cantera_gb300 as gb
from conftest import DATA, MECHS, random_states
assert gb.CHECKED and "_build_checked" in gb.LIB_PATH
out = {{}}
L = gb.library()
for name in ("gri30", "nDodecane", "pdep"):
    f, ph = MECHS[name]
    sol = gb.Solution(os.path.join(DATA, f), ph)
    T, P, Y = random_states(sol.n_species, 200, seed=41)
    out[name + "_w"] = sol.net_production_rates(T, P, Y)
    out[name + "_j"] = sol.net_production_rates_ddCi(T, P, Y)
    rng = np.random.default_rng(5)
    n = 24
    T0 = rng.uniform(1000.0, 1500.0, n)
    Pn = np.full(n, 2e5)
    Y0 = np.tile(Y[:, :1], (1, n)) if name == "pdep" else None
    if Y0 is None:
        fuel = "CH4:1" if name == "gri30" else "c12h26:1"
        ox = "O2:1, N2:3.76" if name == "gri30" else "o2:1, n2:3.76"
        Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, fuel, ox) for p in rng.uniform(0.6, 1.4, n)]).T.copy()
    for lu in (64, 32):
        net = gb.ReactorNet(sol, T0, Pn, Y0, rtol=1e-8, lu_precision=lu)
        net.advance(2e-4)
        T1, Y1 = net.get_state()
        out["%s_T%d" % (name, lu)], out["%s_Y%d" % (name, lu)] = T1, Y1
        net = gb.ReactorNet(sol, T0, Pn, Y0, rtol=1e-8, lu_precision=lu, linear_solver="GMRES")
        net.advance(2e-4)
        T1, Y1 = net.get_state()
        out["%s_Tk%d" % (name, lu)], out["%s_Yk%d" % (name, lu)] = T1, Y1
    st = np.zeros(3, dtype=np.int32)
    rc = L.gb_check_status(sol._h, st.ctypes.data_as(ctypes.c_void_p))
    out[name + "_chk"] = np.array([rc] + st.tolist())
np.savez({out!r}, **out)
'''


def _normal(name):
    import cantera_gb300 as gb
    f, ph = MECHS[name]
    sol = gpu_solution(name)
    T, P, Y = random_states(sol.n_species, 200, seed=41)
    res = {name + "_w": sol.net_production_rates(T, P, Y), name + "_j": sol.net_production_rates_ddCi(T, P, Y)}
    rng = np.random.default_rng(5)
    n = 24
    T0 = rng.uniform(1000.0, 1500.0, n)
    Pn = np.full(n, 2e5)
    if name == "pdep":
        Y0 = np.tile(Y[:, :1], (1, n))
    else:
        fuel = "CH4:1" if name == "gri30" else "c12h26:1"
        ox = "O2:1, N2:3.76" if name == "gri30" else "o2:1, n2:3.76"
        Y0 = np.array([sol.equivalence_ratio_mass_fractions(p, fuel, ox) for p in rng.uniform(0.6, 1.4, n)]).T.copy()
    for lu in (64, 32):
        net = gb.ReactorNet(sol, T0, Pn, Y0, rtol=1e-8, lu_precision=lu)
        net.advance(2e-4)
        T1, Y1 = net.get_state()
        res["%s_T%d" % (name, lu)], res["%s_Y%d" % (name, lu)] = T1, Y1
        net = gb.ReactorNet(sol, T0, Pn, Y0, rtol=1e-8, lu_precision=lu, linear_solver="GMRES")
        net.advance(2e-4)
        T1, Y1 = net.get_state()
        res["%s_Tk%d" % (name, lu)], res["%s_Yk%d" % (name, lu)] = T1, Y1
    return res


def test_checked_build_records_nothing_and_changes_nothing(tmp_path):
    import cantera_gb300 as gb
    from cantera_gb300 import build
    build.build(checked=True)
    out = str(tmp_path / "checked.npz")
    script = tmp_path / "run_checked.py"
    script.write_text(SCRIPT.format(root=ROOT, out=out))
    env = dict(os.environ, GBCHEM_CHECKED="1")
    env.pop("GBCHEM_LIB", None)
    r = subprocess.run([sys.executable, str(script)], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    chk = np.load(out)
    for name in ("gri30", "nDodecane", "pdep"):
        rc, site, idx, bound = chk[name + "_chk"].tolist()
        assert rc == 1, "the checked library must report a checked build"
        assert site == 0, (name, site, idx, bound)
        normal = _normal(name)
        for k, v in normal.items():
            assert np.array_equal(chk[k], v), k
    # the normal library reports no checks
    st = np.zeros(3, dtype=np.int32)
    assert gb.library().gb_check_status(gpu_solution("h2o2")._h, gb._ptr(st)) == 0
