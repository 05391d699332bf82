"""A mechanism with more than 128 state components: GRI-Mech 3.0 with 80 more inert species (argon's
thermodynamics under new names, part of the mixture, so that they weigh in the third-body
concentrations and the heat capacity).  Its 134 components run the integrators' widest register
layout (four 32-lane slots per vector, NS = 8) with the common rate forms, which the reference's
mechanisms here do not reach: the dense path (FP64 and FP32 Newton matrix) against the oracle
with the engine's algorithm, and the Krylov path (FP64 and FP32 factors) against the oracle's
GMRES path with the bars of the reference's test of that solver."""
import os

import numpy as np
import pytest

from conftest import DATA

pytestmark = pytest.mark.gpu

N_EXTRA = 80


def wide_gri30(tmp_path):
    src = open(os.path.join(DATA, "gri30.yaml")).read()
    names = ["XA%d" % i for i in range(N_EXTRA)]
    old_list = "    CH3CHO]\n"
    assert old_list in src
    src = src.replace(old_list, "    CH3CHO, " + ", ".join(names) + "]\n", 1)
    i = src.index("- name: AR\n")
    j = src.index("- name: ", i + 5)
    block = src[i:j]
    extra = "".join(block.replace("- name: AR\n", "- name: %s\n" % nm, 1) for nm in names)
    src = src[:j] + extra + src[j:]
    p = tmp_path / "gri30-wide.yaml"
    p.write_text(src)
    return str(p)


def _states(m, n, seed):
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(1500.0, 1800.0, n)
    P = 101325.0 * 10 ** rng.uniform(0.0, 1.0, n)
    phi = rng.uniform(0.7, 1.3, n)
    Y0 = np.array([m.equivalence_ratio(p, "CH4:1", "O2:1, N2:3.76") for p in phi])
    extra = [m.species_index("XA%d" % i) for i in range(N_EXTRA)]
    Y0 *= 0.9
    Y0[:, extra] += 0.1 / N_EXTRA          # 10 % of the mass in the inert species
    return T0, P, Y0


@pytest.fixture(scope="module")
def wide(tmp_path_factory):
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    path = wide_gri30(tmp_path_factory.mktemp("wide"))
    sol, m = gb.Solution(path, "gri30"), po.Mech(path, "gri30")
    assert sol.n_species == 53 + N_EXTRA and m.K + 1 > 128
    return sol, m


@pytest.mark.parametrize("lu", [64, 32])
def test_dense_path_wide_mechanism(wide, lu):
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = wide
    rtol, atol, t_end = 1e-8, 1e-15, 5e-3
    T0, P, Y0 = _states(m, 32, 3)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol, lu_precision=lu)
    assert net.advance(t_end) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=rtol, atol=atol, analytic=True))
    assert np.all(sto[:, 8] == 0)
    assert np.all(To > T0 + 400)                        # every reactor has ignited and settled
    assert np.max(np.abs(T - To) / To) < 10 * rtol
    major = Yo >= 1e-3
    assert np.max(np.abs(Y.T - Yo)[major] / Yo[major]) < 30 * rtol
    assert np.max(np.abs(net.ignition_times - tio) / tio) < 1e-3


@pytest.mark.parametrize("lu", [64, 32])
def test_krylov_path_wide_mechanism(wide, lu):
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    sol, m = wide
    rtol, atol, t_end = 1e-8, 1e-15, 5e-3
    T0, P, Y0 = _states(m, 32, 5)
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol, lu_precision=lu, linear_solver="GMRES")
    assert net.advance(t_end) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, t_end, po.opts(rtol=rtol, atol=atol, gmres=True))
    assert np.all(sto[:, 8] == 0) and np.all(To > T0 + 400)
    assert np.all(np.abs(T - To) <= 1e-5 * To)
    assert np.all(np.abs(Y.T - Yo) <= 5e-4 * np.abs(Yo) + 1e-6)
    assert np.max(np.abs(net.ignition_times - tio) / tio) < 1e-3
    assert np.all(net.krylov_stats["lin_iters"] > 0)
