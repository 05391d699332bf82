"""Mechanism loader: the YAML subset, reaction classification and unit handling
(reference semantics: src/kinetics/Reaction.cpp:389-555,576-617; src/base/Units.cpp)."""
import os

import numpy as np
import pytest

from conftest import DATA, oracle_mech

R_GAS = 6.02214076e26 * 1.380649e-23


def test_counts():
    for name, K, R in [("h2o2", 10, 29), ("gri30", 53, 325), ("nDodecane", 100, 553)]:
        m = oracle_mech(name)
        assert (m.K, m.R) == (K, R)


def test_three_body_and_units_h2o2():
    m = oracle_mech("h2o2")
    # 2 O + M <=> O2 + M: third order, 1.2e17 cm^6/mol^2/s -> 1.2e11 m^6/kmol^2/s
    T, P = 1500.0, 101325.0
    Y = np.full(m.K, 0.1)
    r = m.rates(T, P, Y)
    assert r["kf"][0] == pytest.approx(1.2e11 / T, rel=1e-14)
    # O + H2 <=> H + OH: 3.87e4 cm^3/mol/s * T^2.7 exp(-6260 cal/mol / RT)
    kf = 3.87e4 * 1e-3 * T ** 2.7 * np.exp(-6260.0 * 4184.0 / R_GAS / T)
    assert r["kf"][2] == pytest.approx(kf, rel=1e-13)
    # H + 2 O2 <=> HO2 + O2 is a three-body reaction with collider O2: rop = kf [O2] [H] [O2]
    c = Y / m.mw * (P * (1.0 / np.sum(Y / m.mw)) / (R_GAS * T))
    kH, kO2 = m.species_index("H"), m.species_index("O2")
    assert r["ropf"][6] == pytest.approx(r["kf"][6] * c[kO2] * c[kH] * c[kO2], rel=1e-13)


def test_troe_matches_formula():
    m = oracle_mech("h2o2")
    T, P = 1200.0, 5 * 101325.0
    Y = np.linspace(0.05, 0.15, m.K)
    Y /= Y.sum()
    r = m.rates(T, P, Y)
    # reaction 22: 2 OH (+M) <=> H2O2 (+M), Troe {A: 0.7346, T3: 94, T1: 1756, T2: 5182}
    rho = P / (R_GAS * T) / np.sum(Y / m.mw)
    c = rho * Y / m.mw
    eff = np.ones(m.K)
    for s, e in [("H2", 2.0), ("H2O", 6.0), ("AR", 0.7)]:
        eff[m.species_index(s)] = e
    M = np.sum(eff * c)
    k0 = 2.3e18 * 1e-6 * T ** -0.9 * np.exp(1700.0 * 4184.0 / R_GAS / T)
    kinf = 7.4e13 * 1e-3 * T ** -0.37
    Pr = k0 * M / kinf
    Fc = (1 - 0.7346) * np.exp(-T / 94.0) + 0.7346 * np.exp(-T / 1756.0) + np.exp(-5182.0 / T)
    lFc = np.log10(Fc)
    cc, nn = -0.4 - 0.67 * lFc, 0.75 - 1.27 * lFc
    f1 = (np.log10(Pr) + cc) / (nn - 0.14 * (np.log10(Pr) + cc))
    F = 10 ** (lFc / (1 + f1 ** 2))
    assert r["kf"][21] == pytest.approx(kinf * Pr / (1 + Pr) * F, rel=1e-12)


def test_reversibility_and_equilibrium():
    m = oracle_mech("gri30")
    T, P = 1800.0, 2 * 101325.0
    Y = np.full(m.K, 1.0 / m.K)
    r = m.rates(T, P, Y)
    assert np.all(r["rkc"][r["rkc"] != 0] > 0)
    # wdot = nu . ropnet (Kinetics::getNetProductionRates)
    assert np.isfinite(r["wdot"]).all()
    assert abs(np.sum(r["wdot"] * m.mw)) < 1e-9 * np.sum(np.abs(r["wdot"] * m.mw))


def _write(tmp_path, text):
    p = os.path.join(str(tmp_path), "m.yaml")
    open(p, "w").write(text)
    return p


def test_yaml_subset(tmp_path):
    from oracle import pyoracle as po
    text = open(os.path.join(DATA, "h2o2.yaml")).read()
    # flow collections across lines, block scalars and quotes are all in the stock file
    assert "description: |-" in text
    p = _write(tmp_path, text.replace("rate-constant: {A: 3.87e+04, b: 2.7, Ea: 6260.0}",
                                      "rate-constant: {A: 3.87e+04,\n    b: 2.7,\n    Ea: '6260.0 cal/mol'}"))
    m2 = po.Mech(p, "ohmech")
    m1 = oracle_mech("h2o2")
    Y = np.full(m1.K, 0.1)
    assert m2.rates(1300.0, 1e5, Y)["kf"][2] == pytest.approx(m1.rates(1300.0, 1e5, Y)["kf"][2], rel=1e-15)


def test_loader_errors(tmp_path):
    from oracle import pyoracle as po
    with pytest.raises(RuntimeError, match="cannot open"):
        po.Mech(os.path.join(str(tmp_path), "missing.yaml"))
    text = open(os.path.join(DATA, "h2o2.yaml")).read().replace("O + H2 <=> H + OH", "O + XX <=> H + OH")
    with pytest.raises(RuntimeError, match="undeclared species 'XX'"):
        po.Mech(_write(tmp_path, text), "ohmech")
    with pytest.raises(RuntimeError, match="only ideal-gas"):
        po.Mech(os.path.join(DATA, "h2o2.yaml"), "ohmech-RK")
