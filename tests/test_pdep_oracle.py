"""The less common rate forms in the oracle and the loader (no GPU): pressure-dependent
Arrhenius (PLOG) and Chebyshev against the known answers of the reference's
test/kinetics/pdep.cpp, chemically activated falloff against test/python/test_kinetics.py
(TestChemicallyActivated), SRI and Tsang falloff against a direct evaluation of the
formulas of src/kinetics/Falloff.cpp, and the loader's handling of the reference's test
mechanisms (sections in other files, explicit units, deprecated and invalid forms)."""
import math

import numpy as np
import pytest

from conftest import MECHS, oracle_mech


def pdep_state(m, X):
    x = np.zeros(m.K)
    for item in X.split(","):
        n, v = item.split(":")
        x[m.species_index(n.strip())] = float(v)
    return m.mole_to_mass(x / x.sum())


def test_pdep_known_answers(goldens):
    """Every EXPECT_NEAR of pdep.cpp: PLOG low / high pressure limits, duplicate-pressure
    sums, exact-pressure corners and Chemkin rates of progress at intermediate pressures;
    Chebyshev rate constants (RMG-py), rates of progress (Chemkin) and range edges, and the
    'molec' quantity units of reaction 7."""
    g = goldens["pdep"]
    m = oracle_mech("pdep")
    assert m.R == 7
    Y = pdep_state(m, g["X"])
    assert len(g["cases"]) == 35
    for c in g["cases"]:
        r = m.rates(c["T"], c["P"], Y)
        if c["quantity"] == "kf_ratio":
            got = r["kf"][c["index"]] - r["kf"][c["other"]] / c["factor"]
            assert abs(got) <= c["tol"], c
        else:
            got = r[c["quantity"]][c["index"]]
            assert abs(got - c["expected"]) <= c["tol"], (c, got)


def test_chemically_activated_known_answers(goldens):
    g = goldens["chemact"]
    m = oracle_mech("chemact")
    Y = m.mole_to_mass(np.array(g["X"]) / np.sum(g["X"]))
    for P, rf in zip(g["P"], g["ropf"]):
        got = m.rates(g["T"], P, Y)["ropf"][0]
        assert abs(got / rf - 1) < g["rel"], (P, got, rf)


# ---- SRI and Tsang: the formulas evaluated directly --------------------------------------
R_CAL = 6.02214076e26 * 1.380649e-23 / 4184.0     # cal/mol/K


def arr(A, b, Ea_cal, T):
    return A * T ** b * math.exp(-Ea_cal / (R_CAL * T))


def falloff_direct(T, M, hi, lo, F):
    klow, khigh = arr(*lo, T), arr(*hi, T)
    pr = M * klow / (khigh + 1e-300)
    return khigh * pr / (1 + pr) * F(T, pr)


def sri_F(a, b, c, d=1.0, e=0.0):
    def F(T, pr):
        lpr = math.log10(max(pr, 1e-300))
        x = a * math.exp(-b / T) + (math.exp(-T / c) if c != 0 else 0.0)
        return x ** (1.0 / (1.0 + lpr * lpr)) * d * T ** e
    return F


def tsang_F(a, b=0.0):
    def F(T, pr):
        lfc = math.log10(max(a + b * T, 1e-300))
        lpr = math.log10(max(pr, 1e-300))
        cc, nn = -0.4 - 0.67 * lfc, 0.75 - 1.27 * lfc
        f1 = (lpr + cc) / (nn - 0.14 * (lpr + cc))
        return 10 ** (lfc / (1 + f1 * f1))
    return F


@pytest.mark.parametrize("T", [400.0, 900.0, 1600.0, 2500.0])
@pytest.mark.parametrize("P", [1e3, 101325.0, 1e7])
def test_sri_falloff_direct(T, P):
    """sri-falloff.yaml (SI units, activation energies in cal/mol): 3- and 5-parameter SRI;
    reaction 2 has a zero efficiency for R1A."""
    m = oracle_mech("sri")
    Y = np.linspace(1, 2, m.K)
    Y /= Y.sum()
    r = m.rates(T, P, Y)
    X = Y / m.mw
    X /= X.sum()
    ctot = P / (8314.46261815324 * T)
    c = {n: X[m.species_index(n)] * ctot for n in ["P2A", "R3", "P1", "R1A"]}
    M1 = ctot + 4.0 * c["P2A"] + 1.0 * c["R3"]
    M2 = ctot - 0.6 * c["P1"] - 1.0 * c["R1A"] + 2.0 * c["R3"]
    k1 = falloff_direct(T, M1, (1e15, -2.0, 1000.0), (4e19, -3.0, 0.0), sri_F(0.54, 201.0, 1024.0))
    k2 = falloff_direct(T, M2, (4e15, -0.5, 100.0), (7e20, -1.0, 0.0), sri_F(1.1, 700.0, 1234.0, 56.0, 0.7))
    assert r["kf"][0] == pytest.approx(k1, rel=1e-12)
    assert r["kf"][1] == pytest.approx(k2, rel=1e-12)


@pytest.mark.parametrize("T", [400.0, 900.0, 1600.0, 2500.0])
@pytest.mark.parametrize("P", [1e3, 101325.0, 1e7])
def test_tsang_falloff_direct(T, P):
    """tsang-falloff.yaml: its species come from gri30.yaml ('gri30.yaml/species: [...]'),
    found through the data directory."""
    m = oracle_mech("tsang")
    assert m.K == 10 and m.R == 2
    Y = np.linspace(1, 2, m.K)
    Y /= Y.sum()
    r = m.rates(T, P, Y)
    X = Y / m.mw
    X /= X.sum()
    ctot = P / (8314.46261815324 * T)
    c = {n: X[m.species_index(n)] * ctot for n in ["CO2", "H2O", "N2", "N2O"]}
    M1 = ctot + 0.5 * c["CO2"] + 7.3 * c["H2O"] + 4.0 * c["N2O"]
    M2 = ctot + 0.6 * c["CO2"] + 4.0 * c["H2O"] + 4.0 * c["N2O"]
    k1 = falloff_direct(T, M1, (1.988e12 * 1e-3, -0.05, -721.0), (5.08e23 * 1e-6, -2.51, -67.6), tsang_F(0.62, 0.0))
    k2 = falloff_direct(T, M2, (8.3e17, -0.93, 1.238e5), (3.57e26 * 1e-3, -2.6, 1.249e5), tsang_F(0.95, -1.0e-4))
    assert r["kf"][0] == pytest.approx(k1, rel=1e-12)
    assert r["kf"][1] == pytest.approx(k2, rel=1e-12)


@pytest.mark.parametrize("name", ["sri", "tsang", "chemact"])
def test_falloff_forms_analytic_jacobian_matches_reference_scheme(name):
    """The analytic d k/d[M] of SRI, Tsang and chemically activated falloff against the
    reference's one-sided difference in [M] (MultiRate.h:135-165)."""
    m = oracle_mech(name)
    rng = np.random.default_rng(7)
    for _ in range(8):
        T = rng.uniform(500, 2500)
        P = 101325.0 * 10 ** rng.uniform(-1, 2)
        Y = rng.dirichlet(0.5 * np.ones(m.K))
        Ja = m.ddci(T, P, Y, mode=1)
        Jr = m.ddci(T, P, Y, mode=0)
        scale = np.max(np.abs(Ja))
        assert np.max(np.abs(Ja - Jr)) <= 1e-6 * scale


def test_plog_and_chebyshev_jacobian_is_mass_action():
    """ddCi holds P fixed, so a PLOG or Chebyshev reaction differentiates like an elementary
    one: d wdot_P1 / d c_R1A = kf_1 c_R1B (P1 appears only in reaction 1, R1A + R1B <=> P1 + H),
    and likewise for the Chebyshev reaction 5 (R5 + H <=> P5A + P5B)."""
    m = oracle_mech("pdep")
    Y = np.linspace(1, 3, m.K)
    Y /= Y.sum()
    T, P = 1200.0, 5e5
    J = m.ddci(T, P, Y, mode=1)
    assert np.array_equal(J, m.ddci(T, P, Y, mode=0))   # no falloff: both schemes agree
    kf = m.rates(T, P, Y)["kf"]
    X = Y / m.mw
    c = X / X.sum() * P / (8314.46261815324 * T)
    i = m.species_index
    assert J[i("P1"), i("R1A")] == pytest.approx(kf[0] * c[i("R1B")], rel=1e-13)
    assert J[i("P5B"), i("R5")] == pytest.approx(kf[4] * c[i("H")], rel=1e-13)


def test_loader_forms():
    from oracle import pyoracle as po
    f = MECHS["pdep"][0]
    # Chebyshev written with the deprecated "(+M)": the collider is dropped
    dep = po.Mech(f, "chebyshev-deprecated")
    assert dep.R == 1
    full = oracle_mech("pdep")
    Yd = np.linspace(1, 2, dep.K)
    Yd /= Yd.sum()
    assert dep.rates(1100.0, 2e6, Yd)["kf"][0] == pytest.approx(full.rates(1100.0, 2e6, Yd)["kf"][6], rel=1e-14)
    # PLOG with an explicit "+ M" is an error
    with pytest.raises(RuntimeError, match="superfluous 'M'"):
        po.Mech(f, "plog-invalid")


def test_unit_expressions_in_yaml(tmp_path):
    """Explicit units on A ('cm^3/molec/s', 'm^3/kmol/s'), activation energies ('kJ/mol',
    'K', 'eV') and PLOG pressures ('bar', 'Pa', 'atm') load to the same rate constants as
    the plain SI numbers."""
    from oracle import pyoracle as po
    head = open(MECHS["pdep"][0]).read().split("reactions:\n- equation")[0]
    head = head.replace("units: {length: cm, time: s, quantity: mol, activation-energy: cal/mol}", "")
    A = 2.5e10   # m^3/kmol/s
    Ea_J = 4.0e7  # J/kmol
    forms = [
        "{A: %r, b: 0.5, Ea: %r}" % (A, Ea_J),
        "{A: %r cm^3/molec/s, b: 0.5, Ea: %r kJ/mol}" % (A * 1e6 / 6.02214076e26, Ea_J / 1e6),
        "{A: %r m^3/kmol/s, b: 0.5, Ea: %r K}" % (A, Ea_J / 8314.46261815324),
        "{A: %r, b: 0.5, Ea: %r eV}" % (A, Ea_J / 6.02214076e26 / 1.602176634e-19),
    ]
    ks = []
    for i, fm in enumerate(forms):
        p = tmp_path / ("u%d.yaml" % i)
        p.write_text(head + "reactions:\n- equation: R1A + R1B => P1 + H\n  rate-constant: " + fm + "\n")
        mm = po.Mech(str(p), "gas")
        ks.append(mm.rates(1000.0, 101325.0, np.ones(mm.K) / mm.K)["kf"][0])
    assert np.allclose(ks, ks[0], rtol=1e-13, atol=0)
    plog = []
    for pa, pb in [("1.0 bar", "10.0 bar"), ("1e5 Pa", "1e6 Pa"), ("%r atm" % (1e5 / 101325), "%r atm" % (1e6 / 101325))]:
        p = tmp_path / "pl.yaml"
        p.write_text(head + "reactions:\n- equation: R1A + R1B => P1 + H\n  type: pressure-dependent-Arrhenius\n"
                     "  rate-constants:\n  - {P: %s, A: 1e10, b: 0, Ea: 0}\n  - {P: %s, A: 1e12, b: 0, Ea: 0}\n" % (pa, pb))
        mm = po.Mech(str(p), "gas")
        plog.append(mm.rates(1000.0, 3e5, np.ones(mm.K) / mm.K)["kf"][0])
    assert np.allclose(plog, plog[0], rtol=1e-12, atol=0)
    # geometric interpolation between the two levels
    assert plog[0] == pytest.approx(1e10 * 100 ** (math.log(3.0) / math.log(10.0)), rel=1e-12)
