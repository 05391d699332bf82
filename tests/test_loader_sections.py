"""Loader features for mechanisms that draw on other files or select reactions (no GPU):
species and reaction sections of another file, the 'declared-species' rule, undeclared
third-body colliders, prefixed units (reference src/thermo/ThermoFactory.cpp:262-304,
src/kinetics/KineticsFactory.cpp:108-218, src/kinetics/Reaction.cpp:858-881,
src/base/Units.cpp:138-195)."""
import os

import numpy as np
import pytest

from conftest import DATA

HEAD = """units: {length: cm, quantity: mol, activation-energy: cal/mol}
phases:
"""


def load(tmp_path, text, phase="gas"):
    from oracle import pyoracle as po
    p = tmp_path / "m.yaml"
    p.write_text(text)
    return po.Mech(str(p), phase)


def test_sections_of_another_file_and_declared_species(tmp_path):
    """Species from gri30.yaml; reactions from gri30.yaml's section with the rule
    'declared-species' keep exactly those among the declared species.  As in the reference
    (Reaction::checkSpecies -> ThirdBody::checkSpecies, src/kinetics/Reaction.cpp:731-733,
    858-881), efficiencies naming undeclared species stay an error unless the phase sets
    'skip-undeclared-third-bodies'."""
    text = HEAD + """- name: gas
  thermo: ideal-gas
  elements: [O, H, N, Ar]
  species:
  - gri30.yaml/species: [H2, H, O, O2, OH, H2O, HO2, H2O2, N2, AR]
  kinetics: gas
  reactions:
  - gri30.yaml/reactions: declared-species
"""
    with pytest.raises(RuntimeError, match="third-body efficiencies for undeclared species"):
        load(tmp_path, text)
    m = load(tmp_path, text + "  skip-undeclared-third-bodies: true\n")
    assert m.K == 10
    # gri30's H/O reactions among these species (its H2/O2 subset); every other reaction names
    # a carbon or nitrogen species that is not declared
    assert 25 <= m.R <= 40
    full = load(tmp_path, HEAD + """- name: gas
  thermo: ideal-gas
  species: [{gri30.yaml/species: all}]
  kinetics: gas
  reactions: [{gri30.yaml/reactions: all}]
""")
    assert full.K == 53 and full.R == 325


def test_undeclared_species_are_errors_unless_declared_species(tmp_path):
    text = HEAD + """- name: gas
  thermo: ideal-gas
  species: [{gri30.yaml/species: [H2, O2, H, O, OH, N2]}]
  kinetics: gas
  reactions: [{gri30.yaml/reactions: all}]
"""
    with pytest.raises(RuntimeError, match="undeclared species"):
        load(tmp_path, text)


def test_undeclared_third_bodies(tmp_path):
    """Efficiencies naming an undeclared species are an error; with
    'skip-undeclared-third-bodies' they are ignored for '+ M' reactions."""
    species = """species:
- name: H
  composition: {H: 1}
  thermo: {model: NASA7, temperature-ranges: [200.0, 3500.0], data: [[2.5, 0, 0, 0, 0, 25473.7, -0.447]]}
- name: H2
  composition: {H: 2}
  thermo: {model: NASA7, temperature-ranges: [200.0, 3500.0], data: [[3.3, 0, 0, 0, 0, -1012.5, -3.29]]}
reactions:
- equation: 2 H + M <=> H2 + M
  type: three-body
  rate-constant: {A: 1.0e+18, b: -1.0, Ea: 0.0}
  efficiencies: {H2: 0.0, AR: 0.63}
"""
    base = HEAD + """- name: gas
  thermo: ideal-gas
  elements: [H]
  species: [H, H2]
  kinetics: gas
"""
    with pytest.raises(RuntimeError, match="undeclared species"):
        load(tmp_path, base + species)
    m = load(tmp_path, base + "  skip-undeclared-third-bodies: true\n" + species)
    assert m.R == 1
    r = m.rates(1500.0, 101325.0, np.array([0.5, 0.5]))
    assert np.isfinite(r["kf"][0]) and r["kf"][0] > 0


@pytest.mark.parametrize("pressure", ["1.0 bar", "100.0 kPa", "0.1 MPa", "1.0e6 dyn/cm^2", "1e5"])
def test_prefixed_pressure_units(tmp_path, pressure):
    """PLOG pressures in any pressure unit (SI prefixes included) or, as a plain number, in Pa."""
    text = HEAD + """- name: gas
  thermo: ideal-gas
  elements: [H]
  species: [H, H2]
  kinetics: gas
species:
- name: H
  composition: {H: 1}
  thermo: {model: NASA7, temperature-ranges: [200.0, 3500.0], data: [[2.5, 0, 0, 0, 0, 25473.7, -0.447]]}
- name: H2
  composition: {H: 2}
  thermo: {model: NASA7, temperature-ranges: [200.0, 3500.0], data: [[3.3, 0, 0, 0, 0, -1012.5, -3.29]]}
reactions:
- equation: H + H => H2
  type: pressure-dependent-Arrhenius
  rate-constants:
  - {P: %s, A: 1.0e+12, b: 0.0, Ea: 0.0}
  - {P: 1.0e7 Pa, A: 1.0e+14, b: 0.0, Ea: 0.0}
""" % pressure
    m = load(tmp_path, text)
    kf = m.rates(1000.0, 1e6, np.array([0.5, 0.5]))["kf"][0]
    # ln k linear in ln P between 1e5 and 1e7 Pa: halfway, the geometric mean (cm^3/mol/s -> m^3/kmol/s)
    assert kf == pytest.approx(1e13 * 1e-3, rel=1e-12)
    assert os.path.exists(os.path.join(DATA, "gri30.yaml"))


def test_unknown_unit_is_an_error(tmp_path):
    text = HEAD + """- name: gas
  thermo: ideal-gas
  elements: [H]
  species: [H, H2]
  kinetics: gas
species:
- name: H
  composition: {H: 1}
  thermo: {model: NASA7, temperature-ranges: [200.0, 3500.0], data: [[2.5, 0, 0, 0, 0, 25473.7, -0.447]]}
- name: H2
  composition: {H: 2}
  thermo: {model: NASA7, temperature-ranges: [200.0, 3500.0], data: [[3.3, 0, 0, 0, 0, -1012.5, -3.29]]}
reactions:
- equation: H + H => H2
  rate-constant: {A: 1.0e+12 cm^3/furlong/s, b: 0.0, Ea: 0.0}
"""
    with pytest.raises(RuntimeError, match="unknown unit"):
        load(tmp_path, text)
