import functools
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
DATA = os.path.join(ROOT, "cantera_gb300", "data")
GOLDEN = os.path.join(ROOT, "tests", "golden")
MECHS = {"h2o2": ("h2o2.yaml", "ohmech"), "gri30": ("gri30.yaml", "gri30"),
         "nDodecane": ("nDodecane_Reitz.yaml", "nDodecane_IG"),
         # the reference's test mechanisms for the less common rate forms (tests/golden)
         "pdep": (os.path.join(GOLDEN, "pdep-test.yaml"), "gas"),
         "chemact": (os.path.join(GOLDEN, "chemically-activated-reaction.yaml"), "gas"),
         "sri": (os.path.join(GOLDEN, "sri-falloff.yaml"), "gas"),
         "tsang": (os.path.join(GOLDEN, "tsang-falloff.yaml"), "gas")}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@functools.lru_cache(maxsize=None)
def oracle_mech(name):
    from oracle import pyoracle as po
    f, ph = MECHS[name]
    return po.Mech(os.path.join(DATA, f), ph)


@functools.lru_cache(maxsize=None)
def gpu_solution(name):
    import cantera_gb300 as gb
    f, ph = MECHS[name]
    return gb.Solution(os.path.join(DATA, f), ph)


def random_states(K, n, seed, Tlo=300.0, Thi=3000.0):
    """Rate-evaluation inputs: T uniform, P log-uniform 0.1-100 atm, Y ~ Dirichlet(0.5)."""
    rng = np.random.default_rng(seed)
    T = rng.uniform(Tlo, Thi, n)
    P = 101325.0 * 10 ** rng.uniform(-1, 2, n)
    Y = rng.dirichlet(0.5 * np.ones(K), n).T.copy()
    return T, P, Y


@pytest.fixture(scope="session")
def goldens():
    import json
    return json.load(open(os.path.join(ROOT, "tests", "golden", "goldens.json")))
