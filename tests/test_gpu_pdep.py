"""The less common rate forms on the GPU (PLOG, Chebyshev, SRI, Tsang, chemically activated
falloff): rates of progress against the reference's known answers (test/kinetics/pdep.cpp,
test/python/test_kinetics.py), net production rates and d(wdot)/dc against the oracle on
the reference's test mechanisms, and the batched integrator on h2o2 variants that use each
form, against the oracle's integrator."""
import math
import os

import numpy as np
import pytest

from conftest import DATA, MECHS, gpu_solution, oracle_mech, random_states

pytestmark = pytest.mark.gpu
WDOT_TOL = 1e-12
JAC_TOL = 1e-12
R_GAS = 8314.46261815324
# pdep-test.yaml: reactants of each reaction and a product that appears in no other one
PDEP_REACTANTS = [["R1A", "R1B"], ["H", "R2"], ["H", "R3"], ["H", "R4"], ["R5", "H"], ["R6"], ["R7", "H"]]
PDEP_PRODUCT = ["P1", "P2B", "P3B", "P4", "P5B", "P6B", "P7B"]


def mole_state(sol, spec):
    x = np.zeros(sol.n_species)
    for item in spec.split(","):
        n, v = item.split(":")
        x[sol.species_names.index(n.strip())] = float(v)
    x /= x.sum()
    y = x * sol.molecular_weights
    return x, y / y.sum()


def test_pdep_known_answers_on_gpu(goldens):
    """Forward rates of progress from the GPU's net production rates: with every product
    at zero concentration, wdot of a product unique to reaction i is ropf_i; kf_i follows by
    dividing by the reactant concentrations."""
    g = goldens["pdep"]
    sol = gpu_solution("pdep")
    x_ref, y_ref = mole_state(sol, g["X"])
    x_all, y_all = mole_state(sol, g["X"] + ", R7:1.0")
    idx = sol.species_names.index
    for c in g["cases"]:
        T, P = c["T"], c["P"]
        use_all = c["quantity"] != "ropf"
        x, y = (x_all, y_all) if use_all else (x_ref, y_ref)
        w = sol.net_production_rates(np.array([T]), np.array([P]), y[:, None].copy())[:, 0]
        conc = x * P / (R_GAS * T)

        def kf(i):
            return w[idx(PDEP_PRODUCT[i])] / np.prod([conc[idx(s)] for s in PDEP_REACTANTS[i]])
        if c["quantity"] == "ropf":
            assert abs(w[idx(PDEP_PRODUCT[c["index"]])] - c["expected"]) <= c["tol"], c
        elif c["quantity"] == "kf":
            assert abs(kf(c["index"]) - c["expected"]) <= max(c["tol"], 1e-12 * c["expected"]), c
        else:
            assert abs(kf(c["index"]) - kf(c["other"]) / c["factor"]) <= c["tol"], c


def test_chemically_activated_known_answers_on_gpu(goldens):
    g = goldens["chemact"]
    sol = gpu_solution("chemact")
    x = np.array(g["X"]) / np.sum(g["X"])
    y = x * sol.molecular_weights
    y /= y.sum()
    # ch3 + oh (+M) <=> ch2o + h2 (+M), products absent: wdot(h2) = ropf
    k = sol.species_names.index("h2")
    for P, rf in zip(g["P"], g["ropf"]):
        w = sol.net_production_rates(np.array([g["T"]]), np.array([P]), y[:, None].copy())[:, 0]
        assert abs(w[k] / rf - 1) < g["rel"], (P, w[k], rf)


@pytest.mark.parametrize("name", ["pdep", "sri", "tsang", "chemact"])
def test_rates_and_jacobian_match_oracle(name):
    sol, m = gpu_solution(name), oracle_mech(name)
    # within the Chebyshev fits' temperature ranges (300-2000 K)
    T, P, Y = random_states(m.K, 2000, seed=21, Tlo=300.0, Thi=2000.0)
    w = sol.net_production_rates(T, P, Y)
    wo, _, gross = m.rates_batch(T, P, Y, gross=True)
    err = np.abs(w - wo)
    assert np.all(err <= WDOT_TOL * gross + 1e-300), np.max(err / (gross + 1e-300))
    J = sol.net_production_rates_ddCi(T[:300], P[:300], Y[:, :300].copy())
    pat = (sol.jac_colptr, sol.jac_rowidx)
    _, Jo = m.rates_batch(T[:300], P[:300], Y[:, :300].copy(), mode=1, pattern=pat)
    scale = np.max(np.abs(Jo), axis=0)
    assert np.all(np.max(np.abs(J - Jo), axis=0) <= JAC_TOL * scale)
    _, Jr = m.rates_batch(T[:300], P[:300], Y[:, :300].copy(), mode=0, pattern=pat)
    assert np.all(np.max(np.abs(J - Jr), axis=0) <= 1e-6 * scale)


def test_pressure_edges_on_gpu():
    """PLOG below the first and above the last pressure (the end levels), at a given
    pressure exactly, and Chebyshev at the ends of its ranges, against the oracle."""
    sol, m = gpu_solution("pdep"), oracle_mech("pdep")
    P = np.array([1e-7, 1.0, 0.01 * 101325, 101325.0, 10 * 101325, 100 * 101325, 1e10, 1e3, 1e7])
    T = np.linspace(300.0, 2000.0, len(P))
    Y = np.ones((m.K, len(P))) / m.K
    w = sol.net_production_rates(T, P, Y)
    wo, _, gross = m.rates_batch(T, P, Y, gross=True)
    assert np.all(np.abs(w - wo) <= WDOT_TOL * gross + 1e-300)


# ---- the integrator on h2o2 variants ------------------------------------------------------
def _cheb_fit(A, b, Ea, Tmin=300.0, Tmax=3000.0, nT=6, p_slope=0.02):
    """Chebyshev coefficients (file units) reproducing A T^b exp(-Ea/RT) over [Tmin, Tmax],
    with a weak pressure dependence in the second pressure column."""
    R_cal = 6.02214076e26 * 1.380649e-23 / 4184.0
    Tg = np.linspace(Tmin, Tmax, 200)
    Tr = (2 / Tg - 1 / Tmin - 1 / Tmax) / (1 / Tmax - 1 / Tmin)
    logk = np.log10(A * Tg ** b * np.exp(-Ea / (R_cal * Tg)))
    c = np.polynomial.chebyshev.chebfit(Tr, logk, nT - 1)
    return [[float(v), p_slope if i == 0 else 0.0] for i, v in enumerate(c)]


def h2o2_variant(tmp_path, form):
    src = open(os.path.join(DATA, "h2o2.yaml")).read()
    troe = "  Troe: {A: 0.7346, T3: 94.0, T1: 1756.0, T2: 5182.0}\n"
    assert troe in src
    if form == "plog_cheb_sri":
        src = src.replace("- equation: H + O2 <=> O + OH  # Reaction 11\n  rate-constant: {A: 2.65e+16, b: -0.6707, Ea: 1.7041e+04}\n",
                          "- equation: H + O2 <=> O + OH  # Reaction 11\n  type: pressure-dependent-Arrhenius\n"
                          "  rate-constants:\n"
                          "  - {P: 0.1 atm, A: 2.12e+16, b: -0.6707, Ea: 1.7041e+04}\n"
                          "  - {P: 1.0 atm, A: 2.65e+16, b: -0.6707, Ea: 1.7041e+04}\n"
                          "  - {P: 10.0 atm, A: 2.65e+16, b: -0.6707, Ea: 1.7041e+04}\n"
                          "  - {P: 10.0 atm, A: 6.6e+15, b: -0.6707, Ea: 1.7041e+04}\n")
        rows = _cheb_fit(2.16e+08, 1.51, 3430.0)
        src = src.replace("- equation: OH + H2 <=> H + H2O  # Reaction 21\n  rate-constant: {A: 2.16e+08, b: 1.51, Ea: 3430.0}\n",
                          "- equation: OH + H2 <=> H + H2O  # Reaction 21\n  type: Chebyshev\n"
                          "  temperature-range: [300.0, 3000.0]\n  pressure-range: [0.01 atm, 100.0 atm]\n"
                          "  data:\n" + "".join("  - [%r, %r]\n" % (a, b) for a, b in rows))
        src = src.replace(troe, "  SRI: {A: 0.45, B: 300.0, C: 900.0, D: 1.2, E: 0.05}\n")
    elif form == "tsang":
        src = src.replace(troe, "  Tsang: {A: 0.55, B: 1.0e-4}\n")
    elif form == "chemact":
        src = src.replace("  type: falloff\n  low-P-rate-constant: {A: 2.3e+18, b: -0.9, Ea: -1700.0}\n"
                          "  high-P-rate-constant: {A: 7.4e+13, b: -0.37, Ea: 0.0}\n",
                          "  type: chemically-activated\n  low-P-rate-constant: {A: 7.4e+13, b: -0.37, Ea: 0.0}\n"
                          "  high-P-rate-constant: {A: 4.0e+7, b: 0.1, Ea: 1000.0}\n")
    p = tmp_path / ("h2o2-%s.yaml" % form)
    p.write_text(src)
    return str(p)


@pytest.mark.parametrize("form", ["plog_cheb_sri", "tsang", "chemact"])
def test_integrator_with_rate_forms_matches_oracle(tmp_path, form):
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    path = h2o2_variant(tmp_path, form)
    sol, m = gb.Solution(path, "ohmech"), po.Mech(path, "ohmech")
    rtol, atol = 1e-8, 1e-15
    rng = np.random.default_rng(31)
    n = 48
    T0 = rng.uniform(1000, 1600, n)
    P = 101325.0 * 10 ** rng.uniform(-0.5, 1.0, n)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in phi])
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol)
    assert net.advance(1e-3) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, 1e-3, po.opts(rtol=rtol, atol=atol, analytic=True))
    assert np.all(sto[:, 8] == 0) and np.all(net.status == 0)
    assert np.max(np.abs(T - To) / To) < 10 * rtol
    d = np.abs(Y.T - Yo)
    major = Yo >= 1e-3
    assert np.max(d[major] / Yo[major]) < 10 * rtol
    assert np.max(np.abs(net.ignition_times - tio) / tio) < 1e-3
    # the variant really differs from the stock mechanism (at a state with radicals present)
    base = gpu_solution("h2o2")
    Tr, Pr, Yr = np.array([1100.0, 1300.0]), np.array([5e4, 2e5]), np.full((m.K, 2), 1.0 / m.K)
    w_var = sol.net_production_rates(Tr, Pr, Yr)
    w_base = base.net_production_rates(Tr, Pr, Yr)
    assert not np.allclose(w_var, w_base, rtol=1e-6, atol=0)
    assert math.isfinite(float(np.sum(T)))


@pytest.mark.parametrize("form,lu", [("plog_cheb_sri", 64), ("plog_cheb_sri", 32), ("tsang", 64), ("chemact", 64)])
def test_krylov_path_with_rate_forms_matches_oracle(tmp_path, form, lu):
    """The Krylov path (mole reactor, GMRES, adaptive preconditioner) on mechanisms with the
    less common rate forms (their own kernel instantiation) against the oracle's GMRES path,
    with the bars of the reference's test of that solver (T 1e-5, Y 5e-4 relative + 1e-6)."""
    import cantera_gb300 as gb
    from oracle import pyoracle as po
    path = h2o2_variant(tmp_path, form)
    sol, m = gb.Solution(path, "ohmech"), po.Mech(path, "ohmech")
    rtol, atol = 1e-8, 1e-15
    rng = np.random.default_rng(37)
    n = 48
    T0 = rng.uniform(1000, 1600, n)
    P = 101325.0 * 10 ** rng.uniform(-0.5, 1.0, n)
    phi = rng.uniform(0.5, 2.0, n)
    Y0 = np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in phi])
    net = gb.ReactorNet(sol, T0, P, Y0.T.copy(), rtol=rtol, atol=atol, linear_solver="GMRES", lu_precision=lu)
    assert net.advance(1e-3) == 0
    T, Y = net.get_state()
    To, Yo, sto, tio = m.advance_batch(T0, P, Y0, 1e-3, po.opts(rtol=rtol, atol=atol, gmres=True))
    assert np.all(sto[:, 8] == 0)
    assert np.all(np.abs(T - To) <= 1e-5 * To)
    assert np.all(np.abs(Y.T - Yo) <= 5e-4 * np.abs(Yo) + 1e-6)
    # ignition delays of the reactors that ignite (a reactor that warms by a few K has its
    # largest dT/dt at the last step, wherever the step sequence puts it)
    ign = (To > T0 + 400) & (tio > 0) & (tio < 1e-3)
    assert ign.sum() >= 40
    assert np.max(np.abs(net.ignition_times[ign] - tio[ign]) / tio[ign]) < 1e-3
    assert np.all(net.krylov_stats["lin_iters"] > 0)
