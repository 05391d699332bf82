"""The cantera-shaped facade (cantera_gb300.compat): state setters and getters, single-state
kinetics and reactor networks built from reactor objects, against the oracle."""
import numpy as np
import pytest

from conftest import gpu_solution, oracle_mech

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ct():
    import cantera_gb300.compat as ct
    return ct


def test_state_setters(ct):
    gas = ct.Solution("gri30.yaml", "gri30")
    gas.TPX = 1200.0, 2 * ct.one_atm, "CH4:1, O2:2, N2:7.52"
    assert gas.T == 1200.0 and gas.P == 2 * ct.one_atm
    X = gas.X
    assert X[gas.species_index("CH4")] == pytest.approx(1 / 10.52, rel=1e-14)
    assert np.sum(gas.Y) == pytest.approx(1.0, rel=1e-14)
    # Y and X are consistent through the molecular weights
    y = X * gas.molecular_weights
    assert np.allclose(gas.Y, y / y.sum(), rtol=1e-14, atol=0)
    # ideal gas
    assert gas.density == pytest.approx(gas.P * gas.mean_molecular_weight / (ct.gas_constant * gas.T), rel=1e-14)
    assert np.sum(gas.concentrations) == pytest.approx(gas.density_mole, rel=1e-13)
    # TP keeps the composition; TDY sets the pressure from the density
    Y0 = gas.Y
    gas.TP = 900.0, None
    assert gas.T == 900.0 and gas.P == 2 * ct.one_atm and np.array_equal(gas.Y, Y0)
    d = gas.density
    gas.TDY = 1800.0, d, None
    assert gas.P == pytest.approx(2 * ct.one_atm * 2.0, rel=1e-13)
    # dict and array compositions
    gas.TPY = 1000.0, ct.one_atm, {"H2": 1.0, "O2": 8.0}
    assert gas.Y[gas.species_index("O2")] == pytest.approx(8 / 9, rel=1e-14)
    gas.Y = np.ones(gas.n_species)
    assert np.allclose(gas.Y, 1.0 / gas.n_species)
    with pytest.raises(ValueError):
        gas.TP = -5.0, ct.one_atm


def test_equivalence_ratio_matches_oracle(ct):
    gas = ct.Solution("gri30.yaml", "gri30")
    m = oracle_mech("gri30")
    for phi in (0.5, 1.0, 1.7):
        gas.set_equivalence_ratio(phi, "CH4:1", "O2:1, N2:3.76")
        assert np.allclose(gas.Y, m.equivalence_ratio(phi, "CH4:1", "O2:1, N2:3.76"), rtol=1e-13, atol=1e-300)


def test_single_state_kinetics_match_oracle(ct):
    gas = ct.Solution("gri30.yaml", "gri30")
    m = oracle_mech("gri30")
    rng = np.random.default_rng(3)
    for _ in range(5):
        gas.TPY = rng.uniform(600, 2500), ct.one_atm * 10 ** rng.uniform(-1, 1.5), rng.dirichlet(0.5 * np.ones(gas.n_species))
        w = gas.net_production_rates
        wo, _, g = m.rates_batch(np.array([gas.T]), np.array([gas.P]), gas.Y[:, None].copy(), gross=True)
        assert np.all(np.abs(w - wo[:, 0]) <= 1e-12 * g[:, 0] + 1e-300)
        J = gas.net_production_rates_ddCi
        assert J.shape == (gas.n_species, gas.n_species) and J.format == "csc"
        Jo = m.ddci(gas.T, gas.P, gas.Y, mode=1)
        assert np.max(np.abs(J.toarray() - Jo)) <= 1e-12 * np.max(np.abs(Jo))


def test_reactor_network_matches_oracle(ct):
    from oracle import pyoracle as po
    gas = ct.Solution("h2o2.yaml", "ohmech")
    m = oracle_mech("h2o2")
    reactors = []
    rng = np.random.default_rng(8)
    T0 = rng.uniform(1000, 1500, 12)
    for i, T in enumerate(T0):
        gas.TP = T, ct.one_atm * (1 + i % 3)
        gas.set_equivalence_ratio(0.6 + 0.1 * i, "H2:1", "O2:1, N2:3.76")
        reactors.append(ct.IdealGasConstPressureReactor(gas, name="r%d" % i))
    net = ct.ReactorNet(reactors)
    rtol = 1e-8
    net.rtol, net.atol = rtol, 1e-15
    assert net.advance(1e-3) == 1e-3 and net.time == 1e-3
    T = np.array([r.T for r in reactors])
    Y = np.array([r.thermo.Y for r in reactors])
    P = np.array([r.thermo.P for r in reactors])
    Y0 = np.array([m.equivalence_ratio(0.6 + 0.1 * i, "H2:1", "O2:1, N2:3.76") for i in range(12)])
    # the facade runs exactly the batched network: bit-identical to driving it directly
    import cantera_gb300 as gb
    direct = gb.ReactorNet(gas._m, T0, P, Y0.T.copy(), rtol=rtol, atol=1e-15)
    assert direct.advance(1e-3) == 0
    Td, Yd = direct.get_state()
    assert np.array_equal(T, Td) and np.array_equal(Y, Yd.T)
    # and agrees with the oracle's integrator (the integrator's own parity tests hold the
    # 10 x rtol bars; near ignition a reactor's error is a time shift)
    To, Yo, st, _ = m.advance_batch(T0, P, Y0, 1e-3, po.opts(rtol=rtol, atol=1e-15, analytic=True))
    assert np.all(st[:, 8] == 0) and np.all(net.status == 0)
    assert np.max(np.abs(T - To) / To) < 100 * rtol
    major = Yo >= 1e-3
    assert np.max(np.abs(Y - Yo)[major] / Yo[major]) < 100 * rtol
    assert np.all(net.solver_stats["steps"] > 0)
    # continuing: the reactors' states follow the network
    net.advance(2e-3)
    assert net.time == 2e-3 and np.all(net.status == 0)
    assert all(r.T != t for r, t in zip(reactors, T))
    assert reactors[0].mass == pytest.approx(reactors[0].density * reactors[0].volume)


def test_reinitialize_and_tolerances(ct):
    gas = ct.Solution("h2o2.yaml", "ohmech")
    gas.TPX = 1100.0, ct.one_atm, "H2:2, O2:1, N2:4"
    a, b = ct.IdealGasConstPressureReactor(gas), ct.IdealGasConstPressureReactor(gas)
    na, nb = ct.ReactorNet([a]), ct.ReactorNet([b])
    for n in (na, nb):
        n.rtol, n.atol = 1e-9, 1e-15
    na.advance(1e-3)
    nb.advance(4e-4)
    nb.reinitialize()            # restart from the state at 4e-4 s, time kept
    assert nb.time == 4e-4
    nb.advance(1e-3)
    assert nb.time == 1e-3
    assert b.T == pytest.approx(a.T, rel=1e-6)
    assert np.allclose(b.thermo.Y, a.thermo.Y, rtol=1e-4, atol=1e-9)


def test_failures_raise(ct):
    gas = ct.Solution("h2o2.yaml", "ohmech")
    gas.TPX = 1200.0, ct.one_atm, "H2:2, O2:1, N2:4"
    r = ct.IdealGasConstPressureReactor(gas)
    net = ct.ReactorNet([r])
    net.max_steps = 5
    with pytest.raises(ct.CanteraError, match="failed"):
        net.advance(1e-3)
    assert net.status[0] != 0
    with pytest.raises(ct.CanteraError, match="failed in their step"):
        net.step()   # a failed reactor stays failed
    with pytest.raises(ValueError, match="another network"):
        ct.ReactorNet([r])
    other = ct.Solution("h2o2.yaml", "ohmech")
    with pytest.raises(NotImplementedError):
        ct.ReactorNet([ct.IdealGasConstPressureReactor(gas), ct.IdealGasConstPressureReactor(other)])


def test_network_state_vector_and_max_order(ct):
    """get_state after an advance: [mass, T, Y] per reactor with the initial mass conserved
    (the volume follows the density), [T, n] for mole reactors; global_component_index into
    it; max_order reaches the integrator at the next (re)initialisation."""
    gas = ct.Solution("h2o2.yaml", "ohmech")
    gas.TPX = 1200.0, ct.one_atm, "H2:2, O2:1, N2:4"
    rho0 = gas.density
    a, b = ct.IdealGasConstPressureReactor(gas, volume=0.5), ct.IdealGasConstPressureReactor(gas)
    net = ct.ReactorNet([a, b])
    net.advance(1e-3)
    y = net.get_state()
    assert y.shape == (net.n_vars,) and net.n_vars == 2 * (gas.n_species + 2)
    assert y[0] == pytest.approx(0.5 * rho0, rel=1e-12) and a.mass == pytest.approx(0.5 * rho0, rel=1e-12)
    assert a.T > 2000.0 and a.volume == pytest.approx(a.mass / a.density, rel=1e-12) and a.volume > 0.75
    i = net.global_component_index("temperature", 1)
    assert y[i] == b.T and net.component_name(i).endswith(": temperature")
    assert np.array_equal(y[net.global_component_index("H2O", 0):][:1], a.thermo.Y[gas.species_index("H2O"):][:1])
    m = ct.IdealGasConstPressureMoleReactor(gas)
    mnet = ct.ReactorNet([m])
    mnet.advance(1e-3)
    z = mnet.get_state()
    assert z[0] == m.T and np.allclose(z[1:] * gas.molecular_weights, m.mass * m.thermo.Y, rtol=1e-14)
    # max order: a new value applies at the next initialisation
    net.max_order = 2
    net.reinitialize()
    net.advance(2e-3)
    assert np.all(net.solver_stats["last_order"] <= 2)
    assert a.mass == pytest.approx(0.5 * rho0, rel=1e-12)


def test_network_get_derivative(ct):
    """ReactorNet.get_derivative in the reference's layouts: [0, dT, dY] per mass-fraction
    reactor (the mass being conserved), [dT, dn] per mole reactor, the amounts' derivatives
    scaled to the reactor's size on either linear solver."""
    gas = ct.Solution("h2o2.yaml", "ohmech")
    gas.TPX = 1100.0, ct.one_atm, "H2:2, O2:1, N2:4"
    a = ct.IdealGasConstPressureReactor(gas, volume=0.5)
    net = ct.ReactorNet([a])
    with pytest.raises(ct.CanteraError):
        net.get_derivative(1)
    net.rtol, net.atol = 1e-10, 1e-16
    net.advance(1e-4)
    d = net.get_derivative(1)
    assert d.shape == (net.n_vars,) and d[0] == 0.0
    y0 = net.get_derivative(0)
    assert y0[0] == pytest.approx(a.mass, rel=1e-14) and y0[1] == pytest.approx(a.T, rel=1e-14)
    moles = {}
    for solver in ("DENSE", "GMRES"):
        m = ct.IdealGasConstPressureMoleReactor(gas, volume=0.5)
        mnet = ct.ReactorNet([m])
        if solver == "GMRES":
            mnet.preconditioner = ct.AdaptivePreconditioner()
        mnet.rtol, mnet.atol = 1e-10, 1e-20
        mnet.advance(1e-4)
        dm = mnet.get_derivative(1)
        assert dm.shape == (mnet.n_vars,)
        # the derivative of the amounts is that of m Y / W
        assert np.allclose(dm[1:] * gas.molecular_weights / m.mass, d[2:], rtol=1e-3, atol=1e-3 * np.max(np.abs(d[2:])))
        assert dm[0] == pytest.approx(d[1], rel=1e-3)
        moles[solver] = mnet.get_derivative(0)[1:]
        assert np.allclose(moles[solver], m.get_state()[1:], rtol=1e-12, atol=1e-30)


def test_species_thermo_and_ideal_gas_properties(ct):
    """The host NASA7 evaluation behind the facade's properties against the oracle's
    (every species of gri30 and n-dodecane, both ranges and the midpoint itself), the reference
    pressure, and the facade's mixture properties from them."""
    import cantera_gb300 as gb
    for name in ("gri30", "nDodecane"):
        sol = gpu_solution(name)
        m = oracle_mech(name)
        T = np.array([300.0, 999.999, 1000.0, 1000.001, 1500.0, 2999.0])
        cp, h, s = sol.species_thermo(T)
        for j, t in enumerate(T):
            co, ho, so = m.thermo(t)
            assert np.allclose(cp[:, j], co, rtol=1e-13, atol=1e-13)
            assert np.allclose(h[:, j], ho, rtol=1e-13, atol=1e-13)
            assert np.allclose(s[:, j], so, rtol=1e-13, atol=1e-13)
        assert sol.reference_pressure == 101325.0
        with pytest.raises(gb.GBError):
            sol.species_thermo(-1.0)
    gas = ct.Solution("gri30.yaml", "gri30")
    gas.TPX = 1400.0, 2 * ct.one_atm, "CH4:1, O2:2, N2:7.52"
    co, ho, so = oracle_mech("gri30").thermo(1400.0)
    X = gas.X
    assert gas.cp_mole == pytest.approx(ct.gas_constant * np.sum(X * co), rel=1e-12)
    assert gas.enthalpy_mass == pytest.approx(ct.gas_constant * 1400.0 * np.sum(X * ho) / gas.mean_molecular_weight,
                                              rel=1e-12)
    nz = X > 0
    s_ref = ct.gas_constant * (np.sum(X * so) - np.sum(X[nz] * np.log(X[nz])) - np.log(2.0))
    assert gas.entropy_mole == pytest.approx(s_ref, rel=1e-12)
