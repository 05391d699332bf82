"""The cantera-shaped facade's state logic (cantera_gb300.compat) without a GPU: the
Solution state setters and getters over a stand-in mechanism object (the kinetics getters
and reactor networks need the engine and are covered by tests/test_gpu_compat.py)."""
import numpy as np
import pytest


class StandInMech:
    """The part of cantera_gb300.Solution the facade's state logic uses."""

    def __init__(self):
        self.species_names = ["H2", "O2", "H2O", "N2"]
        self.n_species = 4
        self.n_reactions = 0
        self.molecular_weights = np.array([2.016, 31.998, 18.015, 28.014])

    def species_index(self, name):
        return self.species_names.index(name)

    def mole_to_mass(self, X):
        y = np.asarray(X) * self.molecular_weights
        return y / y.sum()


@pytest.fixture
def gas():
    from cantera_gb300.compat import Solution
    return Solution(None, _mech=StandInMech())


def test_composition_forms(gas):
    gas.TPX = 1000.0, 2e5, "H2:2, O2:1"
    assert gas.X == pytest.approx([2 / 3, 1 / 3, 0, 0], rel=1e-14)
    gas.X = {"H2": 1.0, "N2": 3.0}
    assert gas.X == pytest.approx([0.25, 0, 0, 0.75], rel=1e-14)
    gas.Y = [1, 1, 0, 2]
    assert gas.Y == pytest.approx([0.25, 0.25, 0, 0.5], rel=1e-14)
    with pytest.raises(ValueError):
        gas.Y = [0, 0, 0, 0]
    with pytest.raises(ValueError):
        gas.X = "H2:1, XX:1"


def test_state_relations(gas):
    from cantera_gb300.compat import gas_constant
    gas.TPY = 1500.0, 3e5, [0.1, 0.2, 0.3, 0.4]
    W = 1 / np.sum(gas.Y / gas.molecular_weights)
    assert gas.mean_molecular_weight == pytest.approx(W, rel=1e-14)
    assert gas.density == pytest.approx(3e5 * W / (gas_constant * 1500.0), rel=1e-14)
    assert gas.density_mole == pytest.approx(3e5 / (gas_constant * 1500.0), rel=1e-14)
    assert gas.concentrations == pytest.approx(gas.density * gas.Y / gas.molecular_weights, rel=1e-14)
    # TP keeps the composition, None leaves a value unchanged
    y = gas.Y
    gas.TP = None, 1e5
    assert gas.T == 1500.0 and gas.P == 1e5 and np.array_equal(gas.Y, y)
    # TDY: density held while T doubles means P doubles
    d = gas.density
    gas.TDY = 3000.0, d, None
    assert gas.P == pytest.approx(2e5, rel=1e-13)
    with pytest.raises(ValueError):
        gas.TP = 300.0, 0.0


def test_copies_are_independent(gas):
    from cantera_gb300.compat import IdealGasConstPressureReactor
    gas.TPX = 1200.0, 1e5, "H2:2, O2:1, N2:4"
    r = IdealGasConstPressureReactor(gas, volume=2.0)
    gas.TPX = 300.0, 1e5, "N2:1"
    assert r.T == 1200.0 and r.thermo.X[0] == pytest.approx(2 / 7)
    assert r.mass == pytest.approx(r.thermo.density * 2.0)
    with pytest.raises(NotImplementedError):
        IdealGasConstPressureReactor(gas, energy="off")


def test_preconditioner_settings_without_engine(gas):
    """The facade's Krylov-path switch (no engine needed until the first advance): an
    AdaptivePreconditioner makes the network's linear solver GMRES, holds the reference's
    defaults and refuses other settings; mass-fraction reactors with it are refused when the
    network is built."""
    import cantera_gb300.compat as ct
    p = ct.AdaptivePreconditioner()
    assert p.linear_solver_type == "GMRES"
    assert (p.threshold, p.ilut_fill_factor, p.ilut_drop_tol) == (0.0, 10, 1e-12)
    p.ilut_drop_tol = 1e-12          # the default is accepted
    with pytest.raises(NotImplementedError):
        p.ilut_fill_factor = 2
    with pytest.raises(NotImplementedError):
        p.threshold = 1e-8
    gas.TPX = 1200.0, ct.one_atm, "H2:2, O2:1, N2:4"
    net = ct.ReactorNet([ct.IdealGasConstPressureMoleReactor(gas), ct.IdealGasConstPressureMoleReactor(gas)])
    assert net.linear_solver_type == "DENSE" and net.preconditioner is None
    net.preconditioner = p
    assert net.linear_solver_type == "GMRES" and net.preconditioner is p
    with pytest.raises(NotImplementedError):
        net.preconditioner = object()
    mixed = ct.ReactorNet([ct.IdealGasConstPressureReactor(gas)])
    mixed.preconditioner = ct.AdaptivePreconditioner()
    with pytest.raises(ct.CanteraError, match="IdealGasConstPressureMoleReactor"):
        mixed.advance(1e-3)


def test_reactor_components_names_and_mass(gas):
    """The reactors' state vectors and names as the reference defines them: [mass,
    temperature, Y] for IdealGasConstPressureReactor, [temperature, n] for the mole reactor;
    unnamed reactors get '<type>_<count>' when added to a network; the mass is fixed at
    initialisation and conserved, the volume follows the density."""
    import cantera_gb300.compat as ct
    gas.TPX = 1200.0, 1e5, "H2:2, O2:1, N2:4"
    a = ct.IdealGasConstPressureReactor(gas, volume=2.0)
    b = ct.IdealGasConstPressureReactor(gas, name="hot")
    c = ct.IdealGasConstPressureMoleReactor(gas)
    net = ct.ReactorNet([a, b])
    assert (a.name, b.name) == ("IdealGasConstPressureReactor_0", "hot")
    assert a.n_vars == 6 and c.n_vars == 5 and net.n_vars == 12
    assert [a.component_name(k) for k in range(6)] == ["mass", "temperature", "H2", "O2", "H2O", "N2"]
    assert [c.component_name(k) for k in range(5)] == ["temperature", "H2", "O2", "H2O", "N2"]
    assert a.component_index("temperature") == 1 and a.component_index("H2O") == 4
    assert c.component_index("temperature") == 0 and c.component_index("H2O") == 3
    with pytest.raises(ct.CanteraError, match="not found"):
        a.component_index("CH4")
    with pytest.raises(IndexError):
        a.component_name(6)
    assert net.component_name(0) == "IdealGasConstPressureReactor_0: mass"
    assert net.component_name(7) == "hot: temperature"
    with pytest.raises(IndexError):
        net.component_name(12)
    assert net.global_component_index("O2", 1) == 6 + 3
    # mass and volume: density x volume until initialised, then the mass is kept
    rho0 = a.density
    assert a.mass == pytest.approx(2.0 * rho0) and a.volume == 2.0
    a._initialize()
    a.thermo.TP = 2400.0, 1e5                      # as an advance would heat it
    assert a.mass == pytest.approx(2.0 * rho0)
    assert a.volume == pytest.approx(4.0) and a.mass == pytest.approx(a.density * a.volume)
    state = a.get_state()
    assert state[0] == pytest.approx(2.0 * rho0) and state[1] == 2400.0
    assert np.allclose(state[2:], a.thermo.Y)
    n = c.get_state()[1:]
    assert np.allclose(n * gas.molecular_weights, c.mass * c.thermo.Y)
    a.insert(gas)                                  # new contents keep the current volume
    assert a.volume == pytest.approx(4.0) and a.mass == pytest.approx(4.0 * gas.density)
    m2 = ct.ReactorNet([ct.IdealGasConstPressureMoleReactor(gas), ct.IdealGasConstPressureReactor(gas)])
    assert [r.name for r in m2.reactors] == ["IdealGasConstPressureMoleReactor_0", "IdealGasConstPressureReactor_0"]


def test_network_integrator_settings_without_engine(gas):
    """max_order is kept for the next initialisation (1..5); the integrator's fixed limits
    (CVODE's defaults) are readable where the reference's are and refuse other values;
    verbose is a flag."""
    import cantera_gb300.compat as ct
    gas.TPX = 1200.0, 1e5, "H2:2, O2:1, N2:4"
    net = ct.ReactorNet([ct.IdealGasConstPressureReactor(gas)])
    assert net.max_order == 5
    net.max_order = 3
    assert net.max_order == 3
    with pytest.raises(ValueError):
        net.max_order = 6
    assert ct.ReactorNet(max_order=2).max_order == 2
    with pytest.raises(AttributeError):
        net.max_err_test_fails
    net.max_err_test_fails = 7
    with pytest.raises(NotImplementedError):
        net.max_err_test_fails = 10
    assert net.max_nonlinear_iterations == 3 and net.max_nonlinear_convergence_failures == 10
    net.max_nonlinear_iterations = 3
    with pytest.raises(NotImplementedError):
        net.max_nonlinear_iterations = 5
    with pytest.raises(NotImplementedError):
        net.max_nonlinear_convergence_failures = 20
    assert net.verbose is False
    net.verbose = 1
    assert net.verbose is True
    with pytest.raises(ct.CanteraError, match="empty"):
        ct.ReactorNet().get_state()


class StandInEngine:
    """The part of cantera_gb300.ReactorNet the facade's get_derivative reads."""

    def __init__(self, d, linear_solver):
        self._d, self.linear_solver = d, linear_solver

    def get_derivative(self, k):
        return self._d * (k + 1)


def test_get_derivative_layouts_without_engine(gas):
    """The facade turns the engine's [T, Y] (dense) or [T, n per m^3 of initial volume] (GMRES)
    derivatives into the reference's per-reactor layouts: [mass or 0, T, Y] for mass-fraction
    reactors, [T, n] for mole reactors (n = m Y / W, or the engine's amounts times the volume
    at initialisation)."""
    import cantera_gb300.compat as ct
    gas.TPX = 1200.0, 1e5, "H2:2, O2:1, N2:4"
    a = ct.IdealGasConstPressureReactor(gas, volume=2.0)
    m = ct.IdealGasConstPressureMoleReactor(gas, volume=3.0)
    net = ct.ReactorNet([a, m])
    with pytest.raises(ct.CanteraError, match="not been integrated"):
        net.get_derivative(1)
    for r in (a, m):
        r._initialize()
    K = gas.n_species
    d = np.arange(2.0 * (K + 1)).reshape(K + 1, 2) + 1.0      # [K + 1, 2 reactors]
    net._engine = StandInEngine(d, "DENSE")
    y1 = net.get_derivative(1)                                 # the stand-in doubles d for k = 1
    assert y1.shape == (net.n_vars,)
    assert y1[0] == 0.0 and y1[1] == 2 * d[0, 0] and np.array_equal(y1[2:2 + K], 2 * d[1:, 0])
    mo = 2 + K
    assert y1[mo] == 2 * d[0, 1]
    assert np.allclose(y1[mo + 1:], m.mass * 2 * d[1:, 1] / gas.molecular_weights, rtol=1e-15)
    y0 = net.get_derivative(0)
    assert y0[0] == a.mass                                     # k = 0: the state, mass included
    net._engine = StandInEngine(d, "GMRES")
    y1 = net.get_derivative(1)
    assert np.allclose(y1[mo + 1:], 3.0 * 2 * d[1:, 1], rtol=1e-15)   # amounts of 1 m^3 x 3 m^3


class OracleThermoMech(StandInMech):
    """A stand-in whose species data come from the oracle's NASA7 evaluation (h2o2)."""

    def __init__(self):
        from conftest import oracle_mech
        self._o = oracle_mech("h2o2")
        self.n_species = self._o.K
        self.species_names = ["s%d" % k for k in range(self._o.K)]
        self.molecular_weights = self._o.mw.copy()
        self.reference_pressure = 101325.0

    def species_thermo(self, T):
        return self._o.thermo(T)


def test_ideal_gas_properties_identities():
    """The facade's ideal-gas properties satisfy the thermodynamic identities: cp = dh/dT and
    s = -dg/dT at constant P and composition (central differences), g = sum X_k mu_k,
    h = sum X_k hbar_k, u = h - RT, cp - cv = R; a species at zero mole fraction enters the
    entropy and chemical potentials through the 1e-300 floor, as in the reference."""
    from cantera_gb300.compat import Solution, gas_constant
    gas = Solution(None, _mech=OracleThermoMech())
    rng = np.random.default_rng(3)
    for T in (600.0, 999.9, 1000.1, 1700.0, 2500.0):        # both NASA7 ranges
        Y = rng.dirichlet(np.ones(gas.n_species))
        Y[2] = 0.0
        gas.TPY = T, 3e5, Y
        X = gas.X
        d = 1e-3
        def at(t, prop):
            gas.TP = t, None
            v = getattr(gas, prop)
            gas.TP = T, None
            return v
        cp_fd = (at(T + d, "enthalpy_mass") - at(T - d, "enthalpy_mass")) / (2 * d)
        assert gas.cp_mass == pytest.approx(cp_fd, rel=1e-7)
        s_fd = -(at(T + d, "gibbs_mole") - at(T - d, "gibbs_mole")) / (2 * d)
        assert gas.entropy_mole == pytest.approx(s_fd, rel=1e-6)
        assert gas.gibbs_mole == pytest.approx(np.sum(X * gas.chemical_potentials), rel=1e-10, abs=1e-3)
        assert gas.enthalpy_mole == pytest.approx(np.sum(X * gas.partial_molar_enthalpies), rel=1e-12)
        assert gas.int_energy_mole == pytest.approx(gas.enthalpy_mole - gas_constant * T, rel=1e-12)
        assert gas.cp_mole - gas.cv_mole == pytest.approx(gas_constant, rel=1e-12)
        assert gas.cp == gas.cp_mass and gas.s == gas.entropy_mass
        mu0 = gas.standard_chemical_potentials
        assert gas.chemical_potentials[2] == pytest.approx(mu0[2] + gas_constant * T * np.log(1e-300), rel=1e-12)
        assert np.all(np.isfinite(gas.partial_molar_entropies))


def test_insert_restarts_the_network(gas):
    """New contents in a reactor of a running network make it restart from the reactors'
    states at the next advance, keeping its time."""
    import cantera_gb300.compat as ct
    gas.TPX = 1200.0, 1e5, "H2:2, O2:1, N2:4"
    r = ct.IdealGasConstPressureReactor(gas)
    net = ct.ReactorNet([r])
    net._engine = StandInEngine(np.zeros((gas.n_species + 1, 1)), "DENSE")
    net._t = 1e-3
    gas.TPX = 900.0, 1e5, "N2:1"
    r.insert(gas)
    assert net._engine is None and net.time == 1e-3 and r.T == 900.0
