"""A ``cantera``-shaped facade over the engine, for scripts written against the reference.

    import cantera_gb300.compat as ct

    gas = ct.Solution("gri30.yaml")
    gas.TPX = 1200.0, ct.one_atm, "CH4:1, O2:2, N2:7.52"
    wdot = gas.net_production_rates                 # this state, kmol/m^3/s
    reactors = []
    for T in (1000.0, 1100.0, 1200.0):
        gas.TP = T, ct.one_atm
        reactors.append(ct.IdealGasConstPressureReactor(gas))
    net = ct.ReactorNet(reactors)
    net.rtol, net.atol = 1e-8, 1e-15
    net.advance(1e-3)
    print([r.T for r in reactors], reactors[0].thermo.Y)

The names and semantics follow the reference's Python interface:
``Solution`` / ``ThermoPhase`` state setters and getters (interfaces/cython/cantera/
thermo.py: ``TP``, ``TPX``, ``TPY``, ``X``, ``Y``, ``set_equivalence_ratio``,
``density``, ``mean_molecular_weight``, ``concentrations``; the ideal-gas properties
``cp``/``cv``/``h``/``u``/``s``/``g`` on mass and mole bases, ``partial_molar_*``,
``chemical_potentials`` and the ``standard_*`` reference-state arrays, from the species' NASA7
data), ``Kinetics``
(interfaces/cython/cantera/kinetics.py:456-461,928-940: ``net_production_rates``,
``net_production_rates_ddCi`` as a scipy CSC matrix), ``IdealGasConstPressureReactor``,
``IdealGasConstPressureMoleReactor``, ``AdaptivePreconditioner`` (interfaces/cython/cantera/
jacobians.py:120-200) and ``ReactorNet`` (interfaces/cython/cantera/reactor.py:1781-2100,
2396-2415: ``advance``, ``step``, ``time``, ``initial_time``, ``reinitialize``, ``rtol``,
``atol``, ``max_steps``, ``max_time_step``, ``max_order``, ``solver_stats``,
``preconditioner``, ``linear_solver_type``, ``initialize``, ``verbose``, ``n_vars``,
``get_state``, ``get_derivative``, ``component_name``, ``global_component_index``; the
integrator limits ``max_err_test_fails``, ``max_nonlinear_iterations``,
``max_nonlinear_convergence_failures`` at CVODE's defaults).  One ``ReactorNet`` over many reactors is one batched GPU network:
every reactor is independent (no walls or inlets), shares the network's mechanism and
tolerances, and reaches each ``advance`` time together.  A network of mole reactors with an
``AdaptivePreconditioner`` runs the engine's GMRES path (the mole-reactor state, the
preconditioner's ILUT, J v products); without one it runs the dense path.  What the batched
engine does not do raises: reactors of different mechanisms in one network, preconditioner
settings other than the reference's defaults; transport properties and other phase models
are not there.
"""
import numpy as np

from . import GBError, ReactorNet as _Net, Solution as _Mech

one_atm = 101325.0
avogadro = 6.02214076e26
gas_constant = avogadro * 1.380649e-23   # J/kmol/K

__all__ = ["Solution", "IdealGasConstPressureReactor", "IdealGasConstPressureMoleReactor",
           "AdaptivePreconditioner", "ReactorNet", "one_atm", "avogadro", "gas_constant", "CanteraError"]
CanteraError = GBError


class Solution:
    """An ideal-gas phase with kinetics: one thermodynamic state over a loaded mechanism."""

    def __init__(self, infile, name="", *, _mech=None):
        self._m = _mech if _mech is not None else _Mech(infile, name)
        self._T = 300.0
        self._P = one_atm
        self._Y = np.zeros(self._m.n_species)
        self._Y[0] = 1.0

    # ---- mechanism ----
    @property
    def species_names(self):
        return list(self._m.species_names)

    @property
    def n_species(self):
        return self._m.n_species

    @property
    def n_reactions(self):
        return self._m.n_reactions

    @property
    def molecular_weights(self):
        return self._m.molecular_weights.copy()

    def species_index(self, name):
        return self._m.species_index(name)

    def _composition(self, comp):
        """A composition as a string 'A:1, B:2', a dict or an array over the species."""
        if isinstance(comp, str):
            v = np.zeros(self.n_species)
            for item in comp.split(","):
                if item.strip():
                    name, x = item.split(":")
                    v[self.species_index(name.strip())] += float(x)
        elif isinstance(comp, dict):
            v = np.zeros(self.n_species)
            for name, x in comp.items():
                v[self.species_index(name)] += float(x)
        else:
            v = np.array(comp, dtype=np.float64).reshape(self.n_species)
        s = v.sum()
        if not s > 0:
            raise ValueError("composition must have a positive sum")
        return v / s

    # ---- state ----
    @property
    def T(self):
        return self._T

    @property
    def P(self):
        return self._P

    @property
    def Y(self):
        return self._Y.copy()

    @Y.setter
    def Y(self, comp):
        self._Y = self._composition(comp)

    @property
    def X(self):
        x = self._Y / self._m.molecular_weights
        return x / x.sum()

    @X.setter
    def X(self, comp):
        self._Y = self._m.mole_to_mass(self._composition(comp))

    @property
    def TP(self):
        return self._T, self._P

    @TP.setter
    def TP(self, v):
        T, P = v
        self._set_TP(T, P)

    @property
    def TPX(self):
        return self._T, self._P, self.X

    @TPX.setter
    def TPX(self, v):
        T, P, X = v
        self._set_TP(T, P)
        if X is not None:
            self.X = X

    @property
    def TPY(self):
        return self._T, self._P, self.Y

    @TPY.setter
    def TPY(self, v):
        T, P, Y = v
        self._set_TP(T, P)
        if Y is not None:
            self.Y = Y

    @property
    def TDY(self):
        return self._T, self.density, self.Y

    @TDY.setter
    def TDY(self, v):
        T, D, Y = v
        if Y is not None:
            self.Y = Y
        T = self._T if T is None else float(T)
        D = self.density if D is None else float(D)
        self._set_TP(T, D * gas_constant * T / self.mean_molecular_weight)

    def _set_TP(self, T, P):
        if T is not None:
            if not T > 0:
                raise ValueError("temperature must be positive")
            self._T = float(T)
        if P is not None:
            if not P > 0:
                raise ValueError("pressure must be positive")
            self._P = float(P)

    def set_equivalence_ratio(self, phi, fuel, oxidizer, basis="mole"):
        """The mixture of fuel and oxidizer with equivalence ratio phi; T and P are kept
        (``ThermoPhase.set_equivalence_ratio``, src/thermo/ThermoPhase.cpp:879-910)."""
        if basis not in ("mole", "molar"):
            raise NotImplementedError("only the molar basis is supported")
        self._Y = self._m.equivalence_ratio_mass_fractions(phi, self._composition(fuel), self._composition(oxidizer))

    @property
    def mean_molecular_weight(self):
        """kg/kmol, from the mass fractions as given (no normalisation)."""
        return 1.0 / np.sum(self._Y / self._m.molecular_weights)

    @property
    def density(self):
        return self._P * self.mean_molecular_weight / (gas_constant * self._T)

    @property
    def density_mole(self):
        return self._P / (gas_constant * self._T)

    @property
    def concentrations(self):
        return self.density * self._Y / self._m.molecular_weights

    # ---- ideal-gas properties of this state (src/thermo/IdealGasPhase.cpp:25-96,
    # include/cantera/thermo/IdealGasPhase.h:294-296; the NASA7 species data evaluated on the host)
    def _ref(self):
        return self._m.species_thermo(self._T)

    @property
    def standard_cp_R(self):
        return self._ref()[0]

    @property
    def standard_enthalpies_RT(self):
        return self._ref()[1]

    @property
    def standard_entropies_R(self):
        return self._ref()[2]

    @property
    def standard_gibbs_RT(self):
        _, h, s = self._ref()
        return h - s

    @property
    def standard_int_energies_RT(self):
        return self._ref()[1] - 1.0

    def _ym(self):
        return self._Y / self._m.molecular_weights

    def _log_x(self):
        """ln max(X_k, 1e-300) (the reference's SmallNumber floor)."""
        return np.log(np.maximum(self._ym() * self.mean_molecular_weight, 1e-300))

    @property
    def partial_molar_enthalpies(self):
        return self._ref()[1] * gas_constant * self._T

    @property
    def partial_molar_int_energies(self):
        return (self._ref()[1] - 1.0) * gas_constant * self._T

    @property
    def partial_molar_cp(self):
        return self._ref()[0] * gas_constant

    @property
    def partial_molar_entropies(self):
        logp = np.log(self._P / self._m.reference_pressure)
        return gas_constant * (self._ref()[2] - logp - self._log_x())

    @property
    def standard_chemical_potentials(self):
        _, h, s = self._ref()
        RT = gas_constant * self._T
        return (h - s) * RT + RT * np.log(self._P / self._m.reference_pressure)

    @property
    def chemical_potentials(self):
        return self.standard_chemical_potentials + gas_constant * self._T * self._log_x()

    def _mean_x(self, v):
        return self.mean_molecular_weight * np.sum(self._ym() * v)

    @property
    def cp_mole(self):
        return gas_constant * self._mean_x(self._ref()[0])

    @property
    def cv_mole(self):
        return self.cp_mole - gas_constant

    @property
    def enthalpy_mole(self):
        return gas_constant * self._T * self._mean_x(self._ref()[1])

    @property
    def int_energy_mole(self):
        return gas_constant * self._T * (self._mean_x(self._ref()[1]) - 1.0)

    @property
    def entropy_mole(self):
        ym, mmw = self._ym(), self.mean_molecular_weight
        sum_xlogx = mmw * np.sum(ym * np.log(np.maximum(ym, 1e-300))) + np.log(mmw)
        return gas_constant * (self._mean_x(self._ref()[2]) - sum_xlogx
                               - np.log(self._P / self._m.reference_pressure))

    @property
    def gibbs_mole(self):
        return self.enthalpy_mole - self._T * self.entropy_mole

    cp_mass = property(lambda self: self.cp_mole / self.mean_molecular_weight)
    cv_mass = property(lambda self: self.cv_mole / self.mean_molecular_weight)
    enthalpy_mass = property(lambda self: self.enthalpy_mole / self.mean_molecular_weight)
    int_energy_mass = property(lambda self: self.int_energy_mole / self.mean_molecular_weight)
    entropy_mass = property(lambda self: self.entropy_mole / self.mean_molecular_weight)
    gibbs_mass = property(lambda self: self.gibbs_mole / self.mean_molecular_weight)
    # the reference's default basis is mass
    cp, cv, h, u, s, g = cp_mass, cv_mass, enthalpy_mass, int_energy_mass, entropy_mass, gibbs_mass

    # ---- kinetics (one state through the batched GPU kernels) ----
    def _one(self):
        return np.array([self._T]), np.array([self._P]), self._Y[:, None].copy()

    @property
    def net_production_rates(self):
        return self._m.net_production_rates(*self._one())[:, 0]

    @property
    def net_production_rates_ddCi(self):
        """d(wdot)/d(c) at constant T and other concentrations, as a scipy CSC matrix on the
        reference's sparsity pattern."""
        import scipy.sparse as sp
        vals = self._m.net_production_rates_ddCi(*self._one())[:, 0]
        K = self.n_species
        return sp.csc_matrix((vals, self._m.jac_rowidx.copy(), self._m.jac_colptr.copy()), shape=(K, K))

    def _copy(self):
        s = Solution(None, _mech=self._m)
        s._T, s._P, s._Y = self._T, self._P, self._Y.copy()
        return s


class IdealGasConstPressureReactor:
    """A constant-pressure ideal-gas reactor holding its own copy of the gas state.  Its
    state vector is [mass, temperature, Y_1..Y_K] (src/zeroD/IdealGasConstPressureReactor.cpp:
    16-26,133-155): the mass is fixed when a network initialises the reactor (as
    density x volume) and conserved, the volume follows as mass / density."""
    _components = ("mass", "temperature")

    def __init__(self, contents, *, name="", volume=1.0, energy="on"):
        if energy != "on":
            raise NotImplementedError("only the energy equation 'on' is supported")
        self.name = name
        self._volume = float(volume)
        self._mass = None
        self._thermo = contents._copy()
        self._net = None

    @property
    def type(self):
        return type(self).__name__

    @property
    def thermo(self):
        """The reactor's gas (its state is the reactor's after each advance)."""
        return self._thermo

    @property
    def T(self):
        return self._thermo.T

    @property
    def density(self):
        return self._thermo.density

    @property
    def mass(self):
        return self._thermo.density * self._volume if self._mass is None else self._mass

    @property
    def volume(self):
        return self._volume if self._mass is None else self._mass / self._thermo.density

    @volume.setter
    def volume(self, v):
        self._volume = float(v)
        self._mass = None

    def _initialize(self):
        self._v_init = self.volume
        self._mass = self._thermo.density * self._v_init

    def insert(self, gas):
        """Replace the contents (and state) of the reactor; its volume is kept, and a network
        holding it restarts from its reactors' states at the next advance (as the reference's
        ReactorBase::setSolution asks its network to reinitialise)."""
        self._volume = self.volume
        self._mass = None
        self._thermo = gas._copy()
        if self._net is not None:
            self._net._engine = None

    @property
    def n_vars(self):
        """Number of components of the reactor's state vector."""
        return len(self._components) + self._thermo.n_species

    def component_index(self, name):
        """Index of a state component: a state variable's name or a species name."""
        if name in self._components:
            return self._components.index(name)
        try:
            k = self._thermo.species_index(name)
        except (ValueError, KeyError, GBError):
            k = -1
        if k is None or k < 0:
            raise CanteraError("%s::componentIndex: Component '%s' not found" % (self.type, name))
        return len(self._components) + int(k)

    def component_name(self, k):
        """Name of the k-th component of the reactor's state vector."""
        nc = len(self._components)
        if 0 <= k < nc:
            return self._components[k]
        if nc <= k < self.n_vars:
            return self._thermo.species_names[k - nc]
        raise IndexError("%s::componentName: component %d outside [0, %d)" % (self.type, k, self.n_vars))

    def get_state(self):
        """The reactor's state vector."""
        return np.concatenate([[self.mass, self.T], self._thermo.Y])


class IdealGasConstPressureMoleReactor(IdealGasConstPressureReactor):
    """A constant-pressure ideal-gas reactor whose integrator state is T and the species
    amounts (IdealGasConstPressureMoleReactor): [temperature, n_1..n_K] in kmol
    (src/zeroD/IdealGasConstPressureMoleReactor.cpp:22-30,274-295); the one reactor type
    that supports the adaptive preconditioner."""
    _components = ("temperature",)

    def get_state(self):
        return np.concatenate([[self.T], self.mass * self._thermo.Y / self._thermo.molecular_weights])


class AdaptivePreconditioner:
    """The reference's preconditioner for GMRES (interfaces/cython/cantera/jacobians.py:
    120-200, src/numerics/AdaptivePreconditioner.cpp): an approximate Jacobian of the mole
    reactors, factored by ILUT.  The engine runs it with the reference's defaults (no
    pruning threshold, drop tolerance 1e-12, fill factor 10); other settings raise."""
    linear_solver_type = "GMRES"
    _defaults = {"threshold": 0.0, "ilut_fill_factor": 10, "ilut_drop_tol": 1e-12}

    def _check(self, name, v):
        if float(v) != float(self._defaults[name]):
            raise NotImplementedError("the engine's preconditioner uses %s = %g" % (name, self._defaults[name]))

    @property
    def threshold(self):
        return self._defaults["threshold"]

    @threshold.setter
    def threshold(self, v):
        self._check("threshold", v)

    @property
    def ilut_fill_factor(self):
        return self._defaults["ilut_fill_factor"]

    @ilut_fill_factor.setter
    def ilut_fill_factor(self, v):
        self._check("ilut_fill_factor", v)

    @property
    def ilut_drop_tol(self):
        return self._defaults["ilut_drop_tol"]

    @ilut_drop_tol.setter
    def ilut_drop_tol(self, v):
        self._check("ilut_drop_tol", v)


class ReactorNet:
    """Independent reactors advanced together as one batched GPU network."""

    # the integrator's fixed limits (CVODE's defaults, which the reference's CVODES keeps unless
    # set): error-test failures per step, Newton iterations per solve, convergence failures
    # per step
    _fixed_limits = {"max_err_test_fails": 7, "max_nonlinear_iterations": 3,
                     "max_nonlinear_convergence_failures": 10}

    def __init__(self, reactors=(), **engine_options):
        self._reactors = []
        self._precon = None
        self._opts = dict(engine_options)
        self._rtol, self._atol = 1e-9, 1e-15
        self._max_steps, self._max_time_step = 20000, 0.0
        self._max_order = int(self._opts.pop("max_order", 5))
        self._verbose = False
        self._counts = {}
        self._t0 = 0.0
        self._t = 0.0
        self._engine = None
        for r in reactors:
            self.add_reactor(r)

    def add_reactor(self, r):
        if self._reactors and r.thermo._m is not self._reactors[0].thermo._m:
            raise NotImplementedError("all reactors of a network must share one Solution's mechanism")
        if r._net is not None and r._net is not self:
            raise ValueError("reactor already belongs to another network")
        r._net = self
        # reproducible names for unnamed reactors, "<type>_<count>" (ReactorNet::updateNames,
        # ReactorBase::setDefaultName: src/zeroD/ReactorNet.cpp:572-575, ReactorBase.cpp:54-65)
        if r.name in ("", "(none)"):
            r.name = "%s_%d" % (r.type, self._counts.get(r.type, 0))
        self._counts[r.type] = self._counts.get(r.type, 0) + 1
        self._reactors.append(r)
        self._engine = None

    def initialize(self):
        """Initialise the integration now (otherwise the first advance or step does)."""
        if self._engine is None:
            self._build()

    @property
    def verbose(self):
        """With True, (re)initialisations print the network's configuration."""
        return self._verbose

    @verbose.setter
    def verbose(self, v):
        self._verbose = bool(v)

    @property
    def max_order(self):
        """Maximum order of the BDF method (1..5), applied at the next (re)initialisation as
        the reference's CVODES does (CVodesIntegrator::applyOptions)."""
        return self._max_order

    @max_order.setter
    def max_order(self, n):
        n = int(n)
        if not 1 <= n <= 5:
            raise ValueError("max_order must be in 1..5")
        self._max_order = n

    def _limit(self, name, n):
        if int(n) != self._fixed_limits[name]:
            raise NotImplementedError("the engine's integrator uses %s = %d" % (name, self._fixed_limits[name]))

    @property
    def max_err_test_fails(self):
        raise AttributeError("unreadable attribute 'max_err_test_fails'")

    @max_err_test_fails.setter
    def max_err_test_fails(self, n):
        self._limit("max_err_test_fails", n)

    @property
    def max_nonlinear_iterations(self):
        return self._fixed_limits["max_nonlinear_iterations"]

    @max_nonlinear_iterations.setter
    def max_nonlinear_iterations(self, n):
        self._limit("max_nonlinear_iterations", n)

    @property
    def max_nonlinear_convergence_failures(self):
        return self._fixed_limits["max_nonlinear_convergence_failures"]

    @max_nonlinear_convergence_failures.setter
    def max_nonlinear_convergence_failures(self, n):
        self._limit("max_nonlinear_convergence_failures", n)

    @property
    def n_vars(self):
        """Number of state variables of the network: the reactors' state vectors together."""
        return sum(r.n_vars for r in self._reactors)

    def _locate(self, i):
        if i < 0:
            raise IndexError("component %d outside [0, %d)" % (i, self.n_vars))
        for r in self._reactors:
            if i < r.n_vars:
                return r, i
            i -= r.n_vars
        raise IndexError("component outside [0, %d)" % self.n_vars)

    def component_name(self, i):
        """Name of the i-th component of the network's state vector, 'reactor: component'
        (ReactorNet::componentName, src/zeroD/ReactorNet.cpp:781-794)."""
        r, k = self._locate(int(i))
        return "%s: %s" % (r.name, r.component_name(k))

    def global_component_index(self, name, reactor):
        """Index in the network's state vector of component `name` of the reactor with index
        `reactor` (ReactorNet::globalComponentIndex, src/zeroD/ReactorNet.cpp:774-779)."""
        offset = sum(r.n_vars for r in self._reactors[:reactor])
        return offset + self._reactors[reactor].component_index(name)

    def get_state(self):
        """The network's state vector: the reactors' state vectors one after another
        (ReactorNet::getState, src/zeroD/ReactorNet.cpp:754-759)."""
        if not self._reactors:
            raise CanteraError("ReactorNet empty or not initialized.")
        self.initialize()
        return np.concatenate([r.get_state() for r in self._reactors])

    def get_derivative(self, k):
        """The k-th time derivative of the network's state vector at the current time, from
        the integrator's step history (ReactorNet::getDerivative, src/zeroD/ReactorNet.cpp:
        721-726): per reactor [mass (0 for k > 0, the mass being conserved), T, Y], or [T, n]
        for a mole reactor.  After step() each reactor's derivative is at its own time."""
        if not self._reactors:
            raise CanteraError("ReactorNet empty or not initialized.")
        if self._engine is None:
            raise CanteraError("the network has not been integrated yet")
        d = self._engine.get_derivative(int(k))
        amounts = self._engine.linear_solver == "GMRES"
        parts = []
        for i, r in enumerate(self._reactors):
            dT, dz = d[0, i], d[1:, i]
            if isinstance(r, IdealGasConstPressureMoleReactor):
                # the GMRES engine integrates the amounts per m^3 of the volume at initialisation
                dn = dz * r._v_init if amounts else r.mass * dz / r.thermo.molecular_weights
                parts.append(np.concatenate([[dT], dn]))
            else:
                parts.append(np.concatenate([[r.mass if k == 0 else 0.0, dT], dz]))
        return np.concatenate(parts)

    @property
    def reactors(self):
        return list(self._reactors)

    def _build(self):
        if not self._reactors:
            raise ValueError("the network has no reactors")
        g = [r.thermo for r in self._reactors]
        T = np.array([s.T for s in g])
        P = np.array([s.P for s in g])
        Y = np.array([s._Y for s in g]).T.copy()
        opts = dict(self._opts)
        if self._precon is not None:
            # ReactorNet::initialize: every reactor must support the preconditioner
            if not all(isinstance(r, IdealGasConstPressureMoleReactor) for r in self._reactors):
                raise CanteraError("the AdaptivePreconditioner needs IdealGasConstPressureMoleReactor reactors")
            opts["linear_solver"] = "GMRES"
        self._engine = _Net(g[0]._m, T, P, Y, rtol=self._rtol, atol=self._atol, max_steps=self._max_steps,
                            max_time_step=self._max_time_step, max_order=self._max_order, **opts)
        self._t0 = self._t
        for r in self._reactors:
            r._initialize()
        if self._verbose:
            print("ReactorNet: %d %s reactor(s), %d species, %s linear solver, rtol %g, atol %g, max order %d, "
                  "t0 = %g" % (len(self._reactors), self._reactors[0].type, g[0].n_species, self.linear_solver_type,
                               self._rtol, self._atol, self._max_order, self._t0))

    def reinitialize(self):
        """Restart the integration from the reactors' current states at the current time."""
        self._build()

    def advance(self, t, apply_limit=True):
        """Advance every reactor to time t; returns t.  Raises if any reactor fails (its
        status is in ``status``; the states of the others are updated)."""
        if self._engine is None:
            self._build()
        if t < self._t:
            raise ValueError("cannot integrate backwards in time")
        failed = self._engine.advance(float(t) - self._t0)
        self._t = float(t)
        T, Y = self._engine.get_state()
        for i, r in enumerate(self._reactors):
            r._thermo._T = float(T[i])
            r._thermo._Y = Y[:, i].copy()
        if failed:
            bad = np.nonzero(self._engine.status)[0]
            raise CanteraError("%d reactor(s) failed to reach t = %g (first: %s)" % (failed, t, bad[:8].tolist()))
        return self._t

    def step(self):
        """Take one internal integrator step (ReactorNet.step: one CVODES step towards
        time + 1, the state at the step's end, no interpolation) and return the new time.
        With one reactor this is the reference's step.  The reactors of a batched network
        are independent, so each takes a step of its own size; the network's time becomes
        the latest of their times (each reactor's state is at its own time, in
        ``reactor_times``), and a later advance(t) needs t >= that time."""
        if self._engine is None:
            self._build()
        times = self._engine.step()
        failed = self._engine.last_step_failures
        self.reactor_times = times + self._t0
        self._t = float(np.max(times)) + self._t0
        T, Y = self._engine.get_state()
        for i, r in enumerate(self._reactors):
            r._thermo._T = float(T[i])
            r._thermo._Y = Y[:, i].copy()
        if failed:
            bad = np.nonzero(self._engine.status)[0]
            raise CanteraError("%d reactor(s) failed in their step (first: %s)" % (failed, bad[:8].tolist()))
        return self._t

    @property
    def time(self):
        return self._t

    @property
    def initial_time(self):
        return self._t0

    @initial_time.setter
    def initial_time(self, t):
        self._t = float(t)
        self._build()

    def _set(self, name, v):
        """Change an integrator setting; a running network takes it from its next step on
        without restarting (as ReactorNet passes it to a live CVODES integrator)."""
        setattr(self, name, v)
        if self._engine is not None:
            setattr(self._engine, name[1:], v)

    @property
    def rtol(self):
        return self._rtol

    @rtol.setter
    def rtol(self, v):
        self._set("_rtol", float(v))

    @property
    def atol(self):
        return self._atol

    @atol.setter
    def atol(self, v):
        self._set("_atol", float(v))

    @property
    def max_steps(self):
        return self._max_steps

    @max_steps.setter
    def max_steps(self, v):
        self._set("_max_steps", int(v))

    @property
    def max_time_step(self):
        return self._max_time_step

    @max_time_step.setter
    def max_time_step(self, v):
        self._set("_max_time_step", float(v))

    @property
    def status(self):
        """Per-reactor status codes (0 = reached the last advance time)."""
        return self._engine.status if self._engine is not None else np.zeros(len(self._reactors), dtype=np.int32)

    @property
    def preconditioner(self):
        return self._precon

    @preconditioner.setter
    def preconditioner(self, precon):
        """ReactorNet.preconditioner: an AdaptivePreconditioner switches the network to GMRES
        (applied at the next initialisation, as in the reference)."""
        if precon is not None and not isinstance(precon, AdaptivePreconditioner):
            raise NotImplementedError("the engine supports the AdaptivePreconditioner only")
        self._precon = precon
        self._engine = None

    @property
    def linear_solver_type(self):
        return "GMRES" if self._precon is not None else "DENSE"

    @property
    def solver_stats(self):
        """Integrator counters (CVodesIntegrator::solverStats names) as arrays over the
        reactors, summed since the last (re)initialisation; with GMRES also lin_iters,
        prec_solves and jt_vec_prod_evals."""
        if self._engine is None:
            return {}
        st = dict(self._engine.solver_stats)
        if self._engine.linear_solver == "GMRES":
            st.update(self._engine.krylov_stats)
        return st
