"""cantera_gb300 - a GB300-native batched engine for Cantera's reactor hot path.

Python mirror of the C ABI in ``include/gbchem.h`` (library ``_build/libgbchem.so``),
shaped like the Cantera objects it stands in for:

* :class:`Solution` - ``ct.Solution(yaml, phase)`` for an ideal-gas mechanism, with the
  batched kinetics getters ``net_production_rates`` and ``net_production_rates_ddCi``
  (Cantera ``Kinetics.net_production_rates`` / ``net_production_rates_ddCi``,
  interfaces/cython/cantera/kinetics.py:456-461,928-940) over many states at once.
* :class:`ReactorNet` - ``ct.ReactorNet`` over ``IdealGasConstPressureReactor`` objects
  (interfaces/cython/cantera/reactor.py:1781-1827), batched: one object advances n
  independent reactors with ``advance(t)``; ``rtol``/``atol``/``max_steps`` setters and
  ``solver_stats`` follow ReactorNet's names.

Arrays are species-major (``Y[k, s]``).  numpy arrays are copied to and from the GPU
inside each call; CUDA torch tensors are passed to the engine as device pointers.
There is no CPU fallback: without the library or a CUDA device every call raises.
"""
import ctypes
import os

import numpy as np

__all__ = ["Solution", "ReactorNet", "library", "DATA_DIR", "GBError"]

HERE = os.path.dirname(os.path.abspath(__file__))
DATA_DIR = os.path.join(HERE, "data")
# GBCHEM_CHECKED=1 loads the bounds-checked build (gb_check_status); GBCHEM_LIB names a library
CHECKED = os.environ.get("GBCHEM_CHECKED", "") not in ("", "0")
LIB_PATH = os.environ.get("GBCHEM_LIB", os.path.join(HERE, "_build_checked" if CHECKED else "_build", "libgbchem.so"))
GB_ERR = -999
GB_DEVICE_POINTERS = 1
STAT_NAMES = ["steps", "rhs_evals", "newton_iters", "lin_setups", "jac_evals",
              "err_test_fails", "conv_fails", "last_order"]
STATUS_NAMES = {0: "ok", 1: "max steps", 2: "error-test failures", 3: "convergence failures",
                4: "non-finite state", 5: "step size too small"}


class GBError(RuntimeError):
    """An engine call returned GB_ERR; the message is the engine's."""


class NetOptions(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("max_steps", ctypes.c_int32), ("max_order", ctypes.c_int32),
                ("max_time_step", ctypes.c_double), ("lu_precision", ctypes.c_int32),
                ("warps_per_block", ctypes.c_int32), ("use_graph", ctypes.c_int32),
                ("matrix_placement", ctypes.c_int32), ("mechanism_in_shared", ctypes.c_int32),
                ("jacobian_reuse", ctypes.c_int32), ("lu_staging", ctypes.c_int32),
                ("linear_solver", ctypes.c_int32)]


_lib = None


def library():
    """Load the engine library (building it first if its sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) or os.environ.get("GBCHEM_REBUILD"):
        from . import build as _build
        _build.build(checked=CHECKED and "GBCHEM_LIB" not in os.environ)
    L = ctypes.CDLL(LIB_PATH)
    I32, D, P = ctypes.c_int32, ctypes.c_double, ctypes.c_void_p
    sig = {
        "gb_mech_load": (I32, [ctypes.c_char_p, ctypes.c_char_p]),
        "gb_add_data_directory": (I32, [ctypes.c_char_p]),
        "gb_mech_del": (I32, [I32]),
        "gb_mech_n_species": (I32, [I32]),
        "gb_mech_n_reactions": (I32, [I32]),
        "gb_mech_species_name": (I32, [I32, I32, I32, ctypes.c_char_p]),
        "gb_mech_species_index": (I32, [I32, ctypes.c_char_p]),
        "gb_mech_molecular_weights": (I32, [I32, I32, P]),
        "gb_kin_net_production_rates": (I32, [I32, I32, P, P, P, I32, P, I32]),
        "gb_kin_jac_nnz": (I32, [I32]),
        "gb_kin_jac_pattern": (I32, [I32, I32, P, I32, P]),
        "gb_kin_net_production_rates_ddCi": (I32, [I32, I32, P, P, P, I32, P, P, I32]),
        "gb_net_default_options": (None, [ctypes.POINTER(NetOptions)]),
        "gb_net_new": (I32, [I32, I32, ctypes.POINTER(NetOptions)]),
        "gb_net_del": (I32, [I32]),
        "gb_net_set_state": (I32, [I32, P, P, P, I32]),
        "gb_net_set_tolerances": (I32, [I32, D, D]),
        "gb_net_set_max_steps": (I32, [I32, I32]),
        "gb_net_set_max_time_step": (I32, [I32, D]),
        "gb_net_advance": (I32, [I32, D]),
        "gb_net_step": (I32, [I32, P, I32]),
        "gb_net_checkpoint_bytes": (ctypes.c_int64, [I32]),
        "gb_net_checkpoint": (I32, [I32, P, ctypes.c_int64]),
        "gb_net_restore": (I32, [I32, P, ctypes.c_int64]),
        "gb_net_time": (D, [I32]),
        "gb_kin_last_kernel_ms": (D, [I32]),
        "gb_check_status": (I32, [I32, P]),
        "gb_net_last_advance_ms": (D, [I32]),
        "gb_net_get_state": (I32, [I32, P, P, I32]),
        "gb_net_get_derivative": (I32, [I32, I32, P, I32]),
        "gb_net_get_status": (I32, [I32, P]),
        "gb_net_solver_stats": (I32, [I32, P]),
        "gb_net_ignition_times": (I32, [I32, P]),
        "gb_net_krylov_stats": (I32, [I32, P]),
        "gb_precond_ilut": (I32, [I32, I32, P, P]),
        "gb_net_launch_info": (I32, [I32, P]),
        "gb_reactor_rhs": (I32, [I32, I32, P, P, P, P, P, I32]),
        "gb_mech_n_elements": (I32, [I32]),
        "gb_mech_element_mass": (I32, [I32, I32, P]),
        "gb_nn_gemm": (I32, [I32, I32, I32, P, ctypes.c_int64, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int64,
                             P, ctypes.c_int64, ctypes.c_int64, I32, ctypes.c_float, P, I32, P, ctypes.c_int64,
                             ctypes.c_int64, I32]),
        "gb_nn_gemm_tc": (I32, [I32, I32, I32, P, ctypes.c_int64, P, ctypes.c_int64, P, ctypes.c_int64, I32,
                                ctypes.c_float, P, I32, P, ctypes.c_int64, I32, P, ctypes.c_int64, I32, P]),
        "gb_nn_transpose": (I32, [I32, I32, P, ctypes.c_int64, P, ctypes.c_int64, P]),
        "gb_nn_sync": (I32, [P]),
        "gb_nn_set_stream": (I32, [P, I32]),
        "gb_nn_adam": (I32, [I32, P, P, P, P, P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, I32]),
        "gb_nn_colsum": (I32, [I32, I32, P, I32, ctypes.c_float, P]),
        "gb_nn_mse": (I32, [I32, I32, I32, P, P, P, P]),
        "gb_nn_features": (I32, [I32, I32, P, P, P, P, P, P, I32]),
        "gb_nn_apply": (I32, [I32, I32, P, I32, P, P, P, P, D, P, P, P, P]),
        "gb_nn_gate": (I32, [I32, I32, D, P, P, P, P, P, P, P, P, P, D, D, D, D, P, P]),
        "gb_get_error": (I32, [I32, ctypes.c_char_p]),
        "gb_mech_structure": (I32, [I32, I32, P]),
        "gb_mech_equivalence_ratio": (I32, [I32, D, P, P, I32, P]),
        "gb_mech_species_thermo": (I32, [I32, I32, P, P, P, P]),
        "gb_mech_reference_pressure": (D, [I32]),
        "gb_measure_fp64": (I32, [P]),
        "gb_check_exp": (I32, [I32, P, P, P]),
        "gb_check_log": (I32, [I32, P, P, P]),
        "gb_reactors_advance_noalloc": (I32, [I32, I32, D, P, P, P, P, ctypes.POINTER(NetOptions), P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    # mechanisms may draw species from the packaged files ("gri30.yaml/species")
    L.gb_add_data_directory(DATA_DIR.encode())
    _lib = L
    return L


def measure_fp64():
    """Device FP64 FMA rate (GFLOP/s) and exp / log cost in FMA-equivalents."""
    r = np.zeros(3)
    _check(library().gb_measure_fp64(_ptr(r)))
    return {"gflops": float(r[0]), "exp_fma": float(r[1]), "log_fma": float(r[2])}


def _check(rc):
    if rc == GB_ERR:
        buf = ctypes.create_string_buffer(4096)
        library().gb_get_error(4096, buf)
        raise GBError(buf.value.decode())
    return rc


def _is_torch_cuda(a):
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


def _after_torch_stream(a):
    """The engine orders its reads of device arrays after the default stream's work; a tensor
    written on another torch stream is waited for here."""
    import torch
    s = torch.cuda.current_stream(a.device)
    if s.cuda_stream != torch.cuda.default_stream(a.device).cuda_stream:
        s.synchronize()


def _ptr(a):
    if a is None:
        return None
    if _is_torch_cuda(a):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _host(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


class Solution:
    """An ideal-gas mechanism loaded into the engine (``ct.Solution(yaml, phase)``)."""

    def __init__(self, infile, name=""):
        path = infile
        if not os.path.exists(path):
            cand = os.path.join(DATA_DIR, infile)
            if os.path.exists(cand):
                path = cand
        self._h = _check(library().gb_mech_load(path.encode(), name.encode()))
        self.source = (os.path.abspath(path), name)
        L = library()
        self.n_species = _check(L.gb_mech_n_species(self._h))
        self.n_reactions = _check(L.gb_mech_n_reactions(self._h))
        buf = ctypes.create_string_buffer(256)
        self.species_names = []
        for k in range(self.n_species):
            _check(L.gb_mech_species_name(self._h, k, 256, buf))
            self.species_names.append(buf.value.decode())
        self.molecular_weights = np.zeros(self.n_species)
        _check(L.gb_mech_molecular_weights(self._h, self.n_species, _ptr(self.molecular_weights)))
        nnz = _check(L.gb_kin_jac_nnz(self._h))
        self.jac_colptr = np.zeros(self.n_species + 1, dtype=np.int32)
        self.jac_rowidx = np.zeros(nnz, dtype=np.int32)
        _check(L.gb_kin_jac_pattern(self._h, self.n_species + 1, _ptr(self.jac_colptr), nnz,
                                     _ptr(self.jac_rowidx)))

    def structure(self):
        """Structure counts used by the FP64 operation model of the benchmark."""
        c = np.zeros(16, dtype=np.int64)
        _check(library().gb_mech_structure(self._h, 16, _ptr(c)))
        keys = ["K", "R", "reversible", "falloff", "troe", "three_body", "tb_entries",
                "gather_entries", "jac_col_entries", "jac_scatter_entries", "reac_slots", "prod_slots",
                "arena_rhs_bytes", "arena_jacobian_bytes", "arena_side_bytes", "arena_bytes"]
        return dict(zip(keys, (int(v) for v in c)))

    def species_index(self, name):
        k = library().gb_mech_species_index(self._h, name.encode())
        if k < 0:
            raise KeyError(name)
        return k

    def composition(self, spec):
        """'CH4:1, O2:2' -> normalised mole fractions over the species."""
        x = np.zeros(self.n_species)
        for item in spec.split(","):
            name, v = item.split(":")
            x[self.species_index(name.strip())] += float(v)
        return x / x.sum()

    def mole_to_mass(self, X):
        y = np.asarray(X, dtype=np.float64) * self.molecular_weights
        return y / y.sum()

    def species_thermo(self, T):
        """cp/R, h/RT and s/R of every species at temperature(s) T (NASA7, host-evaluated):
        arrays [K] for a scalar T, [K, n] for n temperatures."""
        scalar = np.ndim(T) == 0
        Ta = np.ascontiguousarray(np.atleast_1d(np.asarray(T, dtype=np.float64)))
        out = [np.empty((self.n_species, Ta.size)) for _ in range(3)]
        _check(library().gb_mech_species_thermo(self._h, Ta.size, _ptr(Ta), _ptr(out[0]), _ptr(out[1]),
                                                _ptr(out[2])))
        return tuple(o[:, 0].copy() for o in out) if scalar else tuple(out)

    @property
    def reference_pressure(self):
        """Reference pressure of the species' thermodynamic data, Pa."""
        v = library().gb_mech_reference_pressure(self._h)
        if v == -999.999:
            _check(GB_ERR)
        return v

    def equivalence_ratio_mass_fractions(self, phi, fuel, oxidizer):
        """Mass fractions of the fuel/oxidizer mixture with equivalence ratio phi
        (``ThermoPhase.set_equivalence_ratio(phi, fuel, oxidizer)``, molar basis); fuel and
        oxidizer as 'A:1, B:2' strings or mole-fraction arrays over the species."""
        Y = np.zeros(self.n_species)
        comp = lambda c: self.composition(c) if isinstance(c, str) else np.asarray(c, dtype=np.float64)
        f = np.ascontiguousarray(comp(fuel))
        o = np.ascontiguousarray(comp(oxidizer))
        _check(library().gb_mech_equivalence_ratio(self._h, float(phi), _ptr(f), _ptr(o),
                                                   self.n_species, _ptr(Y)))
        return Y

    @property
    def jac_nnz(self):
        return len(self.jac_rowidx)

    def _args(self, T, P, Y):
        if _is_torch_cuda(T):
            _after_torch_stream(T)
            n = T.shape[0]
            return n, T, P, Y, GB_DEVICE_POINTERS
        T = _host(T)
        n = T.shape[0]
        P = _host(np.broadcast_to(np.asarray(P, dtype=np.float64), (n,)))
        Y = _host(Y, (self.n_species, n))
        return n, T, P, Y, 0

    @property
    def last_kernel_ms(self):
        """Device time (ms) of the kernel of the last rates or ddCi call (CUDA events on the
        engine's stream)."""
        return library().gb_kin_last_kernel_ms(self._h)

    def net_production_rates(self, T, P, Y, out=None):
        """wdot[K, n] (kmol/m^3/s) for n states; Y is species-major [K, n]."""
        n, T, P, Y, flags = self._args(T, P, Y)
        if out is None:
            if flags:
                import torch
                out = torch.empty((self.n_species, n), dtype=torch.float64, device=T.device)
            else:
                out = np.empty((self.n_species, n))
        _check(library().gb_kin_net_production_rates(self._h, n, _ptr(T), _ptr(P), _ptr(Y),
                                                      self.n_species * n, _ptr(out), flags))
        return out

    def net_production_rates_ddCi(self, T, P, Y, vals=None, wdot=None):
        """d(wdot)/d(c) values [nnz, n] on the pattern (jac_colptr, jac_rowidx)."""
        n, T, P, Y, flags = self._args(T, P, Y)
        if vals is None:
            if flags:
                import torch
                vals = torch.empty((self.jac_nnz, n), dtype=torch.float64, device=T.device)
            else:
                vals = np.empty((self.jac_nnz, n))
        _check(library().gb_kin_net_production_rates_ddCi(self._h, n, _ptr(T), _ptr(P), _ptr(Y),
                                                           self.jac_nnz, _ptr(vals), _ptr(wdot), flags))
        return vals

    def dense_ddCi(self, vals, s):
        """Dense K x K d(wdot)/dc of state s from pattern values."""
        J = np.zeros((self.n_species, self.n_species))
        v = vals[:, s] if not _is_torch_cuda(vals) else vals[:, s].cpu().numpy()
        for c in range(self.n_species):
            for p in range(self.jac_colptr[c], self.jac_colptr[c + 1]):
                J[self.jac_rowidx[p], c] = v[p]
        return J

    def reactor_rhs(self, T, P, Y):
        """dT/dt [n] and dY/dt [K, n] of constant-pressure ideal-gas reactors at these states
        (IdealGasConstPressureReactor::eval, batched; numpy or torch CUDA arrays)."""
        n, T, P, Y, flags = self._args(T, P, Y)
        if flags:
            import torch
            dT = torch.empty(n, dtype=torch.float64, device=T.device)
            dY = torch.empty((self.n_species, n), dtype=torch.float64, device=T.device)
        else:
            dT, dY = np.empty(n), np.empty((self.n_species, n))
        _check(library().gb_reactor_rhs(self._h, n, _ptr(T), _ptr(P), _ptr(Y), _ptr(dT), _ptr(dY), flags))
        return dT, dY

    def __del__(self):
        try:
            if _lib is not None:
                _lib.gb_mech_del(self._h)
        except Exception:
            pass


LINEAR_SOLVERS = {"DENSE": 0, "GMRES": 1}


class ReactorNet:
    """n independent constant-pressure ideal-gas reactors advanced together.

    linear_solver "DENSE" (default): the mass-fraction reactor with the analytic Jacobian and
    a dense LU.  "GMRES": the reference's preconditioned Krylov path, the mole reactor
    (IdealGasConstPressureMoleReactor) with GMRES and the adaptive preconditioner (ILUT of an
    approximate Jacobian); its per-reactor counters are in krylov_stats."""

    def __init__(self, solution, T, P, Y, rtol=1e-9, atol=1e-15, max_steps=20000, max_order=5,
                 max_time_step=0.0, lu_precision=64, warps_per_block=0, use_graph=False,
                 matrix_placement=0, mechanism_in_shared=0, jacobian_reuse=False, lu_staging=0,
                 linear_solver="DENSE"):
        L = library()
        if str(linear_solver).upper() not in LINEAR_SOLVERS:
            raise ValueError("linear_solver must be one of %s" % sorted(LINEAR_SOLVERS))
        self.linear_solver = str(linear_solver).upper()
        self.solution = solution
        o = NetOptions()
        L.gb_net_default_options(ctypes.byref(o))
        o.rtol, o.atol, o.max_steps, o.max_order = rtol, atol, max_steps, max_order
        o.max_time_step, o.lu_precision = max_time_step, lu_precision
        o.warps_per_block, o.use_graph = warps_per_block, int(use_graph)
        o.matrix_placement = matrix_placement
        o.mechanism_in_shared = mechanism_in_shared
        o.jacobian_reuse = int(jacobian_reuse)
        o.lu_staging = int(lu_staging)
        o.linear_solver = LINEAR_SOLVERS[self.linear_solver]
        n = T.shape[0] if _is_torch_cuda(T) else np.asarray(T).shape[0]
        self.n = n
        self._rtol, self._atol, self._max_steps, self._max_time_step = rtol, atol, max_steps, max_time_step
        self._h = _check(L.gb_net_new(solution._h, n, ctypes.byref(o)))
        self.set_state(T, P, Y)

    # integrator settings, applied from the next step on without restarting the integration
    # (ReactorNet.rtol / atol / max_steps / max_time_step)
    @property
    def rtol(self):
        return self._rtol

    @rtol.setter
    def rtol(self, v):
        _check(library().gb_net_set_tolerances(self._h, float(v), -1.0))
        self._rtol = float(v)

    @property
    def atol(self):
        return self._atol

    @atol.setter
    def atol(self, v):
        _check(library().gb_net_set_tolerances(self._h, -1.0, float(v)))
        self._atol = float(v)

    @property
    def max_steps(self):
        return self._max_steps

    @max_steps.setter
    def max_steps(self, v):
        _check(library().gb_net_set_max_steps(self._h, int(v)))
        self._max_steps = int(v)

    @property
    def max_time_step(self):
        return self._max_time_step

    @max_time_step.setter
    def max_time_step(self, v):
        _check(library().gb_net_set_max_time_step(self._h, float(v)))
        self._max_time_step = float(v)

    def set_state(self, T, P, Y):
        n, T, P, Y, flags = self.solution._args(T, P, Y)
        if n != self.n:
            raise ValueError("expected %d reactors" % self.n)
        _check(library().gb_net_set_state(self._h, _ptr(T), _ptr(P), _ptr(Y), flags))

    def advance(self, t):
        """Advance every reactor to time t; returns the number of failed reactors."""
        return _check(library().gb_net_advance(self._h, float(t)))

    def step(self, times=None):
        """One internal integrator step of every reactor (ReactorNet.step).  Returns each
        reactor's new time ([n]; written into `times` when given, a CUDA tensor or a numpy
        array).  The network's time becomes the latest of them."""
        flags = GB_DEVICE_POINTERS if _is_torch_cuda(times) else 0
        if times is None:
            times = np.empty(self.n)
        self.last_step_failures = _check(library().gb_net_step(self._h, _ptr(times), flags))
        return times

    def checkpoint(self):
        """The network's integrator state (time, records, counters, state) as bytes."""
        L = library()
        nb = L.gb_net_checkpoint_bytes(self._h)
        _check(nb)
        buf = np.empty(nb, dtype=np.uint8)
        _check(L.gb_net_checkpoint(self._h, _ptr(buf), nb))
        return buf.tobytes()

    def restore(self, data):
        """Continue from a checkpoint of a network of the same size and mechanism."""
        buf = np.frombuffer(data, dtype=np.uint8).copy()
        _check(library().gb_net_restore(self._h, _ptr(buf), buf.size))

    @property
    def launch_info(self):
        """blocks, reactors per block, shared bytes per warp, mechanism bytes in shared
        memory, matrix placement (1 shared, 2 global)."""
        v = np.zeros(6, dtype=np.int32)
        _check(library().gb_net_launch_info(self._h, _ptr(v)))
        return dict(zip(["blocks", "warps_per_block", "warp_smem_bytes", "mechanism_smem_bytes",
                         "matrix_placement", "lu_staging_slots"], v.tolist()))

    @property
    def time(self):
        return library().gb_net_time(self._h)

    @property
    def last_kernel_ms(self):
        """Device time (ms) of the integrator launch of the last advance()."""
        return library().gb_net_last_advance_ms(self._h)

    def get_state(self, T=None, Y=None):
        """Temperatures [n] and mass fractions [K, n] at the current time."""
        flags = GB_DEVICE_POINTERS if _is_torch_cuda(T) else 0
        if T is None:
            T = np.empty(self.n)
            Y = np.empty((self.solution.n_species, self.n))
        _check(library().gb_net_get_state(self._h, _ptr(T), _ptr(Y), flags))
        return T, Y

    def get_derivative(self, k, out=None):
        """The k-th time derivative (0..5) of every reactor's integrator state at its output
        time, from the integrator's step history (ReactorNet.get_derivative): [K + 1, n], row 0
        temperature, then the mass fractions (dense solver) or the species amounts in kmol per
        m^3 of initial volume (GMRES).  out: a numpy array or a torch CUDA tensor to fill."""
        flags = GB_DEVICE_POINTERS if _is_torch_cuda(out) else 0
        if out is None:
            out = np.empty((self.solution.n_species + 1, self.n))
        _check(library().gb_net_get_derivative(self._h, int(k), _ptr(out), flags))
        return out

    @property
    def T(self):
        return self.get_state()[0]

    @property
    def Y(self):
        return self.get_state()[1]

    @property
    def status(self):
        s = np.empty(self.n, dtype=np.int32)
        _check(library().gb_net_get_status(self._h, _ptr(s)))
        return s

    @property
    def solver_stats(self):
        """Per-reactor counters as a dict of arrays (CVodesIntegrator::solverStats names)."""
        st = np.empty((self.n, 8), dtype=np.int64)
        _check(library().gb_net_solver_stats(self._h, _ptr(st)))
        return {k: st[:, i] for i, k in enumerate(STAT_NAMES)}

    @property
    def krylov_stats(self):
        """Per-reactor counters of the GMRES path: lin_iters, prec_solves, jt_vec_prod_evals
        (CVodesIntegrator::solverStats names)."""
        st = np.empty((self.n, 3), dtype=np.int64)
        _check(library().gb_net_krylov_stats(self._h, _ptr(st)))
        return {k: st[:, i] for i, k in enumerate(("lin_iters", "prec_solves", "jt_vec_prod_evals"))}

    @property
    def ignition_times(self):
        t = np.empty(self.n)
        _check(library().gb_net_ignition_times(self._h, _ptr(t)))
        return t

    def __del__(self):
        try:
            if _lib is not None:
                _lib.gb_net_del(self._h)
        except Exception:
            pass


def precond_ilut(P):
    """ILUT factors of the adaptive preconditioner (AdaptivePreconditioner::factorize) for a
    batch of matrices P [n, N, N] (or one [N, N]), factored on the GPU one warp per matrix:
    L (unit diagonal, strictly lower part) and U in place, the same shape as P."""
    A = np.ascontiguousarray(P, dtype=np.float64)
    one = A.ndim == 2
    if one:
        A = A[None]
    n, N, N2 = A.shape
    if N != N2:
        raise ValueError("square matrices expected")
    F = np.empty_like(A)
    _check(library().gb_precond_ilut(n, N, _ptr(A), _ptr(F)))
    return F[0] if one else F
