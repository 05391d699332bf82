"""ctypes binding of the CPU oracle (oracle/oracle.cpp).  TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module; the engine itself never does.  ``build()`` compiles the oracle
with the host compiler into ``oracle/_build/liboracle.so``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")
# the same sources built with the reference's release flags (SConstruct:608-610: -O3, the
# compiler's default floating-point contraction): the timed CPU baseline, not the checker
LIB_FAST = os.path.join(HERE, "_build", "liboracle_fast.so")
SOURCES = [
    os.path.join(HERE, "oracle.cpp"),
    os.path.join(ROOT, "cantera_gb300", "csrc", "mechanism.cpp"),
    os.path.join(ROOT, "cantera_gb300", "csrc", "yaml_lite.cpp"),
]
NSTAT = 12
STAT_NAMES = ["steps", "rhs_evals", "newton_iters", "lin_setups", "jac_evals",
              "err_test_fails", "conv_fails", "last_order", "status", "lin_iters", "prec_solves",
              "jtimes_evals"]


def build(force=False, fast=False):
    """Compile the oracle.  The checker (fast=False) is built with -O2 -ffp-contract=off so
    that x86 and Arm agree bit for bit; the timing build (fast=True) with the reference's
    release flags, -O3 and the compiler's default contraction (fused multiply-adds on Arm)."""
    out = LIB_FAST if fast else LIB
    os.makedirs(os.path.dirname(out), exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "oracle.h"), __file__])
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    flags = ["-O3"] if fast else ["-O2", "-ffp-contract=off"]
    tmp = out + ".tmp%d" % os.getpid()
    cmd = ["g++"] + flags + ["-std=c++17", "-fPIC", "-shared", "-o", tmp] + SOURCES + ["-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, out)
    return out


FLAGS = {False: "g++ -O2 -ffp-contract=off", True: "g++ -O3 (default FP contraction)"}


class BdfOpts(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("max_steps", ctypes.c_int32), ("max_order", ctypes.c_int32),
                ("analytic_jacobian", ctypes.c_int32), ("lu_fp32", ctypes.c_int32),
                ("max_time_step", ctypes.c_double), ("jac_reuse", ctypes.c_int32),
                ("mole_reactor", ctypes.c_int32), ("linear_solver", ctypes.c_int32)]


def opts(rtol=1e-9, atol=1e-15, max_steps=20000, max_order=5, analytic=False,
         lu_fp32=False, max_time_step=0.0, jac_reuse=None, mole_reactor=False, gmres=False):
    """Integrator options.  Defaults follow the reference ReactorNet (rtol 1e-9, atol 1e-15,
    20000 steps per advance, order 5, difference-quotient Jacobian kept between setups).
    mole_reactor: the reactor with moles as its state (IdealGasConstPressureMoleReactor);
    gmres: GMRES with the adaptive preconditioner instead of the dense LU (mole reactor only)."""
    if jac_reuse is None:
        jac_reuse = not analytic
    if (mole_reactor or gmres) and analytic:
        raise ValueError("the mole reactor has no analytic Jacobian: use the difference-quotient one")
    return BdfOpts(rtol, atol, max_steps, max_order, int(analytic), int(lu_fp32), max_time_step,
                   int(jac_reuse), int(mole_reactor or gmres), int(gmres))


_libs = {}


def lib(fast=False):
    """The oracle library: the checker build, or with fast=True the timing build."""
    if fast not in _libs:
        L = ctypes.CDLL(build(fast=fast))
        D = ctypes.POINTER(ctypes.c_double)
        I32 = ctypes.c_int32
        L.or_mech_load.restype = I32
        L.or_mech_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.or_last_error.restype = ctypes.c_char_p
        L.or_rates_batch.argtypes = [I32, I32, D, D, D, D, I32, ctypes.POINTER(I32),
                                     ctypes.POINTER(I32), D, D, I32]
        L.or_advance_batch.argtypes = [I32, I32, D, D, D, ctypes.c_double,
                                       ctypes.POINTER(BdfOpts), D, D,
                                       ctypes.POINTER(ctypes.c_int64), D, I32]
        L.or_advance_trajectory.argtypes = [I32, ctypes.c_double, ctypes.c_double, D, I32, D,
                                            ctypes.POINTER(BdfOpts), D,
                                            ctypes.POINTER(ctypes.c_int64)]
        L.or_ignition_by_steps.argtypes = [I32, ctypes.c_double, ctypes.c_double, D,
                                           ctypes.c_double, ctypes.POINTER(BdfOpts), D,
                                           ctypes.POINTER(ctypes.c_int64)]
        L.or_thermo.argtypes = [I32, ctypes.c_double, D, D, D]
        L.or_rates.argtypes = [I32, ctypes.c_double, ctypes.c_double, D, D, D, D, D, D, D]
        L.or_ddci.argtypes = [I32, ctypes.c_double, ctypes.c_double, D, I32, D]
        L.or_reactor_rhs.argtypes = [I32, ctypes.c_double, D, D]
        L.or_mole_reactor_rhs.argtypes = [I32, ctypes.c_double, D, D]
        L.or_mole_precond_jacobian.argtypes = [I32, ctypes.c_double, D, ctypes.c_double, D]
        L.or_ilut.argtypes = [I32, D]
        L.or_ilut.restype = I32
        L.or_prec_order.argtypes = [I32, ctypes.POINTER(I32)]
        L.or_prec_order.restype = I32
        L.or_jac_pattern.argtypes = [I32, I32, ctypes.POINTER(I32), ctypes.POINTER(I32)]
        L.or_jac_pattern.restype = I32
        L.or_equivalence_ratio.argtypes = [I32, ctypes.c_double, D, D, D]
        L.or_mole_to_mass.argtypes = [I32, D, D]
        L.or_molecular_weights.argtypes = [I32, D]
        L.or_species_index.argtypes = [I32, ctypes.c_char_p]
        L.or_add_data_directory.argtypes = [ctypes.c_char_p]
        # files that other mechanism files reference (e.g. "gri30.yaml/species")
        L.or_add_data_directory(os.path.join(ROOT, "cantera_gb300", "data").encode())
        _libs[fast] = L
    return _libs[fast]


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Mech:
    """A mechanism loaded into the oracle."""

    def __init__(self, path, phase="", fast=False):
        """fast=True: the timing build (the reference's compiler flags) instead of the checker."""
        self.L = L = lib(fast)
        self.fast = fast
        self.h = L.or_mech_load(path.encode(), phase.encode())
        if self.h < 0:
            raise RuntimeError(L.or_last_error().decode())
        K = ctypes.c_int32()
        R = ctypes.c_int32()
        L.or_mech_sizes(self.h, ctypes.byref(K), ctypes.byref(R))
        self.K, self.R = K.value, R.value
        self.mw = np.zeros(self.K)
        L.or_molecular_weights(self.h, _p(self.mw))

    def species_index(self, name):
        return self.L.or_species_index(self.h, name.encode())

    def composition(self, spec):
        """'H2:2, O2:1' -> normalised array over species (mole basis)."""
        x = np.zeros(self.K)
        for item in spec.split(","):
            n, v = item.split(":")
            k = self.species_index(n.strip())
            if k < 0:
                raise KeyError(n)
            x[k] += float(v)
        return x / x.sum()

    def mole_to_mass(self, X):
        Y = np.zeros(self.K)
        self.L.or_mole_to_mass(self.h, _p(_c(X)), _p(Y))
        return Y

    def equivalence_ratio(self, phi, fuel, oxidizer):
        Y = np.zeros(self.K)
        self.L.or_equivalence_ratio(self.h, phi, _p(_c(self.composition(fuel))),
                                   _p(_c(self.composition(oxidizer))), _p(Y))
        return Y

    def thermo(self, T):
        cp, h, s = np.zeros(self.K), np.zeros(self.K), np.zeros(self.K)
        self.L.or_thermo(self.h, T, _p(cp), _p(h), _p(s))
        return cp, h, s

    def rates(self, T, P, Y):
        out = {k: np.zeros(self.R) for k in ("kf", "rkc", "ropf", "ropr", "ropnet")}
        wdot = np.zeros(self.K)
        self.L.or_rates(self.h, T, P, _p(_c(Y)), _p(out["kf"]), _p(out["rkc"]), _p(out["ropf"]),
                       _p(out["ropr"]), _p(out["ropnet"]), _p(wdot))
        out["wdot"] = wdot
        return out

    def ddci(self, T, P, Y, mode=0):
        J = np.zeros((self.K, self.K))
        self.L.or_ddci(self.h, T, P, _p(_c(Y)), mode, _p(J))
        return J

    def rates_batch(self, T, P, Y_sm, mode=1, pattern=None, threads=None, gross=False):
        """Species-major batch: Y_sm [K][n].  Returns wdot [K][n], jac [nnz][n] (or None)
        and, with gross=True, the gross-rate scale [K][n] as a third value."""
        n = len(T)
        threads = threads or os.cpu_count()
        wdot = np.zeros((self.K, n))
        gr = np.zeros((self.K, n)) if gross else None
        jac = None
        cp = ri = None
        if pattern is not None:
            colptr, rowidx = pattern
            cp = np.ascontiguousarray(colptr, dtype=np.int32)
            ri = np.ascontiguousarray(rowidx, dtype=np.int32)
            jac = np.zeros((len(ri), n))
        I = ctypes.POINTER(ctypes.c_int32)
        self.L.or_rates_batch(self.h, n, _p(_c(T)), _p(_c(P)), _p(_c(Y_sm)), _p(wdot), mode,
                             cp.ctypes.data_as(I) if cp is not None else None,
                             ri.ctypes.data_as(I) if ri is not None else None,
                             _p(jac) if jac is not None else None, _p(gr), threads)
        if gross:
            return wdot, jac, gr
        return wdot, jac

    def reactor_rhs(self, P, y):
        ydot = np.zeros(self.K + 2)
        self.L.or_reactor_rhs(self.h, P, _p(_c(y)), _p(ydot))
        return ydot

    def mole_reactor_rhs(self, P, z):
        """Mole-reactor right-hand side for z = [T, n_1..n_K] (kmol) at pressure P."""
        zdot = np.zeros(self.K + 1)
        st = self.L.or_mole_reactor_rhs(self.h, P, _p(_c(z)), _p(zdot))
        return zdot, st

    def mole_precond_jacobian(self, P, z, atol=1e-15):
        """The adaptive preconditioner's Jacobian elements [K+1, K+1] at z."""
        J = np.zeros((self.K + 1, self.K + 1))
        st = self.L.or_mole_precond_jacobian(self.h, P, _p(_c(z)), atol, _p(J))
        return J, st

    def prec_order(self):
        """The Krylov path's fill-reducing order of z = [T, n_1..n_K] (order[new] = old)."""
        o = np.zeros(self.K + 1, dtype=np.int32)
        if self.L.or_prec_order(self.h, o.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) != self.K + 1:
            raise RuntimeError(self.L.or_last_error().decode())
        return o

    def jac_pattern(self):
        """The structural pattern of d(wdot)/dc (CSC colptr [K+1], rowidx [nnz])."""
        cp = np.zeros(self.K + 1, dtype=np.int32)
        ri = np.zeros(self.K * self.K, dtype=np.int32)
        I = ctypes.POINTER(ctypes.c_int32)
        nnz = self.L.or_jac_pattern(self.h, len(ri), cp.ctypes.data_as(I), ri.ctypes.data_as(I))
        if nnz < 0:
            raise RuntimeError(self.L.or_last_error().decode())
        return cp, ri[:nnz].copy()

    def advance_batch(self, T0, P, Y0, t_end, o=None, threads=None):
        """Reactor-major Y0 [n][K].  Returns T [n], Y [n][K], stats [n][9], tign [n]."""
        n = len(T0)
        o = o or opts()
        threads = threads or os.cpu_count()
        T = np.zeros(n)
        Y = np.zeros((n, self.K))
        st = np.zeros((n, NSTAT), dtype=np.int64)
        tig = np.zeros(n)
        self.L.or_advance_batch(self.h, n, _p(_c(T0)), _p(_c(P)), _p(_c(Y0)), t_end,
                               ctypes.byref(o), _p(T), _p(Y),
                               st.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _p(tig), threads)
        return T, Y, st, tig

    def trajectory(self, T0, P, Y0, times, o=None):
        o = o or opts()
        times = _c(times)
        out = np.zeros((len(times), self.K + 1))
        st = np.zeros(NSTAT, dtype=np.int64)
        rc = self.L.or_advance_trajectory(self.h, T0, P, _p(_c(Y0)), len(times), _p(times),
                                         ctypes.byref(o), _p(out),
                                         st.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        return out, st, rc

    def ignition_by_steps(self, T0, P, Y0, dT=500.0, o=None):
        o = o or opts()
        t = ctypes.c_double()
        st = np.zeros(NSTAT, dtype=np.int64)
        rc = self.L.or_ignition_by_steps(self.h, T0, P, _p(_c(Y0)), dT, ctypes.byref(o),
                                        ctypes.byref(t),
                                        st.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        return t.value, st, rc


def ilut(A, fast=False):
    """The adaptive preconditioner's ILUT of one N x N matrix (row-major copy): L (unit
    diagonal, strictly lower part) and U in one array."""
    a = np.array(A, dtype=np.float64, order="C", copy=True)
    n = a.shape[0]
    if lib(fast).or_ilut(n, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) != 0:
        raise RuntimeError("or_ilut failed")
    return a
