"""Learned surrogate of the reactor step with a physics gate and a BDF fallback.

A multilayer perceptron maps a reactor state (T, ln P, Box-Cox(Y, lambda 0.1)) to its
change over a fixed step dt (dY, dT, each standardised), learned as the correction to the
explicit step dt f(x0) (f the reactor right-hand side), relative to that step's size:
slow states need almost none.  Training pairs come from the
batched integrator; training and inference run on the engine's own kernels (BF16
tensor-core GEMMs accumulating in FP32 with fused bias/GELU epilogues, the MSE gradient,
bias-gradient sums and Adam; ``gb_nn_*`` in include/gbchem.h).  Each prediction is gated by
element and enthalpy conservation and by the trapezoidal rule with the reactor right-hand
sides at both ends; reactors that fail fall back to the FP64 BDF integrator.

torch provides device memory, the one-off normalisation statistics and the batch
gathers; the network arithmetic (forward, backward, optimiser), the features, the gate and
the integrator are calls into libgbchem.
"""
import ctypes
import math

import numpy as np

from . import GB_DEVICE_POINTERS, ReactorNet, _check, library

PAD_IN = 128      # 2 + K inputs, zero padded (a multiple of 128 for the weight-gradient GEMM)
PAD_OUT = 128     # K + 1 outputs, zero padded


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class Surrogate:
    """MLP ``2+K -> hidden x layers (GELU) -> K+1`` over the step ``dt`` of ``solution``."""

    def __init__(self, solution, dt=1e-6, hidden=512, layers=4, seed=0, device="cuda:0"):
        import torch
        self.torch = torch
        self.sol = solution
        self.K = solution.n_species
        if self.K + 2 > PAD_IN or self.K + 1 > PAD_OUT:
            raise ValueError("mechanism too large for the surrogate's input padding")
        if hidden % 128:
            raise ValueError("hidden width must be a multiple of 128")
        self.dt = float(dt)
        self.dev = torch.device(device)
        dims = [PAD_IN] + [hidden] * layers + [PAD_OUT]
        real_in = [self.K + 2] + [hidden] * layers
        real_out = [hidden] * layers + [self.K + 1]
        g = torch.Generator().manual_seed(seed)
        self.W, self.Wb, self.b, self.mW, self.vW, self.mb, self.vb = [], [], [], [], [], [], []
        for l in range(len(dims) - 1):
            n_out, n_in = dims[l + 1], dims[l]
            w = torch.zeros(n_out, n_in)
            bound = math.sqrt(6.0 / (real_in[l] + real_out[l]))
            w[:real_out[l], :real_in[l]] = (torch.rand(real_out[l], real_in[l], generator=g) * 2 - 1) * bound
            w = w.to(self.dev)
            self.W.append(w)
            self.Wb.append(w.to(torch.bfloat16))
            self.b.append(torch.zeros(n_out, device=self.dev))
            self.mW.append(torch.zeros_like(w))
            self.vW.append(torch.zeros_like(w))
            self.mb.append(torch.zeros(n_out, device=self.dev))
            self.vb.append(torch.zeros(n_out, device=self.dev))
        self.dims = dims
        self.step_count = 0
        self.mu_in = self.sd_in = self.mu_out = self.sd_out = None
        L = library()
        E = L.gb_mech_n_elements(solution._h)
        em = np.zeros(E * self.K)
        _check(L.gb_mech_element_mass(solution._h, E * self.K, em.ctypes.data_as(ctypes.c_void_p)))
        self.elem_mass = torch.tensor(em, device=self.dev)

    # ---- normalisation -------------------------------------------------------------
    FLOOR_Y, FLOOR_T = 1e-12, 1e-6     # the kernels' floors of the correction scale

    def _residual(self, T0, P, Y0, T1, Y1):
        """(x1 - x0 - dt f0) / (dt |f0| + floor), [K+1, n]: the correction the network learns."""
        f0T, f0Y = self.rhs(T0, P, Y0)
        rY = (Y1 - Y0 - self.dt * f0Y) / (self.dt * f0Y.abs() + self.FLOOR_Y)
        rT = (T1 - T0 - self.dt * f0T) / (self.dt * f0T.abs() + self.FLOOR_T)
        return self.torch.cat([rY, rT[None, :]], dim=0)

    def fit_normalization(self, T0, P, Y0, T1, Y1):
        """Per-feature mean and spread of the inputs and of the step corrections (device
        arrays, species-major Y [K, n])."""
        torch = self.torch
        bc = (torch.clamp(Y0, min=0.0) ** 0.1 - 1.0) * 10.0
        feats = torch.cat([T0[None, :], torch.log(P)[None, :], bc], dim=0)        # [K+2, n]
        self.mu_in = feats.mean(dim=1).float()
        self.sd_in = feats.std(dim=1).clamp(min=1e-6).float()
        d = self._residual(T0, P, Y0, T1, Y1)
        self.mu_out = d.mean(dim=1).float()
        self.sd_out = d.std(dim=1).clamp(min=1e-30).float()

    def features(self, T, P, Y):
        n = T.shape[0]
        X = self.torch.zeros(self._rows(n), PAD_IN, dtype=self.torch.bfloat16, device=self.dev)
        _check(library().gb_nn_features(self.sol._h, n, _p(T), _p(P), _p(Y), _p(self.mu_in), _p(self.sd_in),
                                        _p(X), PAD_IN))
        return X

    def targets(self, T0, P, Y0, T1, Y1):
        n = T0.shape[0]
        torch = self.torch
        d = self._residual(T0, P, Y0, T1, Y1).float()
        t = (d - self.mu_out[:, None]) / self.sd_out[:, None]
        out = torch.zeros(self._rows(n), PAD_OUT, device=self.dev)
        out[:n, :self.K + 1] = t.T
        return out

    @staticmethod
    def _rows(n):
        return ((n + 127) // 128) * 128

    # ---- network ---------------------------------------------------------------------
    def _gemm(self, M, N, K, A, sam, sak, B, sbn, sbk, C, scm, scn, c_float, alpha=1.0, bias=None, act=0,
              Z=None, szm=0, szn=0, z_float=1):
        _check(library().gb_nn_gemm(M, N, K, _p(A), sam, sak, _p(B), sbn, sbk, _p(C), scm, scn, c_float, alpha,
                                    _p(bias), act, _p(Z), szm, szn, z_float))

    def forward(self, X, keep=False):
        """Output [M, PAD_OUT] (float) of a padded input batch X [M, PAD_IN] (bf16)."""
        torch = self.torch
        M = X.shape[0]
        A = X
        cache = []
        nl = len(self.W)
        for l in range(nl):
            n_out, n_in = self.dims[l + 1], self.dims[l]
            if l < nl - 1:
                Z = torch.empty(M, n_out, device=self.dev) if keep else None
                C = torch.empty(M, n_out, dtype=torch.bfloat16, device=self.dev)
                self._gemm(M, n_out, n_in, A, n_in, 1, self.Wb[l], n_in, 1, C, n_out, 1, 0, 1.0, self.b[l], 1,
                           Z, n_out, 1, 1)
            else:
                Z = None
                C = torch.empty(M, n_out, device=self.dev)
                self._gemm(M, n_out, n_in, A, n_in, 1, self.Wb[l], n_in, 1, C, n_out, 1, 1, 1.0, self.b[l], 0)
            cache.append((A, Z))
            A = C
        return (A, cache) if keep else A

    def gradients(self, X, Ytarget, n_real):
        """Loss and parameter gradients of a batch (the rows beyond n_real are padding and
        must carry zero targets and zero inputs)."""
        torch = self.torch
        M = X.shape[0]
        out, cache = self.forward(X, keep=True)
        if n_real < M:
            out[n_real:] = 0.0
        loss = torch.zeros(1, device=self.dev)
        dZ = torch.empty(M, PAD_OUT, dtype=torch.bfloat16, device=self.dev)
        _check(library().gb_nn_mse(M, self.K + 1, PAD_OUT, _p(out), _p(Ytarget), _p(dZ), _p(loss)))
        # the loss is averaged over the n_real rows
        scale = M / float(n_real)
        gW, gb = [None] * len(self.W), [None] * len(self.W)
        for l in range(len(self.W) - 1, -1, -1):
            n_out, n_in = self.dims[l + 1], self.dims[l]
            A, _ = cache[l]
            gW[l] = torch.empty(n_out, n_in, device=self.dev)
            # dW = dZ^T A: (n_out x M) (M x n_in)
            self._gemm(n_out, n_in, M, dZ, 1, n_out, A, 1, n_in, gW[l], n_in, 1, 1, scale)
            gb[l] = torch.empty(n_out, device=self.dev)
            _check(library().gb_nn_colsum(M, n_out, _p(dZ), n_out, scale, _p(gb[l])))
            if l > 0:
                _, Zp = cache[l - 1]
                dprev = torch.empty(M, n_in, dtype=torch.bfloat16, device=self.dev)
                # dZ_prev = (dZ W) * GELU'(Z_prev): (M x n_out)(n_out x n_in)
                self._gemm(M, n_in, n_out, dZ, n_out, 1, self.Wb[l], 1, n_in, dprev, n_in, 1, 0, 1.0, None, 2,
                           Zp, n_in, 1, 1)
                dZ = dprev
        return float(loss.item()) * scale, gW, gb

    def adam_step(self, gW, gb, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        L = library()
        for l in range(len(self.W)):
            _check(L.gb_nn_adam(self.W[l].numel(), _p(self.W[l]), _p(self.mW[l]), _p(self.vW[l]), _p(gW[l]),
                                _p(self.Wb[l]), lr, beta1, beta2, eps, self.step_count))
            bb = self.torch.empty(self.b[l].shape, dtype=self.torch.bfloat16, device=self.dev)
            _check(L.gb_nn_adam(self.b[l].numel(), _p(self.b[l]), _p(self.mb[l]), _p(self.vb[l]), _p(gb[l]),
                                _p(bb), lr, beta1, beta2, eps, self.step_count))

    def train(self, X, Yt, n, epochs=10, batch=8192, lr=1e-3, seed=0, log=None):
        """Mini-batch Adam over the n training rows of X [>=n, PAD_IN], Yt [>=n, PAD_OUT]."""
        torch = self.torch
        batch = min(self._rows(batch), self._rows(n))
        g = torch.Generator(device=self.dev).manual_seed(seed)
        losses = []
        for ep in range(epochs):
            perm = torch.randperm(n, device=self.dev, generator=g)
            tot, cnt = 0.0, 0
            for s in range(0, n, batch):
                idx = perm[s:s + batch]
                m = idx.numel()
                Xb = torch.zeros(batch, PAD_IN, dtype=torch.bfloat16, device=self.dev)
                Yb = torch.zeros(batch, PAD_OUT, device=self.dev)
                Xb[:m] = X[idx]
                Yb[:m] = Yt[idx]
                loss, gW, gb = self.gradients(Xb, Yb, m)
                self.adam_step(gW, gb, lr=lr * (0.5 * (1 + math.cos(math.pi * ep / max(1, epochs)))))
                tot += loss * m
                cnt += m
            losses.append(tot / cnt)
            if log:
                log(ep, losses[-1])
        return losses

    # ---- inference with the gate and the fallback -------------------------------------
    def predict(self, T, P, Y, f0=None):
        """Predicted state after dt (device arrays; Y species-major [K, n]) and the
        right-hand side at the start (f0T, f0Y)."""
        torch = self.torch
        n = T.shape[0]
        if f0 is None:
            f0 = self.rhs(T, P, Y)
        X = self.features(T, P, Y)
        O = self.forward(X)
        T1 = torch.empty_like(T)
        Y1 = torch.empty_like(Y)
        _check(library().gb_nn_apply(self.sol._h, n, _p(O), PAD_OUT, _p(self.mu_out), _p(self.sd_out), _p(T), _p(Y),
                                     self.dt, _p(f0[0]), _p(f0[1]), _p(T1), _p(Y1)))
        return T1, Y1, f0

    def rhs(self, T, P, Y):
        torch = self.torch
        dT = torch.empty_like(T)
        dY = torch.empty_like(Y)
        _check(library().gb_reactor_rhs(self.sol._h, T.shape[0], _p(T), _p(P), _p(Y), _p(dT), _p(dY),
                                        GB_DEVICE_POINTERS))
        return dT, dY

    def gate(self, T0, P, Y0, T1, Y1, tol_elem=1e-5, tol_h=1e-5, tol_trap_t=1e-4, tol_trap_y=1e-5, f0=None):
        """accept [n] (int32) and score [n] of predicted steps."""
        torch = self.torch
        n = T0.shape[0]
        f0T, f0Y = self.rhs(T0, P, Y0) if f0 is None else f0
        f1T, f1Y = self.rhs(T1, P, Y1)
        acc = torch.empty(n, dtype=torch.int32, device=self.dev)
        score = torch.empty(n, dtype=torch.float64, device=self.dev)
        _check(library().gb_nn_gate(self.sol._h, n, self.dt, _p(T0), _p(Y0), _p(T1), _p(Y1), _p(f0T), _p(f0Y),
                                    _p(f1T), _p(f1Y), _p(self.elem_mass), tol_elem, tol_h, tol_trap_t, tol_trap_y,
                                    _p(acc), _p(score)))
        return acc, score

    def advance(self, T, P, Y, rtol=1e-8, atol=1e-15, timings=None, **tols):
        """One step dt for every reactor: the surrogate where the gate accepts it, the FP64
        BDF integrator elsewhere.  Returns T1, Y1 and the accepted mask (and, given a dict
        `timings`, the seconds of its phases)."""
        import time
        torch = self.torch

        def mark(name, t0):
            if timings is not None:
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                timings[name] = timings.get(name, 0.0) + (t1 - t0)
                return t1
            return t0
        t0 = time.perf_counter()
        T1, Y1, f0 = self.predict(T, P, Y)
        t0 = mark("predict", t0)
        acc, _ = self.gate(T, P, Y, T1, Y1, f0=f0, **tols)
        t0 = mark("gate", t0)
        rej = torch.nonzero(acc == 0).flatten()
        if rej.numel() > 0:
            Tr, Pr = T[rej].contiguous(), P[rej].contiguous()
            Yr = Y[:, rej].contiguous()
            net = ReactorNet(self.sol, Tr, Pr, Yr, rtol=rtol, atol=atol)
            t0 = mark("fallback_setup", t0)
            net.advance(self.dt)
            t0 = mark("fallback_advance", t0)
            Tf, Yf = torch.empty_like(Tr), torch.empty_like(Yr)
            net.get_state(Tf, Yf)
            T1[rej] = Tf
            Y1[:, rej] = Yf
            t0 = mark("fallback_gather", t0)
        return T1, Y1, acc


def trajectory_states(solution, T0, P, Y0, times, rtol=1e-8, atol=1e-15):
    """States of reactors started at (T0, P, Y0) at each time in `times` (device arrays,
    species-major Y): Ts, Ps, Ys with n_reactors * len(times) columns."""
    import torch
    net = ReactorNet(solution, T0, P, Y0, rtol=rtol, atol=atol, use_graph=False)
    Ts, Ys = [], []
    for t in times:
        if t > 0:
            net.advance(float(t))
        T = torch.empty_like(T0)
        Y = torch.empty_like(Y0)
        net.get_state(T, Y)
        Ts.append(T)
        Ys.append(Y)
    return torch.cat(Ts), P.repeat(len(times)), torch.cat(Ys, dim=1).contiguous()


def generate_pairs(solution, T0, P, Y0, times, dt, rtol=1e-8, atol=1e-15):
    """Training pairs along trajectories: the states of reactors started at (T0, P, Y0) at
    each time in `times`, and the same states advanced by dt.  Device arrays, species-major
    Y; returns Ts, Ps, Ys (inputs) and T1, Y1 (after dt), n_reactors * len(times) columns."""
    import torch
    Ts, Ps, Ys = trajectory_states(solution, T0, P, Y0, times, rtol, atol)
    net2 = ReactorNet(solution, Ts, Ps, Ys, rtol=rtol, atol=atol, use_graph=False)
    net2.advance(dt)
    T1 = torch.empty_like(Ts)
    Y1 = torch.empty_like(Ys)
    net2.get_state(T1, Y1)
    return Ts, Ps, Ys, T1, Y1
