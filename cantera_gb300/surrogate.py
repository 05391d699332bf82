"""Learned surrogate of the reactor step with a physics gate and a BDF fallback.

A multilayer perceptron maps a reactor state (T, ln P, Box-Cox(Y, lambda 0.1)) to its
change over a fixed step dt (dY, dT, each standardised), learned as the correction to the
explicit step dt f(x0) (f the reactor right-hand side), relative to that step's size:
slow states need almost none.  Training pairs come from the
batched integrator; training and inference run on the engine's own kernels (BF16
GEMMs on the tcgen05 tensor cores accumulating in FP32 tensor memory, with fused bias/GELU
epilogues that also write the transposed copies the backward pass reads; the MSE gradient,
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
        self.W, self.Wb, self.WbT, self.b, self.mW, self.vW, self.mb, self.vb = [], [], [], [], [], [], [], []
        for l in range(len(dims) - 1):
            n_out, n_in = dims[l + 1], dims[l]
            w = torch.zeros(n_out, n_in)
            bound = math.sqrt(6.0 / (real_in[l] + real_out[l]))
            w[:real_out[l], :real_in[l]] = (torch.rand(real_out[l], real_in[l], generator=g) * 2 - 1) * bound
            w = w.to(self.dev)
            self.W.append(w)
            self.Wb.append(w.to(torch.bfloat16))
            self.WbT.append(self.Wb[-1].T.contiguous())
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

    # Standardised corrections are heavy-tailed (on the gri30 workload's 2^22 pairs: 99.9th
    # percentile 3.6, 99.99th 29, largest 2,044 standard deviations), and a few such rows set
    # the gradient of a mean-squared loss.  Training targets are clipped at this many standard
    # deviations (0.07 % of the values there); states that need larger corrections are left to
    # the gate and the integrator.
    TARGET_CLIP = 5.0

    def targets(self, T0, P, Y0, T1, Y1):
        n = T0.shape[0]
        torch = self.torch
        d = self._residual(T0, P, Y0, T1, Y1).float()
        t = ((d - self.mu_out[:, None]) / self.sd_out[:, None]).clamp(-self.TARGET_CLIP, self.TARGET_CLIP)
        out = torch.zeros(self._rows(n), PAD_OUT, device=self.dev)
        out[:n, :self.K + 1] = t.T
        return out

    @staticmethod
    def _rows(n):
        return ((n + 127) // 128) * 128

    # ---- network ---------------------------------------------------------------------
    # Every product is one call of the tensor-core GEMM (gb_nn_gemm_tc: tcgen05.mma with
    # TMEM accumulators, TMA-staged K-major operands).  The backward pass needs the layer
    # inputs and the output gradients transposed (the weight gradient dW = dZ^T X reduces
    # over the batch, which must be the K-major dimension of both operands): the forward
    # epilogues write X^T next to X, the backward epilogues dZ^T next to dZ, and W^T is kept
    # beside W.
    def _tc(self, A, B, C, alpha=1.0, bias=None, act=0, Z=None, CT=None, splits=1):
        M, K = A.shape
        N = B.shape[0]
        _check(library().gb_nn_gemm_tc(M, N, K, _p(A), A.stride(0), _p(B), B.stride(0), _p(C), C.stride(0),
                                       int(C.dtype.itemsize == 4), alpha, _p(bias), act, _p(Z),
                                       Z.stride(0) if Z is not None else 0,
                                       int(Z is not None and Z.dtype.itemsize == 4), _p(CT),
                                       CT.stride(0) if CT is not None else 0, splits, self._stream()))

    def _stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def _transpose(self, X, XT):
        _check(library().gb_nn_transpose(X.shape[0], X.shape[1], _p(X), X.stride(0), _p(XT), XT.stride(0),
                                         self._stream()))

    def _refresh_transposed_weights(self):
        for l in range(len(self.Wb)):
            self._transpose(self.Wb[l], self.WbT[l])

    @staticmethod
    def _splits(M, tiles):
        """K-splits of a weight-gradient product (K = batch rows): about one block per SM."""
        s = 1
        while s * 2 * tiles <= 148 and M % (64 * s * 2) == 0:
            s *= 2
        return s

    def forward(self, X, keep=False, buf=None):
        """Output [M, PAD_OUT] (float) of a padded input batch X [M, PAD_IN] (bf16).  keep:
        also the pre-activations and the transposed layer inputs of the backward pass (in
        the training buffers `buf`)."""
        torch = self.torch
        M = X.shape[0]
        A = X
        nl = len(self.W)
        for l in range(nl):
            n_out = self.dims[l + 1]
            if l < nl - 1:
                C = buf["act"][l + 1] if keep else torch.empty(M, n_out, dtype=torch.bfloat16, device=self.dev)
                self._tc(A, self.Wb[l], C, bias=self.b[l], act=1, Z=buf["Z"][l] if keep else None,
                         CT=buf["actT"][l + 1] if keep else None)
            else:
                C = buf["out"] if keep else torch.empty(M, n_out, device=self.dev)
                self._tc(A, self.Wb[l], C, bias=self.b[l], act=0)
            A = C
        return A

    def _buffers(self, M):
        """Device buffers of one training batch of M rows (reused across steps)."""
        torch = self.torch
        bf = torch.bfloat16
        nl = len(self.W)
        d = self.dims
        hid = max(d[1:-1])
        return {"X": torch.zeros(M, PAD_IN, dtype=bf, device=self.dev),
                "Y": torch.zeros(M, PAD_OUT, device=self.dev),
                "act": [None] + [torch.empty(M, d[l], dtype=bf, device=self.dev) for l in range(1, nl)],
                "actT": [torch.empty(d[l], M, dtype=bf, device=self.dev) for l in range(nl)],
                "Z": [torch.empty(M, d[l + 1], device=self.dev) for l in range(nl - 1)],
                "out": torch.empty(M, PAD_OUT, device=self.dev),
                # output-layer gradient (contiguous [M][PAD_OUT]: the MSE kernel's row stride is
                # that of the outputs) and the hidden layers' ping-pong gradients, each with its
                # transposed copy
                "dZo": torch.empty(M, PAD_OUT, dtype=bf, device=self.dev),
                "dZoT": torch.empty(PAD_OUT, M, dtype=bf, device=self.dev),
                "dZ": [torch.empty(M, hid, dtype=bf, device=self.dev) for _ in range(2)],
                "dZT": [torch.empty(hid, M, dtype=bf, device=self.dev) for _ in range(2)],
                "gW": [torch.empty_like(w) for w in self.W],
                "gb": [torch.empty_like(b) for b in self.b],
                "bb": [torch.empty(b.shape, dtype=bf, device=self.dev) for b in self.b],
                "loss": torch.zeros(1, device=self.dev)}

    def _backward(self, buf, n_real):
        """Parameter gradients of the batch in buf (forward pass already run, the rows beyond
        n_real being padding with zero inputs and targets); the batch loss is added to
        buf["loss"] as the mean over all M rows."""
        M = buf["X"].shape[0]
        L = library()
        out = buf["out"]
        if n_real < M:
            out[n_real:] = 0.0
        nl = len(self.W)
        dZ, dZT = buf["dZo"], buf["dZoT"]
        _check(L.gb_nn_mse(M, self.K + 1, PAD_OUT, _p(out), _p(buf["Y"]), _p(dZ), _p(buf["loss"])))
        self._transpose(dZ, dZT)
        scale = M / float(n_real)            # the loss is the mean over the n_real rows
        for l in range(nl - 1, -1, -1):
            n_out, n_in = self.dims[l + 1], self.dims[l]
            tiles = (n_out // 128) * (n_in // (256 if n_in % 256 == 0 else 128))
            # dW = dZ^T X: (n_out x M)(M x n_in), reduced over the batch in K-splits
            self._tc(dZT, buf["actT"][l], buf["gW"][l], alpha=scale, splits=self._splits(M, tiles))
            _check(L.gb_nn_colsum(M, n_out, _p(dZ), dZ.stride(0), scale, _p(buf["gb"][l])))
            if l > 0:
                k = (nl - l) % 2
                dprev, dprevT = buf["dZ"][k], buf["dZT"][k]
                # dZ_prev = (dZ W) * GELU'(Z_prev): (M x n_out)(n_out x n_in) with W^T K-major
                self._tc(dZ, self.WbT[l], dprev, act=2, Z=buf["Z"][l - 1], CT=dprevT)
                dZ, dZT = dprev, dprevT

    def gradients(self, X, Ytarget, n_real):
        """Loss and parameter gradients of a batch (the rows beyond n_real are padding and
        must carry zero targets and zero inputs)."""
        M = X.shape[0]
        buf = self._buffers(M)
        buf["X"].copy_(X)
        buf["Y"].copy_(Ytarget)
        self._transpose(buf["X"], buf["actT"][0])
        self.forward(buf["X"], keep=True, buf=buf)
        self._backward(buf, n_real)
        self.torch.cuda.synchronize()
        _check(library().gb_nn_sync(self._stream()))
        return float(buf["loss"].item()) * M / float(n_real), buf["gW"], buf["gb"]

    def adam_step(self, gW, gb, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, bb=None):
        self.step_count += 1
        L = library()
        for l in range(len(self.W)):
            _check(L.gb_nn_adam(self.W[l].numel(), _p(self.W[l]), _p(self.mW[l]), _p(self.vW[l]), _p(gW[l]),
                                _p(self.Wb[l]), lr, beta1, beta2, eps, self.step_count))
            b16 = bb[l] if bb is not None else self.torch.empty(self.b[l].shape, dtype=self.torch.bfloat16,
                                                                 device=self.dev)
            _check(L.gb_nn_adam(self.b[l].numel(), _p(self.b[l]), _p(self.mb[l]), _p(self.vb[l]), _p(gb[l]),
                                _p(b16), lr, beta1, beta2, eps, self.step_count))
        self._refresh_transposed_weights()

    def train(self, X, Yt, n, epochs=10, batch=16384, lr=1e-3, warmup=0.05, seed=0, log=None):
        """Mini-batch Adam over the n training rows of X [>=n, PAD_IN], Yt [>=n, PAD_OUT]:
        learning rate ramped up linearly over the first `warmup` fraction of the steps, then
        cosine-decayed to zero.  The steps are queued on the current stream without host
        synchronisation; the mean loss of each epoch is read once at its end."""
        torch = self.torch
        batch = min(self._rows(batch), self._rows(n))
        g = torch.Generator(device=self.dev).manual_seed(seed)
        buf = self._buffers(batch)
        L = library()
        _check(L.gb_nn_set_stream(self._stream(), 1))
        losses = []
        steps_per_epoch = (n + batch - 1) // batch
        total = epochs * steps_per_epoch
        nwarm = max(1, int(warmup * total))
        step = 0
        try:
            for ep in range(epochs):
                perm = torch.randperm(n, device=self.dev, generator=g)
                buf["loss"].zero_()
                for s0 in range(0, n, batch):
                    idx = perm[s0:s0 + batch]
                    m = idx.numel()
                    torch.index_select(X, 0, idx, out=buf["X"][:m])
                    torch.index_select(Yt, 0, idx, out=buf["Y"][:m])
                    if m < batch:
                        buf["X"][m:] = 0
                        buf["Y"][m:] = 0
                    self._transpose(buf["X"], buf["actT"][0])
                    self.forward(buf["X"], keep=True, buf=buf)
                    self._backward(buf, m)
                    step += 1
                    f = step / nwarm if step <= nwarm else 0.5 * (1 + math.cos(math.pi * (step - nwarm) / max(1, total - nwarm)))
                    self.adam_step(buf["gW"], buf["gb"], lr=lr * f, bb=buf["bb"])
                _check(L.gb_nn_sync(self._stream()))
                losses.append(float(buf["loss"].item()) * batch / float(n))
                if log:
                    log(ep, losses[-1])
        finally:
            L.gb_nn_set_stream(None, 0)
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
