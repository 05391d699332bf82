"""The learned surrogate's kernels against the CPU restatement (oracle/mlp.py and the
reactor oracle), and a small end-to-end train / gate / fallback run."""
import ctypes

import numpy as np
import pytest

from conftest import gpu_solution, oracle_mech

pytestmark = pytest.mark.gpu


def _dev():
    torch = pytest.importorskip("torch")
    return torch, torch.device("cuda:0")


def _gemm(L, M, N, K, A, sam, sak, B, sbn, sbk, C, scm, scn, cf, alpha=1.0, bias=None, act=0, Z=None, szm=0, szn=0):
    import cantera_gb300 as gb
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    gb._check(L.gb_nn_gemm(M, N, K, p(A), sam, sak, p(B), sbn, sbk, p(C), scm, scn, cf, alpha, p(bias), act, p(Z),
                           szm, szn, 1))


@pytest.mark.parametrize("layout", ["xwt", "dzw", "dztx"])
def test_gemm_layouts_against_numpy(layout):
    """The three products of training (X W^T, dZ W, dZ^T X) with bf16 operands, FP32
    accumulation: within FP32 summation error of the float64 product of the same bf16 values."""
    import cantera_gb300 as gb
    from oracle import mlp
    torch, dev = _dev()
    L = gb.library()
    rng = np.random.default_rng(3)
    M, N, K = 256, 384, 96
    if layout == "xwt":       # A [M][K], B [N][K]
        a = mlp.bf16(rng.normal(size=(M, K)).astype(np.float32)); b = mlp.bf16(rng.normal(size=(N, K)).astype(np.float32))
        A = torch.tensor(a, dtype=torch.bfloat16, device=dev); B = torch.tensor(b, dtype=torch.bfloat16, device=dev)
        args = (A, K, 1, B, K, 1)
        ref = a.astype(np.float64) @ b.astype(np.float64).T
    elif layout == "dzw":     # A [M][K] (k contiguous), B stored [K][N] (B(n,k) = W[k][n])
        a = mlp.bf16(rng.normal(size=(M, K)).astype(np.float32)); w = mlp.bf16(rng.normal(size=(K, N)).astype(np.float32))
        A = torch.tensor(a, dtype=torch.bfloat16, device=dev); B = torch.tensor(w, dtype=torch.bfloat16, device=dev)
        args = (A, K, 1, B, 1, N)
        ref = a.astype(np.float64) @ w.astype(np.float64)
    else:                     # A(m,k) = dZ[k][m] (dZ [K][M]), B(n,k) = X[k][n] (X [K][N])
        dz = mlp.bf16(rng.normal(size=(K, M)).astype(np.float32)); x = mlp.bf16(rng.normal(size=(K, N)).astype(np.float32))
        A = torch.tensor(dz, dtype=torch.bfloat16, device=dev); B = torch.tensor(x, dtype=torch.bfloat16, device=dev)
        args = (A, 1, M, B, 1, N)
        ref = dz.astype(np.float64).T @ x.astype(np.float64)
    C = torch.empty(M, N, device=dev)
    _gemm(L, M, N, K, *args, C, N, 1, 1)
    got = C.cpu().numpy()
    scale = np.sqrt(K) * 4
    assert np.max(np.abs(got - ref)) < 1e-5 * scale


def test_gemm_epilogues_and_argument_checks():
    import cantera_gb300 as gb
    from oracle import mlp
    torch, dev = _dev()
    L = gb.library()
    rng = np.random.default_rng(4)
    M, N, K = 128, 256, 64
    a = mlp.bf16(rng.normal(size=(M, K)).astype(np.float32)); w = mlp.bf16(rng.normal(0, 0.2, size=(N, K)).astype(np.float32))
    bias = rng.normal(size=N).astype(np.float32)
    A = torch.tensor(a, dtype=torch.bfloat16, device=dev); W = torch.tensor(w, dtype=torch.bfloat16, device=dev)
    Bd = torch.tensor(bias, device=dev)
    C = torch.empty(M, N, dtype=torch.bfloat16, device=dev)
    Z = torch.empty(M, N, device=dev)
    _gemm(L, M, N, K, A, K, 1, W, K, 1, C, N, 1, 0, 1.0, Bd, 1, Z, N, 1)
    zref = a.astype(np.float64) @ w.astype(np.float64).T + bias
    assert np.max(np.abs(Z.cpu().numpy() - zref)) < 1e-4
    assert np.max(np.abs(C.float().cpu().numpy() - mlp.gelu(zref))) < 2e-2   # bf16 output
    # multiply by GELU'(Z)
    C2 = torch.empty(M, N, device=dev)
    _gemm(L, M, N, K, A, K, 1, W, K, 1, C2, N, 1, 1, 1.0, None, 2, Z, N, 1)
    ref2 = (a.astype(np.float64) @ w.astype(np.float64).T) * mlp.gelu_grad(Z.cpu().numpy().astype(np.float64))
    assert np.max(np.abs(C2.cpu().numpy() - ref2)) < 1e-4
    # shape and stride requirements are checked before any launch
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert L.gb_nn_gemm(100, N, K, p(A), K, 1, p(W), K, 1, p(C2), N, 1, 1, 1.0, None, 0, None, 0, 0, 1) == -999
    assert L.gb_nn_gemm(M, N, K, p(A), K, 2, p(W), K, 1, p(C2), N, 1, 1, 1.0, None, 0, None, 0, 0, 1) == -999


def test_network_gradients_and_adam_against_oracle():
    """Loss, weight and bias gradients of the whole network (forward + backward kernels) and
    one Adam step, against the CPU restatement with the same bf16 roundings."""
    from cantera_gb300.surrogate import PAD_IN, PAD_OUT, Surrogate
    from oracle import mlp
    torch, dev = _dev()
    sol = gpu_solution("h2o2")
    sur = Surrogate(sol, hidden=128, layers=2, seed=5)
    rng = np.random.default_rng(6)
    M = 128
    X = mlp.bf16(rng.normal(size=(M, PAD_IN)).astype(np.float32))
    X[:, sol.n_species + 2:] = 0.0
    Y = np.zeros((M, PAD_OUT), dtype=np.float32)
    Y[:, :sol.n_species + 1] = rng.normal(size=(M, sol.n_species + 1))
    Xd = torch.tensor(X, dtype=torch.bfloat16, device=dev)
    Yd = torch.tensor(Y, device=dev)
    # give the biases nonzero values so that their path is exercised
    for l in range(len(sur.b)):
        sur.b[l].copy_(torch.tensor(rng.normal(0, 0.1, sur.b[l].shape[0]), dtype=torch.float32))
    sur.b[-1][sol.n_species + 1:] = 0.0
    loss, gW, gb = sur.gradients(Xd, Yd, M)
    Ws = [w.float().cpu().numpy() for w in sur.Wb]
    bs = [b.cpu().numpy().astype(np.float64) for b in sur.b]
    out, cache = mlp.forward(X, Ws, bs)
    dOut, lref = mlp.mse_grad(out[:, :sol.n_species + 1], Y[:, :sol.n_species + 1].astype(np.float64))
    dfull = np.zeros_like(out)
    dfull[:, :sol.n_species + 1] = dOut
    gWr, gbr = mlp.backward(dfull, Ws, cache)
    assert abs(loss - lref) < 2e-2 * lref
    for l in range(len(Ws)):
        g = gW[l].cpu().numpy()
        s = np.max(np.abs(gWr[l])) + 1e-30
        assert np.max(np.abs(g - gWr[l])) < 3e-2 * s, (l, np.max(np.abs(g - gWr[l])) / s)
        gbl = gb[l].cpu().numpy()
        sb = np.max(np.abs(gbr[l])) + 1e-30
        assert np.max(np.abs(gbl - gbr[l])) < 3e-2 * sb, (l, "bias")
    # one Adam step
    w0 = sur.W[0].cpu().numpy().astype(np.float64)
    g0 = gW[0].cpu().numpy().astype(np.float64)
    sur.adam_step(gW, gb, lr=1e-3)
    w1, _, _ = mlp.adam(w0, np.zeros_like(w0), np.zeros_like(w0), g0, 1e-3, 0.9, 0.999, 1e-8, 1)
    assert np.max(np.abs(sur.W[0].cpu().numpy() - w1)) < 1e-6
    assert torch.equal(sur.Wb[0], sur.W[0].to(torch.bfloat16))


def test_reactor_rhs_matches_oracle():
    """Batched IdealGasConstPressureReactor right-hand side against the oracle's."""
    import cantera_gb300 as gb
    torch, dev = _dev()
    for name in ("h2o2", "gri30"):
        sol, m = gpu_solution(name), oracle_mech(name)
        rng = np.random.default_rng(7)
        n = 300
        T = rng.uniform(600, 2800, n)
        P = 101325.0 * 10 ** rng.uniform(-1, 1.5, n)
        Y = rng.dirichlet(0.5 * np.ones(m.K), n)
        dT = np.empty(n)
        dY = np.empty((m.K, n))
        L = gb.library()
        gb._check(L.gb_reactor_rhs(sol._h, n, gb._ptr(T), gb._ptr(P), gb._ptr(np.ascontiguousarray(Y.T)),
                                   gb._ptr(dT), gb._ptr(dY), 0))
        for s in range(n):
            ref = m.reactor_rhs(P[s], np.concatenate([[1.0, T[s]], Y[s]]))
            scale = np.max(np.abs(ref[2:])) + 1e-300
            assert abs(dT[s] - ref[1]) <= 1e-9 * abs(ref[1]) + 1e-9, (name, s)
            assert np.max(np.abs(dY[:, s] - ref[2:])) <= 1e-9 * scale, (name, s)


def test_gate_accepts_integrator_steps_and_rejects_perturbed_ones():
    import torch
    from cantera_gb300.surrogate import Surrogate, generate_pairs
    _, dev = _dev()
    sol = gpu_solution("h2o2")
    m = oracle_mech("h2o2")
    rng = np.random.default_rng(8)
    n = 64
    T0 = torch.tensor(rng.uniform(900, 1300, n), device=dev)
    P = torch.full((n,), 101325.0, device=dev, dtype=torch.float64)
    Y0 = torch.tensor(np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in rng.uniform(0.6, 1.5, n)]).T.copy(),
                      device=dev)
    sur = Surrogate(sol, dt=1e-6, hidden=128, layers=2)
    Ts, Ps, Ys, T1, Y1 = generate_pairs(sol, T0, P, Y0, [0.0, 2e-4], 1e-6, rtol=1e-10, atol=1e-18)
    acc, score = sur.gate(Ts, Ps, Ys, T1, Y1)
    # exact steps pass (except possibly the fastest ones, where the trapezoidal rule is not
    # accurate to the tolerance); shifted temperatures or a lost element fail
    assert acc.float().mean().item() > 0.7
    acc2, _ = sur.gate(Ts, Ps, Ys, T1 + 0.5, Y1)
    assert acc2.sum().item() == 0
    Y1b = Y1.clone()
    Y1b[sol.species_index("H2")] += 1e-3
    acc3, _ = sur.gate(Ts, Ps, Ys, T1, Y1b)
    assert acc3.sum().item() == 0


def test_train_predict_gate_fallback_end_to_end():
    """Train a small surrogate on integrator pairs; the loss falls, and surrogate + gate +
    fallback reproduces the integrator's step to 1e-3 in T and major species (Y > 0.01) while the
    network carries part of the batch (what it gains over the integrator alone)."""
    import torch
    from cantera_gb300.surrogate import Surrogate, generate_pairs
    _, dev = _dev()
    sol = gpu_solution("h2o2")
    m = oracle_mech("h2o2")
    rng = np.random.default_rng(9)
    n = 512
    T0 = torch.tensor(rng.uniform(1000, 1400, n), device=dev)
    P = torch.full((n,), 101325.0, device=dev, dtype=torch.float64)
    Y0 = torch.tensor(np.array([m.equivalence_ratio(p, "H2:1", "O2:1, N2:3.76") for p in rng.uniform(0.6, 1.5, n)]).T.copy(),
                      device=dev)
    times = [0.0, 1e-5, 3e-5, 1e-4, 3e-4, 1e-3]
    Ts, Ps, Ys, T1, Y1 = generate_pairs(sol, T0, P, Y0, times, 1e-6)
    N = Ts.shape[0]
    sur = Surrogate(sol, dt=1e-6, hidden=256, layers=3, seed=1)
    sur.fit_normalization(Ts, Ps, Ys, T1, Y1)
    X = sur.features(Ts, Ps, Ys)
    Yt = sur.targets(Ts, Ps, Ys, T1, Y1)
    losses = sur.train(X, Yt, N, epochs=30, batch=256, lr=1e-3)
    assert losses[-1] < 0.5 * losses[0]
    Tp, Yp, acc = sur.advance(Ts, Ps, Ys)
    frac = acc.float().mean().item()
    T1p, Y1p, f0 = sur.predict(Ts, Ps, Ys)
    _, score = sur.gate(Ts, Ps, Ys, T1p, Y1p, f0=f0)
    print("accepted fraction %.3f, score quantiles %s, losses %s" % (
        frac, np.quantile(score.cpu().numpy(), [0.1, 0.5, 0.9]), losses[::10]))
    assert frac > 0.1
    rel_T = ((Tp - T1).abs() / T1).max().item()
    assert rel_T < 1e-3
    major = Y1 > 1e-2
    rel_Y = ((Yp - Y1).abs()[major] / Y1[major]).max().item()
    assert rel_Y < 1e-3
