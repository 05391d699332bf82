"""The surrogate's CPU restatement (oracle/mlp.py) checked against finite differences, so
that it can serve as the checker of the GPU training kernels."""
import numpy as np

from oracle import mlp


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-30], dtype=np.float32)
    r = mlp.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # ties to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-6
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    dims = [6, 8, 8, 5]
    Ws = [rng.normal(0, 0.5, (dims[i + 1], dims[i])) for i in range(3)]
    bs = [rng.normal(0, 0.1, dims[i + 1]) for i in range(3)]
    X = rng.normal(size=(7, 6))
    Y = rng.normal(size=(7, 5))

    def loss(Ws_, bs_):
        # the same network without bf16 rounding of the intermediates
        A = X
        for l, (W, b) in enumerate(zip(Ws_, bs_)):
            Z = A @ W.T + b
            A = mlp.gelu(Z) if l < 2 else Z
        return ((A - Y) ** 2).mean()

    # exact-arithmetic backward for the check: the restatement with rounding switched off
    A = X
    cache = []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Z = A @ W.T + b
        cache.append((A, Z))
        A = mlp.gelu(Z) if l < 2 else Z
    dOut, _ = mlp.mse_grad(A, Y)
    dZ = dOut
    for l in range(2, -1, -1):
        Al, Zl = cache[l]
        gW = dZ.T @ Al
        h = 1e-6
        W2 = [w.copy() for w in Ws]
        W2[l][1, 2] += h
        W3 = [w.copy() for w in Ws]
        W3[l][1, 2] -= h
        fd = (loss(W2, bs) - loss(W3, bs)) / (2 * h)
        assert abs(fd - gW[1, 2]) < 1e-6 * max(1.0, abs(fd)), (l, fd, gW[1, 2])
        if l > 0:
            dZ = (dZ @ Ws[l]) * mlp.gelu_grad(cache[l - 1][1])


def test_gelu_grad_matches_difference():
    x = np.linspace(-6, 6, 101)
    h = 1e-6
    fd = (mlp.gelu(x + h) - mlp.gelu(x - h)) / (2 * h)
    assert np.max(np.abs(fd - mlp.gelu_grad(x))) < 1e-8


def test_adam_first_step():
    w, m, v = np.ones(3), np.zeros(3), np.zeros(3)
    g = np.array([0.5, -2.0, 0.0])
    w1, m1, v1 = mlp.adam(w, m, v, g, 0.1, 0.9, 0.999, 1e-8, 1)
    # the first bias-corrected step moves every weight with a nonzero gradient by lr
    assert np.allclose(w1[:2], [0.9, 1.1]) and w1[2] == 1.0
