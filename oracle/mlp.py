"""CPU restatement of the surrogate network's arithmetic.  TEST INFRASTRUCTURE ONLY.

The checker for the GPU surrogate kernels (cantera_gb300/csrc/surrogate.cu): the same MLP
(inputs and weights rounded to bfloat16, products accumulated in float32 - here float64,
which bounds the GPU's float32 accumulation error from above), the tanh form of GELU, the
mean-squared-error loss and its gradients by the chain rule, and Adam.  Only tests use it.
"""
import numpy as np


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


C0 = np.sqrt(2.0 / np.pi)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C0 * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C0 * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C0 * (1.0 + 3 * 0.044715 * x * x)


def forward(X, Ws, bs):
    """X [M, K0] (bf16 values); Ws[l] [N_l, K_l] bf16, bs[l] [N_l]; GELU after every layer but
    the last.  Returns the output and the per-layer (input, pre-activation) cache."""
    cache = []
    A = X.astype(np.float64)
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Z = A @ W.astype(np.float64).T + b
        cache.append((A, Z))
        if l < len(Ws) - 1:
            A = bf16(gelu(Z)).astype(np.float64)   # activations are stored as bf16 on the GPU
        else:
            A = Z
    return A, cache


def backward(dOut, Ws, cache):
    """Gradients of the loss w.r.t. every W and b, given dLoss/dOutput [M, N_last]."""
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    dZ = bf16(dOut).astype(np.float64)          # the GPU keeps output gradients in bf16
    for l in range(len(Ws) - 1, -1, -1):
        A, Z = cache[l]
        gW[l] = dZ.T @ A
        gb[l] = dZ.sum(axis=0)
        if l > 0:
            _, Zp = cache[l - 1]
            dA = bf16(dZ).astype(np.float64) @ Ws[l].astype(np.float64)
            dZ = bf16(dA * gelu_grad(Zp)).astype(np.float64)
    return gW, gb


def mse_grad(P, Y):
    M, n = P.shape
    d = P - Y
    return 2.0 * d / (M * n), float((d * d).sum() / (M * n))


def adam(w, m, v, g, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    w = w - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return w, m, v
