"""The surrogate's tcgen05 GEMM (gb_nn_gemm_tc) against a plain PyTorch FP32 reference of
the same products: BF16 operands are exact in FP32, so with FP32 output the only
difference is the order of the FP32 accumulation (tolerance 1e-5 of the row's scale);
BF16 outputs carry one BF16 rounding (tolerance 2^-8 relative)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    import cantera_gb300 as gb
    return gb.library()


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def gemm_tc(A, B, C, alpha=1.0, bias=None, act=0, Z=None, CT=None, splits=1):
    L = _lib()
    M, K = A.shape
    N = B.shape[0]
    rc = L.gb_nn_gemm_tc(M, N, K, _p(A), A.stride(0), _p(B), B.stride(0), _p(C), C.stride(0),
                         int(C.dtype.itemsize == 4), alpha, _p(bias), act, _p(Z),
                         Z.stride(0) if Z is not None else 0, int(Z is not None and Z.dtype.itemsize == 4),
                         _p(CT), CT.stride(0) if CT is not None else 0, splits, None)
    if rc != 0:
        buf = ctypes.create_string_buffer(512)
        L.gb_get_error(512, buf)
        raise RuntimeError(buf.value.decode())
    assert L.gb_nn_sync(None) == 0


def _operands(M, N, K, seed):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = (torch.randn(M, K, device="cuda", generator=g)).to(torch.bfloat16)
    B = (torch.randn(N, K, device="cuda", generator=g) / K ** 0.5).to(torch.bfloat16)
    return A, B


def gelu(x):
    import torch
    return 0.5 * x * (1.0 + torch.tanh(0.7978845608028654 * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    import torch
    t = torch.tanh(0.7978845608028654 * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * 0.7978845608028654 * (1 + 0.134145 * x * x)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 256, 128), (384, 512, 512), (4096, 512, 128),
                                   (4096, 128, 512)])
def test_plain_fp32_output(M, N, K):
    import torch
    A, B = _operands(M, N, K, M + N + K)
    C = torch.full((M, N), float("nan"), device="cuda")
    gemm_tc(A, B, C, alpha=0.5)
    ref = 0.5 * (A.float() @ B.float().T)
    scale = ref.abs().amax(dim=1, keepdim=True) + 1e-30
    assert torch.all((C - ref).abs() <= 1e-5 * scale)


@pytest.mark.parametrize("M,N,K,splits", [(512, 512, 4096, 8), (128, 512, 16384, 16), (512, 128, 2048, 4)])
def test_split_k_accumulates(M, N, K, splits):
    import torch
    A, B = _operands(M, N, K, 7 + splits)
    C = torch.full((M, N), float("nan"), device="cuda")
    gemm_tc(A, B, C, alpha=2.0, splits=splits)
    ref = 2.0 * (A.float() @ B.float().T)
    scale = ref.abs().amax(dim=1, keepdim=True) + 1e-30
    assert torch.all((C - ref).abs() <= 1e-5 * scale)


def test_bias_gelu_keeps_preactivation_and_transpose():
    import torch
    M, N, K = 384, 512, 512
    A, B = _operands(M, N, K, 3)
    bias = torch.randn(N, device="cuda")
    C = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
    Z = torch.empty(M, N, device="cuda")
    CT = torch.empty(N, M, dtype=torch.bfloat16, device="cuda")
    gemm_tc(A, B, C, bias=bias, act=1, Z=Z, CT=CT)
    z = A.float() @ B.float().T + bias
    assert torch.all((Z - z).abs() <= 1e-5 * (z.abs().amax(dim=1, keepdim=True) + 1e-30))
    ref = gelu(Z)
    assert torch.all((C.float() - ref).abs() <= 2 ** -8 * ref.abs() + 1e-6)
    assert torch.equal(CT, C.T.contiguous())


def test_gelu_grad_epilogue_bf16_z():
    import torch
    M, N, K = 256, 512, 256
    A, B = _operands(M, N, K, 4)
    Z = torch.randn(M, N, device="cuda").to(torch.bfloat16)
    C = torch.empty(M, N, device="cuda")
    gemm_tc(A, B, C, act=2, Z=Z)
    ref = (A.float() @ B.float().T) * gelu_grad(Z.float())
    scale = ref.abs().amax(dim=1, keepdim=True) + 1e-30
    assert torch.all((C - ref).abs() <= 1e-5 * scale)


def test_strided_rows_and_rejections():
    """Operands inside wider row-major buffers (lda, ldb, ldc > K, N); invalid shapes and
    layouts are errors, not launches."""
    import torch
    M, N, K = 256, 256, 128
    Abuf = torch.randn(M, K + 64, device="cuda").to(torch.bfloat16)
    Bbuf = torch.randn(N, K + 192, device="cuda").to(torch.bfloat16)
    Cbuf = torch.zeros(M, N + 128, device="cuda")
    A, B, C = Abuf[:, :K], Bbuf[:, :K], Cbuf[:, :N]
    gemm_tc(A, B, C)
    ref = A.float() @ B.float().T
    assert torch.all((C - ref).abs() <= 1e-5 * (ref.abs().amax(dim=1, keepdim=True) + 1e-30))
    assert torch.all(Cbuf[:, N:] == 0)
    L = _lib()
    bad = torch.empty(100, 64, dtype=torch.bfloat16, device="cuda")
    rc = L.gb_nn_gemm_tc(100, 128, 64, _p(bad), 64, _p(B), B.stride(0), _p(C), C.stride(0), 1, 1.0, None, 0,
                         None, 0, 0, None, 0, 1, None)
    assert rc == -999
    rc = L.gb_nn_gemm_tc(256, 256, 96, _p(A), A.stride(0), _p(B), B.stride(0), _p(C), C.stride(0), 1, 1.0, None, 0,
                         None, 0, 0, None, 0, 1, None)
    assert rc == -999


def test_transpose_kernel():
    import torch
    L = _lib()
    X = torch.randn(300, 77, device="cuda").to(torch.bfloat16)
    XT = torch.zeros(77, 320, dtype=torch.bfloat16, device="cuda")
    assert L.gb_nn_transpose(300, 77, _p(X), 77, _p(XT), 320, None) == 0
    assert L.gb_nn_sync(None) == 0
    assert torch.equal(XT[:, :300], X.T) and torch.all(XT[:, 300:] == 0)


def test_tensor_core_path_matches_legacy_gemm():
    """The forward product of a surrogate layer through both GEMMs of the library."""
    import torch
    M, N, K = 512, 512, 128
    A, B = _operands(M, N, K, 9)
    bias = torch.randn(N, device="cuda")
    C1 = torch.empty(M, N, device="cuda")
    gemm_tc(A, B, C1, bias=bias)
    C2 = torch.empty(M, N, device="cuda")
    L = _lib()
    assert L.gb_nn_gemm(M, N, K, _p(A), K, 1, _p(B), K, 1, _p(C2), N, 1, 1, 1.0, _p(bias), 0, None, 0, 0, 1) == 0
    assert torch.allclose(C1, C2, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("M,N,K,splits", [(65536, 512, 256, 1), (40960, 128, 512, 1), (512, 512, 65536, 128)])
def test_persistent_kernel_many_tiles(M, N, K, splits):
    """Grids of more than two waves run the persistent kernel (one CTA per SM walking the
    tiles with two tensor-memory accumulators): plain FP32 output, split-K and (below) the
    full epilogue agree with the FP32 reference."""
    import torch
    A, B = _operands(M, N, K, 11 + splits)
    C = torch.full((M, N), float("nan"), device="cuda")
    gemm_tc(A, B, C, alpha=0.5, splits=splits)
    ref = 0.5 * (A.float() @ B.float().T)
    scale = ref.abs().amax(dim=1, keepdim=True) + 1e-30
    assert torch.all((C - ref).abs() <= 1e-5 * scale)


def test_persistent_kernel_epilogue():
    import torch
    M, N, K = 65536, 512, 512
    A, B = _operands(M, N, K, 5)
    bias = torch.randn(N, device="cuda")
    C = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
    Z = torch.empty(M, N, device="cuda")
    CT = torch.empty(N, M, dtype=torch.bfloat16, device="cuda")
    for _ in range(2):   # the same result on a second call
        gemm_tc(A, B, C, bias=bias, act=1, Z=Z, CT=CT)
        z = A.float() @ B.float().T + bias
        assert torch.all((Z - z).abs() <= 1e-5 * (z.abs().amax(dim=1, keepdim=True) + 1e-30))
        ref = gelu(Z)
        assert torch.all((C.float() - ref).abs() <= 2 ** -8 * ref.abs() + 1e-6)
        assert torch.equal(CT, C.T.contiguous())
