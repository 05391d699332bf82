// surrogate.h - kernels of the learned surrogate: an MLP that maps a reactor state to its
// change over a fixed time step, trained and evaluated on the GPU with BF16 tensor-core
// GEMMs accumulating in FP32, and its physics gate.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "devmech.h"

namespace gbchem {

// C(m, n) = epilogue(alpha * sum_k A(m, k) B(n, k)), element addressing by strides, so
// one kernel serves the forward (X W^T), the input-gradient (dZ W) and the
// weight-gradient (dZ^T X) products.  Requirements (checked by the host wrapper):
// M, N multiples of 128, K a multiple of 32, the contiguous stride of A and of B equal to
// 1 (either along K or along M/N), the other stride a multiple of 8 elements, A and B
// 16-byte aligned.
struct GemmArgs {
    int M, N, K;
    const __nv_bfloat16* A;
    long long sam, sak;          // A(m, k) = A[m * sam + k * sak]
    const __nv_bfloat16* B;
    long long sbn, sbk;          // B(n, k) = B[n * sbn + k * sbk]
    void* C;
    long long scm, scn;          // C(m, n) = C[m * scm + n * scn]
    int cFloat;                  // 1: C is float, 0: bf16
    float alpha;
    const float* bias;           // [N] added before the activation, or null
    int act;                     // 0 none; 1 GELU (pre-activation stored in Z); 2 multiply by GELU'(Z)
    void* Z;
    long long szm, szn;
    int zFloat;
};
cudaError_t launchGemm(const GemmArgs& g, cudaStream_t s);

// The tcgen05 GEMM (umma.cu): C[m][n] = epilogue(alpha * sum_k A[m][k] B[n][k]), A [M][K]
// and B [N][K] BF16, K-major (row strides lda, ldb elements, multiples of 8), FP32
// accumulation in tensor memory; M, N multiples of 128, K of 64 * splits.  Epilogue: + bias
// (float [N]); act 1 = GELU with the pre-activation written to Z (float or bf16, row stride
// ldz) when Z is given, act 2 = multiply by GELU'(Z); C float or bf16 (row stride ldc);
// CT (bf16, may be null) receives C transposed, CT[n * ldct + m].  splits > 1: each CTA
// sums K / splits of the products and adds its tile into FP32 C (zeroed by the caller).
struct UmmaArgs {
    int M, N, K;
    const __nv_bfloat16* A;
    long long lda;
    const __nv_bfloat16* B;
    long long ldb;
    void* C;
    long long ldc;
    int cFloat;
    float alpha;
    const float* bias;
    int act;
    void* Z;
    long long ldz;
    int zFloat;
    __nv_bfloat16* CT;
    long long ldct;
    int splitK;        // set by launchUmma
};
const char* checkUmmaArgs(const UmmaArgs& g, int splits);   // null when the call is valid
cudaError_t launchUmma(const UmmaArgs& g, int splits, cudaStream_t s);
int ummaTakeError();   // 1 if a CTA gave up a bounded wait since the last call (and clears it)

// dst[n * ldd + m] = src[m * lds + n] for m < M, n < N (BF16 transpose through shared memory)
cudaError_t launchTranspose(int M, int N, const __nv_bfloat16* src, long long lds, __nv_bfloat16* dst,
                            long long ldd, cudaStream_t s);

// Adam on FP32 master weights (w, m, v, gradient g, n values); writes the BF16 copy wb.
cudaError_t launchAdam(int n, float* w, float* m, float* v, const float* g, __nv_bfloat16* wb, float lr,
                       float beta1, float beta2, float eps, int step, cudaStream_t s);

// out[n] = alpha * sum_m X[m * ld + n] for n < N (bias gradients; X bf16 [M][ld]).
cudaError_t launchColSum(int M, int N, const __nv_bfloat16* X, int ld, float alpha, float* out, cudaStream_t s);

// MSE gradient and loss: dY[m][j] = 2 (P[m][j] - Y[m][j]) / (M * nout) for j < nout, 0 for
// the padding columns up to ld (bf16 out), loss[0] += sum of squares / (M * nout).
cudaError_t launchMseGrad(int M, int nout, int ld, const float* P, const float* Y, __nv_bfloat16* dY,
                          float* loss, cudaStream_t s);

// Network inputs from reactor states: X[r][0..ldx) (bf16) = normalised (T, ln P, Box-Cox(Y_k)),
// zero padding; states species-major (Y[k * n + r]).  mu/sd [K + 2].
cudaError_t launchFeatures(int n, int K, const double* T, const double* P, const double* Y, const float* mu,
                           const float* sd, __nv_bfloat16* X, int ldx, cudaStream_t s);

// Apply the network output O[r][0..ldo) (float, normalised, component k < K for Y_k, K for
// T) with the output scales mu, sd: v = O sd + mu.  Without f0: x1 = x0 + v.  With the
// right-hand side f0 at x0: x1 = x0 + dt f0 + v (dt |f0| + floor), floor 1e-12 for Y and
// 1e-6 K for T (species-major Y).
cudaError_t launchApplyDelta(int n, int K, const float* O, int ldo, const float* mu, const float* sd,
                             const double* T, const double* Y, double dt, const double* f0T, const double* f0Y,
                             double* Tn, double* Yn, cudaStream_t s);

// The gate: accept[r] = 1 when the predicted state conserves element mass fractions (|dZ_e|
// <= tolElem), enthalpy (|h1 - h0| / (cp0 T0) <= tolH) and satisfies the trapezoidal rule
// over dt, |x1 - x0 - dt/2 (f0 + f1)| <= tolTrap (T relative; Y absolute on the mass-
// fraction scale), given f0, f1 = reactor right-hand sides at the two states.
struct GateArgs {
    int n, K, E;
    double dt;
    const double *T0, *Y0, *T1, *Y1;            // states, species-major Y
    const double *f0T, *f0Y, *f1T, *f1Y;        // right-hand sides, species-major
    const double* elemW;                        // [E][K] element mass per species mass
    const double* nasa;                         // mechanism NASA blocks (device)
    double Rgas;
    const double* rmw;                          // 1/W_k
    double tolElem, tolH, tolTrapT, tolTrapY;
    int* accept;
    double* score;                              // [n] largest normalised gate violation
};
cudaError_t launchGate(const GateArgs& a, cudaStream_t s);

}  // namespace gbchem
