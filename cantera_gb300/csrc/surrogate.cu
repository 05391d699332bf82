// surrogate.cu - kernels of the learned surrogate (see surrogate.h).
//
// The GEMM runs on the tensor cores through mma.sync m16n8k16 (BF16 in, FP32 accumulate):
// 128x128 output tiles per block of 8 warps, each warp 64x32, K staged through shared
// memory 32 at a time.  Its operands are read through strides so that one kernel serves
// X W^T, dZ W and dZ^T X; the epilogue adds the bias and applies GELU (keeping the pre-
// activation for the backward pass) or multiplies by GELU' of a stored pre-activation.
#include "surrogate.h"
#include "nnmath.cuh"

#include <math.h>

namespace gbchem {

namespace {

constexpr int BM = 128, BN = 128, BK = 32, PADK = BK + 8;   // padded rows: conflict-free fragment loads
constexpr int kGemmThreads = 256;


// Load a BMxBK (or BNxBK) tile of an operand, element (row, k) at G[row * srow + k * sk],
// into shared memory rows [row][k].  kContig: sk == 1 (16-byte vectors along k);
// otherwise srow == 1 (16-byte vectors along rows, scattered into the k-major smem layout).
template <bool kContig>
__device__ __forceinline__ void loadTile(__nv_bfloat16 (*S)[PADK], const __nv_bfloat16* G, long long srow,
                                         long long sk, int row0, int k0, int tid) {
    if (kContig) {
        // 128 rows x 4 vectors of 8
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int v = tid + i * kGemmThreads;
            const int r = v >> 2, kq = (v & 3) * 8;
            const uint4 d = *(const uint4*)(G + (long long)(row0 + r) * srow + (long long)(k0 + kq));
            *(uint4*)&S[r][kq] = d;
        }
    } else {
        // 32 k x 16 vectors of 8 rows
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int v = tid + i * kGemmThreads;
            const int k = v >> 4, rq = (v & 15) * 8;
            const uint4 d = *(const uint4*)(G + (long long)(row0 + rq) + (long long)(k0 + k) * sk);
            const __nv_bfloat16* e = (const __nv_bfloat16*)&d;
#pragma unroll
            for (int j = 0; j < 8; j++) S[rq + j][k] = e[j];
        }
    }
}

template <bool aK, bool bK>
__global__ void __launch_bounds__(kGemmThreads) k_gemm(GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[BM][PADK];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][PADK];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 2, wn = warp & 3;            // 2 x 4 warps, 64 x 32 each
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int gq = lane >> 2, tq = lane & 3;
    float acc[4][4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;

    for (int k0 = 0; k0 < g.K; k0 += BK) {
        loadTile<aK>(As, g.A, g.sam, g.sak, m0, k0, tid);
        loadTile<bK>(Bs, g.B, g.sbn, g.sbk, n0, k0, tid);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[4][4], bf[4][2];
#pragma unroll
            for (int mi = 0; mi < 4; mi++) {
                const int r = wm * 64 + mi * 16 + gq;
                af[mi][0] = *(const uint32_t*)&As[r][kk + 2 * tq];
                af[mi][1] = *(const uint32_t*)&As[r + 8][kk + 2 * tq];
                af[mi][2] = *(const uint32_t*)&As[r][kk + 2 * tq + 8];
                af[mi][3] = *(const uint32_t*)&As[r + 8][kk + 2 * tq + 8];
            }
#pragma unroll
            for (int ni = 0; ni < 4; ni++) {
                const int c = wn * 32 + ni * 8 + gq;
                bf[ni][0] = *(const uint32_t*)&Bs[c][kk + 2 * tq];
                bf[ni][1] = *(const uint32_t*)&Bs[c][kk + 2 * tq + 8];
            }
#pragma unroll
            for (int mi = 0; mi < 4; mi++)
#pragma unroll
                for (int ni = 0; ni < 4; ni++) {
                    float* d = acc[mi][ni];
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                        : "r"(af[mi][0]), "r"(af[mi][1]), "r"(af[mi][2]), "r"(af[mi][3]), "r"(bf[ni][0]),
                          "r"(bf[ni][1]));
                }
        }
        __syncthreads();
    }
    // epilogue
#pragma unroll
    for (int mi = 0; mi < 4; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int m = m0 + wm * 64 + mi * 16 + gq + (c >= 2 ? 8 : 0);
                const int n = n0 + wn * 32 + ni * 8 + 2 * tq + (c & 1);
                float v = g.alpha * acc[mi][ni][c];
                if (g.bias) v += g.bias[n];
                if (g.act == 1) {
                    if (g.Z) {   // training keeps the pre-activation for the backward pass
                        const long long zi = (long long)m * g.szm + (long long)n * g.szn;
                        if (g.zFloat) ((float*)g.Z)[zi] = v;
                        else ((__nv_bfloat16*)g.Z)[zi] = __float2bfloat16(v);
                    }
                    v = gelu(v);
                } else if (g.act == 2) {
                    const long long zi = (long long)m * g.szm + (long long)n * g.szn;
                    const float z = g.zFloat ? ((const float*)g.Z)[zi] : __bfloat162float(((const __nv_bfloat16*)g.Z)[zi]);
                    v *= geluGrad(z);
                }
                const long long ci = (long long)m * g.scm + (long long)n * g.scn;
                if (g.cFloat) ((float*)g.C)[ci] = v;
                else ((__nv_bfloat16*)g.C)[ci] = __float2bfloat16(v);
            }
}

__global__ void k_adam(int n, float* w, float* m, float* v, const float* g, __nv_bfloat16* wb, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        wb[i] = __float2bfloat16(wi);
    }
}

// one block per 32 columns: 8 row groups of 32 threads, partial sums combined in shared memory
__global__ void k_colsum(int M, int N, const __nv_bfloat16* X, int ld, float alpha, float* out) {
    __shared__ float part[8][32];
    const int c = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int n = blockIdx.x * 32 + c;
    float s = 0.f;
    if (n < N)
        for (int m = g; m < M; m += 8) s += __bfloat162float(X[(long long)m * ld + n]);
    part[g][c] = s;
    __syncthreads();
    if (g == 0 && n < N) {
        float t = 0.f;
        for (int q = 0; q < 8; q++) t += part[q][c];
        out[n] = alpha * t;
    }
}

__global__ void k_mse(int M, int nout, int ld, const float* P, const float* Y, __nv_bfloat16* dY, float* loss) {
    __shared__ float red[256];
    float part = 0.f;
    const float scale = 1.f / ((float)M * (float)nout);
    const long long total = (long long)M * ld;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(i % ld);
        float d = 0.f;
        if (j < nout) {
            d = P[i] - Y[i];
            part += d * d;
        }
        dY[i] = __float2bfloat16(2.f * d * scale);
    }
    red[threadIdx.x] = part;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] * scale);
}

__device__ __forceinline__ double boxcox(double y) { return (pow(fmax(y, 0.0), 0.1) - 1.0) * 10.0; }

__global__ void k_features(int n, int K, const double* T, const double* P, const double* Y, const float* mu,
                           const float* sd, __nv_bfloat16* X, int ldx) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    __nv_bfloat16* x = X + (long long)r * ldx;
    x[0] = __float2bfloat16((float)((T[r] - mu[0]) / sd[0]));
    x[1] = __float2bfloat16((float)((log(P[r]) - mu[1]) / sd[1]));
    for (int k = 0; k < K; k++)
        x[2 + k] = __float2bfloat16((float)((boxcox(Y[(long long)k * n + r]) - mu[2 + k]) / sd[2 + k]));
    for (int j = K + 2; j < ldx; j++) x[j] = __float2bfloat16(0.f);
}

// with the explicit step, the network's outputs are corrections relative to its size,
// (x1 - x0 - dt f0) / (dt |f0| + floor), so that slow states need a correction near zero
constexpr double kFloorY = 1e-12, kFloorT = 1e-6;

__global__ void k_apply(int n, int K, const float* O, int ldo, const float* mu, const float* sd, const double* T,
                        const double* Y, double dt, const double* f0T, const double* f0Y, double* Tn, double* Yn) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float* o = O + (long long)r * ldo;
    for (int k = 0; k < K; k++) {
        const long long i = (long long)k * n + r;
        const double v = (double)o[k] * sd[k] + mu[k];
        Yn[i] = f0Y ? Y[i] + dt * f0Y[i] + v * (dt * fabs(f0Y[i]) + kFloorY) : Y[i] + v;
    }
    const double v = (double)o[K] * sd[K] + mu[K];
    Tn[r] = f0T ? T[r] + dt * f0T[r] + v * (dt * fabs(f0T[r]) + kFloorT) : T[r] + v;
}

// h/RT and cp/R of species k at T from the Horner-form NASA block
__device__ __forceinline__ void nasaHc(const double* nasa, int k, double T, double& hRT, double& cpR) {
    const double* a = nasa + (size_t)k * kNasaStride;
    const double* p = (T <= a[0]) ? a + 1 : a + 1 + kNasaRange;
    cpR = fma(fma(fma(fma(p[4], T, p[3]), T, p[2]), T, p[1]), T, p[0]);
    hRT = fma(fma(fma(fma(p[10], T, p[9]), T, p[8]), T, p[7]), T, p[0]) + p[5] / T;
}

__global__ void k_gate(GateArgs a) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.n) return;
    const int n = a.n;
    const double T0 = a.T0[r], T1 = a.T1[r];
    double h0 = 0.0, h1 = 0.0, cp0 = 0.0, trapY = 0.0;
    for (int k = 0; k < a.K; k++) {
        const long long i = (long long)k * n + r;
        const double y0 = a.Y0[i], y1 = a.Y1[i];
        double hr0, c0, hr1, c1;
        nasaHc(a.nasa, k, T0, hr0, c0);
        nasaHc(a.nasa, k, T1, hr1, c1);
        h0 += y0 * hr0 * T0 * a.rmw[k];
        h1 += y1 * hr1 * T1 * a.rmw[k];
        cp0 += y0 * c0 * a.rmw[k];
        const double res = y1 - y0 - 0.5 * a.dt * (a.f0Y[i] + a.f1Y[i]);
        trapY = fmax(trapY, fabs(res));
    }
    double elem = 0.0;
    for (int e = 0; e < a.E; e++) {
        double z0 = 0.0, z1 = 0.0;
        for (int k = 0; k < a.K; k++) {
            const long long i = (long long)k * n + r;
            const double w = a.elemW[(size_t)e * a.K + k];
            z0 += w * a.Y0[i];
            z1 += w * a.Y1[i];
        }
        elem = fmax(elem, fabs(z1 - z0));
    }
    // (h in units of R: sum Y_k (h_k/RT) T / W_k; cp likewise)
    const double dh = fabs(h1 - h0) / (cp0 * T0);
    const double trapT = fabs(T1 - T0 - 0.5 * a.dt * (a.f0T[r] + a.f1T[r])) / T0;
    double score = elem / a.tolElem;
    score = fmax(score, dh / a.tolH);
    score = fmax(score, trapT / a.tolTrapT);
    score = fmax(score, trapY / a.tolTrapY);
    const bool finite = isfinite(T1) && isfinite(score);
    a.score[r] = finite ? score : INFINITY;
    a.accept[r] = (finite && score <= 1.0) ? 1 : 0;
}

}  // namespace

// 32 x 32 tiles through padded shared memory: coalesced reads of src rows, coalesced
// writes of dst rows
__global__ void k_transpose(int M, int N, const __nv_bfloat16* src, long long lds, __nv_bfloat16* dst,
                            long long ldd) {
    __shared__ __nv_bfloat16 t[32][34];
    const int m0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8 threads
#pragma unroll
    for (int i = ty; i < 32; i += 8)
        if (m0 + i < M && n0 + tx < N) t[i][tx] = src[(size_t)(m0 + i) * lds + n0 + tx];
    __syncthreads();
#pragma unroll
    for (int i = ty; i < 32; i += 8)
        if (n0 + i < N && m0 + tx < M) dst[(size_t)(n0 + i) * ldd + m0 + tx] = t[tx][i];
}

cudaError_t launchTranspose(int M, int N, const __nv_bfloat16* src, long long lds, __nv_bfloat16* dst,
                            long long ldd, cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    dim3 grid((N + 31) / 32, (M + 31) / 32);
    k_transpose<<<grid, 256, 0, s>>>(M, N, src, lds, dst, ldd);
    return cudaGetLastError();
}

cudaError_t launchGemm(const GemmArgs& g, cudaStream_t s) {
    dim3 grid(g.N / BN, g.M / BM);
    const bool aK = g.sak == 1, bK = g.sbk == 1;
    if (aK && bK) k_gemm<true, true><<<grid, kGemmThreads, 0, s>>>(g);
    else if (aK) k_gemm<true, false><<<grid, kGemmThreads, 0, s>>>(g);
    else if (bK) k_gemm<false, true><<<grid, kGemmThreads, 0, s>>>(g);
    else k_gemm<false, false><<<grid, kGemmThreads, 0, s>>>(g);
    return cudaGetLastError();
}

cudaError_t launchAdam(int n, float* w, float* m, float* v, const float* g, __nv_bfloat16* wb, float lr, float beta1,
                       float beta2, float eps, int step, cudaStream_t s) {
    const float c1 = 1.f / (1.f - powf(beta1, (float)step));
    const float c2 = 1.f / (1.f - powf(beta2, (float)step));
    k_adam<<<(n + 255) / 256, 256, 0, s>>>(n, w, m, v, g, wb, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launchColSum(int M, int N, const __nv_bfloat16* X, int ld, float alpha, float* out, cudaStream_t s) {
    k_colsum<<<(N + 31) / 32, 256, 0, s>>>(M, N, X, ld, alpha, out);
    return cudaGetLastError();
}

cudaError_t launchMseGrad(int M, int nout, int ld, const float* P, const float* Y, __nv_bfloat16* dY, float* loss,
                          cudaStream_t s) {
    k_mse<<<512, 256, 0, s>>>(M, nout, ld, P, Y, dY, loss);
    return cudaGetLastError();
}

cudaError_t launchFeatures(int n, int K, const double* T, const double* P, const double* Y, const float* mu,
                           const float* sd, __nv_bfloat16* X, int ldx, cudaStream_t s) {
    k_features<<<(n + 127) / 128, 128, 0, s>>>(n, K, T, P, Y, mu, sd, X, ldx);
    return cudaGetLastError();
}

cudaError_t launchApplyDelta(int n, int K, const float* O, int ldo, const float* mu, const float* sd,
                             const double* T, const double* Y, double dt, const double* f0T, const double* f0Y,
                             double* Tn, double* Yn, cudaStream_t s) {
    k_apply<<<(n + 127) / 128, 128, 0, s>>>(n, K, O, ldo, mu, sd, T, Y, dt, f0T, f0Y, Tn, Yn);
    return cudaGetLastError();
}

cudaError_t launchGate(const GateArgs& a, cudaStream_t s) {
    k_gate<<<(a.n + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace gbchem
