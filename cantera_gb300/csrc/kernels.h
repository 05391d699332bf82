// kernels.h - launch interface between the host library (capi.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "devmech.h"

namespace gbchem {

struct RatesParams {
    DevMech m;
    int n;
    const double* T;
    const double* P;
    const double* Y;      // [K][n]
    double* wdot;         // [K][n] or null
    double* jac;          // [nnz][n] or null
    int* counter;         // [2]: tile (wdot) or state (Jacobian) counter, then an error
                          // flag, both zeroed before launch (the flag is set when a block's
                          // bulk copy of the mechanism did not complete)
    int warpDoubles;      // shared-memory doubles per warp
    int mechSmem;         // bytes of the mechanism arena copied into shared memory
    int tileDoubles;      // the block's state tile (wdot alone; 0 with the Jacobian)
    double* ext;          // with the Jacobian: kfe and rkc (2R doubles) of each resident warp in
                          // global memory (block b, warp w at ext + (b * warps + w) * 2R), so
                          // that more warps fit in shared memory; null: in the warp's slice
};
constexpr int kRatesTile = 32;   // consecutive states per block tile of the rates kernel
// the block's state tile in shared memory: rows T, P, Y_0..Y_{K-1} of kRatesTile + 1 doubles
__host__ __device__ inline int ratesTileDoubles(const DevMech& m) {
    return ((m.K + 2) * (kRatesTile + 1) + 1) & ~1;
}

// batched reactor right-hand side (IdealGasConstPressureReactor::eval over [T, Y])
struct RhsParams {
    DevMech m;
    int n;
    const double* T;
    const double* P;
    const double* Y;      // [K][n]
    double* dTdt;         // [n]
    double* dYdt;         // [K][n]
    int warpDoubles;
};
int rhsWarpDoubles(const DevMech& m);
cudaError_t launchReactorRhs(const RhsParams& p, int blocks, int warpsPerBlock, cudaStream_t stream);

struct BdfParams {
    DevMech m;
    int n;
    double t0, tout;
    double rtol, atol, hmaxInv;
    int maxSteps, maxOrder;
    const double* P;      // [n]
    double* T;            // [n]   in: initial state of fresh reactors; out: T(tout)
    double* Y;            // [K][n]
    double* rec;          // [n][recStride] integrator records (flags 0 = fresh)
    int recStride;
    long long* stats;     // [n][8]
    int* status;          // [n]
    double* tign;         // [n]
    int* counter;         // work counter (zeroed before launch)
    const int* order;     // [n] queue order (null: identity)
    int ld;               // leading dimension of the Newton matrix
    int warpDoubles;
    int mechSmem;         // bytes of the mechanism arena copied into shared memory (multiple of 16)
    void* Mbuf;           // Newton matrices in global memory, one slot of Mstride bytes per
                          // resident warp (L2 resident); null: in the warp's shared slice
    long long Mstride;
    int luSlots;          // shared-memory staging buffers per block for factorisations of
    int luSlotBytes;      // global-memory matrices (0: none); bytes per buffer (multiple of 16)
    void* JSbuf;          // with global matrices: the Jacobian scratch (kfe, rkc: 2R doubles) and
    long long JSstride;   // the Nordsieck array of each resident warp, one slot of JSstride
                          // bytes; else null
    void* Jbuf;           // kept Jacobians (FP64), one slot of Jstride bytes per resident warp;
                          // null: a new Jacobian at every linear-solver setup
    long long Jstride;
    int oneStep;          // 1: each reactor takes one internal step (its state at the new
                          // internal time is written, no interpolation); 0: step past tout
    double* tnow;         // [n] internal time of each reactor after the launch (or null)
    long long* kstats;    // Krylov path: [n][3] linear iterations, preconditioner solves,
                          // J v products (null otherwise)
    double* kzBuf;        // Krylov path: the preconditioned basis vectors, kKrylovMaxl N-vectors
                          // per resident warp (null otherwise)
};

constexpr int kBdfMaxThreads = 256;   // at most 8 warps per block
constexpr int kKrylovMaxl = 5;         // Krylov path: at most 5 Krylov vectors (CVODE's default)
constexpr int kMaxLuSlots = 4;         // shared-memory factorisation buffers per block
int bdfRecordStride(int N);
int bdfNordsieckDoubles(int N);
// Where the host finds a reactor's step history in its integrator record: rec[j N + i] =
// h^j y_i^(j) / j! (the Nordsieck array, j = 0..qmax, scaled by the current step size h), then
// the step scalars at (qmax + 1) N + {tn, h, q, flags}; flags & initFlag: integrated at least
// once since the last reset.
struct BdfRecordLayout { int qmax, tn, h, q, flags, initFlag; };
BdfRecordLayout bdfRecordLayout();
int bdfWarpDoubles(const DevMech& m, int ld, bool fp32);
int bdfWarpDoublesNoMatrix(const DevMech& m);   // the slice when the matrix (and the Jacobian
                                                 // scratch kfe, rkc) are in global memory
int ratesWarpDoubles(const DevMech& m, bool jac);   // the pattern-sized Jacobian only with jac;
                                                     // with jac, kfe and rkc in RatesParams::ext
cudaError_t launchRates(const RatesParams& p, int blocks, int warpsPerBlock, cudaStream_t stream);
cudaError_t launchBdf(const BdfParams& p, int blocks, int warpsPerBlock, bool fp32, cudaStream_t stream);
// resident blocks per SM of the integrator kernel for this launch shape (registers included)
int bdfBlocksPerSm(int N, bool fp32, int warpsPerBlock, size_t smem, bool extra);
// the instantiations for mechanisms with the less common rate forms (kernels_x.cu)
cudaError_t launchReactorRhsX(const RhsParams& p, int blocks, int warpsPerBlock, cudaStream_t stream);
cudaError_t launchRatesX(const RatesParams& p, int blocks, int warpsPerBlock, cudaStream_t stream);
cudaError_t launchBdfX(const BdfParams& p, int blocks, int warpsPerBlock, bool fp32, cudaStream_t stream);
int bdfBlocksPerSmX(bool fp32, int warpsPerBlock, size_t smem);
// the Krylov path (krylov.cu): the mole reactor with GMRES and the adaptive preconditioner;
// its per-warp slice adds bdfKrylovDoubles(N) doubles (the Krylov basis and GMRES scalars),
// Jbuf (the preconditioner's Jacobian) is required and the matrix slot holds its factors
int bdfKrylovDoubles(int N);
// FP64 preconditioner factors (krylov.cu) or FP32 ones (krylov32.cu; the ILUT and the
// triangular solves in FP32, everything else FP64)
cudaError_t launchBdfKrylov64(const BdfParams& p, int blocks, int warpsPerBlock, cudaStream_t stream);
cudaError_t launchBdfKrylov32(const BdfParams& p, int blocks, int warpsPerBlock, cudaStream_t stream);
int bdfBlocksPerSmKrylov64(int N, bool extra, int warpsPerBlock, size_t smem);
int bdfBlocksPerSmKrylov32(int N, bool extra, int warpsPerBlock, size_t smem);
// batched ILUT of n matrices stored transposed in a[n][N][ld] (in place), reciprocal pivots
// to dinv[n][N], rn[n][N] scratch (device pointers)
cudaError_t launchIlut(int n, int N, int ld, double* a, double* dinv, double* rn, cudaStream_t stream);
// FP64 throughput probe: returns {GFLOP/s of FMA, exp cost, log cost in FMA-equivalents}
cudaError_t measureFp64(double* results, int smCount);
cudaError_t checkExp(int n, const double* x, double* mine, double* lib);
cudaError_t checkLog(int n, const double* x, double* mine, double* lib);

}  // namespace gbchem
