// umma.cu - the surrogate network's GEMM on the 5th-generation tensor cores (tcgen05).
//
// C(m, n) = epilogue(alpha * sum_k A[m][k] B[n][k]) with BF16 operands, both K-major (row
// m of A and row n of B contiguous along k), FP32 accumulation in tensor memory (TMEM).
//
// One CTA of 4 warps computes a 128 x BN output tile (BN = 128 or 256):
//   * warp 0, one lane: the producer.  It streams 64-wide K slices of the A tile (128 rows)
//     and the B tile (BN rows) into a ring of shared-memory stages with TMA
//     (cp.async.bulk.tensor, 128-byte swizzle), each stage guarded by a "full" mbarrier
//     that counts the bytes in and an "empty" mbarrier that the tensor cores release.
//   * warp 1, one lane: the MMA issuer.  Per stage, four tcgen05.mma (M = 128, N = BN,
//     K = 16) read both operands from shared memory through matrix descriptors and
//     accumulate into a 128-lane x BN-column FP32 tile in TMEM; tcgen05.commit then frees
//     the stage, and after the last slice signals the accumulator.
//   * all four warps: the epilogue.  Warp w reads TMEM lanes 32w..32w+31 (its rows) 32
//     columns at a time with tcgen05.ld, applies alpha, the bias and the activation (GELU
//     keeping the pre-activation, or the GELU' multiplier of a stored pre-activation), and
//     writes C row segments and, when asked, the transposed copy C^T (coalesced: a warp's
//     lanes hold consecutive rows).  With split-K (gridDim.z > 1) each CTA reduces a K range
//     and adds its partial tile into FP32 C with vector atomics.
// Every mbarrier wait is bounded in time (%globaltimer); a wait that runs out sets the
// error flag, and the CTA skips ahead to releasing its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "nnmath.cuh"
#include "surrogate.h"

namespace gbchem {

namespace {

constexpr int kUmmaThreads = 128;
constexpr int kBK = 64;                         // K slice per stage: one 128-byte swizzle row
constexpr uint64_t kWaitLimitNs = 2000000000ull;   // 2 s per wait
__device__ int g_ummaError;                     // set when a CTA gave up a wait

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globalTimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbarTryWait(uint32_t mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
    return done != 0;
}

// wait for phase `parity`, at most kWaitLimitNs; false when the limit passed
__device__ __forceinline__ bool mbarWait(uint32_t mbar, uint32_t parity) {
    if (mbarTryWait(mbar, parity)) return true;
    const uint64_t t0 = globalTimer();
    for (;;) {
#pragma unroll 1
        for (int i = 0; i < 64; i++)
            if (mbarTryWait(mbar, parity)) return true;
        if (globalTimer() - t0 > kWaitLimitNs) return false;
    }
}

__device__ __forceinline__ void mbarInit(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbarExpectTx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// 2-D tiled TMA load of box {c0 (inner, along K), c1 (rows)} into shared memory
__device__ __forceinline__ void tmaLoad2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(dst), "l"((uint64_t)map), "r"(mbar), "r"(c0), "r"(c1) : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA with the
// 128-byte swizzle: rows of 128 bytes (64 BF16 along K), 8-row groups 1024 bytes apart
// (stride byte offset), descriptor version 1, layout SWIZZLE_128B.  The leading byte
// offset is not used by this layout.
__device__ __forceinline__ uint64_t smemDescSw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address >> 4, bits 0-13
    d |= (uint64_t)1 << 16;                           // leading byte offset (unused)
    d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset >> 4, bits 32-45
    d |= (uint64_t)1 << 46;                           // version
    d |= (uint64_t)2 << 61;                           // SWIZZLE_128B
    return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t instrDescBf16(int M, int N) {
    return (1u << 4)                       // D format F32
           | (1u << 7)                     // A format BF16
           | (1u << 10)                    // B format BF16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void ummaF16(uint32_t tmemD, uint64_t aDesc, uint64_t bDesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmemD), "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void ummaCommit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmemLoad32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Stages are few enough (2 of 48 KB, or 3 of 32 KB) that two CTAs fit an SM: one CTA's
// epilogue then overlaps the other's loads and MMAs (measured on 65,536 x 512 x 512: 105 us
// against 114 us with one CTA of 4 stages per SM); their 2 x BN tensor-memory columns fit the
// SM's 512.
template <int BN>
struct UmmaCfg {
    static constexpr int kStages = BN == 256 ? 2 : 3;
    static constexpr int kABytes = 128 * kBK * 2;                 // 16 KB
    static constexpr int kBBytes = BN * kBK * 2;                  // 16 or 32 KB
    static constexpr int kStageBytes = kABytes + kBBytes;
    static constexpr int kTmemCols = BN;                          // power of two >= 32
    // dynamic shared memory: 1 KB alignment slack, the stages, then the barriers
    static constexpr int kSmem = 1024 + kStages * kStageBytes + 256;
};

// One 32-column chunk of a tile row: v = the row's FP32 accumulators of columns n..n+31.
// alpha, bias, activation; stores of C (and Z, C^T); with split-K an atomic add into C.
__device__ __forceinline__ void epilogueChunk(const UmmaArgs& g, int row, int n, float* v) {
    if (g.splitK) {
        float* C = (float*)g.C + (size_t)row * g.ldc + n;
#pragma unroll
        for (int i = 0; i < 32; i += 4)
            atomicAdd((float4*)(C + i), make_float4(g.alpha * v[i], g.alpha * v[i + 1], g.alpha * v[i + 2],
                                                    g.alpha * v[i + 3]));
        return;
    }
#pragma unroll
    for (int i = 0; i < 32; i++) {
        float x = g.alpha * v[i];
        if (g.bias) x += g.bias[n + i];
        v[i] = x;
    }
    if (g.act == 1) {
        if (g.Z) {   // the pre-activation, kept for the backward pass
            if (g.zFloat) {
                float4* Z = (float4*)((float*)g.Z + (size_t)row * g.ldz + n);
#pragma unroll
                for (int i = 0; i < 8; i++) Z[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            } else {
                __nv_bfloat162* Z = (__nv_bfloat162*)((__nv_bfloat16*)g.Z + (size_t)row * g.ldz + n);
#pragma unroll
                for (int i = 0; i < 16; i++) Z[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
            }
        }
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = gelu(v[i]);
    } else if (g.act == 2) {
        if (g.zFloat) {
            const float4* Z = (const float4*)((const float*)g.Z + (size_t)row * g.ldz + n);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const float4 z = Z[i];
                v[4 * i] *= geluGrad(z.x);
                v[4 * i + 1] *= geluGrad(z.y);
                v[4 * i + 2] *= geluGrad(z.z);
                v[4 * i + 3] *= geluGrad(z.w);
            }
        } else {
            const __nv_bfloat162* Z = (const __nv_bfloat162*)((const __nv_bfloat16*)g.Z + (size_t)row * g.ldz + n);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const float2 z = __bfloat1622float2(Z[i]);
                v[2 * i] *= geluGrad(z.x);
                v[2 * i + 1] *= geluGrad(z.y);
            }
        }
    }
    if (g.cFloat) {
        float4* C = (float4*)((float*)g.C + (size_t)row * g.ldc + n);
#pragma unroll
        for (int i = 0; i < 8; i++) C[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    } else {
        uint4* C = (uint4*)((__nv_bfloat16*)g.C + (size_t)row * g.ldc + n);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            __nv_bfloat162 h[4];
#pragma unroll
            for (int j = 0; j < 4; j++) h[j] = __floats2bfloat162_rn(v[8 * i + 2 * j], v[8 * i + 2 * j + 1]);
            C[i] = *(const uint4*)h;
        }
    }
    if (g.CT) {   // transposed copy: lanes hold consecutive rows, so each column is one 64-byte run
        __nv_bfloat16* CT = (__nv_bfloat16*)g.CT;
#pragma unroll
        for (int i = 0; i < 32; i++) CT[(size_t)(n + i) * g.ldct + row] = __float2bfloat16(v[i]);
    }
}

template <int BN>
__global__ void __launch_bounds__(kUmmaThreads, 2)
k_umma_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, UmmaArgs g) {
    using Cfg = UmmaCfg<BN>;
    constexpr int S = Cfg::kStages;
    extern __shared__ __align__(1024) uint8_t dsm[];
    // stages must start on 1024-byte boundaries (the swizzle pattern's period)
    uint8_t* base = (uint8_t*)(((uintptr_t)dsm + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(base + S * Cfg::kStageBytes);   // full[S], empty[S], acc
    uint32_t* tmemSlot = (uint32_t*)(bars + 2 * S + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * BN, m0 = blockIdx.y * 128;
    const int kPer = g.K / (int)gridDim.z;                      // K range of this CTA
    const int kBeg = (int)blockIdx.z * kPer;
    const int nk = kPer / kBK;

    const uint32_t fullB = smemAddr(bars), emptyB = smemAddr(bars + S), accB = smemAddr(bars + 2 * S);
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbarInit(fullB + 8 * s, 1);
            mbarInit(emptyB + 8 * s, 1);
        }
        mbarInit(accB, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapB) : "memory");
    }
    if (warp == 2) {   // one warp allocates the accumulator columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                     "r"(Cfg::kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmemSlot;
    __shared__ int s_fail;
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();

    if (warp == 0 && lane == 0) {
        // producer
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % S;
            if (!mbarWait(emptyB + 8 * s, ((kb / S) & 1) ^ 1)) { s_fail = 1; break; }
            const uint32_t a = smemAddr(base + s * Cfg::kStageBytes);
            const uint32_t b = a + Cfg::kABytes;
            mbarExpectTx(fullB + 8 * s, Cfg::kStageBytes);
            tmaLoad2d(a, &mapA, kBeg + kb * kBK, m0, fullB + 8 * s);
            tmaLoad2d(b, &mapB, kBeg + kb * kBK, n0, fullB + 8 * s);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = instrDescBf16(128, BN);
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % S;
            if (!mbarWait(fullB + 8 * s, (kb / S) & 1)) { s_fail = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smemAddr(base + s * Cfg::kStageBytes);
            const uint64_t ad = smemDescSw128(a), bd = smemDescSw128(a + Cfg::kABytes);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; kk++)   // K = 16 per MMA: 32 bytes along the swizzled row
                ummaF16(tmem, ad + 2 * kk, bd + 2 * kk, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            ummaCommit(emptyB + 8 * s);
        }
        ummaCommit(accB);
    }
    __syncthreads();   // the roles are done (s_fail is final)

    // epilogue: wait for the accumulator (bounded, block-uniform outcome), then
    // TMEM -> registers -> global
    const bool ok = __syncthreads_and(mbarWait(accB, 0) && !s_fail) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32];
            tmemLoad32(tbase + (uint32_t)c0, v);
            epilogueChunk(g, row, n0 + c0, v);
        }
    } else if (lane == 0) {
        atomicExch(&g_ummaError, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 2)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Persistent form: one CTA per SM walks the tiles (t = blockIdx.x, + gridDim.x, ...; split-K
// ranges are tiles too) with warp-specialised roles and two TMEM accumulators, so that the
// epilogue of one tile overlaps the loads and MMAs of the next:
//   warp 0, one lane: TMA producer over a 4- or 6-stage ring (as above, the ring's position
//     running on across tiles);
//   warp 1, one lane: MMA issuer, accumulating tile i into accumulator i % 2 after the
//     epilogue has released it (mbarrier accEmpty), signalling accFull when its MMAs complete;
//   warps 2..5: the epilogue (warp w reads TMEM lanes 32 (w % 4) .. + 31), each warp's first
//     lane arriving on accEmpty once its rows are read.
// A wait that runs out sets s_abort: every role stops at its next tile, the MMA warp drains
// its issued MMAs (a final commit, bounded wait) before the tensor memory is released.
// ---------------------------------------------------------------------------
constexpr int kUmmaPThreads = 192;

template <int BN>
struct UmmaPCfg {
    static constexpr int kStages = BN == 256 ? 4 : 6;
    static constexpr int kABytes = 128 * kBK * 2;
    static constexpr int kBBytes = BN * kBK * 2;
    static constexpr int kStageBytes = kABytes + kBBytes;
    static constexpr int kTmemCols = 2 * BN;                      // two accumulators (<= 512)
    static constexpr int kSmem = 1024 + kStages * kStageBytes + 256;
};

__device__ __forceinline__ void mbarArrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

template <int BN>
__global__ void __launch_bounds__(kUmmaPThreads, 1)
k_umma_gemm_persistent(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                       UmmaArgs g, int splits) {
    using Cfg = UmmaPCfg<BN>;
    constexpr int S = Cfg::kStages;
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* base = (uint8_t*)(((uintptr_t)dsm + 1023) & ~(uintptr_t)1023);
    // barriers: full[S], empty[S], accFull[2], accEmpty[2], drain
    uint64_t* bars = (uint64_t*)(base + S * Cfg::kStageBytes);
    uint32_t* tmemSlot = (uint32_t*)(bars + 2 * S + 5);
    __shared__ int s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gx = g.N / BN, gy = g.M / 128;
    const int ntiles = gx * gy * splits;
    const int kPer = g.K / splits;
    const int nk = kPer / kBK;
    const uint32_t fullB = smemAddr(bars), emptyB = smemAddr(bars + S), accFullB = smemAddr(bars + 2 * S),
                   accEmptyB = smemAddr(bars + 2 * S + 2), drainB = smemAddr(bars + 2 * S + 4);
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; i++) {
            mbarInit(fullB + 8 * i, 1);
            mbarInit(emptyB + 8 * i, 1);
        }
        for (int b = 0; b < 2; b++) {
            mbarInit(accFullB + 8 * b, 1);
            mbarInit(accEmptyB + 8 * b, 4);   // one arrival per epilogue warp
        }
        mbarInit(drainB, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapB) : "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                     "r"(Cfg::kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmemSlot;
    volatile int* abortFlag = &s_abort;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            for (int t = blockIdx.x; t < ntiles && !*abortFlag; t += gridDim.x) {
                const int z = t / (gx * gy), r = t - z * gx * gy;
                const int m0 = (r / gx) * 128, n0 = (r % gx) * BN, kBeg = z * kPer;
                for (int kb = 0; kb < nk; kb++, it++) {
                    const int st = it % S;
                    if (!mbarWait(emptyB + 8 * st, ((it / S) & 1) ^ 1)) { *abortFlag = 1; break; }
                    const uint32_t a = smemAddr(base + st * Cfg::kStageBytes);
                    mbarExpectTx(fullB + 8 * st, Cfg::kStageBytes);
                    tmaLoad2d(a, &mapA, kBeg + kb * kBK, m0, fullB + 8 * st);
                    tmaLoad2d(a + Cfg::kABytes, &mapB, kBeg + kb * kBK, n0, fullB + 8 * st);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = instrDescBf16(128, BN);
            int it = 0, i = 0;
            for (int t = blockIdx.x; t < ntiles && !*abortFlag; t += gridDim.x, i++) {
                const int b = i & 1;
                if (!mbarWait(accEmptyB + 8 * b, ((i >> 1) & 1) ^ 1)) { *abortFlag = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(b * BN);
                bool fail = false;
                for (int kb = 0; kb < nk; kb++, it++) {
                    const int st = it % S;
                    if (!mbarWait(fullB + 8 * st, (it / S) & 1)) { fail = true; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a = smemAddr(base + st * Cfg::kStageBytes);
                    const uint64_t ad = smemDescSw128(a), bd = smemDescSw128(a + Cfg::kABytes);
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; kk++)
                        ummaF16(acc, ad + 2 * kk, bd + 2 * kk, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
                    ummaCommit(emptyB + 8 * st);
                }
                if (fail) { *abortFlag = 1; break; }
                ummaCommit(accFullB + 8 * b);
            }
            // every issued MMA has completed before the tensor memory is released
            ummaCommit(drainB);
            if (!mbarWait(drainB, 0)) *abortFlag = 1;
        }
    } else {
        const int ew = warp & 3;                       // TMEM lanes 32 ew .. 32 ew + 31
        int i = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int b = i & 1;
            const bool ok = mbarWait(accFullB + 8 * b, (i >> 1) & 1);
            if (__all_sync(0xffffffffu, ok && !*abortFlag) == 0) { if (lane == 0) *abortFlag = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int z = t / (gx * gy), r = t - z * gx * gy;
            const int m0 = (r / gx) * 128, n0 = (r % gx) * BN;
            const int row = m0 + ew * 32 + lane;
            const uint32_t tbase = tmem + ((uint32_t)(ew * 32) << 16) + (uint32_t)(b * BN);
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                float v[32];
                tmemLoad32(tbase + (uint32_t)c0, v);
                epilogueChunk(g, row, n0 + c0, v);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbarArrive(accEmptyB + 8 * b);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && *abortFlag) atomicExch(&g_ummaError, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols)
                     : "memory");
}

// the driver's tensor-map encoder, looked up once through the runtime (the library does
// not link the driver library itself)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return nullptr;
        fn = (EncodeTiledFn)p;
    }
    return fn;
}

// K-major BF16 matrix [rows][K] with row stride ld elements; box 64 (K) x boxRows
bool makeMap(CUtensorMap* map, const void* ptr, int rows, int K, long long ld, int boxRows) {
    EncodeTiledFn fn = encoder();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)boxRows};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launchUmmaT(const UmmaArgs& g, int splits, cudaStream_t s) {
    CUtensorMap ma, mb;
    if (!makeMap(&ma, g.A, g.M, g.K, g.lda, 128) || !makeMap(&mb, g.B, g.N, g.K, g.ldb, BN))
        return cudaErrorInvalidValue;
    constexpr int smem = UmmaCfg<BN>::kSmem;
    cudaError_t e = cudaFuncSetAttribute(k_umma_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(g.N / BN, g.M / 128, splits);
    k_umma_gemm<BN><<<grid, kUmmaThreads, smem, s>>>(ma, mb, g);
    return cudaGetLastError();
}

}  // namespace

const char* checkUmmaArgs(const UmmaArgs& g, int splits) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return "M, N and K must be positive";
    if (g.M % 128) return "M must be a multiple of 128";
    if (g.N % 128) return "N must be a multiple of 128";
    if (splits < 1 || g.K % (kBK * splits)) return "K must be a multiple of 64 * splits";
    if (g.lda < g.K || g.ldb < g.K || g.lda % 8 || g.ldb % 8) return "lda, ldb must be >= K and multiples of 8";
    if (((uintptr_t)g.A | (uintptr_t)g.B) & 15) return "A and B must be 16-byte aligned";
    if (g.ldc < g.N || (g.cFloat ? g.ldc % 4 : g.ldc % 8) || ((uintptr_t)g.C & 15))
        return "C: ldc >= N, rows 16-byte aligned";
    if (splits > 1 && (!g.cFloat || g.act || g.bias || g.CT)) return "split-K accumulates plain FP32 only";
    if (g.act && !g.Z && g.act == 2) return "act 2 needs Z";
    if (g.Z && (g.ldz < g.N || (g.zFloat ? g.ldz % 4 : g.ldz % 2) || ((uintptr_t)g.Z & 15)))
        return "Z: ldz >= N, rows aligned";
    if (g.CT && g.ldct < g.M) return "CT: ldct >= M";
    if (!encoder()) return "cuTensorMapEncodeTiled is not available from the driver";
    return nullptr;
}

namespace {
template <int BN>
cudaError_t launchUmmaPersistentT(const UmmaArgs& g, int splits, int ctas, cudaStream_t s) {
    CUtensorMap ma, mb;
    if (!makeMap(&ma, g.A, g.M, g.K, g.lda, 128) || !makeMap(&mb, g.B, g.N, g.K, g.ldb, BN))
        return cudaErrorInvalidValue;
    constexpr int smem = UmmaPCfg<BN>::kSmem;
    cudaError_t e = cudaFuncSetAttribute(k_umma_gemm_persistent<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_umma_gemm_persistent<BN><<<ctas, kUmmaPThreads, smem, s>>>(ma, mb, g, splits);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launchUmma(const UmmaArgs& g0, int splits, cudaStream_t s) {
    UmmaArgs g = g0;
    g.splitK = splits > 1 ? 1 : 0;
    const int BN = g.N % 256 == 0 ? 256 : 128;
    const long long tiles = (long long)(g.N / BN) * (g.M / 128) * splits;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    // many tiles: one persistent CTA per SM overlapping each tile's epilogue with the next
    // tile's mainloop; a grid of at most two waves of the two-CTA kernel does that already
    if (tiles > 2LL * sms) {
        const int ctas = (int)std::min<long long>(tiles, sms);
        return BN == 256 ? launchUmmaPersistentT<256>(g, splits, ctas, s) : launchUmmaPersistentT<128>(g, splits, ctas, s);
    }
    if (BN == 256) return launchUmmaT<256>(g, splits, s);
    return launchUmmaT<128>(g, splits, s);
}

int ummaTakeError() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_ummaError, sizeof(int)) != cudaSuccess) return -1;
    if (v) {
        int z = 0;
        cudaMemcpyToSymbol(g_ummaError, &z, sizeof(int));
    }
    return v;
}

}  // namespace gbchem
