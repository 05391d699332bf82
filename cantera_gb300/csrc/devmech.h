// devmech.h - the mechanism as the GPU reads it: one device allocation holding flat
// arrays, addressed through the pointers below.  Built on the host from a Mechanism
// (mechanism.h) by packDevMech() in capi.cu.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
struct int4 { int x, y, z, w; };
#else
#include <cuda_runtime.h>
#endif

namespace gbchem {

// four doubles, 32-byte aligned (loaded as two 16-byte vector loads)
struct alignas(32) D4 { double x, y, z, w; };

constexpr int kMaxSpecies = 255;   // limits of the GPU path (checked at load time)
constexpr int kMaxN = kMaxSpecies + 1;   // integrated components: T and the species
// NASA7 block per species: Tmid, then per range (low, high) kNasaRange values
// a0..a6, a1/2, a2/3, a3/4, a4/5, a2/2, a3/3, a4/4 (the scaled coefficients of the
// Horner forms of h/RT and s/R), padded to kNasaStride.
constexpr int kNasaRange = 14;
constexpr int kNasaStride = 32;

// rinfo.x bit fields
constexpr int kKindMask = 0x7;      // RateKind
constexpr int kRevBit = 1 << 3;     // reversible
constexpr int kRBucketShift = 4;    // reactant StoichBucket (3 bits)
constexpr int kPBucketShift = 7;    // product StoichBucket (3 bits)
constexpr int kDnIntBit = 1 << 10;  // dn is an integer in [-3, 3]
constexpr int kNoExpBit = 1 << 11;  // b = 0 and Ea = 0: k = A
constexpr int kChemActBit = 1 << 12;  // chemically-activated falloff: k = klow F / (1 + Pr)
// rate kinds (the RateKind values of mechanism.h)
constexpr int kKindLindemann = 2, kKindTroe = 3, kKindPlog = 4, kKindCheb = 5, kKindSri = 6, kKindTsang = 7;

struct DevMech {
    int K, R, N, NF, NTB, nnz;
    double Pref, Rgas;
    // the arena holding every array below, and the ends (16-byte rounded) of its parts:
    // [0, hotBytes) what a right-hand side reads, [hotBytes, jacBytes) what a Jacobian
    // adds, [jacBytes, sideBytes) the general side lists
    const char* arena;
    int hotBytes, jacBytes, sideBytes;
    // species [K]
    const double* mw;
    const double* rmw;
    const double* nasa;          // [K][kNasaStride]
    // reactions [R]
    const int4* rinfo;           // x flags, y third-body index (-1), z falloff index (-1),
                                 // w offset of the reaction's table in pdep (-1)
    const D4* rarr;         // A, b, Ea/R, dn
    const int4* rk;              // reactant species repeated by coefficient (x,y,z; -1 unused), w = count
    const int4* pk;              // product species, same form
    const int* sidePtr;          // [2R+1] general side lists (used by CN buckets): side 2i reactants, 2i+1 products
    const int* sideK;
    const double* sideNu;
    const double* sideOrd;
    const int* rsPtr;            // [R+1] species of reaction i with net stoichiometric coefficient
    const int* rsK;
    const double* rsNu;
    // falloff [NF]
    const D4* fo1;          // A0, b0, Ea0/R, then Troe a | SRI a | Tsang a
    const D4* fo2;          // Troe 1/T3, 1/T1, T2, 1 | SRI b, c, d, e | Tsang b, 0, 0, 0 | Lindemann 0
    // third bodies [NTB]
    const int* tbRxn;
    const double* tbDef;
    const int* tbMA;
    const int* tbPtr;            // [NTB+1]
    const int* tbK;
    const double* tbE;           // efficiency - default
    // wdot gather: species k -> (reaction, net coefficient)
    const int* spPtr;            // [K+1]
    const int* spRxn;
    const double* spNu;
    // the same entries cut into tasks of bounded length for a balanced warp gather:
    // task t sums entries [taskPtr[t], taskPtr[t+1]) of one species; lane l runs tasks
    // laneTasks[laneTaskPtr[l] .. laneTaskPtr[l+1]); species k adds the partial sums of
    // tasks spTasks[spTaskPtr[k] .. spTaskPtr[k+1]) in order
    int NT;
    const int* taskPtr;          // [NT+1] into spRxn / spNu
    const int* laneTaskPtr;      // [33]
    const int* laneTasks;
    const int* spTaskPtr;        // [K+1]
    const int* spTasks;
    // d(wdot)/dc columns: column j -> (reaction, efficiency - default of j or 0)
    const int* colPtr;           // [K+1]
    const int* colRxn;
    const double* colE;
    const int* laneColPtr;       // [33] columns assigned to each lane (balanced by work)
    const int* laneCols;
    // dense default-efficiency part: species k -> (third-body index, S_net[k][i] * default)
    const int* gsPtr;            // [K+1]
    const int* gsTb;
    const double* gsCoef;
    // output pattern of d(wdot)/dc (CSC): jcPtr[K+1], jrIdx[nnz], jpCol[nnz] (column of each slot)
    const int* jcPtr;
    const int* jrIdx;
    const int* jpCol;
    // the less common rate forms (last, so that the fields above keep their offsets)
    int NX;                      // reactions of those forms (PLOG, Chebyshev, SRI, Tsang,
                                 // chemically activated), evaluated out of line
    // pressure-dependent reactions, one table per reaction at rinfo.w (doubles):
    //   PLOG:      L, then L levels (ln P, first, end) with first/end offsets (from the table
    //              start) of the level's (A, b, Ea/R) triples, which follow; the first and
    //              last levels are the sentinels at ln P = -1000 and +1000
    //   Chebyshev: nT, nP, TrNum, TrDen, PrNum, PrDen, then nT x nP coefficients (row-major)
    const double* pdep;
    // the pattern slot of each scatter of the column lists (the rates kernel accumulates
    // d(wdot)/dc directly on the output pattern): column j's scatters start at
    // colSlotStart[j]; then, for each entry e of column j in order and each species of
    // reaction colRxn[e] with a net coefficient (rsPtr order), the slot of (species, j) in
    // jcPtr/jrIdx, or -1
    const int* colSlotStart;     // [K+1]
    const int* colSlot;
    // fill-reducing ordering of the Krylov path's preconditioner over z = [T, n]: precOrder[new]
    // = old, N entries (preconditionerOrdering)
    const int* precOrder;
    // bounds-check record of the checked build (GBCHEM_CHECKED): first failing site, its
    // index, its bound; written only by the checked build's kernels
    int* chk;
};

// Bounds-checked build.  Every index that comes from the mechanism's tables (species,
// reactions, third bodies, falloff records, gather tasks, Jacobian columns and slots) or
// from a queue passes through GB_IX(m, i, n, site).  In the normal build that is just i.
// With GBCHEM_CHECKED an index outside [0, n) records (site, i, n) in m.chk (the first
// violation wins) and is replaced by 0, so that the access itself stays in bounds and the
// kernel runs on; the host reads the record with gb_check_status.
#if defined(__CUDACC__) && defined(GBCHEM_CHECKED)
__device__ __forceinline__ int gbCheckIx(const DevMech& m, long long i, long long n, int site) {
    if ((unsigned long long)i < (unsigned long long)n) return (int)i;
    if (m.chk && atomicCAS(m.chk, 0, site) == 0) {
        m.chk[1] = (int)i;
        m.chk[2] = (int)n;
    }
    return 0;
}
// the used fields (the first min(w, 3)) of an expanded species list
__device__ __forceinline__ int4 gbCheckIx4(const DevMech& m, int4 e, int n, int site) {
    if (e.w > 0) e.x = gbCheckIx(m, e.x, n, site);
    if (e.w > 1) e.y = gbCheckIx(m, e.y, n, site);
    if (e.w > 2) e.z = gbCheckIx(m, e.z, n, site);
    return e;
}
#define GB_IX(m, i, n, site) gbCheckIx((m), (i), (n), (site))
#define GB_IX4(m, e, n, site) gbCheckIx4((m), (e), (n), (site))
#else
#define GB_IX(m, i, n, site) (i)
#define GB_IX4(m, e, n, site) (e)
#endif
enum { GB_SITE_SPECIES = 1, GB_SITE_SIDE = 2, GB_SITE_TB_SPECIES = 3, GB_SITE_TB = 4, GB_SITE_FALLOFF = 5,
       GB_SITE_GATHER_RXN = 6, GB_SITE_TASK = 7, GB_SITE_COLUMN = 8, GB_SITE_COL_RXN = 9, GB_SITE_SLOT = 10,
       GB_SITE_NET_SPECIES = 11, GB_SITE_DENSE_TB = 12, GB_SITE_PATTERN_ROW = 13, GB_SITE_QUEUE = 14,
       GB_SITE_PREC_ORDER = 15 };

// every array of a DevMech
#define GB_DEVMECH_ARRAYS(X) \
    X(mw) X(rmw) X(nasa) X(rinfo) X(rarr) X(rk) X(pk) X(sidePtr) X(sideK) X(sideNu) X(sideOrd) \
    X(rsPtr) X(rsK) X(rsNu) X(fo1) X(fo2) X(tbRxn) X(tbDef) X(tbMA) X(tbPtr) X(tbK) X(tbE) \
    X(spPtr) X(spRxn) X(spNu) X(taskPtr) X(laneTaskPtr) X(laneTasks) X(spTaskPtr) X(spTasks) \
    X(colPtr) X(colRxn) X(colE) X(laneColPtr) X(laneCols) X(gsPtr) X(gsTb) X(gsCoef) \
    X(jcPtr) X(jrIdx) X(jpCol) X(pdep) X(colSlotStart) X(colSlot) X(precOrder)

#ifdef __CUDACC__
// Point the arrays that lie in the first `bytes` of the arena at a copy of that prefix
// at `copy` (shared memory).
__device__ __forceinline__ void rebaseMech(DevMech& d, const char* copy, int bytes) {
#define GB_REBASE(f)                                                                      \
    {                                                                                     \
        const char* q = (const char*)d.f;                                                 \
        if (q >= d.arena && q < d.arena + bytes) d.f = (decltype(d.f))(copy + (q - d.arena)); \
    }
    GB_DEVMECH_ARRAYS(GB_REBASE)
#undef GB_REBASE
}

// Block prologue of the kernels: copy `bytes` (a multiple of 16) of the arena into the
// start of dynamic shared memory and build the block's DevMech in `sm` (shared).  The
// caller synchronises the block afterwards.
__device__ __forceinline__ void loadMech(const DevMech& src, DevMech& sm, char* dyn, int bytes) {
    const int4* from = (const int4*)src.arena;
    int4* to = (int4*)dyn;
    for (int q = threadIdx.x; q < bytes / 16; q += blockDim.x) to[q] = from[q];
    if (threadIdx.x == 0) {
        sm = src;
        if (bytes > 0) rebaseMech(sm, dyn, bytes);
    }
}

// Bounded wait for phase `parity` of the mbarrier at shared address `mbar`; false when
// `limit` polls pass without it (each poll may suspend the thread briefly in hardware).
__device__ __forceinline__ bool mbarWaitBounded(uint32_t mbar, uint32_t parity, int limit) {
    for (int it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

constexpr int kBulkChunk = 32768;          // bytes per bulk copy instruction
constexpr int kBulkWaitPolls = 1 << 22;    // polls before a block gives up on its copy

// Block prologue with the bulk-copy (TMA) engine: one thread arms the block's mbarrier with
// the byte count and issues cp.async.bulk copies of the arena prefix [0, bytes) (a
// multiple of 16; the arena is 256-byte aligned, `dyn` 128-byte aligned) into shared
// memory; every thread waits (bounded) for the mbarrier's first phase.  Builds the block's
// DevMech in `sm` as loadMech does.  Returns false in every thread of the block when the
// copy did not complete within the limit.
__device__ __forceinline__ bool loadMechBulk(const DevMech& src, DevMech& sm, char* dyn, int bytes,
                                             uint64_t* mbar) {
    const uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar);
    if (threadIdx.x == 0) {
        sm = src;
        if (bytes > 0) {
            rebaseMech(sm, dyn, bytes);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(dyn);
            for (int off = 0; off < bytes; off += kBulkChunk) {
                const int sz = bytes - off < kBulkChunk ? bytes - off : kBulkChunk;
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                    ::"r"(dst + off), "l"(src.arena + off), "r"(sz), "r"(mb) : "memory");
            }
        }
    }
    __syncthreads();
    bool ok = true;
    if (bytes > 0) ok = mbarWaitBounded(mb, 0, kBulkWaitPolls);
    return __syncthreads_and(ok) != 0;
}
#endif

}  // namespace gbchem
