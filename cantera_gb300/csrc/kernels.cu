// kernels.cu - GPU kernels of the engine: batched net production rates and their
// concentration Jacobian, and the batched BDF reactor integrator.
//
// Both kernels are persistent: a grid sized to fill every SM, one state (reactor) per
// warp at a time, and a device-side work counter from which a warp takes its next state
// as soon as it finishes the previous one.  Reactors of very different stiffness
// (igniting next to inert) therefore never leave warps idle until the queue runs dry.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "kernels.h"
#include "kinetics.cuh"

namespace gbchem {

// =============================================================================
// Rates and d(wdot)/dc over a batch of states (Kinetics::getNetProductionRates,
// Kinetics::netProductionRates_ddCi)
// =============================================================================
// A block takes tiles of kRatesTile consecutive states from an atomic counter.  The tile's
// T, P and Y[K] rows are loaded into shared memory with one coalesced 256-byte request per
// row (lanes across states); each warp then evaluates whole states (lanes across species,
// reactions and Jacobian columns) and writes wdot back into its state's column of the
// tile, which the block stores with coalesced rows.  With d(wdot)/dc (several times the work
// of a state's wdot) warps take single states instead, and the Jacobian is accumulated per
// warp directly on the output pattern (nnz doubles: no dense K x K scratch, no gather).  The
// mechanism prefix the call reads is staged into shared memory by the bulk-copy engine.
template <bool kX>
__global__ void __launch_bounds__(256, 1) k_rates(RatesParams p) {
    extern __shared__ __align__(128) double smem[];
    __shared__ uint64_t s_tab[kGbxTableWords];
    __shared__ DevMech s_mech;
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ int s_tile;
    if (!loadMechBulk(p.m, s_mech, (char*)smem, p.mechSmem, &s_mbar)) {
        if (threadIdx.x == 0) atomicExch(p.counter + 1, 1);
        return;
    }
    gbx_load_table(s_tab);   // (its barrier also publishes s_mech)
    const DevMech& m = s_mech;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int W = blockDim.x >> 5;
    const int K = m.K, n = p.n;
    constexpr int LD = kRatesTile + 1;        // padded row: column reads hit distinct banks
    double* tile = smem + p.mechSmem / 8;     // rows: T, P, then Y_k / wdot_k, each LD doubles
    double* base = tile + p.tileDoubles + (size_t)warp * p.warpDoubles;
    KinScratch s;
    double* ext = p.ext ? p.ext + (size_t)(blockIdx.x * W + warp) * 2 * m.R : nullptr;
    const int kinD = KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT, ext != nullptr);
    s.carve(base, m.K, m.R, m.NTB, m.NF, m.NT, ext);
    s.tab = s_tab;
    double* Yl = base + kinD;
    double* gk = Yl + K;
    double* Js = gk + K;                      // [nnz] this warp's d(wdot)/dc on the pattern
    const bool jac = p.jac != nullptr;
    KinState st;
    if (jac) {
        // d(wdot)/dc: a state costs several wdot evaluations, so keeping every warp busy
        // matters more than coalesced input rows: each warp takes single states from the
        // counter and writes its state's wdot and pattern values itself (the warps of a block
        // work on neighbouring states at the same time, so a slot's neighbouring values merge
        // in L2 before they are written back)
        for (;;) {
            int idx = 0;
            if (lane == 0) idx = atomicAdd(p.counter, 1);
            idx = __shfl_sync(0xffffffffu, idx, 0);
            if (idx >= n) break;
            for (int k = lane; k < K; k += 32) Yl[k] = p.Y[(size_t)k * n + idx];
            const double T = p.T[idx], P = p.P[idx];
            __syncwarp();
            warpState(m, T, P, Yl, s, st, lane);
            __syncwarp();
            warpRates<kX>(m, s, st, lane, true);
            if (p.wdot)
                for (int k = lane; k < K; k += 32) p.wdot[(size_t)k * n + idx] = s.wdot[k];
            for (int q = lane; q < m.nnz; q += 32) Js[q] = 0.0;
            __syncwarp();
            warpJacSparse(m, s, Js, lane);
            warpDenseG(m, s, gk, lane);
            double* out = p.jac + idx;
            for (int q = lane; q < m.nnz; q += 32)
                out[(size_t)q * n] = Js[q] + gk[GB_IX(m, m.jrIdx[q], K, GB_SITE_PATTERN_ROW)];
            __syncwarp();
        }
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(p.counter, 1);
        __syncthreads();
        const long long s0 = (long long)s_tile * kRatesTile;
        if (s0 >= n) break;
        const int ns = (int)min((long long)kRatesTile, (long long)n - s0);
        // coalesced tile load: row r by warp r mod W, lane = state
#pragma unroll 1
        for (int r = warp; r < K + 2; r += W) {
            const double* src = r == 0 ? p.T : (r == 1 ? p.P : p.Y + (size_t)(r - 2) * n);
            if (lane < ns) tile[r * LD + lane] = src[s0 + lane];
        }
        __syncthreads();
        // warp w on states w, w+W, ... of the tile
#pragma unroll 1
        for (int j = warp; j < ns; j += W) {
            for (int k = lane; k < K; k += 32) Yl[k] = tile[(2 + k) * LD + j];
            const double T = tile[j], P = tile[LD + j];
            __syncwarp();
            warpState(m, T, P, Yl, s, st, lane);
            __syncwarp();
            warpRates<kX>(m, s, st, lane, false);
            for (int k = lane; k < K; k += 32) tile[(2 + k) * LD + j] = s.wdot[k];
            __syncwarp();
        }
        __syncthreads();
        if (p.wdot) {
#pragma unroll 1
            for (int r = warp; r < K; r += W)
                if (lane < ns) p.wdot[(size_t)r * n + s0 + lane] = tile[(2 + r) * LD + lane];
        }
        __syncthreads();
    }
}

// =============================================================================
// Batched BDF integrator (the CVODES algorithm as the reference configures it:
// src/numerics/CVodesIntegrator.cpp:281-529, src/zeroD/ReactorNet.cpp:164-169)
// =============================================================================
namespace {
constexpr int QMAX = 5;
constexpr double BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, ADDON = 1e-6;
constexpr double ETA_FIX_MAX = 1.5;
constexpr double ETA_MAX_FIRST = 1e4, ETA_MAX_EARLY = 10.0, ETA_MAX_GENERAL = 10.0;
constexpr int SMALL_NST = 10;
constexpr double ETA_MIN_EF = 0.1, ETA_MAX_EF = 0.2, ETA_CF = 0.25;
constexpr int SMALL_NEF = 2, MXNEF1 = 3, MXNEF = 7, MXNCF = 10;
constexpr int MAXCOR = 3;
constexpr double NLSCOEF = 0.1, CRDOWN = 0.3, RDIV = 2.0;
constexpr int MSBP = 20;
constexpr int MSBJ = 51;
constexpr double DGMAX_JBAD = 0.2;
constexpr double DGMAX = 0.3;
constexpr double UROUND = 2.220446049250313e-16;
enum { ST_OK = 0, ST_MAX_STEPS = 1, ST_ERR_FAIL = 2, ST_CONV_FAIL = 3, ST_NONFINITE = 4, ST_H_TOO_SMALL = 5 };
enum { NLS_OK = 0, NLS_RECOVER = 1 };

// scalar slots of the per-reactor record (after zn[QMAX+1][N])
enum {
    R_TN = 0, R_H, R_HSCALE, R_HPRIME, R_ETA, R_ETAMAX, R_TAU = 6, R_TQ = 13, R_GAMMAP = 19, R_CRATE,
    R_SAVEDTQ5, R_IGN = 22, R_Q = 30, R_QPRIME, R_QWAIT, R_NST, R_NSTLP, R_NSAMP, R_FLAGS, R_STATUS,
    R_L = 38, R_NSCAL = 44
};
enum { F_HASPREV = 1, F_HASRIGHT = 2, F_AWAIT = 4, F_INIT = 8 };
}  // namespace

struct BdfScal {
    double tn, h, hscale, hprime, eta, etamax, gamma, gammap, gamrat, crate, acnrm, saved_tq5;
    double tau[QMAX + 2], tq[6], l[QMAX + 1];
    int q, qprime, qwait, L, nst, nstlp, nstlj;
    bool haveLU, haveJ;
    // ignition marker
    int status0;
};

// Per-warp bookkeeping touched only by lane 0 (kept out of registers): the ignition
// marker and the solver counters.
struct WarpAux {
    double ls_t, ls_v, pv_t, pv_v, bs_t, bs_v, nx_t, nx_v;
    long long nrhs, nni, nsetups, nje, netf, ncfn;
    long long nli, nps, njtv;   // Krylov path: linear iterations, preconditioner solves, J v products
    int nsamp, flags;
};
constexpr int kAuxDoubles = (int)((sizeof(WarpAux) + 7) / 8);

// ---------------------------------------------------------------------------
// The large per-warp routines are kept out of line (one copy of their code: the
// integrator reaches them from several places) and take plain arguments, so that the
// integrator's own state stays in registers.  A warp's shared-memory slice starts with
// the KinState of its last right-hand side (kStateSlots doubles), then the kinetics
// scratch.
// ---------------------------------------------------------------------------
// division and square root for the integrator's scalar step control, out of line: one copy
// of their code instead of one per use (the step logic runs once per step, its code size
// matters more than a call)
GB_TU_LOCAL __device__ __noinline__ double ddiv(double a, double b) { return a / b; }
GB_TU_LOCAL __device__ __noinline__ double dsqrt(double a) { return sqrt(a); }

constexpr int kStateSlots = 16;
static_assert(kKinStateDoubles <= 15, "state slots");

// finite (not inf, not NaN) on the integer pipe
__device__ __forceinline__ bool finiteBits(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}
__device__ __forceinline__ void storeState(double* base, const KinState& st) {
    base[0] = st.T; base[1] = st.P; base[2] = st.RT; base[3] = st.rho;
    base[4] = st.mmw; base[5] = st.ctot; base[6] = st.lnT; base[7] = st.recipT;
    base[8] = st.rrho; base[9] = st.lnPP; base[10] = st.lnC0; base[11] = st.RTP; base[12] = st.PRT;
}

// slot kExtSlot of the state slots holds the address of the warp's external Jacobian
// scratch (kfe, rkc) or null
constexpr int kExtSlot = 15;
__device__ __forceinline__ double* extScratch(const double* base) {
    return reinterpret_cast<double* const*>(base + kExtSlot)[0];
}
__device__ __forceinline__ void carveScratch(const DevMech& m, double* base, const uint64_t* tab, KinScratch& s) {
    s.carve(base + kStateSlots, m.K, m.R, m.NTB, m.NF, m.NT, extScratch(base));
    s.tab = tab;
}
__device__ __forceinline__ void loadState(const double* base, KinState& st) {
    st.T = base[0]; st.P = base[1]; st.RT = base[2]; st.rho = base[3];
    st.mmw = base[4]; st.ctot = base[5]; st.lnT = base[6]; st.recipT = base[7];
    st.rrho = base[8]; st.lnPP = base[9]; st.lnC0 = base[10]; st.RTP = base[11]; st.PRT = base[12];
}

// reactor right-hand side at z = [T, Y]; returns true when every derivative is finite
// (with forJac the kinetics scratch also keeps what d(wdot)/dc needs: the right-hand side
// that precedes a Jacobian evaluation).  kMole: the state is z = [T, n_1..n_K] of
// IdealGasConstPressureMoleReactor (src/zeroD/IdealGasConstPressureMoleReactor.cpp:53-104):
// dn_k/dt = wdot_k V with V = mass / rho, and m cp dT/dt = -sum_k h_k wdot_k V, which is the
// same dT/dt as the mass-fraction form.
template <bool kX, bool kMole = false>
__device__ __noinline__ bool devRhs(const DevMech& m, double* base, const uint64_t* tab, double P,
                                    const double* z, double* zdot, int lane, bool forJac) {
    KinScratch s;
    carveScratch(m, base, tab, s);
    KinState st;
    warpState<kMole>(m, z[0], P, z + 1, s, st, lane);
    __syncwarp();
    warpRates<kX>(m, s, st, lane, forJac);
    if (lane == 0) storeState(base, st);
    double ph = 0.0, pc = 0.0;
#pragma unroll 1
    for (int k = lane; k < m.K; k += 32) {
        ph += s.wdot[k] * s.hRT[k];
        pc += s.c[k] * s.cpR[k];
    }
    // dT/dt = -sum(h_k wdot_k) / (rho cp_mass) = -T sum(h_k/RT wdot_k) / sum(c_k cp_k/R)
    const double hw = warpSum(ph);
    const double dTdt = -(hw * st.T) / warpSum(pc);
    bool ok = finiteBits(dTdt);
    if (lane == 0) zdot[0] = dTdt;
    const double rrho = st.rrho;
    if (kMole) {
        double pm = 0.0;
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) pm += z[1 + k] * m.mw[k];
        const double vol = warpSum(pm) * rrho;
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) {
            const double v = s.wdot[k] * vol;
            zdot[1 + k] = v;
            ok = ok && finiteBits(v);
        }
    } else {
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) {
            const double v = s.wdot[k] * m.mw[k] * rrho;
            zdot[1 + k] = v;
            ok = ok && finiteBits(v);
        }
    }
    __syncwarp();
    return __all_sync(0xffffffffu, ok);
}

    // LU with partial pivoting in place (row-major, leading dimension ld).  Afterwards
// piv[] holds the gather permutation (row i of P*b is b[piv[i]]) and dinv[] the
// reciprocal diagonal of U, both in shared memory.
__device__ __forceinline__ unsigned long long absKey(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFULL;
}
__device__ __forceinline__ unsigned long long absKey(float x) {
    return (unsigned long long)((unsigned)__float_as_int(x) & 0x7FFFFFFFu);
}

// Left-looking LU with partial pivoting and lazy row interchanges: P A = L U with row k of
// P A being the stored (physical) row piv[k].  Column j is computed in registers (lane l holds
// rows l, l + 32, ... of it): the eliminations of the earlier pivots are applied in pivot order
// (step k: u = the column's value in row piv[k], broadcast by a shuffle; every row not yet a
// pivot at step k subtracts its stored multiplier a[r][k] times u), then the pivot is the
// largest remaining entry and the remaining rows become multipliers.  Each entry of the
// matrix is stored once (the right-looking form rewrites the trailing submatrix at every
// pivot, and a global store goes to L2); the multipliers are re-read, from L1.  Row r of the
// result holds, for r = piv[k], the multipliers L[k][0..k-1] and then U[k][k..N-1].
template <typename MT, int S>
__device__ __forceinline__ bool luLeft(MT* a, int N, int ld, int* piv, double* dinv, int lane) {
    int pidx[S];   // pivot index of the lane's rows (N: not a pivot yet)
#pragma unroll
    for (int t = 0; t < S; t++) pidx[t] = N;
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        MT c[S], m1[S], m2[S];
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int r = lane + 32 * t;
            c[t] = r < N ? a[(size_t)r * ld + j] : (MT)0;
            m1[t] = (r < N && j > 0) ? a[(size_t)r * ld] : (MT)0;
            m2[t] = (r < N && j > 1) ? a[(size_t)r * ld + 1] : (MT)0;
        }
        int p1 = j > 0 ? piv[0] : 0;
#pragma unroll 1
        for (int k = 0; k < j; k++) {
            MT mul[S];
#pragma unroll
            for (int t = 0; t < S; t++) {
                mul[t] = m1[t];
                m1[t] = m2[t];
                const int r = lane + 32 * t;
                if (r < N && k + 2 < j) m2[t] = a[(size_t)r * ld + k + 2];
            }
            const int pk = p1;
            if (k + 1 < j) p1 = piv[k + 1];
            MT sel = c[0];
#pragma unroll
            for (int t = 1; t < S; t++)
                if ((pk >> 5) == t) sel = c[t];
            const MT u = __shfl_sync(0xffffffffu, sel, pk & 31);
#pragma unroll
            for (int t = 0; t < S; t++)
                if (pidx[t] > k) c[t] -= mul[t] * u;
        }
        // pivot: the largest remaining |entry| (integer compare of the bits with the sign
        // cleared; the caller has checked that M is finite), lowest row on ties
        unsigned long long bv = 0ULL;
        int bi = N;
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int r = lane + 32 * t;
            if (r < N && pidx[t] == N) {
                const unsigned long long v = absKey(c[t]);
                if (v > bv || bi == N) { bv = v; bi = r; }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (oi < N && (bi == N || ov > bv || (ov == bv && oi < bi))) { bv = ov; bi = oi; }
        }
        if (bv == 0ULL) return false;
        MT psel = c[0];
#pragma unroll
        for (int t = 1; t < S; t++)
            if ((bi >> 5) == t) psel = c[t];
        const MT pv = __shfl_sync(0xffffffffu, psel, bi & 31);
        const MT inv = (MT)1 / pv;
        if (lane == 0) {
            piv[j] = bi;
            dinv[j] = (double)inv;
        }
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int r = lane + 32 * t;
            if (r == bi) pidx[t] = j;
            else if (pidx[t] == N) c[t] *= inv;
            if (r < N) a[(size_t)r * ld + j] = c[t];
        }
        __syncwarp();
    }
    return true;
}

// Right-looking LU with partial pivoting and physical row interchanges (row k of P A stored
// in row k), for the larger matrices, where the trailing updates' parallel work beats the
// left-looking form's sequential chain of N^2 / 2 shuffles (n-dodecane, N = 101: 646 against
// 514 reactors/s), blocked by panels of four columns.  Step k of the unblocked form: the
// pivot is the largest |a[i][k]|, i >= k (integer compare of the bits with the sign cleared;
// the caller has checked that the matrix is finite; lowest row on ties); rows k and the
// pivot's are interchanged in full; the multipliers a[i][k] *= 1 / a[k][k]; every trailing
// entry a[i][j] (i, j > k) = fma(-a[i][k], a[k][j], a[i][j]).  Here a panel's four columns are
// factored first (those steps restricted to the panel's columns), and only then are its four
// pivots applied to the rest of the matrix, each trailing entry loaded and stored once per
// panel instead of once per pivot (a global store goes to L2).  Every entry receives the same
// fused multiply-adds in the same pivot order, with the same operands (a row interchange inside
// the panel moves a row's multipliers with its not-yet-updated trailing part), so the factors
// are bit for bit those of the unblocked form.
template <typename MT>
__device__ __forceinline__ bool luRightPanel4(MT* a, int N, int ld, int* piv, double* dinv, int lane) {
    constexpr int B = 4;
    if (lane == 0)
        for (int i = 0; i < N; i++) piv[i] = i;
    __syncwarp();
#pragma unroll 1
    for (int k0 = 0; k0 < N; k0 += B) {
        const int kend = min(k0 + B, N);
        // the panel: columns k0 .. kend - 1
#pragma unroll 1
        for (int k = k0; k < kend; k++) {
            unsigned long long bv = 0ULL;
            int bi = N;
            for (int i = k + lane; i < N; i += 32) {
                const unsigned long long v = absKey(a[(size_t)i * ld + k]);
                if (v > bv || bi == N) { bv = v; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
            }
            if (bv == 0ULL) return false;
            if (bi != k) {
                for (int j = lane; j < N; j += 32) {
                    MT t = a[(size_t)k * ld + j];
                    a[(size_t)k * ld + j] = a[(size_t)bi * ld + j];
                    a[(size_t)bi * ld + j] = t;
                }
                if (lane == 0) { int t = piv[k]; piv[k] = piv[bi]; piv[bi] = t; }
            }
            __syncwarp();
            const MT inv = (MT)1 / a[(size_t)k * ld + k];
            if (lane == 0) dinv[k] = (double)inv;
            // multipliers of column k, then pivot k applied to the panel's later columns
#pragma unroll 1
            for (int i = k + 1 + lane; i < N; i += 32) {
                MT* r = a + (size_t)i * ld;
                const MT l = r[k] * inv;
                r[k] = l;
                for (int j = k + 1; j < kend; j++) r[j] = fma(-l, a[(size_t)k * ld + j], r[j]);
            }
            __syncwarp();
        }
        const int nb = kend - k0;
        // the trailing columns: the panel's rows first (row k0 + p receives pivots k0 .. k0 + p - 1
        // in order), then the rows below (all the panel's pivots in order), lanes over columns
#pragma unroll 1
        for (int j = kend + lane; j < N; j += 32) {
            MT u[B];
#pragma unroll
            for (int p = 0; p < B; p++) u[p] = p < nb ? a[(size_t)(k0 + p) * ld + j] : (MT)0;
#pragma unroll
            for (int p = 1; p < B; p++) {
                if (p >= nb) break;
                const MT* r = a + (size_t)(k0 + p) * ld + k0;
#pragma unroll
                for (int q = 0; q < p; q++) u[p] = fma(-r[q], u[q], u[p]);
                a[(size_t)(k0 + p) * ld + j] = u[p];
            }
            int i = kend;
            for (; i + 4 <= N; i += 4) {
                MT l[4][B], v[4];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    const MT* row = a + (size_t)(i + r) * ld;
#pragma unroll
                    for (int p = 0; p < B; p++) l[r][p] = p < nb ? row[k0 + p] : (MT)0;
                    v[r] = row[j];
                }
#pragma unroll
                for (int r = 0; r < 4; r++) {
#pragma unroll
                    for (int p = 0; p < B; p++)
                        if (p < nb) v[r] = fma(-l[r][p], u[p], v[r]);
                    a[(size_t)(i + r) * ld + j] = v[r];
                }
            }
            for (; i < N; i++) {
                MT* row = a + (size_t)i * ld;
                MT v = row[j];
#pragma unroll
                for (int p = 0; p < B; p++)
                    if (p < nb) v = fma(-row[k0 + p], u[p], v);
                row[j] = v;
            }
        }
        __syncwarp();
    }
    return true;
}

// The factorisation of an integrator instantiation with NS register slots per lane (N <= 32
// NS): left-looking up to 64 components (h2o2 +5 %, gri30 +0.7 % FP64 / +3.7 % FP32 reactors/s
// over the right-looking form), right-looking in panels of four beyond (n-dodecane, same factors
// as the unblocked form: +9 % FP64, +14 % FP32 reactors/s).  kLazyRows<NS> tells the solve
// which layout the factors have.
template <int NS>
constexpr bool kLazyRows = NS <= 2;

template <typename MT, int NS>
__device__ __noinline__ bool devLuFactor(MT* a, int N, int ld, int* piv, double* dinv, int lane) {
    __syncwarp();
    bool ok;
    if constexpr (kLazyRows<NS>) ok = luLeft<MT, NS>(a, N, ld, piv, dinv, lane);
    else ok = luRightPanel4<MT>(a, N, ld, piv, dinv, lane);
    __syncwarp();
    return ok;
}

// Shared-memory staging of a factorisation whose matrix lives in global memory: a block
// owns a few matrix-sized buffers; a warp that finds one free (atomic claim, never a wait)
// copies its matrix in, factors it there and copies the factors back, otherwise it factors
// in place.
struct LuPool {
    char* buf;        // nslots buffers of slotBytes (shared memory), or null
    int* flags;       // nslots claim flags (shared memory)
    int nslots;
    int slotBytes;
};

template <typename MT, int NS>
__device__ __noinline__ bool devLuStaged(MT* M, int N, int ld, int* piv, double* dinv, int lane, LuPool pool) {
    int slot = -1;
    if (pool.nslots > 0 && lane == 0) {
        for (int q = 0; q < pool.nslots && slot < 0; q++)
            if (atomicCAS(&pool.flags[q], 0, 1) == 0) slot = q;
    }
    slot = __shfl_sync(0xffffffffu, slot, 0);
    if (slot < 0) return devLuFactor<MT, NS>(M, N, ld, piv, dinv, lane);
    MT* S = (MT*)(pool.buf + (size_t)slot * pool.slotBytes);
    const int n = N * ld;
#pragma unroll 1
    for (int q = lane; q < n; q += 32) S[q] = M[q];
    __syncwarp();
    const bool ok = devLuFactor<MT, NS>(S, N, ld, piv, dinv, lane);
#pragma unroll 1
    for (int q = lane; q < n; q += 32) M[q] = S[q];
    __syncwarp();
    __threadfence_block();
    if (lane == 0) atomicExch(&pool.flags[slot], 0);
    __syncwarp();
    return ok;
}

// Newton matrix M = I - gamma*J (J analytic in the species columns, one-sided
// difference in T), stored TRANSPOSED (element M[r][c] at A[c*ld + r]) and factored in
// place: the factorisation of A = M^T pivots on M's columns, and the triangular solves
// then read rows of A, which are contiguous (coalesced when A lives in global memory).
// The kinetics scratch must hold the state y (the last right-hand side was evaluated at y,
// giving ftemp).  kJacOnly: store J (transposed, no identity) and skip the factorisation.
// Returns false if J is not finite or M singular.
template <typename MT, bool kJacOnly, bool kX, int NS>
__device__ __noinline__ bool devSetup(const DevMech& mm, double* base, const uint64_t* tab, MT* A, int ld,
                                      double gamma, double P, const double* y, const double* ftemp,
                                      double* v1, double* v2, double* tempv, int* piv, double* dinv,
                                      int lane, LuPool pool) {
    const int K = mm.K, N = mm.N;
    KinScratch s;
    carveScratch(mm, base, tab, s);
    KinState st;
    loadState(base, st);
#pragma unroll 1
    for (int q = lane; q < N * ld; q += 32) A[q] = (MT)0;
    __syncwarp();
    MT* Jt = A + ld + 1;   // Jc^T: Jc[k][j] at Jt[j*ld + k]
    warpJacC<MT, true>(mm, s, Jt, ld, lane);
    // v1 = X (mole fractions); v2[k] = (Jc X)_k
    const double rct = st.RTP;   // 1/ctot
#pragma unroll 1
    for (int k = lane; k < K; k += 32) v1[k] = s.c[k] * rct;
    __syncwarp();
#pragma unroll 1
    for (int k = lane; k < K; k += 32) {
        double a = 0.0;
#pragma unroll 1
        for (int l = 0; l < K; l++) a += (double)Jt[(size_t)l * ld + k] * v1[l];
        v2[k] = a;
    }
    double pcp = 0.0;
#pragma unroll 1
    for (int k = lane; k < K; k += 32) pcp += v1[k] * s.cpR[k];
    const double cpmix = warpSum(pcp);
    __syncwarp();
    // hJ_j = sum_k h_k Jc[k][j]
    double phj = 0.0;
#pragma unroll 1
    for (int j = lane; j < K; j += 32) {
        const MT* row = Jt + (size_t)j * ld;
        double a = 0.0;
#pragma unroll 1
        for (int k = 0; k < K; k++) a += s.hRT[k] * (double)row[k];
        tempv[j] = a;
        phj += a * v1[j];
    }
    const double hJX = warpSum(phj);
    const double rho = st.rho, mmw = st.mmw;
    // 1/(rho R cp_mix/mmw) = 1/(R ctot cp_mix) = (RT/P) / (R cp_mix)
    const double rD = st.RTP / (mm.Rgas * cpmix);
    const double G = ftemp[0];
    // v2[k] <- W_k (Jc X)_k - wdot_k W_k mmw / rho: J[1+k][1+j] = (W_k Jc_kj - v2[k]) / W_j
    const double c1 = mmw * st.rrho;
#pragma unroll 1
    for (int k = lane; k < K; k += 32) v2[k] = mm.mw[k] * (v2[k] - s.wdot[k] * c1);
    __syncwarp();
    // species block of M = I - gamma J: M_kj = delta_kj - gamma/W_j (W_k Jc_kj - v2_k), by
    // rows of A (lanes along k)
    bool fin = true;
#pragma unroll 1
    for (int j = 0; j < K; j++) {
        const double gj = -gamma * mm.rmw[j];
        MT* row = Jt + (size_t)j * ld;
#pragma unroll 1
        for (int k = lane; k < K; k += 32) {
            double v = fma(mm.mw[k], (double)row[k], -v2[k]) * gj;
            if (!kJacOnly && k == j) v += 1.0;
            fin = fin && finiteBits(v);
            row[k] = (MT)v;
        }
    }
    // T row of M (column 0 of A)
    const double hscale = rho * st.RT, cpscale = rho * mm.Rgas;
#pragma unroll 1
    for (int j = lane; j < K; j += 32) {
        const double rWj = mm.rmw[j];
        const double dH = hscale * rWj * (tempv[j] - hJX);
        const double dD = cpscale * rWj * (s.cpR[j] - cpmix);
        const double v = (dH + G * dD) * rD * gamma;   // -gamma * J[0][1+j]
        fin = fin && finiteBits(v);
        A[(size_t)(1 + j) * ld] = (MT)v;
    }
    __syncwarp();
    // T column of M (row 0 of A): one-sided difference
    const double T0 = y[0];
    const double dT = sqrt(UROUND) * fmax(1.0, fabs(T0));
#pragma unroll 1
    for (int i = lane; i < N; i += 32) tempv[i] = y[i];
    __syncwarp();
    if (lane == 0) tempv[0] = T0 + dT;
    __syncwarp();
    bool ok = devRhs<kX>(mm, base, tab, P, tempv, v1, lane, false);
    const double gdT = -gamma / dT;
#pragma unroll 1
    for (int i = lane; i < N; i += 32) {
        double v = (v1[i] - ftemp[i]) * gdT;
        if (!kJacOnly && i == 0) v += 1.0;
        fin = fin && finiteBits(v);
        A[i] = (MT)v;
    }
    __syncwarp();
    ok = __all_sync(0xffffffffu, ok && fin);
    if (!ok) return false;
    if (kJacOnly) return true;
    return devLuStaged<MT, NS>(A, N, ld, piv, dinv, lane, pool);
}

// A = M^T = I - gamma J^T from a kept Jacobian (stored transposed, FP64), then the LU
// factorisation of A.
template <typename MT, int NS>
__device__ __noinline__ bool devFormLU(MT* M, const double* J, int N, int ld, double gamma, int* piv, double* dinv,
                                       int lane, LuPool pool) {
    bool fin = true;
#pragma unroll 1
    for (int i = 0; i < N; i++) {
#pragma unroll 1
        for (int j = lane; j < N; j += 32) {
            double v = -gamma * J[(size_t)i * ld + j];
            if (i == j) v += 1.0;
            fin = fin && finiteBits(v);
            M[(size_t)i * ld + j] = (MT)v;
        }
    }
    __syncwarp();
    if (!__all_sync(0xffffffffu, fin)) return false;
    return devLuStaged<MT, NS>(M, N, ld, piv, dinv, lane, pool);
}

// Solve (P^T L U) x = b in place.  The vector lives in registers (element i in lane
// i % 32, slot i / 32); every substitution step broadcasts one element by a shuffle.
template <typename MT, int S>
__device__ __noinline__ void devLuSolve(const MT* a, double* b, int N, int ld, const int* piv, const double* dinv,
                                        int lane) {
    // a holds the factors of A = M^T: P A = L U, row k of P A coming from row piv[k] of A and
    // stored in row piv[k] of a (left-looking form) or in row k (right-looking form), so
    // M = U^T L^T P and M x = b is solved by U^T w = b (forward), L^T z = w (backward),
    // x[piv[i]] = z[i].  Step k of either sweep reads the stored row of k (coalesced); the rows
    // of steps k+1 and k+2 are in flight meanwhile.  The vector lives in registers: element i
    // in lane i % 32, slot i / 32.
    auto row = [&](int k) -> const MT* { return a + (size_t)(kLazyRows<S> ? piv[k] : k) * ld; };
    MT x[S];
#pragma unroll
    for (int t = 0; t < S; t++) {
        const int i = lane + 32 * t;
        x[t] = (i < N) ? (MT)b[i] : (MT)0;
    }
    MT n1[S], n2[S];
    // forward: U^T w = b; w_k = b_k / U_kk, then b_i -= U[k][i] w_k for i > k
    const MT* r1 = row(0);
    const MT* r2 = row(N > 1 ? 1 : 0);
#pragma unroll
    for (int t = 0; t < S; t++) {
        const int i = lane + 32 * t;
        n1[t] = (i < N) ? r1[i] : (MT)0;
        n2[t] = (i < N && N > 1) ? r2[i] : (MT)0;
    }
    MT nd1 = (MT)dinv[0];
    MT nd2 = (N > 1) ? (MT)dinv[1] : (MT)0;
#pragma unroll
    for (int tk = 0; tk < S; tk++) {
        const int kend = min(N, 32 * (tk + 1));
        for (int k = 32 * tk; k < kend; k++) {
            MT cur[S];
            const MT dk = nd1;
            nd1 = nd2;
            if (k + 2 < N) nd2 = (MT)dinv[k + 2];
            const MT* rn = row(k + 2 < N ? k + 2 : 0);
#pragma unroll
            for (int t = 0; t < S; t++) {
                cur[t] = n1[t];
                n1[t] = n2[t];
                const int i = lane + 32 * t;
                if (i < N && k + 2 < N) n2[t] = rn[i];
            }
            if (lane == (k & 31)) x[tk] = x[tk] * dk;
            const MT wk = __shfl_sync(0xffffffffu, x[tk], k & 31);
#pragma unroll
            for (int t = tk; t < S; t++) {
                const int i = lane + 32 * t;
                if (i > k && i < N) x[t] -= cur[t] * wk;
            }
        }
    }
    // backward: L^T z = w (unit diagonal); w_i -= L[k][i] z_k for i < k
    const MT* b1 = row(N - 1);
    const MT* b2 = row(N > 1 ? N - 2 : 0);
#pragma unroll
    for (int t = 0; t < S; t++) {
        const int i = lane + 32 * t;
        n1[t] = (i < N) ? b1[i] : (MT)0;
        n2[t] = (i < N && N > 1) ? b2[i] : (MT)0;
    }
#pragma unroll
    for (int tk = S - 1; tk >= 0; tk--) {
        const int kbeg = min(N, 32 * (tk + 1)) - 1;
        for (int k = kbeg; k >= 32 * tk; k--) {
            MT cur[S];
            const MT* rp = row(k > 1 ? k - 2 : 0);
#pragma unroll
            for (int t = 0; t < S; t++) {
                cur[t] = n1[t];
                n1[t] = n2[t];
                const int i = lane + 32 * t;
                if (i < N && k > 1) n2[t] = rp[i];
            }
            const MT zk = __shfl_sync(0xffffffffu, x[tk], k & 31);
#pragma unroll
            for (int t = 0; t <= tk; t++) {
                const int i = lane + 32 * t;
                if (i < k) x[t] -= cur[t] * zk;
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < S; t++) {
        const int i = lane + 32 * t;
        if (i < N) b[piv[i]] = (double)x[t];
    }
    __syncwarp();
}


// =============================================================================
// Krylov linear solver: GMRES preconditioned by an incomplete LU of I - gamma Jp, where Jp
// is the adaptive preconditioner's approximate Jacobian of the mole reactor
// (IdealGasConstPressureMoleReactor::getJacobianElements,
// src/zeroD/IdealGasConstPressureMoleReactor.cpp:106-221; AdaptivePreconditioner,
// src/numerics/AdaptivePreconditioner.cpp:17-81; the solver CVODE runs for it,
// src/numerics/CVodesIntegrator.cpp:67-80).  The matrices are stored transposed (row j holds
// column j), so that the factorisation's updates and both triangular sweeps read and write
// whole rows (coalesced).
// =============================================================================
constexpr int kMaxl = kKrylovMaxl;     // Krylov vectors (CVODE's default)
[[maybe_unused]] constexpr double kEplifac = 0.05;     // linear tolerance factor (CVODE's default)
[[maybe_unused]] constexpr double kIlutTau = 1e-12;    // drop tolerance the adaptive preconditioner gives ILUT
[[maybe_unused]] constexpr int kIlutFillFactor = 10;   // ILUT's fill factor (the library default it keeps)
// GMRES scalars per warp: H[(kMaxl + 1)][kMaxl], cs[kMaxl], sn[kMaxl], g[kMaxl + 1], y[kMaxl],
// rho (padded to an even count)
constexpr int kGmresScalars = ((kMaxl + 1) * kMaxl + 2 * kMaxl + (kMaxl + 1) + kMaxl + 1 + 1) & ~1;

// The preconditioner's Jacobian Jp at the state y, its components clipped below at atol
// (AdaptivePreconditioner::stateAdjustment), into Jt = Jp^T (FP64, leading dimension ld):
// the T column by a one-sided difference with dT = T sqrt(eps) (perturbed state first, as the
// reference), the species block d(dn_k/dt)/dn_j = d(wdot_k)/dc_j (ddCi; the -n_i/(V N) terms of
// the exact derivative are left out, as there), and the T row
// d(dT/dt)/dn_j = (cp_j qdot - m cp sum_k h_k d(dn_k/dt)/dn_j) / (m cp)^2, qdot = sum_k h_k dn_k/dt.
// Scratch: four N-vectors at w.  Returns false when a right-hand side is not finite.
template <bool kX>
__device__ __noinline__ bool devPrecJac(const DevMech& mm, double* base, const uint64_t* tab, double* Jt, int ld,
                                        double P, double atol, const double* y, double* w, int lane) {
    const int K = mm.K, N = mm.N;
    double* zc = w;
    double* zp = w + N;
    double* fc = w + 2 * N;
    double* fp = w + 3 * N;
#pragma unroll 1
    for (int i = lane; i < N; i += 32) {
        const double v = fmax(y[i], atol);
        zc[i] = v;
        zp[i] = v;
    }
    __syncwarp();
    const double dT = zc[0] * sqrt(UROUND);
    if (lane == 0) zp[0] = zc[0] + dT;
    __syncwarp();
    bool ok = devRhs<kX, true>(mm, base, tab, P, zp, fp, lane, false);
    ok = devRhs<kX, true>(mm, base, tab, P, zc, fc, lane, true) && ok;
    if (!ok) return false;
#pragma unroll 1
    for (int q = lane; q < N * ld; q += 32) Jt[q] = 0.0;
    __syncwarp();
    // T column of Jp = row 0 of Jt
#pragma unroll 1
    for (int j = lane; j < N; j += 32) Jt[j] = (fp[j] - fc[j]) / dT;
    KinScratch s;
    carveScratch(mm, base, tab, s);
    KinState st;
    loadState(base, st);
    // species block: d(wdot_k)/dc_j at Jt[(1 + j) ld + 1 + k], then the default-efficiency part
    // g_k that every column shares
    double* Jsp = Jt + ld + 1;
    warpJacC<double, true>(mm, s, Jsp, ld, lane);
    double* g = fp;
    warpDenseG(mm, s, g, lane);
    bool anyG = false;
#pragma unroll 1
    for (int k = lane; k < K; k += 32) anyG = anyG || g[k] != 0.0;
    if (__any_sync(0xffffffffu, anyG)) {
#pragma unroll 1
        for (int j = 0; j < K; j++) {
            double* row = Jsp + (size_t)j * ld;
#pragma unroll 1
            for (int k = lane; k < K; k += 32) row[k] += g[k];
        }
    }
    __syncwarp();
    // T row: h_k = (h_k/RT) RT, qdot = sum_k h_k wdot_k V, m cp = V R sum_k c_k cp_k/R
    double pm = 0.0, pq = 0.0, pc = 0.0;
#pragma unroll 1
    for (int k = lane; k < K; k += 32) {
        pm += zc[1 + k] * mm.mw[k];
        pq += s.hRT[k] * s.wdot[k];
        pc += s.c[k] * s.cpR[k];
    }
    const double vol = warpSum(pm) * st.rrho;
    const double qdot = warpSum(pq) * st.RT * vol;
    const double mcp = vol * mm.Rgas * warpSum(pc);
    const double denom = 1.0 / (mcp * mcp);
#pragma unroll 1
    for (int j = lane; j < K; j += 32) {
        const double* row = Jsp + (size_t)j * ld;
        double hs = 0.0;
#pragma unroll 1
        for (int k = 0; k < K; k++) hs += row[k] * (s.hRT[k] * st.RT);
        const double cpj = s.cpR[j] * mm.Rgas;
        Jt[(size_t)(1 + j) * ld] = (cpj * qdot - mcp * hs) * denom;
    }
    __syncwarp();
    return true;
}

// Keep the `fill` largest entries (by magnitude) among those of w[] that `part` selects and
// clear the others (ILUT's fill limit): the fill-th largest magnitude is found bit by bit on
// the magnitudes' bit patterns; entries equal to it are kept in index order.
template <typename MT, int S>
__device__ __forceinline__ void ilutFillLimit(MT (&w)[S], const bool (&part)[S], int fill, int lane) {
    unsigned long long key[S];
#pragma unroll
    for (int t = 0; t < S; t++) key[t] = part[t] ? absKey(w[t]) : 0ULL;
    auto countGe = [&](unsigned long long v) {
        int c = 0;
#pragma unroll
        for (int t = 0; t < S; t++) c += __popc(__ballot_sync(0xffffffffu, part[t] && key[t] >= v));
        return c;
    };
    unsigned long long T = 0;
#pragma unroll 1
    for (int b = 62; b >= 0; b--) {
        const unsigned long long cand = T | (1ULL << b);
        if (countGe(cand) >= fill) T = cand;
    }
    int need = fill - (T == ~0ULL ? 0 : countGe(T + 1));
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int t = 0; t < S; t++) {
        const unsigned eq = __ballot_sync(0xffffffffu, part[t] && key[t] == T);
        const int rank = __popc(eq & lt);
        if (part[t] && (key[t] < T || (key[t] == T && rank >= need))) w[t] = (MT)0;
        need -= __popc(eq);
    }
}

// ILUT(p, tau) of P in place, P stored transposed (a[j ld + i] = P[i][j]), with the rules of
// Saad's dual-threshold incomplete LU as the adaptive preconditioner uses it: row by row, a
// multiplier at or below tau is dropped, then the entries of the finished row below tau times
// its 2-norm (of the row before elimination), then all but the p largest of its L part and of
// its U part, p = 10 nnz(P) / N + 1, and a zero pivot becomes sqrt(tau) times the row norm.
// Carried out right-looking: at step k row k has received every update it gets in the
// row-by-row (IKJ) order, in the same order, so it is finished and dropped before its U part
// updates the rows below.  Afterwards a holds L (unit diagonal, strictly lower part) and U,
// dinv[] the reciprocal diagonal of U.  rn: N doubles of scratch.  MT: the element type of the
// factors (double; float for the FP32 preconditioner, whose arithmetic is FP32 too).
template <typename MT, int S>
__device__ __noinline__ void devIlut(MT* a, int N, int ld, double* dinv, double* rn, int lane) {
    int cnt = 0;
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        const MT* row = a + (size_t)j * ld;
#pragma unroll 1
        for (int i = lane; i < N; i += 32) cnt += row[i] != (MT)0;
    }
    const long long nnz = __reduce_add_sync(0xffffffffu, cnt);
    const int fill = (int)(nnz * kIlutFillFactor / N) + 1;
    // 2-norms of the rows of P (columns of a)
#pragma unroll 1
    for (int i = lane; i < N; i += 32) {
        double q = 0.0;
#pragma unroll 1
        for (int j = 0; j < N; j++) {
            const double v = (double)a[(size_t)j * ld + i];
            q += v * v;
        }
        rn[i] = sqrt(q);
    }
    __syncwarp();
    const double sqrtTau = sqrt(kIlutTau);
#pragma unroll 1
    for (int k = 0; k < N; k++) {
        // finish row k of P (column k of a): threshold drops, fill limits, zero pivot
        MT w[S];
        bool inL[S], inU[S];
        const double rnk = rn[k];
        const double thr = kIlutTau * rnk;
        int cL = 0, cU = 0;
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int j = lane + 32 * t;
            MT v = (j < N) ? a[(size_t)j * ld + k] : (MT)0;
            if (j != k && !(fabs((double)v) > thr)) v = (MT)0;
            w[t] = v;
            inL[t] = j < k;
            inU[t] = j > k && j < N;
            cL += __popc(__ballot_sync(0xffffffffu, inL[t] && v != (MT)0));
            cU += __popc(__ballot_sync(0xffffffffu, inU[t] && v != (MT)0));
        }
        if (cL > fill) ilutFillLimit<MT, S>(w, inL, fill, lane);
        if (cU > fill) ilutFillLimit<MT, S>(w, inU, fill, lane);
        MT dk = (MT)0;
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int j = lane + 32 * t;
            if (j == k && w[t] == (MT)0) w[t] = (MT)(sqrtTau * rnk);
            if (j < N) a[(size_t)j * ld + k] = w[t];
            if (t == (k >> 5)) dk = w[t];
        }
        dk = __shfl_sync(0xffffffffu, dk, k & 31);
        if (lane == 0) dinv[k] = 1.0 / (double)dk;
        // multipliers of column k (row k of a): f_i = P[i][k] / P[k][k], dropped at or below tau
        MT f[S];
        bool anyF[S];
        MT* rk = a + (size_t)k * ld;
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int i = lane + 32 * t;
            MT v = (MT)0;
            if (i > k && i < N) {
                const MT p = rk[i];
                if (p != (MT)0) {
                    v = p / dk;
                    if (fabs((double)v) <= kIlutTau) v = (MT)0;
                    rk[i] = v;
                }
            }
            f[t] = v;
            anyF[t] = __any_sync(0xffffffffu, v != (MT)0);
        }
        // rows i > k: P[i][j] -= f_i P[k][j] for the kept entries P[k][j], j > k (row j of a),
        // walking the set bits of the kept entries' mask four rows at a time: the four rows'
        // loads are issued before any store (the rows are distinct, so the order of the updates
        // of each element is unchanged)
#pragma unroll
        for (int tj = 0; tj < S; tj++) {
            if (32 * tj + 31 <= k) continue;
            const int j0 = 32 * tj;
            unsigned msk = __ballot_sync(0xffffffffu, w[tj] != (MT)0 && j0 + lane > k && j0 + lane < N);
#pragma unroll 1
            while (msk) {
                int jq[4];
                MT u[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    jq[q] = msk ? __ffs(msk) - 1 : -1;
                    if (msk) msk &= msk - 1;
                    u[q] = __shfl_sync(0xffffffffu, w[tj], jq[q] < 0 ? 0 : jq[q]);
                }
                MT v[S][4];
#pragma unroll
                for (int t = 0; t < S; t++) {
                    const int i = lane + 32 * t;
                    const bool act = anyF[t] && i > k && i < N;
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        v[t][q] = (act && jq[q] >= 0) ? a[(size_t)(j0 + jq[q]) * ld + i] : (MT)0;
                }
#pragma unroll
                for (int t = 0; t < S; t++) {
                    const int i = lane + 32 * t;
                    const bool act = anyF[t] && i > k && i < N;
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (act && jq[q] >= 0) a[(size_t)(j0 + jq[q]) * ld + i] = fma(-f[t], u[q], v[t][q]);
                }
            }
        }
        __syncwarp();
    }
}

// Solve (L U) x' = b' in place with the factors of devIlut of the reordered matrix, b'[i] =
// b[q[i]] and b[q[i]] = x'[i] (q: the fill-reducing order): L w = b' forward (unit lower;
// column k of L is row k of a), then U x' = w backward (column j of U is row j of a, its
// diagonal from dinv).  The vector lives in registers (element i in lane i % 32, slot i / 32); every
// substitution step broadcasts one element by a shuffle.  The factors are usually in L2 (one
// matrix per resident warp), so the rows of the next kIluAhead steps are in flight meanwhile.
[[maybe_unused]] constexpr int kIluAhead = 4;
template <typename MT, int S>
__device__ __noinline__ void devIluSolve(const MT* a, double* b, int N, int ld, const double* dinv, const DevMech& m,
                                         int lane) {
    const int* q = m.precOrder;
    MT x[S], nr[kIluAhead][S];
    int qi[S];
#pragma unroll
    for (int t = 0; t < S; t++) {
        const int i = lane + 32 * t;
        qi[t] = (i < N) ? GB_IX(m, q[i], N, GB_SITE_PREC_ORDER) : 0;
        x[t] = (i < N) ? (MT)b[qi[t]] : (MT)0;
    }
#pragma unroll
    for (int p = 0; p < kIluAhead; p++) {
        const MT* r = a + (size_t)(p < N ? p : 0) * ld;
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int i = lane + 32 * t;
            nr[p][t] = (i < N && p < N) ? r[i] : (MT)0;
        }
    }
#pragma unroll
    for (int tk = 0; tk < S; tk++) {
        const int kend = min(N, 32 * (tk + 1));
        for (int k = 32 * tk; k < kend; k++) {
            MT cur[S];
            const int kn = k + kIluAhead;
            const MT* rn = a + (size_t)(kn < N ? kn : 0) * ld;
#pragma unroll
            for (int t = 0; t < S; t++) {
                cur[t] = nr[0][t];
#pragma unroll
                for (int p = 0; p + 1 < kIluAhead; p++) nr[p][t] = nr[p + 1][t];
                const int i = lane + 32 * t;
                if (i < N && kn < N) nr[kIluAhead - 1][t] = rn[i];
            }
            const MT wk = __shfl_sync(0xffffffffu, x[tk], k & 31);
            if (wk == (MT)0) continue;
#pragma unroll
            for (int t = tk; t < S; t++) {
                const int i = lane + 32 * t;
                if (i > k && i < N) x[t] -= cur[t] * wk;
            }
        }
    }
    MT nd[kIluAhead];
#pragma unroll
    for (int p = 0; p < kIluAhead; p++) {
        const int k = N - 1 - p;
        const MT* r = a + (size_t)(k >= 0 ? k : 0) * ld;
        nd[p] = (k >= 0) ? (MT)dinv[k] : (MT)0;
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int i = lane + 32 * t;
            nr[p][t] = (i < N && k >= 0) ? r[i] : (MT)0;
        }
    }
#pragma unroll
    for (int tk = S - 1; tk >= 0; tk--) {
        const int kbeg = min(N, 32 * (tk + 1)) - 1;
        for (int k = kbeg; k >= 32 * tk; k--) {
            MT cur[S];
            const int kn = k - kIluAhead;
            const MT dk = nd[0];
#pragma unroll
            for (int p = 0; p + 1 < kIluAhead; p++) nd[p] = nd[p + 1];
            if (kn >= 0) nd[kIluAhead - 1] = (MT)dinv[kn];
            const MT* rp = a + (size_t)(kn >= 0 ? kn : 0) * ld;
#pragma unroll
            for (int t = 0; t < S; t++) {
                cur[t] = nr[0][t];
#pragma unroll
                for (int p = 0; p + 1 < kIluAhead; p++) nr[p][t] = nr[p + 1][t];
                const int i = lane + 32 * t;
                if (i < N && kn >= 0) nr[kIluAhead - 1][t] = rp[i];
            }
            if (lane == (k & 31)) x[tk] = x[tk] * dk;
            const MT zk = __shfl_sync(0xffffffffu, x[tk], k & 31);
            if (zk == (MT)0) continue;
#pragma unroll
            for (int t = 0; t <= tk; t++) {
                const int i = lane + 32 * t;
                if (i < k) x[t] -= cur[t] * zk;
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < S; t++) {
        const int i = lane + 32 * t;
        if (i < N) b[qi[t]] = (double)x[t];
    }
    __syncwarp();
}

// One reactor per warp.  kKry: the mole reactor with GMRES and the adaptive preconditioner
// (the Krylov path) instead of the mass-fraction reactor with a dense LU.
template <bool kX, bool kKry = false>
struct BdfWarp {
    const DevMech* m;
    int N, Nnorm, lane, ld;
    double P, rtol, atol, hmaxInv;
    int maxOrder;
    double* base;            // the warp's shared-memory slice
    const uint64_t* tab;     // exp table (block shared)
    WarpAux* aux;            // lane 0 only
    double* Jsv;             // the kept Jacobian (global slot), or null: a new one at every setup
    LuPool pool;             // shared-memory staging buffers for the factorisation
    double *zn, *ewt, *acor, *y, *ftemp, *tempv, *v1, *v2, *dinv;
    int* piv;
    double* V;               // Krylov path: the Krylov basis, (kMaxl + 1) N-vectors
    double* Hs;              // Krylov path: the GMRES scalars (kGmresScalars)
    double* Zs;              // Krylov path: the preconditioned basis vectors, kMaxl N-vectors (global)

    __device__ double wrms(const double* v) const {
        double a = 0.0;
#pragma unroll 1
        for (int i = lane; i < N; i += 32) { double x = v[i] * ewt[i]; a += x * x; }
        return dsqrt(ddiv(warpSum(a), Nnorm));
    }
    __device__ double* Z(int j) const { return zn + (size_t)j * N; }
    // x^p for x >= 0 in the step-size heuristics, through the engine's exp and log
    __device__ double epow(double x, double p) const { return gbx_exp(p * gbx_log(x, tab), tab); }
    __device__ void setEwt(const double* yv) {
#pragma unroll 1
        for (int i = lane; i < N; i += 32) ewt[i] = 1.0 / (rtol * fabs(yv[i]) + atol);
        __syncwarp();
    }
    __device__ bool rhs(const double* z, double* zdot, BdfScal& S, bool forJac = false) {
        if (lane == 0) aux->nrhs++;
        return devRhs<kX, kKry>(*m, base, tab, P, z, zdot, lane, forJac);
    }
    // Linear-solver setup.  With a kept Jacobian, CVODE's policy decides when to evaluate a
    // new one (first step, 51 steps since the last, a convergence failure with a stale one
    // and a small change of gamma, or a failure of the previous step); otherwise M is formed
    // from the kept one.  convfail: 0 none, 1 retry after a failure with a stale Jacobian,
    // 2 the previous attempt at this step failed.  fresh: a new Jacobian was evaluated.
    template <typename MT, int NS>
    __device__ bool setup(MT* M, BdfScal& S, int convfail, bool& fresh) {
        if constexpr (kKry) {
            // preconditioner setup as CVODE's linear-solver interface drives it for a
            // matrix-free solver (cvLsSetup): the preconditioner's Jacobian is evaluated anew on
            // the same conditions as a kept dense one, otherwise only gamma changes; then the
            // incomplete factorisation of I - gamma Jp
            const double dgamma = fabs(ddiv(S.gamma, S.gammap) - 1.0);
            fresh = !S.haveJ || S.nst == 0 || S.nst >= S.nstlj + MSBJ || (convfail == 1 && dgamma < DGMAX_JBAD) ||
                    convfail == 2;
            if (lane == 0) aux->nsetups++;
            if (fresh) {
                if (lane == 0) { aux->nje++; aux->nrhs += 2; }
                const bool ok = devPrecJac<kX>(*m, base, tab, Jsv, ld, P, atol, y, V, lane);
                S.nstlj = S.nst;
                S.haveJ = ok;
                if (!ok) return false;
            }
            // P' = Q P Q^T in the fill-reducing order (Eigen's IncompleteLUT orders the matrix
            // before the factorisation), stored transposed: M[b][a] = P[q[a]][q[b]] =
            // delta - gamma Jp^T[q[b]][q[a]]
            const double g = S.gamma;
            const int* q = m->precOrder;
#pragma unroll 1
            for (int b = 0; b < N; b++) {
                const int jb = GB_IX(*m, q[b], N, GB_SITE_PREC_ORDER);
                const double* src = Jsv + (size_t)jb * ld;
                MT* dst = M + (size_t)b * ld;
#pragma unroll 1
                for (int a = lane; a < N; a += 32) {
                    const int ia = GB_IX(*m, q[a], N, GB_SITE_PREC_ORDER);
                    double v = -g * src[ia];
                    if (ia == jb) v += 1.0;
                    dst[a] = (MT)v;
                }
            }
            __syncwarp();
            devIlut<MT, NS>(M, N, ld, dinv, V, lane);
            return true;
        }
        if (!Jsv) {
            if (lane == 0) { aux->nje++; aux->nsetups++; aux->nrhs++; }   // nrhs: the difference in T
            fresh = true;
            return devSetup<MT, false, kX, NS>(*m, base, tab, M, ld, S.gamma, P, y, ftemp, v1, v2, tempv, piv, dinv, lane, pool);
        }
        const double dgamma = fabs(ddiv(S.gamma, S.gammap) - 1.0);
        fresh = !S.haveJ || S.nst == 0 || S.nst >= S.nstlj + MSBJ || (convfail == 1 && dgamma < DGMAX_JBAD) ||
                convfail == 2;
        if (lane == 0) aux->nsetups++;
        if (fresh) {
            if (lane == 0) { aux->nje++; aux->nrhs++; }
            const bool ok = devSetup<double, true, kX, NS>(*m, base, tab, Jsv, ld, -1.0, P, y, ftemp, v1, v2, tempv, piv, dinv,
                                                   lane, LuPool{nullptr, nullptr, 0, 0});
            S.nstlj = S.nst;
            S.haveJ = ok;
            if (!ok) return false;
        }
        return devFormLU<MT, NS>(M, Jsv, N, ld, S.gamma, piv, dinv, lane, pool);
    }

    template <typename MT, int S>
    __device__ void luSolve(const MT* a, double* b) { devLuSolve<MT, S>(a, b, N, ld, piv, dinv, lane); }

    // J v by the difference quotient (f(y + sig v) - f(y)) / sig, sig = 1 / ||v||_wrms, shrunk by
    // 1/4 (at most three tries) when f is not finite (CVODE's default Jacobian-times-vector
    // product); y and f(y) are the current Newton iterate.  work: an N-vector of scratch.
    __device__ bool jtimes(const double* v, double* Jv, double* work, BdfScal& S) {
        double sig = ddiv(1.0, wrms(v));
        bool ok = false;
        for (int it = 0; it < 3; it++) {
#pragma unroll 1
            for (int i = lane; i < N; i += 32) work[i] = y[i] + sig * v[i];
            __syncwarp();
            if (lane == 0) aux->njtv++;
            ok = rhs(work, Jv, S);
            if (ok) break;
            sig *= 0.25;
        }
        if (!ok) return false;
        const double siginv = ddiv(1.0, sig);
#pragma unroll 1
        for (int i = lane; i < N; i += 32) Jv[i] = (Jv[i] - ftemp[i]) * siginv;
        __syncwarp();
        return true;
    }
    template <typename MT, int NS>
    __device__ void precSolve(const MT* Ft, double* x) {
        if (lane == 0) aux->nps++;
        devIluSolve<MT, NS>(Ft, x, N, ld, dinv, *m, lane);
    }
    // (I - gamma J) x = b in place by right-preconditioned GMRES, as CVODE's iterative
    // linear-solver interface runs SUNDIALS' SPGMR for the reference's preconditioned solver
    // (src/numerics/CVodesIntegrator.cpp:67-80; cvLsSolve): tolerance eplifac tq[4] in the
    // weighted RMS norm (sqrt(N) times it in the scaled 2-norm), the error weights as both
    // scaling vectors, zero initial guess, at most kMaxl Krylov vectors, no restarts, modified
    // Gram-Schmidt with one reorthogonalisation when the new vector's norm collapses by the
    // factor 1000, Givens rotations for the least-squares problem (lane 0 holds it).  A
    // right-hand side already below the tolerance is the solution on the first Newton
    // iteration and zero afterwards.  Returns 0, or 1 (recoverable: not converged and, after
    // the first Newton iteration, only reduced).
    template <typename MT, int NS>
    __device__ int gmres(const MT* Ft, double* b, BdfScal& S, int mnewt) {
        const double deltar = kEplifac * S.tq[4];
        if (wrms(b) <= deltar) {
            if (mnewt > 0) {
#pragma unroll 1
                for (int i = lane; i < N; i += 32) b[i] = 0.0;
                __syncwarp();
            }
            return 0;
        }
        const double delta = deltar * dsqrt((double)N);
        double* H = Hs;                              // H[i][l] at H[i * kMaxl + l]
        double* cs = Hs + (kMaxl + 1) * kMaxl;
        double* sn = cs + kMaxl;
        double* g = sn + kMaxl;
        double* yv = g + kMaxl + 1;
        double* z = v1;
        double* Az = v2;
        double q = 0.0;
#pragma unroll 1
        for (int i = lane; i < N; i += 32) {
            const double x = ewt[i] * b[i];
            V[i] = x;
            q += x * x;
        }
        const double beta = dsqrt(warpSum(q));
#pragma unroll 1
        for (int i = lane; i < N; i += 32) V[i] = V[i] / beta;
        if (lane == 0) {
            g[0] = beta;
#pragma unroll 1
            for (int j = 1; j <= kMaxl; j++) g[j] = 0.0;
        }
        __syncwarp();
        double rho = beta;
        bool converged = false;
        int mv = 0;
        while (mv < kMaxl) {
            const int l = mv;
            const double* vl = V + (size_t)l * N;
            double* vn = V + (size_t)(l + 1) * N;
#pragma unroll 1
            for (int i = lane; i < N; i += 32) z[i] = vl[i] / ewt[i];
            __syncwarp();
            precSolve<MT, NS>(Ft, z);
            // keep z_l = P^-1 S^-1 v_l: the solution P^-1 S^-1 (V y) is sum_l y_l z_l
            double* zl = Zs + (size_t)l * N;
#pragma unroll 1
            for (int i = lane; i < N; i += 32) zl[i] = z[i];
            if (!jtimes(z, Az, b, S)) return 1;
            double pk = 0.0;
#pragma unroll 1
            for (int i = lane; i < N; i += 32) {
                const double x = ewt[i] * (z[i] - S.gamma * Az[i]);
                vn[i] = x;
                pk += x * x;
            }
            const double vk = dsqrt(warpSum(pk));
#pragma unroll 1
            for (int i2 = 0; i2 <= l; i2++) {
                const double* vi = V + (size_t)i2 * N;
                double pd = 0.0;
#pragma unroll 1
                for (int i = lane; i < N; i += 32) pd += vi[i] * vn[i];
                const double h = warpSum(pd);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) vn[i] -= h * vi[i];
                if (lane == 0) H[i2 * kMaxl + l] = h;
            }
            double pn = 0.0;
#pragma unroll 1
            for (int i = lane; i < N; i += 32) pn += vn[i] * vn[i];
            double vnorm = dsqrt(warpSum(pn));
            const double fac = 1000.0 * vk;
            if (fac + vnorm == fac) {
#pragma unroll 1
                for (int i2 = 0; i2 <= l; i2++) {
                    const double* vi = V + (size_t)i2 * N;
                    double pd = 0.0;
#pragma unroll 1
                    for (int i = lane; i < N; i += 32) pd += vi[i] * vn[i];
                    const double pr = warpSum(pd);
#pragma unroll 1
                    for (int i = lane; i < N; i += 32) vn[i] -= pr * vi[i];
                    if (lane == 0) H[i2 * kMaxl + l] += pr;
                }
                pn = 0.0;
#pragma unroll 1
                for (int i = lane; i < N; i += 32) pn += vn[i] * vn[i];
                vnorm = dsqrt(warpSum(pn));
            }
            double rl = 0.0;
            if (lane == 0) {
                H[(l + 1) * kMaxl + l] = vnorm;
#pragma unroll 1
                for (int i2 = 0; i2 < l; i2++) {
                    const double t1 = H[i2 * kMaxl + l], t2 = H[(i2 + 1) * kMaxl + l];
                    H[i2 * kMaxl + l] = cs[i2] * t1 + sn[i2] * t2;
                    H[(i2 + 1) * kMaxl + l] = -sn[i2] * t1 + cs[i2] * t2;
                }
                const double hl = H[l * kMaxl + l], hl1 = H[(l + 1) * kMaxl + l];
                const double d = hypot(hl, hl1);
                cs[l] = hl / d;
                sn[l] = hl1 / d;
                H[l * kMaxl + l] = d;
                H[(l + 1) * kMaxl + l] = 0.0;
                g[l + 1] = -sn[l] * g[l];
                g[l] = cs[l] * g[l];
                rl = fabs(g[l + 1]);
            }
            rho = __shfl_sync(0xffffffffu, rl, 0);
            mv++;
            if (rho <= delta) { converged = true; break; }
            if (vnorm == 0.0) break;
#pragma unroll 1
            for (int i = lane; i < N; i += 32) vn[i] = vn[i] / vnorm;
            __syncwarp();
        }
        if (lane == 0) {
            aux->nli += mv;
#pragma unroll 1
            for (int i2 = mv - 1; i2 >= 0; i2--) {
                double sacc = g[i2];
#pragma unroll 1
                for (int j = i2 + 1; j < mv; j++) sacc -= H[i2 * kMaxl + j] * yv[j];
                yv[i2] = sacc / H[i2 * kMaxl + i2];
            }
        }
        __syncwarp();
        // x = P^-1 S^-1 (V y) = sum_j y_j z_j: the preconditioned vectors kept during the
        // iterations (the reference's SPGMR forms V y and applies the preconditioner once more;
        // the same vector by linearity, one solve fewer)
#pragma unroll 1
        for (int i = lane; i < N; i += 32) {
            double sacc = 0.0;
#pragma unroll 1
            for (int j = 0; j < mv; j++) sacc += yv[j] * Zs[(size_t)j * N + i];
            b[i] = sacc;
        }
        __syncwarp();
        if (converged) return 0;
        if (rho < beta && mnewt == 0) return 0;
        return 1;
    }

    __device__ void predict(BdfScal& S) {
        S.tn += S.h;
#pragma unroll 1
        for (int k = 1; k <= S.q; k++)
#pragma unroll 1
            for (int j = S.q; j >= k; j--) {
                double* a = Z(j - 1);
                const double* b = Z(j);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) a[i] += b[i];
            }
        __syncwarp();
    }
    __device__ void restore(BdfScal& S, double saved_t) {
        S.tn = saved_t;
#pragma unroll 1
        for (int k = 1; k <= S.q; k++)
#pragma unroll 1
            for (int j = S.q; j >= k; j--) {
                double* a = Z(j - 1);
                const double* b = Z(j);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) a[i] -= b[i];
            }
        __syncwarp();
    }
    __device__ void rescale(BdfScal& S) {
        double f = S.eta;
#pragma unroll 1
        for (int j = 1; j <= S.q; j++) {
            double* a = Z(j);
#pragma unroll 1
            for (int i = lane; i < N; i += 32) a[i] *= f;
            f *= S.eta;
        }
        __syncwarp();
        S.h = S.hscale * S.eta;
        S.hscale = S.h;
    }
    __device__ void setCoefficients(BdfScal& S) {
        const int q = S.q;
#pragma unroll 1
        for (int i = 0; i <= QMAX; i++) S.l[i] = 0.0;
        S.l[0] = S.l[1] = 1.0;
        double xi_inv = 1.0, xistar_inv = 1.0, alpha0 = -1.0, alpha0_hat = -1.0, hsum = S.h;
        if (q > 1) {
#pragma unroll 1
            for (int j = 2; j < q; j++) {
                hsum += S.tau[j - 1];
                xi_inv = ddiv(S.h, hsum);
                alpha0 -= ddiv(1.0, j);
#pragma unroll 1
                for (int i = j; i >= 1; i--) S.l[i] += S.l[i - 1] * xi_inv;
            }
            alpha0 -= ddiv(1.0, q);
            xistar_inv = -S.l[1] - alpha0;
            hsum += S.tau[q - 1];
            xi_inv = ddiv(S.h, hsum);
            alpha0_hat = -S.l[1] - xi_inv;
#pragma unroll 1
            for (int i = q; i >= 1; i--) S.l[i] += S.l[i - 1] * xistar_inv;
        }
        const double lq = S.l[q];
        double A1 = 1.0 - alpha0_hat + alpha0;
        double A2 = 1.0 + q * A1;
        S.tq[2] = fabs(ddiv(A1, alpha0 * A2));
        S.tq[5] = fabs(ddiv(A2 * xistar_inv, lq * xi_inv));
        if (S.qwait == 1) {
            if (q > 1) {
                double C = ddiv(xistar_inv, lq);
                double A3 = alpha0 + ddiv(1.0, q);
                double A4 = alpha0_hat + xi_inv;
                double Cpinv = ddiv(1.0 - A4 + A3, A3);
                S.tq[1] = fabs(C * Cpinv);
            } else {
                S.tq[1] = 1.0;
            }
            double hs = hsum + S.tau[q];
            double xi2 = ddiv(S.h, hs);
            double A5 = alpha0 - ddiv(1.0, q + 1);
            double A6 = alpha0_hat - xi2;
            double Cppinv = ddiv(1.0 - A6 + A5, A2);
            S.tq[3] = fabs(ddiv(Cppinv, xi2 * (q + 2) * A5));
        }
        S.tq[4] = ddiv(NLSCOEF, S.tq[2]);
    }

    template <typename MT, int NS>
    __device__ int newton(MT* M, BdfScal& S, bool callSetup, bool prevFailed) {
        const double rl1 = ddiv(1.0, S.l[1]);
        bool jcur = false;
        int convfail = prevFailed ? 2 : 0;
        for (;;) {
#pragma unroll 1
            for (int i = lane; i < N; i += 32) { y[i] = zn[i]; acor[i] = 0.0; }
            __syncwarp();
            if (!rhs(y, ftemp, S, callSetup)) return NLS_RECOVER;
            if (callSetup) {
                callSetup = false;
                bool fresh = true;
                bool ok = setup<MT, NS>(M, S, convfail, fresh);
                S.gammap = S.gamma;
                S.gamrat = 1.0;
                S.crate = 1.0;
                S.nstlp = S.nst;
                S.haveLU = ok;
                jcur = fresh;
                if (!ok) return NLS_RECOVER;
            }
            double delp = 0.0, del = 0.0;
            int mm = 0;
            bool retry = false;
            const double* z1 = Z(1);
            for (;;) {
                if (lane == 0) aux->nni++;
#pragma unroll 1
                for (int i = lane; i < N; i += 32) tempv[i] = S.gamma * ftemp[i] - (rl1 * z1[i] + acor[i]);
                __syncwarp();
                if constexpr (kKry) {
                    // an iterative solve uses the current gamma: no correction for its change
                    if (gmres<MT, NS>(M, tempv, S, mm) != 0) { retry = !jcur; break; }
                } else {
                    luSolve<MT, NS>(M, tempv);
                    if (S.gamrat != 1.0) {
                        double f = ddiv(2.0, 1.0 + S.gamrat);
#pragma unroll 1
                        for (int i = lane; i < N; i += 32) tempv[i] *= f;
                        __syncwarp();
                    }
                }
                del = wrms(tempv);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) { acor[i] += tempv[i]; y[i] = zn[i] + acor[i]; }
                __syncwarp();
                if (!isfinite(del)) { retry = !jcur; break; }
                if (mm > 0) S.crate = fmax(CRDOWN * S.crate, ddiv(del, delp));
                double dcon = ddiv(del * fmin(1.0, S.crate), S.tq[4]);
                if (dcon <= 1.0) {
                    S.acnrm = (mm == 0) ? del : wrms(acor);
                    return NLS_OK;
                }
                mm++;
                if (mm == MAXCOR || (mm >= 2 && del > RDIV * delp)) { retry = !jcur; break; }
                delp = del;
                if (!rhs(y, ftemp, S)) { retry = !jcur; break; }
            }
            if (retry && S.haveLU) { callSetup = true; convfail = 1; continue; }
            return NLS_RECOVER;
        }
    }

    // Nordsieck order change (see the CPU restatement for the polynomial construction)
    // w(x) = x^2 prod_{j=1}^{nf}(x + xi_j): coefficients w[2..nf+2]
    __device__ void orderPoly(const BdfScal& S, int nf, double (&w)[QMAX + 2]) const {
#pragma unroll 1
        for (int i = 0; i < QMAX + 2; i++) w[i] = 0.0;
        w[2] = 1.0;
        double hsum = 0.0;
#pragma unroll 1
        for (int j = 1; j <= nf; j++) {
            hsum += S.tau[j];
            const double xi = ddiv(hsum, S.hscale);
#pragma unroll 1
            for (int i = j + 2; i >= 2; i--) w[i] = w[i] * xi + w[i - 1];
        }
    }
    __device__ void decreaseOrder(BdfScal& S) {
        double w[QMAX + 2];
        orderPoly(S, S.q - 2, w);
        const double* zq = Z(S.q);
#pragma unroll 1
        for (int j = 2; j < S.q; j++) {
            double* a = Z(j);
#pragma unroll 1
            for (int i = lane; i < N; i += 32) a[i] -= w[j] * zq[i];
        }
        __syncwarp();
        double* a = Z(S.q);
#pragma unroll 1
        for (int i = lane; i < N; i += 32) a[i] = 0.0;
        __syncwarp();
    }
    __device__ void increaseOrder(BdfScal& S, double lq_prev) {
        double w[QMAX + 2];
        orderPoly(S, S.q - 1, w);
        const double c = ddiv(lq_prev, S.q + 1);
        const double* sv = Z(QMAX);
#pragma unroll 1
        for (int i = lane; i < N; i += 32) tempv[i] = c * sv[i];
        __syncwarp();
#pragma unroll 1
        for (int j = 2; j <= S.q; j++) {
            double* a = Z(j);
#pragma unroll 1
            for (int i = lane; i < N; i += 32) a[i] += w[j] * tempv[i];
        }
        double* top = Z(S.q + 1);
#pragma unroll 1
        for (int i = lane; i < N; i += 32) top[i] = tempv[i];
        __syncwarp();
    }

    // lane 0 only
    __device__ void recordSample(double t, double v) {
        if (lane != 0) return;
        WarpAux& A = *aux;
        if (A.flags & F_AWAIT) { A.nx_t = t; A.nx_v = v; A.flags = (A.flags & ~F_AWAIT) | F_HASRIGHT; }
        if (A.nsamp == 0 || v > A.bs_v) {
            A.pv_t = A.ls_t; A.pv_v = A.ls_v;
            A.flags = (A.nsamp > 0) ? (A.flags | F_HASPREV) : (A.flags & ~F_HASPREV);
            A.bs_t = t; A.bs_v = v;
            A.flags = (A.flags | F_AWAIT) & ~F_HASRIGHT;
        }
        A.ls_t = t; A.ls_v = v;
        A.nsamp++;
    }
    __device__ double ignitionTime() const {
        const WarpAux& A = *aux;
        if (!(A.flags & F_HASPREV) || !(A.flags & F_HASRIGHT)) return A.bs_t;
        double t0 = A.pv_t, t1 = A.bs_t, t2 = A.nx_t;
        double s0 = ddiv(A.bs_v - A.pv_v, t1 - t0), s1 = ddiv(A.nx_v - A.bs_v, t2 - t1);
        double curv = ddiv(s1 - s0, t2 - t0);
        if (!(curv < 0)) return t1;
        double tv = 0.5 * (t0 + t1) - ddiv(s0, 2.0 * curv);
        return fmin(fmax(tv, t0), t2);
    }

    __device__ double initialStep(BdfScal& S, double tout) {
        const double tdist = fabs(tout - S.tn);
        const double tround = UROUND * fmax(fabs(S.tn), fabs(tout));
        const double hlb = 100.0 * tround;
        const double* z0 = Z(0);
        const double* z1 = Z(1);
        double hi = 0.0;
#pragma unroll 1
        for (int i = lane; i < N; i += 32) hi = fmax(hi, fabs(z1[i]) / (0.1 * fabs(z0[i]) + atol));
        double hub_inv = warpMax(hi);
        double hub = 0.1 * tdist;
        if (hub * hub_inv > 1.0) hub = ddiv(1.0, hub_inv);
        if (hub < hlb) return dsqrt(hlb * hub);
        double hg = dsqrt(hlb * hub);
        double hnew = hg;
        for (int count = 1; count <= 4; count++) {
#pragma unroll 1
            for (int i = lane; i < N; i += 32) y[i] = z0[i] + hg * z1[i];
            __syncwarp();
            if (!rhs(y, tempv, S)) { hg *= 0.2; continue; }
#pragma unroll 1
            for (int i = lane; i < N; i += 32) tempv[i] = (tempv[i] - z1[i]) / hg;
            __syncwarp();
            double yddnrm = wrms(tempv);
            hnew = (yddnrm * hub * hub > 2.0) ? dsqrt(ddiv(2.0, yddnrm)) : dsqrt(hg * hub);
            if (count == 4) break;
            double hrat = ddiv(hnew, hg);
            if (hrat > 0.5 && hrat < 2.0) break;
            if (count > 1 && hrat > 2.0) { hnew = hg; break; }
            hg = hnew;
        }
        double h0 = 0.5 * hnew;
        h0 = fmin(fmax(h0, hlb), hub);
        if (hmaxInv > 0) h0 = fmin(h0, ddiv(1.0, hmaxInv));
        return h0;
    }

    __device__ void prepareNext(BdfScal& S, double dsm) {
        if (S.etamax == 1.0) {
            S.qwait = max(S.qwait, 2);
            S.qprime = S.q;
            S.hprime = S.h;
            S.eta = 1.0;
            S.etamax = (S.nst <= SMALL_NST) ? ETA_MAX_EARLY : ETA_MAX_GENERAL;
            return;
        }
        const int L = S.L;
        double etaq = ddiv(1.0, epow(BIAS2 * dsm, ddiv(1.0, L)) + ADDON);
        if (S.qwait != 0) {
            S.eta = etaq;
            S.qprime = S.q;
        } else {
            S.qwait = 2;
            double etaqm1 = 0.0, etaqp1 = 0.0;
            if (S.q > 1) {
                double ddn = wrms(Z(S.q)) * S.tq[1];
                etaqm1 = ddiv(1.0, epow(BIAS1 * ddn, ddiv(1.0, S.q)) + ADDON);
            }
            if (S.q != maxOrder && S.saved_tq5 != 0.0) {
                const double hr = ddiv(S.h, S.tau[2]);
                double hp = hr;
#pragma unroll 1
                for (int i = 2; i <= L; i++) hp *= hr;
                double cquot = ddiv(S.tq[5], S.saved_tq5) * hp;
                const double* sv = Z(QMAX);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) tempv[i] = acor[i] - cquot * sv[i];
                __syncwarp();
                double dup = wrms(tempv) * S.tq[3];
                etaqp1 = ddiv(1.0, epow(BIAS3 * dup, ddiv(1.0, L + 1)) + ADDON);
            }
            double etam = fmax(etaqm1, fmax(etaq, etaqp1));
            if (etam < ETA_FIX_MAX) {
                S.eta = 1.0;
                S.qprime = S.q;
            } else if (etam == etaq) {
                S.eta = etaq;
                S.qprime = S.q;
            } else if (etam == etaqm1) {
                S.eta = etaqm1;
                S.qprime = S.q - 1;
            } else {
                S.eta = etaqp1;
                S.qprime = S.q + 1;
                double* sv = Z(QMAX);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) sv[i] = acor[i];
                __syncwarp();
            }
        }
        if (S.eta < ETA_FIX_MAX) {
            S.eta = 1.0;
            S.qprime = S.q;
        } else {
            S.eta = fmin(S.eta, S.etamax);
            if (hmaxInv > 0) S.eta /= fmax(1.0, fabs(S.h) * S.eta * hmaxInv);
        }
        S.hprime = S.h * S.eta;
        S.etamax = (S.nst <= SMALL_NST) ? ETA_MAX_EARLY : ETA_MAX_GENERAL;
    }

    // one internal step; returns a status code
    template <typename MT, int NS>
    __device__ int step(MT* M, BdfScal& S) {
        const double saved_t = S.tn;
        int ncf = 0, nef = 0;
        bool prevConvFail = false;
        if (S.nst > 0) {
            if (S.qprime != S.q) {
                if (S.qprime == S.q + 1) increaseOrder(S, S.l[S.q]);
                else decreaseOrder(S);
                S.q = S.qprime;
                S.L = S.q + 1;
                S.qwait = S.L;
            }
            if (S.hprime != S.h) {
                S.eta = ddiv(S.hprime, S.h);
                rescale(S);
            }
        }
        setEwt(Z(0));
        for (;;) {
            predict(S);
            setCoefficients(S);
            S.gamma = ddiv(S.h, S.l[1]);
            if (S.nst == 0) S.gammap = S.gamma;
            S.gamrat = (S.nst > 0) ? ddiv(S.gamma, S.gammap) : 1.0;
            bool callSetup = (S.nst == 0) || prevConvFail || (S.nst >= S.nstlp + MSBP) ||
                             (fabs(S.gamrat - 1.0) > DGMAX) || !S.haveLU;
            int nls = newton<MT, NS>(M, S, callSetup, prevConvFail);
            if (nls != NLS_OK) {
                if (lane == 0) aux->ncfn++;
                ncf++;
                restore(S, saved_t);
                if (ncf == MXNCF) return ST_CONV_FAIL;
                S.eta = ETA_CF;
                rescale(S);
                prevConvFail = true;
                S.etamax = 1.0;
                if (fabs(S.h) < 10.0 * UROUND * fmax(1.0, fabs(S.tn))) return ST_H_TOO_SMALL;
                continue;
            }
            double dsm = S.acnrm * S.tq[2];
            if (dsm > 1.0) {
                if (lane == 0) aux->netf++;
                nef++;
                restore(S, saved_t);
                if (nef == MXNEF) return ST_ERR_FAIL;
                S.etamax = 1.0;
                if (nef <= MXNEF1) {
                    S.eta = ddiv(1.0, epow(BIAS2 * dsm, ddiv(1.0, S.L)) + ADDON);
                    S.eta = fmax(ETA_MIN_EF, S.eta);
                    if (nef >= SMALL_NEF) S.eta = fmin(S.eta, ETA_MAX_EF);
                    rescale(S);
                } else {
                    S.eta = ETA_MIN_EF;
                    S.h *= S.eta;
                    S.hscale = S.h;
                    S.qwait = 10;
                    if (S.q > 1) { S.q = 1; S.L = 2; }
                    if (!rhs(Z(0), tempv, S)) return ST_NONFINITE;
                    double* z1 = Z(1);
#pragma unroll 1
                    for (int i = lane; i < N; i += 32) z1[i] = S.h * tempv[i];
                    for (int j = 2; j <= QMAX; j++) {
                        double* a = Z(j);
#pragma unroll 1
                        for (int i = lane; i < N; i += 32) a[i] = 0.0;
                    }
                    __syncwarp();
                }
                if (fabs(S.h) < 10.0 * UROUND * fmax(1.0, fabs(S.tn))) return ST_H_TOO_SMALL;
                continue;
            }
            // accepted
            S.nst++;
#pragma unroll
            for (int i = QMAX; i >= 2; i--)
                if (i <= S.q) S.tau[i] = S.tau[i - 1];
            if (S.q == 1 && S.nst > 1) S.tau[2] = S.tau[1];
            S.tau[1] = S.h;
#pragma unroll
            for (int j = 0; j <= QMAX; j++) {
                if (j <= S.q) {
                    double* a = Z(j);
                    const double lj = S.l[j];
#pragma unroll 1
                    for (int i = lane; i < N; i += 32) a[i] += lj * acor[i];
                }
            }
            __syncwarp();
            S.qwait--;
            if (S.qwait == 1 && S.q != QMAX) {
                double* sv = Z(QMAX);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) sv[i] = acor[i];
                __syncwarp();
                S.saved_tq5 = S.tq[5];
            }
            recordSample(S.tn, ddiv(zn[N], S.h));
            prepareNext(S, dsm);
            return ST_OK;
        }
    }
};

template <typename MT, int NS, bool kX, bool kKry>
__global__ void __launch_bounds__(kBdfMaxThreads, 1) k_bdf(BdfParams p) {
    extern __shared__ __align__(128) double smem[];
    __shared__ uint64_t s_tab[kGbxTableWords];
    __shared__ DevMech s_mech;
    __shared__ int s_luflags[kMaxLuSlots];
    if (threadIdx.x < kMaxLuSlots) s_luflags[threadIdx.x] = 0;
    loadMech(p.m, s_mech, (char*)smem, p.mechSmem);
    gbx_load_table(s_tab);   // (its barrier also completes the mechanism copy)
    const DevMech& m = s_mech;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    double* base = smem + p.mechSmem / 8 + (size_t)warp * p.warpDoubles;
    BdfWarp<kX, kKry> W;
    W.m = &m;
    W.N = m.N;
    // error-norm divisor: the reference's state has the mass as well for the mass-fraction
    // reactor (K + 2 components), T and the K amounts for the mole reactor
    W.Nnorm = kKry ? m.N : m.N + 1;
    W.lane = lane;
    W.ld = p.ld;
    W.rtol = p.rtol;
    W.atol = p.atol;
    W.hmaxInv = p.hmaxInv;
    W.maxOrder = p.maxOrder;
    const int N = m.N;
    const bool ext = p.JSbuf != nullptr;
    const int kinD = kStateSlots + KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT, ext);
    if (lane == 0)
        reinterpret_cast<double**>(base + kExtSlot)[0] =
            ext ? (double*)((char*)p.JSbuf + (size_t)(blockIdx.x * (blockDim.x >> 5) + warp) * p.JSstride) : nullptr;
    __syncwarp();
    W.base = base;
    W.tab = s_tab;
    double* q = base + kinD;
    W.aux = (WarpAux*)q; q += kAuxDoubles;
    // with global matrices the Nordsieck array lives in the warp's global slot too, after the
    // Jacobian scratch (more shared memory left as L1)
    if (ext) W.zn = extScratch(base) + 2 * m.R;
    else { W.zn = q; q += (QMAX + 1) * N; }
    W.ewt = q; q += N;
    W.acor = q; q += N;
    W.y = q; q += N;
    W.ftemp = q; q += N;
    W.tempv = q; q += N;
    W.v1 = q; q += N;
    W.v2 = q; q += N;
    W.dinv = q; q += N;
    W.piv = (int*)q; q += (N + 1) / 2;
    if (kKry) {
        W.V = q; q += (kMaxl + 1) * N;
        W.Hs = q; q += kGmresScalars;
        W.Zs = p.kzBuf + (size_t)(blockIdx.x * (blockDim.x >> 5) + warp) * kMaxl * N;
    } else {
        W.V = W.Hs = W.Zs = nullptr;
    }
    MT* M = p.Mbuf ? (MT*)((char*)p.Mbuf + (size_t)(blockIdx.x * (blockDim.x >> 5) + warp) * p.Mstride)
                   : (MT*)q;
    W.Jsv = p.Jbuf ? (double*)((char*)p.Jbuf + (size_t)(blockIdx.x * (blockDim.x >> 5) + warp) * p.Jstride) : nullptr;
    // staging buffers follow the warps' slices
    W.pool.buf = (char*)(smem + p.mechSmem / 8 + (size_t)(blockDim.x >> 5) * p.warpDoubles);
    W.pool.flags = s_luflags;
    W.pool.nslots = p.Mbuf ? p.luSlots : 0;
    W.pool.slotBytes = p.luSlotBytes;

    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(p.counter, 1);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= p.n) break;
        const int r = p.order ? GB_IX(m, p.order[idx], p.n, GB_SITE_QUEUE) : idx;
        double* rec = p.rec + (size_t)r * p.recStride;
        const double* rs = rec + (QMAX + 1) * N;
        long long* stt = p.stats + (size_t)r * 8;
        long long* kst = kKry ? p.kstats + (size_t)r * 3 : nullptr;
        W.P = p.P[r];
        BdfScal S;
        const bool fresh = !(((int)rs[R_FLAGS]) & F_INIT);
        if (fresh) {
            // zn[0] = state, zn[1] = h*f(state)
            double* z0 = W.zn;
            const double T0 = p.T[r];
            if (lane == 0) z0[0] = T0;
            if (kKry) {
                // amounts in an initial volume of 1 m^3: n_k = rho Y_k / W_k
                double py = 0.0;
#pragma unroll 1
                for (int k = lane; k < m.K; k += 32) py += p.Y[(size_t)k * p.n + r] * m.rmw[k];
                const double rho = (W.P / (m.Rgas * T0)) / warpSum(py);
#pragma unroll 1
                for (int k = lane; k < m.K; k += 32) z0[1 + k] = rho * p.Y[(size_t)k * p.n + r] * m.rmw[k];
            } else {
#pragma unroll 1
                for (int k = lane; k < m.K; k += 32) z0[1 + k] = p.Y[(size_t)k * p.n + r];
            }
#pragma unroll 1
            for (int j = 1; j <= QMAX; j++)
#pragma unroll 1
                for (int i = lane; i < N; i += 32) W.zn[(size_t)j * N + i] = 0.0;
            __syncwarp();
            S.tn = p.t0;
            if (lane == 0) {
                WarpAux& A = *W.aux;
                A.nrhs = A.nni = A.nsetups = A.nje = A.netf = A.ncfn = 0;
                A.nli = A.nps = A.njtv = 0;
                A.flags = F_INIT; A.nsamp = 0;
                A.ls_t = A.ls_v = A.pv_t = A.pv_v = A.bs_t = A.bs_v = A.nx_t = A.nx_v = 0.0;
            }
            S.nst = 0; S.nstlp = 0; S.nstlj = 0;
            S.haveLU = false; S.haveJ = false;
#pragma unroll 1
            for (int i = 0; i < QMAX + 2; i++) S.tau[i] = 0.0;
#pragma unroll 1
            for (int i = 0; i < 6; i++) S.tq[i] = 0.0;
#pragma unroll 1
            for (int i = 0; i <= QMAX; i++) S.l[i] = 0.0;
            S.saved_tq5 = 0.0; S.crate = 1.0; S.gammap = 0.0; S.gamrat = 1.0; S.acnrm = 0.0;
            W.setEwt(z0);
            int status = ST_OK;
            if (!W.rhs(z0, W.Z(1), S)) status = ST_NONFINITE;
            if (status == ST_OK) {
                double h0 = W.initialStep(S, p.tout);
                double* z1 = W.Z(1);
#pragma unroll 1
                for (int i = lane; i < N; i += 32) z1[i] *= h0;
                __syncwarp();
                S.h = S.hscale = S.hprime = h0;
                S.eta = 1.0;
                S.q = S.qprime = 1; S.L = 2; S.qwait = 2; S.etamax = ETA_MAX_FIRST;
                S.tau[1] = h0;
                W.recordSample(S.tn, ddiv(z1[0], h0));
            } else {
                S.h = S.hscale = S.hprime = 0.0;
                S.q = S.qprime = 1; S.L = 2; S.qwait = 2; S.etamax = ETA_MAX_FIRST; S.eta = 1.0;
            }
            S.status0 = status;
        } else {
#pragma unroll 1
            for (int i = lane; i < (QMAX + 1) * N; i += 32) W.zn[i] = rec[i];
            __syncwarp();
            S.tn = rs[R_TN]; S.h = rs[R_H]; S.hscale = rs[R_HSCALE]; S.hprime = rs[R_HPRIME];
            S.eta = rs[R_ETA]; S.etamax = rs[R_ETAMAX];
#pragma unroll 1
            for (int i = 0; i < QMAX + 2; i++) S.tau[i] = rs[R_TAU + i];
#pragma unroll 1
            for (int i = 0; i < 6; i++) S.tq[i] = rs[R_TQ + i];
#pragma unroll 1
            for (int i = 0; i <= QMAX; i++) S.l[i] = rs[R_L + i];
            S.gammap = rs[R_GAMMAP]; S.crate = rs[R_CRATE]; S.saved_tq5 = rs[R_SAVEDTQ5];
            if (lane == 0) {
                WarpAux& A = *W.aux;
                A.ls_t = rs[R_IGN + 0]; A.ls_v = rs[R_IGN + 1]; A.pv_t = rs[R_IGN + 2]; A.pv_v = rs[R_IGN + 3];
                A.bs_t = rs[R_IGN + 4]; A.bs_v = rs[R_IGN + 5]; A.nx_t = rs[R_IGN + 6]; A.nx_v = rs[R_IGN + 7];
                A.nsamp = (int)rs[R_NSAMP];
                A.flags = (int)rs[R_FLAGS];
                A.nrhs = stt[1]; A.nni = stt[2]; A.nsetups = stt[3]; A.nje = stt[4]; A.netf = stt[5]; A.ncfn = stt[6];
                if (kKry) { A.nli = kst[0]; A.nps = kst[1]; A.njtv = kst[2]; }
            }
            S.q = (int)rs[R_Q]; S.qprime = (int)rs[R_QPRIME]; S.qwait = (int)rs[R_QWAIT];
            S.nst = (int)rs[R_NST]; S.nstlp = (int)rs[R_NSTLP];
            S.L = S.q + 1;
            S.haveLU = false;   // the factorisation and the Jacobian are not kept between advance calls
            S.haveJ = false;
            S.nstlj = S.nst;
            S.gamrat = 1.0; S.acnrm = 0.0;
            S.status0 = (int)rs[R_STATUS];
        }
        int status = S.status0;
        long long count = 0;
        while (status == ST_OK && S.tn < p.tout) {
            if (count >= p.maxSteps) { status = ST_MAX_STEPS; break; }
            status = W.template step<MT, NS>(M, S);
            count++;
            if (p.oneStep) break;
        }
        // output: interpolate to tout (or the last state on failure; the state at the new
        // internal time after one step)
        const double sfac = (status == ST_OK && S.h != 0.0 && !p.oneStep) ? ddiv(p.tout - S.tn, S.h) : 0.0;
        if (kKry) {
            // the state at tout, then mass fractions from the amounts: Y_k = n_k W_k / mass
            double pm = 0.0;
#pragma unroll 1
            for (int i = lane; i < N; i += 32) {
                double v = W.zn[(size_t)S.q * N + i];
#pragma unroll 1
                for (int j = S.q - 1; j >= 0; j--) v = W.zn[(size_t)j * N + i] + sfac * v;
                if (status != ST_OK) v = W.zn[i];
                W.tempv[i] = v;
                if (i > 0) pm += v * m.mw[i - 1];
            }
            const double rmass = 1.0 / warpSum(pm);
#pragma unroll 1
            for (int i = lane; i < N; i += 32) {
                const double v = W.tempv[i];
                if (i == 0) p.T[r] = v;
                else p.Y[(size_t)(i - 1) * p.n + r] = v * m.mw[i - 1] * rmass;
            }
            __syncwarp();
        } else {
#pragma unroll 1
            for (int i = lane; i < N; i += 32) {
                double v = W.zn[(size_t)S.q * N + i];
#pragma unroll 1
                for (int j = S.q - 1; j >= 0; j--) v = W.zn[(size_t)j * N + i] + sfac * v;
                if (status != ST_OK) v = W.zn[i];
                if (i == 0) p.T[r] = v;
                else p.Y[(size_t)(i - 1) * p.n + r] = v;
            }
        }
        // save the integrator record
#pragma unroll 1
        for (int i = lane; i < (QMAX + 1) * N; i += 32) rec[i] = W.zn[i];
        if (lane == 0) {
            double* o = rec + (QMAX + 1) * N;
            o[R_TN] = S.tn; o[R_H] = S.h; o[R_HSCALE] = S.hscale; o[R_HPRIME] = S.hprime;
            o[R_ETA] = S.eta; o[R_ETAMAX] = S.etamax;
#pragma unroll 1
            for (int i = 0; i < QMAX + 2; i++) o[R_TAU + i] = S.tau[i];
#pragma unroll 1
            for (int i = 0; i < 6; i++) o[R_TQ + i] = S.tq[i];
#pragma unroll 1
            for (int i = 0; i <= QMAX; i++) o[R_L + i] = S.l[i];
            o[R_GAMMAP] = S.gammap; o[R_CRATE] = S.crate; o[R_SAVEDTQ5] = S.saved_tq5;
            const WarpAux& A = *W.aux;
            o[R_IGN + 0] = A.ls_t; o[R_IGN + 1] = A.ls_v; o[R_IGN + 2] = A.pv_t; o[R_IGN + 3] = A.pv_v;
            o[R_IGN + 4] = A.bs_t; o[R_IGN + 5] = A.bs_v; o[R_IGN + 6] = A.nx_t; o[R_IGN + 7] = A.nx_v;
            o[R_Q] = S.q; o[R_QPRIME] = S.qprime; o[R_QWAIT] = S.qwait; o[R_NST] = S.nst;
            o[R_NSTLP] = S.nstlp; o[R_NSAMP] = A.nsamp; o[R_FLAGS] = A.flags | F_INIT; o[R_STATUS] = status;
            stt[0] = S.nst; stt[1] = A.nrhs; stt[2] = A.nni; stt[3] = A.nsetups; stt[4] = A.nje;
            stt[5] = A.netf; stt[6] = A.ncfn; stt[7] = S.q;
            if (kKry) { kst[0] = A.nli; kst[1] = A.nps; kst[2] = A.njtv; }
            p.status[r] = status;
            p.tign[r] = W.ignitionTime();
            if (p.tnow) p.tnow[r] = S.tn;
        }
        __syncwarp();
    }
}

// =============================================================================
// Batched reactor right-hand side: one warp per state (grid-stride over states)
// =============================================================================
template <bool kX>
__global__ void __launch_bounds__(256, 1) k_reactor_rhs(RhsParams p) {
    extern __shared__ __align__(128) double smem[];
    __shared__ uint64_t s_tab[kGbxTableWords];
    __shared__ DevMech s_mech;
    loadMech(p.m, s_mech, (char*)smem, 0);
    gbx_load_table(s_tab);
    const DevMech& m = s_mech;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    double* base = smem + (size_t)warp * p.warpDoubles;
    double* z = base + kStateSlots + KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT);
    double* zd = z + m.N;
    if (lane == 0) reinterpret_cast<double**>(base + kExtSlot)[0] = nullptr;
    __syncwarp();
    for (int r = blockIdx.x * wpb + warp; r < p.n; r += gridDim.x * wpb) {
        if (lane == 0) z[0] = p.T[r];
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) z[1 + k] = p.Y[(size_t)k * p.n + r];
        __syncwarp();
        devRhs<kX>(m, base, s_tab, p.P[r], z, zd, lane, false);
        if (lane == 0) p.dTdt[r] = zd[0];
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) p.dYdt[(size_t)k * p.n + r] = zd[1 + k];
        __syncwarp();
    }
}

template <bool kX>
cudaError_t launchReactorRhsT(const RhsParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    size_t smem = (size_t)p.warpDoubles * 8 * warpsPerBlock;
    cudaError_t e = cudaFuncSetAttribute(k_reactor_rhs<kX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_reactor_rhs<kX><<<blocks, 32 * warpsPerBlock, smem, stream>>>(p);
    return cudaGetLastError();
}

template <typename MT, int NS, bool kX, bool kKry = false>
cudaError_t launchBdfT(const BdfParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    size_t smem = (size_t)p.mechSmem + (size_t)p.warpDoubles * 8 * warpsPerBlock +
                  (size_t)(p.Mbuf ? p.luSlots : 0) * p.luSlotBytes;
    cudaError_t e = cudaFuncSetAttribute(k_bdf<MT, NS, kX, kKry>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // the rest of the SM's 256 KB of L1/shared storage is L1: ask for the smallest carveout
    // that holds the block (static tables and the per-block reservation included)
    const int pct = (int)std::min<size_t>(100, ((smem + 4096 + 1024) * 100 + 233471) / 233472);
    e = cudaFuncSetAttribute(k_bdf<MT, NS, kX, kKry>, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    k_bdf<MT, NS, kX, kKry><<<blocks, 32 * warpsPerBlock, smem, stream>>>(p);
    return cudaGetLastError();
}

template <bool kX>
cudaError_t launchRatesT(const RatesParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    size_t smem = (size_t)p.mechSmem + (size_t)p.tileDoubles * 8 + (size_t)p.warpDoubles * 8 * warpsPerBlock;
    cudaError_t e = cudaFuncSetAttribute(k_rates<kX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_rates<kX><<<blocks, 32 * warpsPerBlock, smem, stream>>>(p);
    return cudaGetLastError();
}

template <typename MT, int NS, bool kX, bool kKry = false>
int bdfBlocksPerSmT(int warpsPerBlock, size_t smem) {
    int nb = 0;
    if (cudaFuncSetAttribute(k_bdf<MT, NS, kX, kKry>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bdf<MT, NS, kX, kKry>, 32 * warpsPerBlock, smem) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}

#ifdef GB_KERNELS_EXTRA
// Mechanisms with the less common rate forms (DevMech::NX > 0): their own instantiations
// (kX), compiled in a module of their own (kernels_x.cu) so that the common instantiations
// keep their register allocation; the integrator uses the widest register slots (NS = 8,
// any N).
cudaError_t launchReactorRhsX(const RhsParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    return launchReactorRhsT<true>(p, blocks, warpsPerBlock, stream);
}
cudaError_t launchRatesX(const RatesParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    return launchRatesT<true>(p, blocks, warpsPerBlock, stream);
}
cudaError_t launchBdfX(const BdfParams& p, int blocks, int warpsPerBlock, bool fp32, cudaStream_t stream) {
    return fp32 ? launchBdfT<float, 8, true>(p, blocks, warpsPerBlock, stream)
                : launchBdfT<double, 8, true>(p, blocks, warpsPerBlock, stream);
}
int bdfBlocksPerSmX(bool fp32, int warpsPerBlock, size_t smem) {
    return fp32 ? bdfBlocksPerSmT<float, 8, true>(warpsPerBlock, smem)
                : bdfBlocksPerSmT<double, 8, true>(warpsPerBlock, smem);
}
#elif defined(GB_KERNELS_KRYLOV)
// The Krylov path's instantiations (krylov.cu with FP64 preconditioner factors, krylov32.cu
// with FP32 ones; everything else FP64): the factors in the matrix slot; mechanisms with the
// less common rate forms use the widest register slots.
#if GB_KERNELS_KRYLOV == 32
#define GB_KMT float
#define GB_KLAUNCH launchBdfKrylov32
#define GB_KBLOCKS bdfBlocksPerSmKrylov32
#else
#define GB_KMT double
#define GB_KLAUNCH launchBdfKrylov64
#define GB_KBLOCKS bdfBlocksPerSmKrylov64
#endif
cudaError_t GB_KLAUNCH(const BdfParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    if (p.m.NX) return launchBdfT<GB_KMT, 8, true, true>(p, blocks, warpsPerBlock, stream);
    const int N = p.m.N;
    if (N <= 64) return launchBdfT<GB_KMT, 2, false, true>(p, blocks, warpsPerBlock, stream);
    if (N <= 128) return launchBdfT<GB_KMT, 4, false, true>(p, blocks, warpsPerBlock, stream);
    return launchBdfT<GB_KMT, 8, false, true>(p, blocks, warpsPerBlock, stream);
}
int GB_KBLOCKS(int N, bool extra, int warpsPerBlock, size_t smem) {
    if (extra) return bdfBlocksPerSmT<GB_KMT, 8, true, true>(warpsPerBlock, smem);
    if (N <= 64) return bdfBlocksPerSmT<GB_KMT, 2, false, true>(warpsPerBlock, smem);
    if (N <= 128) return bdfBlocksPerSmT<GB_KMT, 4, false, true>(warpsPerBlock, smem);
    return bdfBlocksPerSmT<GB_KMT, 8, false, true>(warpsPerBlock, smem);
}
#undef GB_KMT
#undef GB_KLAUNCH
#undef GB_KBLOCKS
#if GB_KERNELS_KRYLOV != 32

// Batched incomplete factorisation: one warp per matrix (grid-stride), each stored transposed
// in a[m][N][ld] and factored in place, its reciprocal pivots to dinv[m][N]; rn[m][N] scratch.
template <int S>
__global__ void __launch_bounds__(256) k_ilut(int n, int N, int ld, double* a, double* dinv, double* rn) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int r = blockIdx.x * wpb + (threadIdx.x >> 5); r < n; r += gridDim.x * wpb)
        devIlut<double, S>(a + (size_t)r * N * ld, N, ld, dinv + (size_t)r * N, rn + (size_t)r * N, lane);
}
cudaError_t launchIlut(int n, int N, int ld, double* a, double* dinv, double* rn, cudaStream_t stream) {
    const int blocks = std::max(1, std::min((n + 7) / 8, 4096));
    if (N <= 64) k_ilut<2><<<blocks, 256, 0, stream>>>(n, N, ld, a, dinv, rn);
    else if (N <= 128) k_ilut<4><<<blocks, 256, 0, stream>>>(n, N, ld, a, dinv, rn);
    else if (N <= 256) k_ilut<8><<<blocks, 256, 0, stream>>>(n, N, ld, a, dinv, rn);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}
#endif  // GB_KERNELS_KRYLOV != 32
#else
int rhsWarpDoubles(const DevMech& m) {
    const int tot = kStateSlots + KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT) + 2 * m.N;
    return (tot + 1) & ~1;
}

cudaError_t launchReactorRhs(const RhsParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    return p.m.NX ? launchReactorRhsX(p, blocks, warpsPerBlock, stream)
                  : launchReactorRhsT<false>(p, blocks, warpsPerBlock, stream);
}

int bdfRecordStride(int N) { return (QMAX + 1) * N + R_NSCAL; }
int bdfNordsieckDoubles(int N) { return (QMAX + 1) * N; }
BdfRecordLayout bdfRecordLayout() { return {QMAX, R_TN, R_H, R_Q, R_FLAGS, F_INIT}; }

int bdfWarpDoubles(const DevMech& m, int ld, bool fp32) {
    int N = m.N;
    int kinD = kStateSlots + KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT);
    int vec = (QMAX + 1) * N + 8 * N + (N + 1) / 2 + kAuxDoubles;
    int mat = fp32 ? (N * ld + 1) / 2 : N * ld;
    int tot = kinD + vec + mat;
    return (tot + 1) & ~1;   // keep each warp's slice 16-byte aligned
}

int bdfWarpDoublesNoMatrix(const DevMech& m) {
    int N = m.N;
    int kinD = kStateSlots + KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT, true);
    int vec = 8 * N + (N + 1) / 2 + kAuxDoubles;   // the Nordsieck array is in the global slot
    return (kinD + vec + 1) & ~1;
}

int bdfKrylovDoubles(int N) { return (((kMaxl + 1) * N + kGmresScalars) + 1) & ~1; }

int ratesWarpDoubles(const DevMech& m, bool jac) {
    int kinD = KinScratch::doubles(m.K, m.R, m.NTB, m.NF, m.NT, jac);
    int tot = kinD + 2 * m.K + (jac ? m.nnz : 0);
    return (tot + 1) & ~1;
}

cudaError_t launchRates(const RatesParams& p, int blocks, int warpsPerBlock, cudaStream_t stream) {
    return p.m.NX ? launchRatesX(p, blocks, warpsPerBlock, stream)
                  : launchRatesT<false>(p, blocks, warpsPerBlock, stream);
}

int bdfBlocksPerSm(int N, bool fp32, int warpsPerBlock, size_t smem, bool extra) {
    if (extra) return bdfBlocksPerSmX(fp32, warpsPerBlock, smem);
    if (fp32) {
        if (N <= 64) return bdfBlocksPerSmT<float, 2, false>(warpsPerBlock, smem);
        if (N <= 128) return bdfBlocksPerSmT<float, 4, false>(warpsPerBlock, smem);
        return bdfBlocksPerSmT<float, 8, false>(warpsPerBlock, smem);
    }
    if (N <= 64) return bdfBlocksPerSmT<double, 2, false>(warpsPerBlock, smem);
    if (N <= 128) return bdfBlocksPerSmT<double, 4, false>(warpsPerBlock, smem);
    return bdfBlocksPerSmT<double, 8, false>(warpsPerBlock, smem);
}

cudaError_t launchBdf(const BdfParams& p, int blocks, int warpsPerBlock, bool fp32, cudaStream_t stream) {
    if (p.m.NX) return launchBdfX(p, blocks, warpsPerBlock, fp32, stream);
    // register slots of the Newton vector per lane: 32 components each
    const int N = p.m.N;
    if (N <= 64) return fp32 ? launchBdfT<float, 2, false>(p, blocks, warpsPerBlock, stream)
                             : launchBdfT<double, 2, false>(p, blocks, warpsPerBlock, stream);
    if (N <= 128) return fp32 ? launchBdfT<float, 4, false>(p, blocks, warpsPerBlock, stream)
                              : launchBdfT<double, 4, false>(p, blocks, warpsPerBlock, stream);
    return fp32 ? launchBdfT<float, 8, false>(p, blocks, warpsPerBlock, stream)
                : launchBdfT<double, 8, false>(p, blocks, warpsPerBlock, stream);
}

// -----------------------------------------------------------------------------
// FP64 probe: eight independent FMA chains per thread (enough to fill the pipe), and
// chains of exp / log of varying arguments, over a grid that covers every SM.
// -----------------------------------------------------------------------------
__global__ void k_probe_fma(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_probe_exp(double* out, int iters, int useLog) {
    double s = 0, x = useLog ? 1.5 + threadIdx.x * 1e-4 : -1.0 - threadIdx.x * 1e-4;
    for (int i = 0; i < iters; i++) {
        s += useLog ? log(x) : exp(x);
        x += 1e-7;
        s += useLog ? log(x * 0.5) : exp(x * 0.5);
        x += 1e-7;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_check_exp(int n, const double* x, double* mine, double* lib) {
    __shared__ uint64_t s_tab[kGbxTableWords];
    gbx_load_table(s_tab);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mine[i] = fexp(x[i], s_tab);
        lib[i] = exp(x[i]);
    }
}

__global__ void k_check_log(int n, const double* x, double* mine, double* lib) {
    __shared__ uint64_t s_tab[kGbxTableWords];
    gbx_load_table(s_tab);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mine[i] = gbx_log(x[i], s_tab);
        lib[i] = log(x[i]);
    }
}

cudaError_t checkLog(int n, const double* x, double* mine, double* lib) {
    k_check_log<<<256, 256>>>(n, x, mine, lib);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaDeviceSynchronize();
}

cudaError_t checkExp(int n, const double* x, double* mine, double* lib) {
    k_check_exp<<<256, 256>>>(n, x, mine, lib);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaDeviceSynchronize();
}

cudaError_t measureFp64(double* results, int smCount) {
    const int threads = 256, blocks = smCount * 8;
    double* d = nullptr;
    cudaError_t e = cudaMalloc(&d, (size_t)threads * blocks * sizeof(double));
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float ms = 0.f;
    const int it = 4096;
    double best = 0.0, bestExpRate = 0.0, bestLogRate = 0.0;
    for (int rep = 0; rep < 6; rep++) {
        cudaEventRecord(a);
        k_probe_fma<<<blocks, threads>>>(d, it, 1.0000001, 1e-9);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        const double fmaPerS = 8.0 * it * threads * blocks / (ms * 1e-3);
        best = fmax(best, fmaPerS);
        cudaEventRecord(a);
        k_probe_exp<<<blocks, threads>>>(d, it / 8, 0);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        bestExpRate = fmax(bestExpRate, 2.0 * (it / 8) * threads * blocks / (ms * 1e-3));
        cudaEventRecord(a);
        k_probe_exp<<<blocks, threads>>>(d, it / 8, 1);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        bestLogRate = fmax(bestLogRate, 2.0 * (it / 8) * threads * blocks / (ms * 1e-3));
    }
    // costs relative to the best FMA rate, each at its own best (clocks settle during the reps)
    const double bestExp = best / bestExpRate, bestLog = best / bestLogRate;
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    results[0] = 2.0 * best / 1e9;
    results[1] = bestExp;
    results[2] = bestLog;
    return e;
}

#endif  // GB_KERNELS_EXTRA

}  // namespace gbchem
