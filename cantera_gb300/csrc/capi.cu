// capi.cu - host side of the engine and its C ABI (include/gbchem.h).
//
// Handles index process-wide tables, as Cantera's CLib Cabinet does
// (interfaces/clib/src/Cabinet.h); every entry point catches exceptions and turns
// them into GB_ERR plus a thread-local message (interfaces/clib/src/clib_utils.h:32-52).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gbchem.h"
#include "devmech.h"
#include "kernels.h"
#include "mechanism.h"
#include "surrogate.h"

using namespace gbchem;

namespace {

thread_local std::string g_error;
// the stream of the surrogate's calls (gb_nn_*) on this host thread, and whether they
// return without waiting for their work (gb_nn_set_stream)
thread_local cudaStream_t g_nnStream = nullptr;
thread_local bool g_nnAsync = false;

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};
void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Device buffer with RAII.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { if (p) cudaFree(p); }
    void ensure(size_t b) {
        if (b <= bytes) return;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        ck(cudaMalloc(&p, std::max<size_t>(b, 256)), "cudaMalloc");
        bytes = b;
    }
    template <class T> T* as() const { return (T*)p; }
};

// Arena builder for the packed mechanism: appends arrays with 32-byte alignment.
struct Arena {
    std::vector<char> data;
    template <class T> size_t add(const std::vector<T>& v) {
        size_t off = (data.size() + 31) & ~size_t(31);
        data.resize(off + v.size() * sizeof(T) + 32);
        if (!v.empty()) std::memcpy(data.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

struct MechEntry {
    Mechanism m;
    DBuf arena;
    DevMech dm{};
    std::vector<int32_t> jcPtr, jrIdx;
    cudaStream_t stream = nullptr;
    int smCount = 0;
    int device = -1;      // the CUDA device the mechanism's arena and stream live on
    // kinetics workspace
    DBuf dT, dP, dY, dW, dJ, dCounter, dExt;
    DBuf dChk;                                  // bounds-check record (checked build)
    cudaEvent_t evA = nullptr, evB = nullptr;   // around the last kinetics kernel launch
    cudaEvent_t evCaller = nullptr;             // the caller's default-stream work (afterCallerWork)
    double lastMs = 0.0;
    ~MechEntry() {
        if (evA) cudaEventDestroy(evA);
        if (evB) cudaEventDestroy(evB);
        if (evCaller) cudaEventDestroy(evCaller);
        if (stream) cudaStreamDestroy(stream);
    }
};

// Device arrays a caller hands in (GB_DEVICE_POINTERS) have usually just been written by its
// kernels on the default stream, and the engine's stream is a non-blocking one, which does not
// wait for the default stream by itself: make it wait for the work already issued to the legacy
// and the per-thread default streams before it reads them (an event dependency, no host
// synchronisation).  Arrays written on another stream must be synchronised by the caller.
void afterCallerWork(MechEntry& e) {
    if (!e.evCaller) ck(cudaEventCreateWithFlags(&e.evCaller, cudaEventDisableTiming), "event");
    ck(cudaEventRecord(e.evCaller, cudaStreamLegacy), "record the default stream's work");
    ck(cudaStreamWaitEvent(e.stream, e.evCaller, 0), "wait for the default stream's work");
    ck(cudaEventRecord(e.evCaller, cudaStreamPerThread), "record the per-thread stream's work");
    ck(cudaStreamWaitEvent(e.stream, e.evCaller, 0), "wait for the per-thread stream's work");
}

struct NetEntry {
    int mech;
    int n;
    gb_net_options opts;
    double time = 0.0;
    int warpsPerBlock = 0, blocks = 0, ld = 0, warpDoubles = 0, recStride = 0;
    DBuf dP, dT, dY, dRec, dStats, dStatus, dTign, dCounter, dOrder, dM, dJ, dJS, dTnow, dKStats, dKz;
    bool krylov = false;  // the mole reactor with GMRES and the adaptive preconditioner
    size_t JSstride = 0;  // bytes per Jacobian-scratch slot in dJS (with global matrices)
    size_t Jstride = 0;   // bytes per kept-Jacobian slot in dJ (0: no Jacobian reuse)
    size_t Mstride = 0;   // bytes per Newton-matrix slot in dM (0: matrices in shared memory)
    bool matGlobal = false;
    int mechSmem = 0;     // bytes of the mechanism arena each block copies into shared memory
    int luSlots = 0, luSlotBytes = 0;   // shared-memory factorisation buffers per block
    bool haveOrder = false;
    cudaGraphExec_t graph = nullptr;
    double graphTout = -1.0;
    cudaEvent_t evA = nullptr, evB = nullptr;
    double lastMs = 0.0;
    ~NetEntry() {
        if (graph) cudaGraphExecDestroy(graph);
        if (evA) cudaEventDestroy(evA);
        if (evB) cudaEventDestroy(evB);
    }
};

std::mutex g_mu;
std::vector<std::unique_ptr<MechEntry>> g_mechs;
std::vector<std::unique_ptr<NetEntry>> g_nets;

MechEntry& mech(int32_t h) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (h < 0 || h >= (int32_t)g_mechs.size() || !g_mechs[h]) throw std::runtime_error("invalid mechanism handle " + std::to_string(h));
    return *g_mechs[h];
}
// The mechanism's device arrays and stream belong to the device that was current at
// gb_mech_load; a kernel launched with another device current would read another GPU's
// memory, so every call that launches work checks the current device first.
void requireMechDevice(const MechEntry& e) {
    int dev = -1;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != e.device)
        throw std::runtime_error("the current CUDA device (" + std::to_string(dev) +
                                 ") is not the device the mechanism was loaded on (" +
                                 std::to_string(e.device) + ")");
}

NetEntry& net(int32_t h) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (h < 0 || h >= (int32_t)g_nets.size() || !g_nets[h]) throw std::runtime_error("invalid reactor network handle " + std::to_string(h));
    return *g_nets[h];
}

template <class F> int32_t guarded(F&& f) {
    try {
        return f();
    } catch (std::exception& e) {
        g_error = e.what();
        return GB_ERR;
    } catch (...) {
        g_error = "unknown error";
        return GB_ERR;
    }
}

// ---------------------------------------------------------------------------
// Mechanism -> device layout
// ---------------------------------------------------------------------------
void packDevMech(MechEntry& e) {
    const Mechanism& m = e.m;
    const int K = m.K, R = m.R;
    if (K > kMaxSpecies) throw std::runtime_error("mechanism has more species than the GPU path supports");
    std::vector<double> rmw(K), nasa((size_t)K * kNasaStride, 0.0);
    for (int k = 0; k < K; k++) {
        rmw[k] = 1.0 / m.mw[k];
        nasa[(size_t)k * kNasaStride] = m.nasaTmid[k];
        for (int r = 0; r < 2; r++) {
            const double* a = r == 0 ? &m.nasaLow[7 * k] : &m.nasaHigh[7 * k];
            double* d = &nasa[(size_t)k * kNasaStride + 1 + r * kNasaRange];
            for (int j = 0; j < 7; j++) d[j] = a[j];
            d[7] = a[1] / 2.0; d[8] = a[2] / 3.0; d[9] = a[3] / 4.0; d[10] = a[4] / 5.0;
            d[11] = a[2] / 2.0; d[12] = a[3] / 3.0; d[13] = a[4] / 4.0;
        }
    }
    // Device reaction order: falloff (Troe, then Lindemann), the other falloff forms (SRI,
    // Tsang, chemically activated), three-body, pressure-dependent Arrhenius, Chebyshev,
    // reversible, then irreversible reactions, and within each group those whose rate
    // constant needs an exponential first.  A warp evaluates 32 consecutive reactions at a
    // time, so grouping keeps its lanes on the same code path.  Results are per species and
    // do not depend on this order (beyond summation order).
    auto group = [&](int i) {
        if (m.kind[i] == kTroe && !m.chemAct[i]) return 0;
        if (m.kind[i] == kLindemann && !m.chemAct[i]) return 1;
        if (isFalloffKind(m.kind[i])) return 2;
        if (m.kind[i] == kThreeBody) return 3;
        if (m.kind[i] == kPlog) return 4;
        if (m.kind[i] == kChebyshev) return 5;
        return m.reversible[i] ? 6 : 7;
    };
    auto noExp = [&](int i) { return m.kind[i] <= kThreeBody && m.b[i] == 0.0 && m.EaR[i] == 0.0; };
    std::vector<int> perm(R), inv(R);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) {
        int ga = group(a), gb = group(b);
        if (ga != gb) return ga < gb;
        return (int)noExp(a) < (int)noExp(b);
    });
    for (int ni = 0; ni < R; ni++) inv[perm[ni]] = ni;

    std::vector<int4> rinfo(R), rk(R), pk(R);
    std::vector<D4> rarr(R);
    std::vector<int> sidePtr(1, 0), sideK;
    std::vector<double> sideNu, sideOrd;
    std::vector<D4> fo1, fo2;
    std::vector<double> pdep;
    std::vector<int> rsPtr(1, 0), rsK;
    std::vector<double> rsNu;
    std::vector<std::map<int, double>> net(R);
    for (int ni = 0; ni < R; ni++) {
        const int i = perm[ni];
        int flags = m.kind[i] & kKindMask;
        if (m.reversible[i]) flags |= kRevBit;
        flags |= (m.reacBucket[i] & 7) << kRBucketShift;
        flags |= (m.prodBucket[i] & 7) << kPBucketShift;
        if (m.chemAct[i]) flags |= kChemActBit;
        int fo = -1;
        if (isFalloffKind(m.kind[i])) {
            fo = (int)fo1.size();
            const double* x = &m.falloffX[5 * i];
            if (m.kind[i] == kSri) {
                fo1.push_back(D4{m.A0[i], m.b0[i], m.Ea0R[i], x[0]});
                fo2.push_back(D4{x[1], x[2], x[3], x[4]});
            } else if (m.kind[i] == kTsang) {
                fo1.push_back(D4{m.A0[i], m.b0[i], m.Ea0R[i], x[0]});
                fo2.push_back(D4{x[1], 0.0, 0.0, 0.0});
            } else {
                fo1.push_back(D4{m.A0[i], m.b0[i], m.Ea0R[i], m.troe[4 * i]});
                fo2.push_back(D4{m.troe[4 * i + 1], m.troe[4 * i + 2], m.troe[4 * i + 3], m.kind[i] == kTroe ? 1.0 : 0.0});
            }
        }
        int pd = -1;
        if (m.kind[i] == kPlog) {
            pd = (int)pdep.size();
            const int l0 = m.plogPtr[i], l1 = m.plogPtr[i + 1], L = l1 - l0;
            const int q0 = m.plogFirst[l0];          // first rate of the reaction
            int nrates = 0;
            for (int l = l0; l < l1; l++) nrates = std::max(nrates, m.plogLast[l] - q0);
            pdep.push_back((double)L);
            const int rbase = 1 + 3 * L;             // offset of the first rate triple
            for (int l = l0; l < l1; l++) {
                pdep.push_back(m.plogLogP[l]);
                pdep.push_back((double)(rbase + 3 * (m.plogFirst[l] - q0)));
                pdep.push_back((double)(rbase + 3 * (m.plogLast[l] - q0)));
            }
            for (int q = q0; q < q0 + nrates; q++) {
                pdep.push_back(m.plogA[q]);
                pdep.push_back(m.plogB[q]);
                pdep.push_back(m.plogEaR[q]);
            }
        } else if (m.kind[i] == kChebyshev) {
            pd = (int)pdep.size();
            pdep.push_back((double)m.chebNT[i]);
            pdep.push_back((double)m.chebNP[i]);
            for (int j = 0; j < 4; j++) pdep.push_back(m.chebLim[4 * i + j]);
            for (int q = m.chebPtr[i]; q < m.chebPtr[i + 1]; q++) pdep.push_back(m.chebCoef[q]);
        }
        if (m.dn[i] == std::floor(m.dn[i]) && std::fabs(m.dn[i]) <= 3.0) flags |= kDnIntBit;
        if (noExp(i)) flags |= kNoExpBit;
        rinfo[ni] = int4{flags, m.tbOfRxn[i], fo, pd};
        rarr[ni] = D4{m.A[i], m.b[i], m.EaR[i], m.dn[i]};
        auto expand = [&](const int32_t* ks, const double* nus, int n) {
            int4 e4{-1, -1, -1, 0};
            int cnt = 0;
            int* slot[3] = {&e4.x, &e4.y, &e4.z};
            for (int j = 0; j < n; j++)
                for (int r = 0; r < (int)nus[j] && cnt < 3; r++) *slot[cnt++] = ks[j];
            e4.w = cnt;
            return e4;
        };
        rk[ni] = expand(&m.reacK[m.reacPtr[i]], &m.reacNu[m.reacPtr[i]], m.reacPtr[i + 1] - m.reacPtr[i]);
        pk[ni] = expand(&m.prodK[m.prodPtr[i]], &m.prodNu[m.prodPtr[i]], m.prodPtr[i + 1] - m.prodPtr[i]);
        for (int j = m.reacPtr[i]; j < m.reacPtr[i + 1]; j++) {
            sideK.push_back(m.reacK[j]); sideNu.push_back(m.reacNu[j]); sideOrd.push_back(m.reacOrder[j]);
            net[ni][m.reacK[j]] -= m.reacNu[j];
        }
        sidePtr.push_back((int)sideK.size());
        for (int j = m.prodPtr[i]; j < m.prodPtr[i + 1]; j++) {
            sideK.push_back(m.prodK[j]); sideNu.push_back(m.prodNu[j]); sideOrd.push_back(m.prodNu[j]);
            net[ni][m.prodK[j]] += m.prodNu[j];
        }
        sidePtr.push_back((int)sideK.size());
        for (auto& kv : net[ni])
            if (kv.second != 0.0) { rsK.push_back(kv.first); rsNu.push_back(kv.second); }
        rsPtr.push_back((int)rsK.size());
    }
    // species gather lists (net coefficients)
    std::vector<std::vector<std::pair<int, double>>> bySpecies(K);
    for (int i = 0; i < R; i++)
        for (int q = rsPtr[i]; q < rsPtr[i + 1]; q++) bySpecies[rsK[q]].push_back({i, rsNu[q]});
    std::vector<int> spPtr(1, 0), spRxn;
    std::vector<double> spNu;
    for (int k = 0; k < K; k++) {
        for (auto& pr : bySpecies[k]) { spRxn.push_back(pr.first); spNu.push_back(pr.second); }
        spPtr.push_back((int)spRxn.size());
    }
    // gather tasks: species lists cut into pieces of at most `cap` entries, pieces dealt
    // to lanes heaviest first onto the least-loaded lane
    std::vector<int> taskPtr(1, 0), taskSp;
    {
        const int E = spPtr.back();
        const int cap = std::max(8, (E + 31) / 32);
        for (int k = 0; k < K; k++)
            for (int a0 = spPtr[k]; a0 < spPtr[k + 1]; a0 += cap) {
                taskPtr.push_back(std::min(a0 + cap, spPtr[k + 1]));
                taskSp.push_back(k);
            }
    }
    const int NT = (int)taskSp.size();
    std::vector<int> laneTaskPtr(1, 0), laneTasks, spTaskPtr(1, 0), spTasks;
    {
        std::vector<int> ord(NT);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
            return taskPtr[a + 1] - taskPtr[a] > taskPtr[b + 1] - taskPtr[b];
        });
        std::vector<std::vector<int>> lt(32);
        std::vector<int> ld(32, 0);
        for (int t : ord) {
            int l = (int)(std::min_element(ld.begin(), ld.end()) - ld.begin());
            lt[l].push_back(t);
            ld[l] += taskPtr[t + 1] - taskPtr[t] + 2;
        }
        for (int l = 0; l < 32; l++) {
            for (int t : lt[l]) laneTasks.push_back(t);
            laneTaskPtr.push_back((int)laneTasks.size());
        }
        for (int k = 0; k < K; k++) {
            for (int t = 0; t < NT; t++)
                if (taskSp[t] == k) spTasks.push_back(t);
            spTaskPtr.push_back((int)spTasks.size());
        }
    }
    // third bodies
    std::vector<int> tbRxn(m.tbRxn.size()), tbMA(m.tbMassAction.begin(), m.tbMassAction.end());
    for (size_t t = 0; t < tbRxn.size(); t++) tbRxn[t] = inv[m.tbRxn[t]];
    std::vector<int> tbPtr(m.tbPtr.begin(), m.tbPtr.end()), tbK(m.tbSpecies.begin(), m.tbSpecies.end());
    std::vector<double> tbDef(m.tbDefault), tbE(m.tbEffMinusDefault);
    // Jacobian columns: dependencies of each reaction through mass action and the
    // non-default part of its third-body efficiencies
    std::vector<std::vector<std::pair<int, double>>> cols(K);
    for (int ni = 0; ni < R; ni++) {
        const int i = perm[ni];
        std::map<int, double> deps;
        for (int j = m.reacPtr[i]; j < m.reacPtr[i + 1]; j++) deps[m.reacK[j]] += 0.0;
        if (m.reversible[i])
            for (int j = m.prodPtr[i]; j < m.prodPtr[i + 1]; j++) deps[m.prodK[j]] += 0.0;
        int t = m.tbOfRxn[i];
        if (t >= 0)
            for (int q = m.tbPtr[t]; q < m.tbPtr[t + 1]; q++)
                if (m.tbEffMinusDefault[q] != 0.0) deps[m.tbSpecies[q]] = m.tbEffMinusDefault[q];
        for (auto& kv : deps) cols[kv.first].push_back({ni, kv.second});
    }
    std::vector<int> colPtr(1, 0), colRxn;
    std::vector<double> colE;
    std::vector<long> work(K, 0);
    for (int j = 0; j < K; j++) {
        for (auto& pr : cols[j]) {
            colRxn.push_back(pr.first);
            colE.push_back(pr.second);
            work[j] += 1 + (rsPtr[pr.first + 1] - rsPtr[pr.first]);
        }
        colPtr.push_back((int)colRxn.size());
    }
    // balance columns over 32 lanes: heaviest first onto the least-loaded lane
    std::vector<int> order(K);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
    std::vector<std::vector<int>> laneList(32);
    std::vector<long> load(32, 0);
    for (int j : order) {
        int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        laneList[l].push_back(j);
        load[l] += work[j];
    }
    std::vector<int> laneColPtr(1, 0), laneCols;
    for (int l = 0; l < 32; l++) {
        for (int j : laneList[l]) laneCols.push_back(j);
        laneColPtr.push_back((int)laneCols.size());
    }
    // dense default-efficiency part
    std::vector<int> gsPtr(1, 0), gsTb;
    std::vector<double> gsCoef;
    {
        std::vector<std::vector<std::pair<int, double>>> gl(K);
        for (int t = 0; t < m.nThirdBody(); t++) {
            if (m.tbDefault[t] == 0.0) continue;
            int i = inv[m.tbRxn[t]];
            for (int q = rsPtr[i]; q < rsPtr[i + 1]; q++) gl[rsK[q]].push_back({t, rsNu[q] * m.tbDefault[t]});
        }
        for (int k = 0; k < K; k++) {
            for (auto& pr : gl[k]) { gsTb.push_back(pr.first); gsCoef.push_back(pr.second); }
            gsPtr.push_back((int)gsTb.size());
        }
    }
    // output pattern
    jacobianPattern(m, e.jcPtr, e.jrIdx);
    std::vector<int> jpCol(e.jrIdx.size());
    for (int c = 0; c < K; c++)
        for (int q = e.jcPtr[c]; q < e.jcPtr[c + 1]; q++) jpCol[q] = c;
    std::vector<int> jcPtr(e.jcPtr.begin(), e.jcPtr.end()), jrIdx(e.jrIdx.begin(), e.jrIdx.end());
    // the pattern slot of every scatter of a column entry: column j, its entries e (reaction
    // i) in order, the species r of reaction i with a net coefficient in order ->
    // slot of (r, j), or -1 (not a structural nonzero)
    std::vector<int> colSlotStart(1, 0), colSlot;
    for (int j = 0; j < K; j++) {
        std::map<int, int> slotOfRow;
        for (int q = jcPtr[j]; q < jcPtr[j + 1]; q++) slotOfRow[jrIdx[q]] = q;
        for (int e2 = colPtr[j]; e2 < colPtr[j + 1]; e2++) {
            const int i = colRxn[e2];
            for (int r = rsPtr[i]; r < rsPtr[i + 1]; r++) {
                auto it = slotOfRow.find(rsK[r]);
                colSlot.push_back(it == slotOfRow.end() ? -1 : it->second);
            }
        }
        colSlotStart.push_back((int)colSlot.size());
    }

    // Arena order by use: what every right-hand side reads, then what a Jacobian reads,
    // then the general (CN) side lists, then the rest.  Kernels copy a prefix of the arena
    // into shared memory when it fits, so the hottest data goes first.
    Arena a;
    size_t o_nasa = a.add(nasa), o_rmw = a.add(rmw), o_mw = a.add(m.mw);
    size_t o_rinfo = a.add(rinfo), o_rarr = a.add(rarr), o_rk = a.add(rk), o_pk = a.add(pk);
    size_t o_fo1 = a.add(fo1), o_fo2 = a.add(fo2);
    size_t o_tbPtr = a.add(tbPtr), o_tbK = a.add(tbK), o_tbE = a.add(tbE), o_tbDef = a.add(tbDef);
    size_t o_taskPtr = a.add(taskPtr), o_ltp = a.add(laneTaskPtr), o_lt = a.add(laneTasks),
           o_stp = a.add(spTaskPtr), o_st = a.add(spTasks);
    size_t o_spRxn = a.add(spRxn), o_spNu = a.add(spNu);
    const size_t hotEnd = a.data.size();
    size_t o_lcp = a.add(laneColPtr), o_lc = a.add(laneCols);
    size_t o_colPtr = a.add(colPtr), o_colRxn = a.add(colRxn), o_colE = a.add(colE);
    size_t o_rsPtr = a.add(rsPtr), o_rsK = a.add(rsK), o_rsNu = a.add(rsNu);
    size_t o_gsPtr = a.add(gsPtr), o_gsTb = a.add(gsTb), o_gsCoef = a.add(gsCoef);
    size_t o_colSlotStart = a.add(colSlotStart), o_colSlot = a.add(colSlot);
    const size_t jacEnd = a.data.size();
    size_t o_sidePtr = a.add(sidePtr), o_sideK = a.add(sideK), o_sideNu = a.add(sideNu), o_sideOrd = a.add(sideOrd);
    const size_t sideEnd = a.data.size();
    size_t o_spPtr = a.add(spPtr), o_tbRxn = a.add(tbRxn), o_tbMA = a.add(tbMA);
    size_t o_jcPtr = a.add(jcPtr), o_jrIdx = a.add(jrIdx), o_jpCol = a.add(jpCol);
    size_t o_pdep = a.add(pdep);
    const std::vector<int32_t> precOrder = preconditionerOrdering(m);
    size_t o_precOrder = a.add(precOrder);
    e.arena.ensure(a.data.size());
    ck(cudaMemcpy(e.arena.p, a.data.data(), a.data.size(), cudaMemcpyHostToDevice), "upload mechanism");
    char* b = e.arena.as<char>();
    DevMech& d = e.dm;
    auto up16 = [](size_t v) { return (int)((v + 15) & ~size_t(15)); };
    d.arena = b;
    d.hotBytes = up16(hotEnd); d.jacBytes = up16(jacEnd); d.sideBytes = up16(sideEnd);
    d.K = K; d.R = R; d.N = K + 1; d.NF = (int)fo1.size(); d.NTB = m.nThirdBody(); d.nnz = (int)jrIdx.size();
    d.NX = 0;
    for (int i = 0; i < R; i++) d.NX += (m.kind[i] > kTroe || m.chemAct[i]) ? 1 : 0;
    d.Pref = m.Pref; d.Rgas = gasConstant();
    d.mw = (const double*)(b + o_mw); d.rmw = (const double*)(b + o_rmw); d.nasa = (const double*)(b + o_nasa);
    d.rinfo = (const int4*)(b + o_rinfo); d.rarr = (const D4*)(b + o_rarr);
    d.rk = (const int4*)(b + o_rk); d.pk = (const int4*)(b + o_pk);
    d.sidePtr = (const int*)(b + o_sidePtr); d.sideK = (const int*)(b + o_sideK);
    d.sideNu = (const double*)(b + o_sideNu); d.sideOrd = (const double*)(b + o_sideOrd);
    d.rsPtr = (const int*)(b + o_rsPtr); d.rsK = (const int*)(b + o_rsK); d.rsNu = (const double*)(b + o_rsNu);
    d.fo1 = (const D4*)(b + o_fo1); d.fo2 = (const D4*)(b + o_fo2);
    d.tbRxn = (const int*)(b + o_tbRxn); d.tbDef = (const double*)(b + o_tbDef); d.tbMA = (const int*)(b + o_tbMA);
    d.tbPtr = (const int*)(b + o_tbPtr); d.tbK = (const int*)(b + o_tbK); d.tbE = (const double*)(b + o_tbE);
    d.spPtr = (const int*)(b + o_spPtr); d.spRxn = (const int*)(b + o_spRxn); d.spNu = (const double*)(b + o_spNu);
    d.NT = NT;
    d.taskPtr = (const int*)(b + o_taskPtr); d.laneTaskPtr = (const int*)(b + o_ltp); d.laneTasks = (const int*)(b + o_lt);
    d.spTaskPtr = (const int*)(b + o_stp); d.spTasks = (const int*)(b + o_st);
    d.colPtr = (const int*)(b + o_colPtr); d.colRxn = (const int*)(b + o_colRxn); d.colE = (const double*)(b + o_colE);
    d.laneColPtr = (const int*)(b + o_lcp); d.laneCols = (const int*)(b + o_lc);
    d.gsPtr = (const int*)(b + o_gsPtr); d.gsTb = (const int*)(b + o_gsTb); d.gsCoef = (const double*)(b + o_gsCoef);
    d.jcPtr = (const int*)(b + o_jcPtr); d.jrIdx = (const int*)(b + o_jrIdx); d.jpCol = (const int*)(b + o_jpCol);
    d.pdep = (const double*)(b + o_pdep);
    d.colSlotStart = (const int*)(b + o_colSlotStart); d.colSlot = (const int*)(b + o_colSlot);
    d.precOrder = (const int*)(b + o_precOrder);
}

// dynamic shared memory a block may use: the opt-in maximum less the kernels' static
// tables (exp/log tables, kGbxTableWords words) and a margin
int maxSmemPerBlock() {
    int dev = 0, v = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device attribute");
    return v - 4096;
}

// Copy n*count doubles to a device buffer unless they are already on the device.
const double* stage(const double* src, size_t count, DBuf& buf, bool device, cudaStream_t s) {
    if (device) return src;
    buf.ensure(count * sizeof(double));
    ck(cudaMemcpyAsync(buf.p, src, count * sizeof(double), cudaMemcpyHostToDevice, s), "copy to device");
    return buf.as<double>();
}

int32_t runRates(int32_t h, int32_t n, const double* T, const double* P, const double* Y, double* wdot,
                 double* vals, int32_t flags) {
    MechEntry& e = mech(h);
    requireMechDevice(e);
    if (n < 0) throw std::runtime_error("negative number of states");
    if (n == 0) return 0;
    const bool dev = (flags & GB_DEVICE_POINTERS) != 0;
    const int K = e.m.K;
    cudaStream_t s = e.stream;
    if (dev) afterCallerWork(e);
    const double* dT = stage(T, n, e.dT, dev, s);
    const double* dP = stage(P, n, e.dP, dev, s);
    const double* dY = stage(Y, (size_t)K * n, e.dY, dev, s);
    double* dW = nullptr;
    double* dJ = nullptr;
    if (wdot) {
        if (dev) dW = wdot;
        else { e.dW.ensure((size_t)K * n * 8); dW = e.dW.as<double>(); }
    }
    if (vals) {
        if (dev) dJ = vals;
        else { e.dJ.ensure((size_t)e.dm.nnz * n * 8); dJ = e.dJ.as<double>(); }
    }
    e.dCounter.ensure(2 * sizeof(int));
    ck(cudaMemsetAsync(e.dCounter.p, 0, 2 * sizeof(int), s), "memset");
    RatesParams p{};
    p.m = e.dm; p.n = n; p.T = dT; p.P = dP; p.Y = dY; p.wdot = dW; p.jac = dJ;
    p.counter = e.dCounter.as<int>();
    p.warpDoubles = ratesWarpDoubles(e.dm, dJ != nullptr);
    p.tileDoubles = dJ ? 0 : ratesTileDoubles(e.dm);
    // the mechanism data the call reads goes into shared memory when 8 warps still fit
    // next to the block's state tile
    const int budget = maxSmemPerBlock() - p.tileDoubles * 8;
    const int want = dJ ? e.dm.sideBytes : e.dm.hotBytes;
    p.mechSmem = (budget - want) / (p.warpDoubles * 8) >= 8 ? want : 0;
    int wpb = std::max(1, std::min(8, (budget - p.mechSmem) / (p.warpDoubles * 8)));
    if (budget - p.mechSmem < p.warpDoubles * 8) throw std::runtime_error("mechanism too large for the rates kernel's shared memory");
    const int perBlock = p.mechSmem + p.tileDoubles * 8 + p.warpDoubles * 8 * wpb + 1024;
    int blocksPerSm = std::max(1, (228 * 1024) / perBlock);
    // wdot alone: a tile of 32 states per block at a time; with the Jacobian: a state per warp
    const long long units = dJ ? ((long long)n + wpb - 1) / wpb : ((long long)n + kRatesTile - 1) / kRatesTile;
    int blocks = (int)std::min<long long>((long long)e.smCount * blocksPerSm, units);
    if (dJ) {   // kfe and rkc of each resident warp (the Jacobian's per-reaction data)
        e.dExt.ensure((size_t)blocks * wpb * 2 * e.dm.R * 8);
        p.ext = e.dExt.as<double>();
    }
    if (!e.evA) {
        ck(cudaEventCreate(&e.evA), "event");
        ck(cudaEventCreate(&e.evB), "event");
    }
    ck(cudaEventRecord(e.evA, s), "event record");
    ck(launchRates(p, blocks, wpb, s), "rates kernel launch");
    ck(cudaEventRecord(e.evB, s), "event record");
    if (wdot && !dev) ck(cudaMemcpyAsync(wdot, dW, (size_t)K * n * 8, cudaMemcpyDeviceToHost, s), "copy wdot");
    if (vals && !dev) ck(cudaMemcpyAsync(vals, dJ, (size_t)e.dm.nnz * n * 8, cudaMemcpyDeviceToHost, s), "copy jac");
    ck(cudaStreamSynchronize(s), "rates kernel");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, e.evA, e.evB), "event time");
    e.lastMs = ms;
    int flags2[2] = {0, 0};
    ck(cudaMemcpy(flags2, e.dCounter.p, sizeof(flags2), cudaMemcpyDeviceToHost), "copy flags");
    if (flags2[1]) throw std::runtime_error("rates kernel: the bulk copy of the mechanism into shared memory did not complete");
    return 0;
}

// Launch shape of the integrator: where the Newton matrices live, how much of the
// mechanism each block copies into shared memory, reactors (warps) per block.  A block's
// dynamic shared memory is the mechanism prefix plus one slice per warp.  Automatic choice:
// a block of 8 warps with the matrices in shared memory and as much of the mechanism as
// fits; if 8 such warps do not fit, the matrices move to global memory (an L2-resident
// slot per warp).
void chooseBdfLaunch(const MechEntry& me, const gb_net_options& o, int n, bool fp32, int ld, NetEntry& ne) {
    const DevMech& d = me.dm;
    const int budget = maxSmemPerBlock();
    const int kry = ne.krylov ? bdfKrylovDoubles(d.N) : 0;   // the Krylov basis and GMRES scalars
    const int wdShared = bdfWarpDoubles(d, ld, fp32) + kry;
    const int wdGlobal = bdfWarpDoublesNoMatrix(d) + kry;
    const int maxW = o.warps_per_block > 0 ? std::min(o.warps_per_block, kBdfMaxThreads / 32) : kBdfMaxThreads / 32;
    auto mechBytes = [&](int level) {
        return level == 4 ? d.sideBytes : (level == 3 ? d.jacBytes : (level == 2 ? d.hotBytes : 0));
    };
    std::vector<int> places;
    if (o.matrix_placement != 2) places.push_back(1);
    if (o.matrix_placement != 1) places.push_back(2);
    // first candidate (in preference order) that holds a full block; else the largest block.
    // Measured on GB300 (gri30): a mechanism copy that costs resident warps, or that takes
    // the L1 share the global matrices live in, is slower than none, so the automatic
    // choice copies the mechanism only next to shared-memory matrices.
    int bestFit = 0, bestPlace = 0, bestMech = 0;
    bool full = false;
    for (int pl : places) {
        std::vector<int> levels;
        if (o.mechanism_in_shared != 0) levels = {o.mechanism_in_shared};
        else if (pl == 1) levels = {4, 3, 2, 1};
        else levels = {1};
        for (int lv : levels) {
            const int mech = mechBytes(lv);
            const int wd = pl == 2 ? wdGlobal : wdShared;
            const int fit = std::min((budget - mech) / (wd * 8), maxW);
            if (fit > bestFit) { bestFit = fit; bestPlace = pl; bestMech = mech; }
            if (fit >= maxW) { full = true; break; }
        }
        if (full) break;
    }
    if (bestFit < 1) throw std::runtime_error("mechanism too large for one warp's shared memory");
    ne.matGlobal = bestPlace == 2;
    ne.mechSmem = bestMech;
    ne.warpDoubles = ne.matGlobal ? wdGlobal : wdShared;
    ne.warpsPerBlock = bestFit;
    // with global matrices, the shared memory left over holds factorisation buffers
    ne.luSlots = 0;
    ne.luSlotBytes = ((d.N * ld * (fp32 ? 4 : 8)) + 15) & ~15;
    // automatic: none - on gri30 every staging buffer cost more in L1 capacity (the global
    // matrices' cache) than it saved in the factorisation (8 warps/SM: 5,942 reactors/s with
    // none, 5,689 / 5,560 / 5,419 with 1 / 2 / 3 buffers)
    if (ne.matGlobal && o.lu_staging > 0 && !ne.krylov) {
        const int room = (budget - ne.mechSmem - ne.warpDoubles * 8 * bestFit) / ne.luSlotBytes;
        const int cap = std::min(o.lu_staging, kMaxLuSlots);
        ne.luSlots = std::max(0, std::min(room, cap));
    }
    const int perBlock = ne.mechSmem + ne.warpDoubles * 8 * bestFit + ne.luSlots * ne.luSlotBytes;
    const int blocksPerSm = ne.krylov ? (fp32 ? bdfBlocksPerSmKrylov32(d.N, d.NX > 0, bestFit, (size_t)perBlock)
                                              : bdfBlocksPerSmKrylov64(d.N, d.NX > 0, bestFit, (size_t)perBlock))
                                      : bdfBlocksPerSm(d.N, fp32, bestFit, (size_t)perBlock, d.NX > 0);
    ne.blocks = std::min(me.smCount * blocksPerSm, (n + bestFit - 1) / bestFit);
}

void netLaunch(NetEntry& ne, MechEntry& me, double t0, double tout, bool oneStep = false) {
    BdfParams p{};
    p.oneStep = oneStep ? 1 : 0;
    p.tnow = ne.dTnow.p ? ne.dTnow.as<double>() : nullptr;
    p.m = me.dm; p.n = ne.n; p.t0 = t0; p.tout = tout;
    p.rtol = ne.opts.rtol; p.atol = ne.opts.atol;
    p.hmaxInv = ne.opts.max_time_step > 0 ? 1.0 / ne.opts.max_time_step : 0.0;
    p.maxSteps = ne.opts.max_steps; p.maxOrder = ne.opts.max_order;
    p.P = ne.dP.as<double>(); p.T = ne.dT.as<double>(); p.Y = ne.dY.as<double>();
    p.rec = ne.dRec.as<double>(); p.recStride = ne.recStride;
    p.stats = ne.dStats.as<long long>(); p.status = ne.dStatus.as<int>(); p.tign = ne.dTign.as<double>();
    p.counter = ne.dCounter.as<int>(); p.order = ne.haveOrder ? ne.dOrder.as<int>() : nullptr;
    p.ld = ne.ld; p.warpDoubles = ne.warpDoubles;
    p.Mbuf = ne.Mstride ? ne.dM.p : nullptr; p.Mstride = (long long)ne.Mstride;
    p.Jbuf = ne.Jstride ? ne.dJ.p : nullptr; p.Jstride = (long long)ne.Jstride;
    p.JSbuf = ne.JSstride ? ne.dJS.p : nullptr; p.JSstride = (long long)ne.JSstride;
    p.mechSmem = ne.mechSmem;
    p.luSlots = ne.luSlots; p.luSlotBytes = ne.luSlotBytes;
    p.kstats = ne.krylov ? ne.dKStats.as<long long>() : nullptr;
    p.kzBuf = ne.krylov ? ne.dKz.as<double>() : nullptr;
    ck(cudaMemsetAsync(ne.dCounter.p, 0, sizeof(int), me.stream), "memset");
    if (ne.krylov)
        ck(ne.opts.lu_precision == 32 ? launchBdfKrylov32(p, ne.blocks, ne.warpsPerBlock, me.stream)
                                      : launchBdfKrylov64(p, ne.blocks, ne.warpsPerBlock, me.stream),
           "integrator launch (Krylov)");
    else ck(launchBdf(p, ne.blocks, ne.warpsPerBlock, ne.opts.lu_precision == 32, me.stream), "integrator launch");
}


// ---------------------------------------------------------------------------
// Allocation-free advance.  Some callers cannot call cudaMalloc at all: a host code whose
// own caching allocator owns every byte of the device (a CFD solver that calls chemistry
// once per cell batch inside its time loop) or a process whose device memory is fully
// budgeted.  gb_reactors_advance_noalloc serves them: its integrator records live in this
// fixed array that the module carries, so the call allocates nothing, neither through
// the CUDA runtime nor through any library.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;   // 16 MiB per device
static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noallocMu;                           // held for the whole call
void* g_noallocAddr[kNoAllocMaxDevices] = {};      // per device, looked up once

// Device address of this device's copy of the scratch array.  The first lookup on a
// device loads the module there (lazy loading), which the CUDA driver may not do inside a
// stream capture, so the first call on each device must precede any capture.
void* noallocScratch(int dev) {
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw std::runtime_error("device ordinal out of range");
    if (!g_noallocAddr[dev]) {
        void* a = nullptr;
        ck(cudaGetSymbolAddress(&a, g_noallocScratch), "cudaGetSymbolAddress(scratch)");
        if (!a) throw std::runtime_error("cudaGetSymbolAddress returned a null scratch address");
        g_noallocAddr[dev] = a;
    }
    return g_noallocAddr[dev];
}

size_t alignUp256(size_t b) { return (b + 255) & ~size_t(255); }

// Reactors that fit the scratch array for a mechanism with N = K + 1 state components:
// one work counter (256 bytes), then per reactor its record, its 8 counters and its
// ignition time.
int noallocCapacity(int N) {
    const size_t per = (size_t)bdfRecordStride(N) * 8 + 64 + 8;
    const size_t avail = kNoAllocScratchBytes - 256 - 3 * 256;
    return (int)std::min<size_t>(avail / per, (size_t)INT32_MAX);
}

void requireDevicePointer(const void* ptr, int dev, const char* what) {
    cudaPointerAttributes a{};
    ck(cudaPointerGetAttributes(&a, ptr), what);
    const bool ok = (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
    if (!ok) throw std::runtime_error(std::string(what) + " must be a device pointer on the current device");
}
// end of a surrogate call: wait for its work unless this thread asked for asynchronous calls
void nnFinish(const char* what) {
    if (!g_nnAsync) ck(cudaStreamSynchronize(g_nnStream), what);
}
}  // namespace

extern "C" {

int32_t gb_get_error(int32_t buflen, char* buf) {
    if (buf && buflen > 0) {
        std::strncpy(buf, g_error.c_str(), (size_t)buflen - 1);
        buf[buflen - 1] = '\0';
    }
    return (int32_t)g_error.size();
}

int32_t gb_add_data_directory(const char* dir) {
    return guarded([&]() -> int32_t {
        if (!dir) throw std::runtime_error("null directory");
        addDataDirectory(dir);
        return 0;
    });
}

int32_t gb_mech_load(const char* path, const char* phase) {
    return guarded([&]() -> int32_t {
        if (!path) throw std::runtime_error("null path");
        auto e = std::make_unique<MechEntry>();
        e->m = loadMechanism(path, phase ? phase : "");
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        ck(cudaDeviceGetAttribute(&e->smCount, cudaDevAttrMultiProcessorCount, dev), "device attribute");
        e->device = dev;
        ck(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "stream");
        packDevMech(*e);
        e->dChk.ensure(4 * sizeof(int));
        ck(cudaMemset(e->dChk.p, 0, 4 * sizeof(int)), "memset");
        e->dm.chk = e->dChk.as<int>();
        std::lock_guard<std::mutex> lk(g_mu);
        g_mechs.push_back(std::move(e));
        return (int32_t)g_mechs.size() - 1;
    });
}

int32_t gb_mech_del(int32_t h) {
    return guarded([&]() -> int32_t {
        mech(h);
        std::lock_guard<std::mutex> lk(g_mu);
        g_mechs[h].reset();
        return 0;
    });
}

int32_t gb_mech_n_species(int32_t h) { return guarded([&]() -> int32_t { return mech(h).m.K; }); }
int32_t gb_mech_n_reactions(int32_t h) { return guarded([&]() -> int32_t { return mech(h).m.R; }); }

int32_t gb_mech_species_name(int32_t h, int32_t k, int32_t buflen, char* buf) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        if (k < 0 || k >= e.m.K) throw std::runtime_error("species index out of range");
        const std::string& s = e.m.speciesNames[k];
        if (buf && buflen > 0) {
            std::strncpy(buf, s.c_str(), (size_t)buflen - 1);
            buf[buflen - 1] = '\0';
        }
        return (int32_t)s.size();
    });
}

int32_t gb_mech_species_index(int32_t h, const char* name) {
    return guarded([&]() -> int32_t { return mech(h).m.speciesIndex(name ? name : ""); });
}

int32_t gb_mech_molecular_weights(int32_t h, int32_t buflen, double* mw) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        if (buflen < e.m.K) throw std::runtime_error("buffer too small for molecular weights");
        std::copy(e.m.mw.begin(), e.m.mw.end(), mw);
        return 0;
    });
}

int32_t gb_mech_equivalence_ratio(int32_t h, double phi, const double* fuelX, const double* oxX,
                                  int32_t buflen, double* Y) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        if (buflen < e.m.K) throw std::runtime_error("buffer too small for mass fractions");
        if (!fuelX || !oxX || !Y) throw std::runtime_error("null array argument");
        equivalenceRatioMassFractions(e.m, phi, fuelX, oxX, Y);
        return 0;
    });
}

int32_t gb_mech_species_thermo(int32_t h, int32_t n, const double* T, double* cp_R, double* h_RT, double* s_R) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        const Mechanism& m = e.m;
        if (n < 0) throw std::runtime_error("negative number of temperatures");
        if (!T || !cp_R || !h_RT || !s_R) throw std::runtime_error("null array argument");
        for (int s = 0; s < n; s++) {
            const double t = T[s];
            if (!(t > 0.0)) throw std::runtime_error("temperature must be positive");
            const double lt = std::log(t), rt = 1.0 / t;
            for (int k = 0; k < m.K; k++) {
                // NASA7: the low range up to and including the midpoint temperature
                const double* a = (t <= m.nasaTmid[k] ? m.nasaLow.data() : m.nasaHigh.data()) + 7 * (size_t)k;
                const size_t o = (size_t)k * n + s;
                cp_R[o] = a[0] + t * (a[1] + t * (a[2] + t * (a[3] + t * a[4])));
                h_RT[o] = a[0] + t * (a[1] / 2 + t * (a[2] / 3 + t * (a[3] / 4 + t * a[4] / 5))) + a[5] * rt;
                s_R[o] = a[0] * lt + t * (a[1] + t * (a[2] / 2 + t * (a[3] / 3 + t * a[4] / 4))) + a[6];
            }
        }
        return 0;
    });
}

double gb_mech_reference_pressure(int32_t h) {
    try {
        return mech(h).m.Pref;
    } catch (std::exception& ex) {
        g_error = ex.what();
        return -999.999;
    }
}

int32_t gb_kin_net_production_rates(int32_t h, int32_t n, const double* T, const double* P, const double* Y,
                                    int32_t bufLen, double* wdot, int32_t flags) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        if ((int64_t)bufLen < (int64_t)e.m.K * n) throw std::runtime_error("wdot buffer too small: need K*n");
        if (!T || !P || !Y || !wdot) throw std::runtime_error("null array argument");
        return runRates(h, n, T, P, Y, wdot, nullptr, flags);
    });
}

int32_t gb_mech_structure(int32_t h, int32_t ncounts, int64_t* counts) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        const Mechanism& m = e.m;
        if (ncounts < 12) throw std::runtime_error("need 12 counts");
        int64_t rev = 0, fo = 0, troe = 0, rslots = 0, pslots = 0;
        for (int i = 0; i < m.R; i++) {
            rev += m.reversible[i];
            fo += isFalloffKind(m.kind[i]);
            troe += (m.kind[i] == kTroe);
            for (int j = m.reacPtr[i]; j < m.reacPtr[i + 1]; j++) rslots += (int64_t)m.reacNu[j];
            for (int j = m.prodPtr[i]; j < m.prodPtr[i + 1]; j++) pslots += (int64_t)m.prodNu[j];
        }
        // gather / Jacobian list sizes are those of the packed device layout
        std::vector<int> spPtr(e.m.K + 1), colPtr(e.m.K + 1), rsPtr(e.m.R + 1);
        ck(cudaMemcpy(spPtr.data(), e.dm.spPtr, spPtr.size() * 4, cudaMemcpyDeviceToHost), "copy");
        ck(cudaMemcpy(colPtr.data(), e.dm.colPtr, colPtr.size() * 4, cudaMemcpyDeviceToHost), "copy");
        ck(cudaMemcpy(rsPtr.data(), e.dm.rsPtr, rsPtr.size() * 4, cudaMemcpyDeviceToHost), "copy");
        std::vector<int> colRxn(colPtr.back());
        if (!colRxn.empty())
            ck(cudaMemcpy(colRxn.data(), e.dm.colRxn, colRxn.size() * 4, cudaMemcpyDeviceToHost), "copy");
        int64_t scatter = 0;
        for (int r : colRxn) scatter += rsPtr[r + 1] - rsPtr[r];
        counts[0] = m.K; counts[1] = m.R; counts[2] = rev; counts[3] = fo; counts[4] = troe;
        counts[5] = m.nThirdBody(); counts[6] = (int64_t)m.tbSpecies.size(); counts[7] = spPtr.back();
        counts[8] = colPtr.back(); counts[9] = scatter; counts[10] = rslots; counts[11] = pslots;
        if (ncounts >= 16) {   // the device arena: what a right-hand side reads, + a Jacobian, + side lists, total
            counts[12] = e.dm.hotBytes; counts[13] = e.dm.jacBytes; counts[14] = e.dm.sideBytes;
            counts[15] = (int64_t)e.arena.bytes;
        }
        return 0;
    });
}

int32_t gb_measure_fp64(double* results) {
    return guarded([&]() -> int32_t {
        int dev = 0, sms = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
        ck(measureFp64(results, sms), "fp64 probe");
        return 0;
    });
}

int32_t gb_check_log(int32_t n, const double* x, double* mine, double* lib) {
    return guarded([&]() -> int32_t {
        if (n < 0 || !x || !mine || !lib) throw std::runtime_error("bad arguments");
        ck(checkLog(n, x, mine, lib), "log check");
        return 0;
    });
}

int32_t gb_check_exp(int32_t n, const double* x, double* mine, double* lib) {
    return guarded([&]() -> int32_t {
        if (n < 0 || !x || !mine || !lib) throw std::runtime_error("bad arguments");
        ck(checkExp(n, x, mine, lib), "exp check");
        return 0;
    });
}

int32_t gb_kin_jac_nnz(int32_t h) {
    return guarded([&]() -> int32_t { return (int32_t)mech(h).jrIdx.size(); });
}

int32_t gb_kin_jac_pattern(int32_t h, int32_t ncolptr, int32_t* colptr, int32_t nnz, int32_t* rowidx) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        if (ncolptr < (int32_t)e.jcPtr.size() || nnz < (int32_t)e.jrIdx.size())
            throw std::runtime_error("pattern buffers too small");
        std::copy(e.jcPtr.begin(), e.jcPtr.end(), colptr);
        std::copy(e.jrIdx.begin(), e.jrIdx.end(), rowidx);
        return 0;
    });
}

int32_t gb_kin_net_production_rates_ddCi(int32_t h, int32_t n, const double* T, const double* P, const double* Y,
                                         int32_t nnz, double* vals, double* wdot, int32_t flags) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        if (nnz < (int32_t)e.jrIdx.size()) throw std::runtime_error("nnz smaller than the Jacobian pattern");
        if (!T || !P || !Y || !vals) throw std::runtime_error("null array argument");
        return runRates(h, n, T, P, Y, wdot, vals, flags);
    });
}

void gb_net_default_options(gb_net_options* o) {
    if (!o) return;
    o->rtol = 1e-9;
    o->atol = 1e-15;
    o->max_steps = 20000;
    o->max_order = 5;
    o->max_time_step = 0.0;
    o->lu_precision = 64;
    o->warps_per_block = 0;
    o->use_graph = 0;
    o->matrix_placement = 0;
    o->mechanism_in_shared = 0;
    o->jacobian_reuse = 0;
    o->lu_staging = 0;
    o->linear_solver = 0;
}

int32_t gb_net_new(int32_t h, int32_t n, const gb_net_options* opts) {
    return guarded([&]() -> int32_t {
        MechEntry& me = mech(h);
        requireMechDevice(me);
        if (n <= 0) throw std::runtime_error("a reactor network needs n > 0 reactors");
        auto ne = std::make_unique<NetEntry>();
        ne->mech = h;
        ne->n = n;
        if (opts) ne->opts = *opts;
        else gb_net_default_options(&ne->opts);
        if (ne->opts.lu_precision != 32 && ne->opts.lu_precision != 64)
            throw std::runtime_error("lu_precision must be 32 or 64");
        if (ne->opts.max_order < 1 || ne->opts.max_order > 5) throw std::runtime_error("max_order must be 1..5");
        if (!(ne->opts.rtol > 0) || !(ne->opts.atol > 0)) throw std::runtime_error("tolerances must be positive");
        if (ne->opts.linear_solver != 0 && ne->opts.linear_solver != 1)
            throw std::runtime_error("linear_solver must be 0 (dense) or 1 (GMRES with the adaptive preconditioner)");
        ne->krylov = ne->opts.linear_solver == 1;
        const int N = me.dm.N;
        const bool fp32 = ne->opts.lu_precision == 32;
        ne->ld = fp32 ? (N % 2 == 0 ? N + 1 : N) : (N % 2 == 0 ? N + 1 : N);
        if (ne->opts.matrix_placement < 0 || ne->opts.matrix_placement > 2)
            throw std::runtime_error("matrix_placement must be 0, 1 or 2");
        if (ne->opts.mechanism_in_shared < 0 || ne->opts.mechanism_in_shared > 4)
            throw std::runtime_error("mechanism_in_shared must be 0..4");
        ne->recStride = bdfRecordStride(N);
        chooseBdfLaunch(me, ne->opts, n, fp32, ne->ld, *ne);
        const int wpb = ne->warpsPerBlock;
        const bool matGlobal = ne->matGlobal;
        if (matGlobal) {
            const size_t elt = fp32 ? 4 : 8;
            ne->Mstride = ((size_t)N * ne->ld * elt + 255) & ~size_t(255);
            ne->dM.ensure(ne->Mstride * (size_t)ne->blocks * wpb);
            ne->JSstride = (((size_t)2 * me.m.R + bdfNordsieckDoubles(N)) * 8 + 255) & ~size_t(255);
            ne->dJS.ensure(ne->JSstride * (size_t)ne->blocks * wpb);
        }
        if (ne->opts.jacobian_reuse || ne->krylov) {   // the Krylov path keeps the preconditioner's Jacobian
            ne->Jstride = ((size_t)N * ne->ld * 8 + 255) & ~size_t(255);
            ne->dJ.ensure(ne->Jstride * (size_t)ne->blocks * wpb);
        }
        if (ne->krylov) {
            ne->dKStats.ensure((size_t)n * 3 * 8);
            ck(cudaMemset(ne->dKStats.p, 0, (size_t)n * 24), "memset");
            ne->dKz.ensure((size_t)kKrylovMaxl * N * 8 * ne->blocks * wpb);   // preconditioned vectors per warp
        }
        const int K = me.m.K;
        ne->dP.ensure((size_t)n * 8);
        ne->dT.ensure((size_t)n * 8);
        ne->dY.ensure((size_t)K * n * 8);
        ne->dRec.ensure((size_t)n * ne->recStride * 8);
        ne->dStats.ensure((size_t)n * 8 * 8);
        ne->dStatus.ensure((size_t)n * 4);
        ne->dTign.ensure((size_t)n * 8);
        ne->dCounter.ensure(sizeof(int));
        ck(cudaEventCreate(&ne->evA), "event");
        ck(cudaEventCreate(&ne->evB), "event");
        ck(cudaMemset(ne->dRec.p, 0, (size_t)n * ne->recStride * 8), "memset");
        ck(cudaMemset(ne->dStats.p, 0, (size_t)n * 64), "memset");
        ck(cudaMemset(ne->dStatus.p, 0, (size_t)n * 4), "memset");
        std::lock_guard<std::mutex> lk(g_mu);
        g_nets.push_back(std::move(ne));
        return (int32_t)g_nets.size() - 1;
    });
}

int32_t gb_net_launch_info(int32_t h, int32_t* info) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        if (!info) throw std::runtime_error("null array argument");
        info[0] = ne.blocks; info[1] = ne.warpsPerBlock; info[2] = ne.warpDoubles * 8;
        info[3] = ne.mechSmem; info[4] = ne.matGlobal ? 2 : 1; info[5] = ne.luSlots;
        return 0;
    });
}

int32_t gb_net_del(int32_t h) {
    return guarded([&]() -> int32_t {
        net(h);
        std::lock_guard<std::mutex> lk(g_mu);
        g_nets[h].reset();
        return 0;
    });
}

int32_t gb_net_set_state(int32_t h, const double* T, const double* P, const double* Y, int32_t flags) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        if (!T || !P || !Y) throw std::runtime_error("null array argument");
        const int K = me.m.K, n = ne.n;
        auto kind = (flags & GB_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        cudaStream_t s = me.stream;
        if (flags & GB_DEVICE_POINTERS) afterCallerWork(me);
        ck(cudaMemcpyAsync(ne.dT.p, T, (size_t)n * 8, kind, s), "copy T");
        ck(cudaMemcpyAsync(ne.dP.p, P, (size_t)n * 8, kind, s), "copy P");
        ck(cudaMemcpyAsync(ne.dY.p, Y, (size_t)K * n * 8, kind, s), "copy Y");
        ck(cudaMemsetAsync(ne.dRec.p, 0, (size_t)n * ne.recStride * 8, s), "reset records");
        ck(cudaMemsetAsync(ne.dStats.p, 0, (size_t)n * 64, s), "reset stats");
        if (ne.krylov) ck(cudaMemsetAsync(ne.dKStats.p, 0, (size_t)n * 24, s), "reset Krylov stats");
        ck(cudaMemsetAsync(ne.dStatus.p, 0, (size_t)n * 4, s), "reset status");
        // queue order: hottest reactors first (they take the most steps), so the
        // longest integrations start early and the tail of the queue is short
        std::vector<double> hT(n);
        if (flags & GB_DEVICE_POINTERS) ck(cudaMemcpyAsync(hT.data(), T, (size_t)n * 8, cudaMemcpyDeviceToHost, s), "copy T");
        else std::copy(T, T + n, hT.begin());
        ck(cudaStreamSynchronize(s), "set state");
        std::vector<int> ord(n);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return hT[a] > hT[b]; });
        ne.dOrder.ensure((size_t)n * 4);
        ck(cudaMemcpy(ne.dOrder.p, ord.data(), (size_t)n * 4, cudaMemcpyHostToDevice), "copy order");
        ne.haveOrder = true;
        ne.time = 0.0;
        return 0;
    });
}

// a captured advance holds the old settings: drop it so that the next advance re-captures
static void dropGraph(NetEntry& ne) {
    if (ne.graph) {
        cudaGraphExecDestroy(ne.graph);
        ne.graph = nullptr;
    }
    ne.graphTout = -1.0;
}

int32_t gb_net_set_tolerances(int32_t h, double rtol, double atol) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        if (!std::isfinite(rtol) || !std::isfinite(atol)) throw std::runtime_error("tolerances must be finite");
        if (rtol > 0.0) ne.opts.rtol = rtol;
        if (atol > 0.0) ne.opts.atol = atol;
        dropGraph(ne);
        return 0;
    });
}

int32_t gb_net_set_max_steps(int32_t h, int32_t max_steps) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        if (max_steps <= 0) throw std::runtime_error("max_steps must be positive");
        ne.opts.max_steps = max_steps;
        dropGraph(ne);
        return 0;
    });
}

int32_t gb_net_set_max_time_step(int32_t h, double max_time_step) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        if (!(max_time_step >= 0.0) || !std::isfinite(max_time_step))
            throw std::runtime_error("max_time_step must be finite and >= 0");
        ne.opts.max_time_step = max_time_step;
        dropGraph(ne);
        return 0;
    });
}

int32_t gb_net_advance(int32_t h, double t) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        if (t < ne.time) throw std::runtime_error("cannot integrate backwards in time");
        if (t == ne.time) return 0;
        cudaStream_t s = me.stream;
        ck(cudaEventRecord(ne.evA, s), "event record");
        if (ne.opts.use_graph) {
            if (!ne.graph || ne.graphTout != t) {
                if (ne.graph) { cudaGraphExecDestroy(ne.graph); ne.graph = nullptr; }
                cudaGraph_t g;
                ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
                netLaunch(ne, me, ne.time, t);
                ck(cudaStreamEndCapture(s, &g), "end capture");
                ck(cudaGraphInstantiate(&ne.graph, g, 0), "graph instantiate");
                cudaGraphDestroy(g);
                ne.graphTout = t;
            }
            ck(cudaGraphLaunch(ne.graph, s), "graph launch");
        } else {
            netLaunch(ne, me, ne.time, t);
        }
        ck(cudaEventRecord(ne.evB, s), "event record");
        ck(cudaStreamSynchronize(s), "integrator");
        float ms = 0.f;
        ck(cudaEventElapsedTime(&ms, ne.evA, ne.evB), "event time");
        ne.lastMs = ms;
        ne.time = t;
        std::vector<int> st(ne.n);
        ck(cudaMemcpy(st.data(), ne.dStatus.p, (size_t)ne.n * 4, cudaMemcpyDeviceToHost), "copy status");
        int bad = 0;
        for (int v : st) bad += (v != 0);
        return bad;
    });
}

int32_t gb_net_step(int32_t h, double* times, int32_t flags) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        cudaStream_t s = me.stream;
        ne.dTnow.ensure((size_t)ne.n * 8);
        ck(cudaEventRecord(ne.evA, s), "event record");
        // one CV_ONE_STEP call per reactor towards time + 1 (the reference's tout), no graph:
        // the captured advance stays valid for the next gb_net_advance
        netLaunch(ne, me, ne.time, ne.time + 1.0, true);
        ck(cudaEventRecord(ne.evB, s), "event record");
        ck(cudaStreamSynchronize(s), "integrator step");
        float ms = 0.f;
        ck(cudaEventElapsedTime(&ms, ne.evA, ne.evB), "event time");
        ne.lastMs = ms;
        std::vector<double> tn(ne.n);
        ck(cudaMemcpy(tn.data(), ne.dTnow.p, (size_t)ne.n * 8, cudaMemcpyDeviceToHost), "copy times");
        if (times) {
            auto kind = (flags & GB_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
            ck(cudaMemcpy(times, ne.dTnow.p, (size_t)ne.n * 8, kind), "copy times");
        }
        // the network's time: the latest reactor time, from which every reactor can go on
        // (an advance to an earlier time would have to reach back past a reactor's last step)
        ne.time = *std::max_element(tn.begin(), tn.end());
        std::vector<int> st(ne.n);
        ck(cudaMemcpy(st.data(), ne.dStatus.p, (size_t)ne.n * 4, cudaMemcpyDeviceToHost), "copy status");
        int bad = 0;
        for (int v : st) bad += (v != 0);
        return bad;
    });
}

/* ---- checkpoint / restore of a network's integrator records ------------------------- */
namespace {
constexpr int64_t kCkptMagic = 0x4B43504B43424747LL;   // "GGBCKPCK"
constexpr int64_t kCkptVersion = 1;
struct CkptLayout {
    size_t header, rec, stats, status, tign, T, P, Y, kstats, total;
};
CkptLayout ckptLayout(const NetEntry& ne, int K) {
    CkptLayout L{};
    const size_t n = (size_t)ne.n;
    auto up8 = [](size_t b) { return (b + 7) & ~size_t(7); };
    L.header = 8 * 8 + 8;                               // 8 int64 fields, then the time
    L.rec = L.header;
    L.stats = L.rec + n * ne.recStride * 8;
    L.status = L.stats + n * 64;
    L.tign = L.status + up8(n * 4);
    L.T = L.tign + n * 8;
    L.P = L.T + n * 8;
    L.Y = L.P + n * 8;
    L.kstats = L.Y + (size_t)K * n * 8;                // the Krylov path's counters (its networks only)
    L.total = L.kstats + (ne.krylov ? n * 24 : 0);
    return L;
}
}  // namespace

int64_t gb_net_checkpoint_bytes(int32_t h) {
    try {
        NetEntry& ne = net(h);
        return (int64_t)ckptLayout(ne, mech(ne.mech).m.K).total;
    } catch (std::exception& e) {
        g_error = e.what();
        return GB_ERR;
    }
}

int32_t gb_net_checkpoint(int32_t h, void* buf, int64_t bytes) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        const int K = me.m.K;
        const CkptLayout L = ckptLayout(ne, K);
        if (!buf || bytes < (int64_t)L.total) throw std::runtime_error("checkpoint buffer smaller than gb_net_checkpoint_bytes");
        char* b = (char*)buf;
        int64_t hd[8] = {kCkptMagic, kCkptVersion, ne.n, me.dm.N, ne.recStride, K, ne.krylov ? 1 : 0, 0};
        std::memcpy(b, hd, sizeof(hd));
        std::memcpy(b + 64, &ne.time, 8);
        const size_t n = (size_t)ne.n;
        ck(cudaStreamSynchronize(me.stream), "checkpoint");
        ck(cudaMemcpy(b + L.rec, ne.dRec.p, n * ne.recStride * 8, cudaMemcpyDeviceToHost), "checkpoint records");
        ck(cudaMemcpy(b + L.stats, ne.dStats.p, n * 64, cudaMemcpyDeviceToHost), "checkpoint stats");
        ck(cudaMemcpy(b + L.status, ne.dStatus.p, n * 4, cudaMemcpyDeviceToHost), "checkpoint status");
        ck(cudaMemcpy(b + L.tign, ne.dTign.p, n * 8, cudaMemcpyDeviceToHost), "checkpoint ignition");
        ck(cudaMemcpy(b + L.T, ne.dT.p, n * 8, cudaMemcpyDeviceToHost), "checkpoint T");
        ck(cudaMemcpy(b + L.P, ne.dP.p, n * 8, cudaMemcpyDeviceToHost), "checkpoint P");
        ck(cudaMemcpy(b + L.Y, ne.dY.p, (size_t)K * n * 8, cudaMemcpyDeviceToHost), "checkpoint Y");
        if (ne.krylov) ck(cudaMemcpy(b + L.kstats, ne.dKStats.p, n * 24, cudaMemcpyDeviceToHost), "checkpoint Krylov stats");
        return 0;
    });
}

int32_t gb_net_restore(int32_t h, const void* buf, int64_t bytes) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        const int K = me.m.K;
        const CkptLayout L = ckptLayout(ne, K);
        if (!buf || bytes < (int64_t)L.header) throw std::runtime_error("checkpoint buffer too small for this network");
        const char* b = (const char*)buf;
        int64_t hd[8];
        std::memcpy(hd, b, sizeof(hd));
        if (hd[0] != kCkptMagic || hd[1] != kCkptVersion) throw std::runtime_error("not a reactor-network checkpoint");
        if (hd[2] != ne.n || hd[3] != me.dm.N || hd[4] != ne.recStride || hd[5] != K)
            throw std::runtime_error("checkpoint of a network of another size or mechanism");
        if (hd[6] != (ne.krylov ? 1 : 0))
            throw std::runtime_error("checkpoint of a network with the other linear solver (its records hold other state variables)");
        if (bytes < (int64_t)L.total) throw std::runtime_error("checkpoint buffer too small for this network");
        double t = 0.0;
        std::memcpy(&t, b + 64, 8);
        if (!std::isfinite(t) || t < 0.0) throw std::runtime_error("checkpoint time is not valid");
        const size_t n = (size_t)ne.n;
        cudaStream_t s = me.stream;
        ck(cudaStreamSynchronize(s), "restore");
        ck(cudaMemcpy(ne.dRec.p, b + L.rec, n * ne.recStride * 8, cudaMemcpyHostToDevice), "restore records");
        ck(cudaMemcpy(ne.dStats.p, b + L.stats, n * 64, cudaMemcpyHostToDevice), "restore stats");
        ck(cudaMemcpy(ne.dStatus.p, b + L.status, n * 4, cudaMemcpyHostToDevice), "restore status");
        ck(cudaMemcpy(ne.dTign.p, b + L.tign, n * 8, cudaMemcpyHostToDevice), "restore ignition");
        ck(cudaMemcpy(ne.dT.p, b + L.T, n * 8, cudaMemcpyHostToDevice), "restore T");
        ck(cudaMemcpy(ne.dP.p, b + L.P, n * 8, cudaMemcpyHostToDevice), "restore P");
        ck(cudaMemcpy(ne.dY.p, b + L.Y, (size_t)K * n * 8, cudaMemcpyHostToDevice), "restore Y");
        if (ne.krylov) ck(cudaMemcpy(ne.dKStats.p, b + L.kstats, n * 24, cudaMemcpyHostToDevice), "restore Krylov stats");
        // queue order as gb_net_set_state makes it (hottest first); it only schedules
        std::vector<double> hT(n);
        std::memcpy(hT.data(), b + L.T, n * 8);
        std::vector<int> ord(n);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return hT[a] > hT[c]; });
        ne.dOrder.ensure(n * 4);
        ck(cudaMemcpy(ne.dOrder.p, ord.data(), n * 4, cudaMemcpyHostToDevice), "restore order");
        ne.haveOrder = true;
        ne.time = t;
        dropGraph(ne);
        return 0;
    });
}

int32_t gb_check_status(int32_t h, int32_t* out) {
    return guarded([&]() -> int32_t {
        MechEntry& me = mech(h);
        requireMechDevice(me);
        if (!out) throw std::runtime_error("null array argument");
        int v[4] = {0, 0, 0, 0};
        ck(cudaDeviceSynchronize(), "check status");
        ck(cudaMemcpy(v, me.dChk.p, sizeof(v), cudaMemcpyDeviceToHost), "check status");
        ck(cudaMemset(me.dChk.p, 0, sizeof(v)), "check status");
        out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
#ifdef GBCHEM_CHECKED
        return 1;
#else
        return 0;
#endif
    });
}

double gb_kin_last_kernel_ms(int32_t h) {
    try {
        return mech(h).lastMs;
    } catch (std::exception& e) {
        g_error = e.what();
        return -999.999;
    }
}

double gb_net_time(int32_t h) {
    try {
        return net(h).time;
    } catch (std::exception& e) {
        g_error = e.what();
        return -999.999;
    }
}

double gb_net_last_advance_ms(int32_t h) {
    try {
        return net(h).lastMs;
    } catch (std::exception& e) {
        g_error = e.what();
        return -999.999;
    }
}

int32_t gb_net_get_state(int32_t h, double* T, double* Y, int32_t flags) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        auto kind = (flags & GB_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (T) ck(cudaMemcpy(T, ne.dT.p, (size_t)ne.n * 8, kind), "copy T");
        if (Y) ck(cudaMemcpy(Y, ne.dY.p, (size_t)me.m.K * ne.n * 8, kind), "copy Y");
        return 0;
    });
}

int32_t gb_net_get_derivative(int32_t h, int32_t k, double* out, int32_t flags) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        MechEntry& me = mech(ne.mech);
        requireMechDevice(me);
        const BdfRecordLayout L = bdfRecordLayout();
        if (!out) throw std::runtime_error("null array argument");
        if (k < 0 || k > L.qmax) throw std::runtime_error("derivative order k must be in 0.." + std::to_string(L.qmax));
        const int N = me.m.K + 1, n = ne.n;
        const size_t stride = (size_t)ne.recStride;
        std::vector<double> rec((size_t)n * stride);
        ck(cudaStreamSynchronize(me.stream), "integrator");
        ck(cudaMemcpy(rec.data(), ne.dRec.p, rec.size() * 8, cudaMemcpyDeviceToHost), "copy records");
        // c[j] = j! / (j - k)! for j >= k
        double c[16] = {0.0};
        for (int j = k; j <= L.qmax; j++) {
            double v = 1.0;
            for (int i = j - k + 1; i <= j; i++) v *= i;
            c[j] = v;
        }
        std::vector<double> res((size_t)N * n);
        for (int r = 0; r < n; r++) {
            const double* z = rec.data() + (size_t)r * stride;
            const double* o = z + (size_t)(L.qmax + 1) * N;
            if (!(((int)o[L.flags]) & L.initFlag))
                throw std::runtime_error("reactor " + std::to_string(r) + " has not been integrated since its state was set");
            const double tn = o[L.tn], hh = o[L.h];
            const int q = (int)o[L.q];
            // the reactor's output time: the network's time after an advance (within the last
            // step, tn >= t), its own internal time after a step or a failure (tn <= t)
            const double t = std::min(ne.time, tn);
            const double s = hh != 0.0 ? (t - tn) / hh : 0.0;
            const double hk = (k == 0) ? 1.0 : (hh != 0.0 ? std::pow(hh, -k) : 0.0);
            for (int i = 0; i < N; i++) {
                double v = 0.0;
                if (q >= k) {
                    v = c[q] * z[(size_t)q * N + i];
                    for (int j = q - 1; j >= k; j--) v = c[j] * z[(size_t)j * N + i] + s * v;
                }
                res[(size_t)i * n + r] = v * hk;
            }
        }
        auto kind = (flags & GB_DEVICE_POINTERS) ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
        ck(cudaMemcpy(out, res.data(), res.size() * 8, kind), "copy derivative");
        return 0;
    });
}

int32_t gb_net_get_status(int32_t h, int32_t* status) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        ck(cudaMemcpy(status, ne.dStatus.p, (size_t)ne.n * 4, cudaMemcpyDeviceToHost), "copy status");
        return 0;
    });
}

int32_t gb_net_solver_stats(int32_t h, int64_t* stats) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        ck(cudaMemcpy(stats, ne.dStats.p, (size_t)ne.n * 64, cudaMemcpyDeviceToHost), "copy stats");
        return 0;
    });
}

int32_t gb_net_krylov_stats(int32_t h, int64_t* stats) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        if (!stats) throw std::runtime_error("null array argument");
        if (!ne.krylov) throw std::runtime_error("the network uses the dense linear solver (linear_solver 0)");
        ck(cudaMemcpy(stats, ne.dKStats.p, (size_t)ne.n * 24, cudaMemcpyDeviceToHost), "copy Krylov stats");
        return 0;
    });
}

int32_t gb_precond_ilut(int32_t n, int32_t N, const double* P, double* F) {
    return guarded([&]() -> int32_t {
        if (n <= 0 || N <= 0 || N > 256) throw std::runtime_error("need n > 0 matrices of order 1..256");
        if (!P || !F) throw std::runtime_error("null array argument");
        int dev = -1;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        const int ld = (N % 2 == 0) ? N + 1 : N;
        const size_t per = (size_t)N * ld;
        std::vector<double> h((size_t)n * per, 0.0);
        for (int r = 0; r < n; r++)   // transposed: row j holds column j
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++) h[r * per + (size_t)j * ld + i] = P[((size_t)r * N + i) * N + j];
        DBuf a, dinv, rn;
        a.ensure(h.size() * 8);
        dinv.ensure((size_t)n * N * 8);
        rn.ensure((size_t)n * N * 8);
        ck(cudaMemcpy(a.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice), "copy matrices");
        ck(launchIlut(n, N, ld, a.as<double>(), dinv.as<double>(), rn.as<double>(), nullptr), "ILUT launch");
        ck(cudaMemcpy(h.data(), a.p, h.size() * 8, cudaMemcpyDeviceToHost), "copy factors");
        for (int r = 0; r < n; r++)
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++) F[((size_t)r * N + i) * N + j] = h[r * per + (size_t)j * ld + i];
        return 0;
    });
}

int32_t gb_net_ignition_times(int32_t h, double* tign) {
    return guarded([&]() -> int32_t {
        NetEntry& ne = net(h);
        ck(cudaMemcpy(tign, ne.dTign.p, (size_t)ne.n * 8, cudaMemcpyDeviceToHost), "copy tign");
        return 0;
    });
}

int32_t gb_reactors_advance_noalloc(int32_t h, int32_t n, double t_end, double* T, const double* P,
                                    double* Y, int32_t* status, const gb_net_options* opts,
                                    void* stream) {
    return guarded([&]() -> int32_t {
        MechEntry& me = mech(h);
        requireMechDevice(me);
        if (n <= 0) throw std::runtime_error("need n > 0 reactors");
        if (!T || !P || !Y || !status) throw std::runtime_error("null array argument");
        if (!(t_end > 0) || !std::isfinite(t_end)) throw std::runtime_error("t_end must be positive and finite");
        gb_net_options o;
        if (opts) o = *opts;
        else gb_net_default_options(&o);
        if (o.lu_precision != 32 && o.lu_precision != 64) throw std::runtime_error("lu_precision must be 32 or 64");
        if (o.max_order < 1 || o.max_order > 5) throw std::runtime_error("max_order must be 1..5");
        if (!(o.rtol > 0) || !(o.atol > 0)) throw std::runtime_error("tolerances must be positive");
        if (o.linear_solver != 0)
            throw std::runtime_error("the allocation-free advance runs the dense linear solver only (linear_solver 0)");
        const int N = me.dm.N;
        const int cap = noallocCapacity(N);
        if (n > cap)
            throw std::runtime_error("gb_reactors_advance_noalloc: n = " + std::to_string(n) +
                                     " exceeds the maximum of " + std::to_string(cap) +
                                     " reactors that its 16 MiB scratch holds for this mechanism");
        cudaStream_t s = (cudaStream_t)stream;
        // the call synchronises its stream and queries pointers, neither of which a stream
        // capture allows: refuse before touching the stream
        cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
        ck(cudaStreamIsCapturing(s, &cap_status), "cudaStreamIsCapturing");
        if (cap_status != cudaStreamCaptureStatusNone)
            throw std::runtime_error("gb_reactors_advance_noalloc cannot be called while its stream is being captured");
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        requireDevicePointer(T, dev, "T");
        requireDevicePointer(P, dev, "P");
        requireDevicePointer(Y, dev, "Y");
        requireDevicePointer(status, dev, "status");

        const bool fp32 = o.lu_precision == 32;
        const int ld = (N % 2 == 0) ? N + 1 : N;
        const int warpDoubles = bdfWarpDoubles(me.dm, ld, fp32);
        const int recStride = bdfRecordStride(N);
        const int fit = maxSmemPerBlock() / (warpDoubles * 8);
        if (fit < 1) throw std::runtime_error("mechanism too large for one warp's shared memory");
        const int wpb = std::min(std::min(o.warps_per_block > 0 ? o.warps_per_block : 8, kBdfMaxThreads / 32), fit);
        // resident blocks per SM from the occupancy calculator (registers included), as the
        // network path chooses its grid
        const int blocksPerSm = bdfBlocksPerSm(N, fp32, wpb, (size_t)warpDoubles * 8 * wpb, me.dm.NX > 0);
        const int blocks = std::min(me.smCount * blocksPerSm, (n + wpb - 1) / wpb);

        std::lock_guard<std::mutex> lk(g_noallocMu);
        char* base = (char*)noallocScratch(dev);
        int* counter = (int*)base;
        const size_t recBytes = (size_t)n * recStride * 8;
        double* rec = (double*)(base + 256);
        long long* stats = (long long*)(base + 256 + alignUp256(recBytes));
        double* tign = (double*)((char*)stats + alignUp256((size_t)n * 64));
        // Must start at zero: the work counter, and each record (a record whose flags
        // word is zero makes the kernel start that reactor from T, P, Y at time 0).
        ck(cudaMemsetAsync(counter, 0, sizeof(int), s), "reset counter");
        ck(cudaMemsetAsync(rec, 0, recBytes, s), "reset records");
        BdfParams p{};
        p.m = me.dm; p.n = n; p.t0 = 0.0; p.tout = t_end;
        p.rtol = o.rtol; p.atol = o.atol;
        p.hmaxInv = o.max_time_step > 0 ? 1.0 / o.max_time_step : 0.0;
        p.maxSteps = o.max_steps; p.maxOrder = o.max_order;
        p.P = P; p.T = T; p.Y = Y;
        p.rec = rec; p.recStride = recStride;
        p.stats = stats; p.status = status; p.tign = tign;
        p.counter = counter; p.order = nullptr;
        p.ld = ld; p.warpDoubles = warpDoubles;
        ck(launchBdf(p, blocks, wpb, fp32, s), "integrator launch");
        ck(cudaStreamSynchronize(s), "integrator");
        return 0;
    });
}

/* ---- batched reactor right-hand side ---------------------------------------------- */
int32_t gb_reactor_rhs(int32_t h, int32_t n, const double* T, const double* P, const double* Y, double* dTdt,
                       double* dYdt, int32_t flags) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        requireMechDevice(e);
        if (n < 0) throw std::runtime_error("negative number of states");
        if (n == 0) return 0;
        if (!T || !P || !Y || !dTdt || !dYdt) throw std::runtime_error("null array argument");
        const bool dev = (flags & GB_DEVICE_POINTERS) != 0;
        const int K = e.m.K;
        cudaStream_t s = e.stream;
        if (dev) afterCallerWork(e);
        const double* dT = stage(T, n, e.dT, dev, s);
        const double* dP = stage(P, n, e.dP, dev, s);
        const double* dY = stage(Y, (size_t)K * n, e.dY, dev, s);
        double* oT = dTdt;
        double* oY = dYdt;
        if (!dev) {
            e.dW.ensure((size_t)(K + 1) * n * 8);
            oY = e.dW.as<double>();
            oT = oY + (size_t)K * n;
        }
        RhsParams p{};
        p.m = e.dm; p.n = n; p.T = dT; p.P = dP; p.Y = dY; p.dTdt = oT; p.dYdt = oY;
        p.warpDoubles = rhsWarpDoubles(e.dm);
        const int wpb = std::max(1, std::min(8, maxSmemPerBlock() / (p.warpDoubles * 8)));
        const int blocksPerSm = std::max(1, (228 * 1024) / (p.warpDoubles * 8 * wpb + 1024));
        const int blocks = std::max(1, std::min(e.smCount * blocksPerSm, (n + wpb - 1) / wpb));
        ck(launchReactorRhs(p, blocks, wpb, s), "reactor rhs launch");
        if (!dev) {
            ck(cudaMemcpyAsync(dYdt, oY, (size_t)K * n * 8, cudaMemcpyDeviceToHost, s), "copy dYdt");
            ck(cudaMemcpyAsync(dTdt, oT, (size_t)n * 8, cudaMemcpyDeviceToHost, s), "copy dTdt");
        }
        ck(cudaStreamSynchronize(s), "reactor rhs");
        return 0;
    });
}

int32_t gb_mech_n_elements(int32_t h) {
    return guarded([&]() -> int32_t { return (int32_t)mech(h).m.elementNames.size(); });
}

int32_t gb_mech_element_mass(int32_t h, int32_t buflen, double* out) {
    return guarded([&]() -> int32_t {
        const Mechanism& m = mech(h).m;
        const int E = (int)m.elementNames.size(), K = m.K;
        if (!out || buflen < E * K) throw std::runtime_error("element mass buffer too small");
        for (int e = 0; e < E; e++)
            for (int k = 0; k < K; k++) out[(size_t)e * K + k] = m.atoms[(size_t)k * E + e] * m.elementWeights[e] / m.mw[k];
        return 0;
    });
}

/* ---- learned surrogate: tensor-core MLP operations (device pointers) ---------------- */
int32_t gb_nn_gemm(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, int64_t sak, const void* B,
                   int64_t sbn, int64_t sbk, void* C, int64_t scm, int64_t scn, int32_t c_float, float alpha,
                   const float* bias, int32_t act, void* Z, int64_t szm, int64_t szn, int32_t z_float) {
    return guarded([&]() -> int32_t {
        if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 128 || K % 32)
            throw std::runtime_error("gemm: M and N must be positive multiples of 128, K of 32");
        if (!A || !B || !C) throw std::runtime_error("gemm: null operand");
        if (!((sak == 1 && sam % 8 == 0) || (sam == 1 && sak % 8 == 0)))
            throw std::runtime_error("gemm: A needs a unit stride and the other a multiple of 8");
        if (!((sbk == 1 && sbn % 8 == 0) || (sbn == 1 && sbk % 8 == 0)))
            throw std::runtime_error("gemm: B needs a unit stride and the other a multiple of 8");
        if (((uintptr_t)A & 15) || ((uintptr_t)B & 15)) throw std::runtime_error("gemm: A and B must be 16-byte aligned");
        if (act < 0 || act > 2 || (act == 2 && !Z)) throw std::runtime_error("gemm: bad activation arguments");
        GemmArgs g{};
        g.M = M; g.N = N; g.K = K;
        g.A = (const __nv_bfloat16*)A; g.sam = sam; g.sak = sak;
        g.B = (const __nv_bfloat16*)B; g.sbn = sbn; g.sbk = sbk;
        g.C = C; g.scm = scm; g.scn = scn; g.cFloat = c_float;
        g.alpha = alpha; g.bias = bias; g.act = act; g.Z = Z; g.szm = szm; g.szn = szn; g.zFloat = z_float;
        ck(launchGemm(g, g_nnStream), "gemm launch");
        nnFinish("gemm");
        return 0;
    });
}

int32_t gb_nn_set_stream(void* stream, int32_t async) {
    return guarded([&]() -> int32_t {
        g_nnStream = (cudaStream_t)stream;
        g_nnAsync = async != 0;
        return 0;
    });
}

int32_t gb_nn_gemm_tc(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb,
                      void* C, int64_t ldc, int32_t c_float, float alpha, const float* bias, int32_t act, void* Z,
                      int64_t ldz, int32_t z_float, void* CT, int64_t ldct, int32_t splits, void* stream) {
    return guarded([&]() -> int32_t {
        if (!A || !B || !C) throw std::runtime_error("gemm_tc: null operand");
        if (act < 0 || act > 2) throw std::runtime_error("gemm_tc: act must be 0, 1 or 2");
        UmmaArgs g{};
        g.M = M; g.N = N; g.K = K;
        g.A = (const __nv_bfloat16*)A; g.lda = lda;
        g.B = (const __nv_bfloat16*)B; g.ldb = ldb;
        g.C = C; g.ldc = ldc; g.cFloat = c_float;
        g.alpha = alpha; g.bias = bias; g.act = act; g.Z = Z; g.ldz = ldz; g.zFloat = z_float;
        g.CT = (__nv_bfloat16*)CT; g.ldct = ldct;
        if (const char* why = checkUmmaArgs(g, splits)) throw std::runtime_error(std::string("gemm_tc: ") + why);
        cudaStream_t s = (cudaStream_t)stream;
        if (splits > 1)   // the CTAs add their partial tiles into C
            ck(cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, (size_t)M, s), "gemm_tc: clear C");
        ck(launchUmma(g, splits, s), "gemm_tc launch");
        return 0;
    });
}

int32_t gb_nn_transpose(int32_t M, int32_t N, const void* src, int64_t lds, void* dst, int64_t ldd, void* stream) {
    return guarded([&]() -> int32_t {
        if (M < 0 || N < 0 || lds < N || ldd < M) throw std::runtime_error("transpose: bad sizes");
        if (M && N && (!src || !dst)) throw std::runtime_error("transpose: null array");
        ck(launchTranspose(M, N, (const __nv_bfloat16*)src, lds, (__nv_bfloat16*)dst, ldd, (cudaStream_t)stream),
           "transpose launch");
        return 0;
    });
}

int32_t gb_nn_sync(void* stream) {
    return guarded([&]() -> int32_t {
        ck(cudaStreamSynchronize((cudaStream_t)stream), "surrogate stream");
        const int e = ummaTakeError();
        if (e < 0) throw std::runtime_error("gemm_tc: cannot read the error flag");
        if (e) throw std::runtime_error("gemm_tc: a tensor-core GEMM block gave up waiting for its operands or "
                                        "its accumulator (bounded wait ran out); its output tile is not written");
        return 0;
    });
}

int32_t gb_nn_adam(int32_t n, float* w, float* m, float* v, const float* g, void* wb, float lr, float beta1,
                   float beta2, float eps, int32_t step) {
    return guarded([&]() -> int32_t {
        if (n < 0 || !w || !m || !v || !g || !wb || step < 1) throw std::runtime_error("adam: bad arguments");
        ck(launchAdam(n, w, m, v, g, (__nv_bfloat16*)wb, lr, beta1, beta2, eps, step, g_nnStream), "adam launch");
        nnFinish("adam");
        return 0;
    });
}

int32_t gb_nn_colsum(int32_t M, int32_t N, const void* X, int32_t ld, float alpha, float* out) {
    return guarded([&]() -> int32_t {
        if (M < 0 || N < 0 || ld < N || !X || !out) throw std::runtime_error("colsum: bad arguments");
        ck(launchColSum(M, N, (const __nv_bfloat16*)X, ld, alpha, out, g_nnStream), "colsum launch");
        nnFinish("colsum");
        return 0;
    });
}

int32_t gb_nn_mse(int32_t M, int32_t nout, int32_t ld, const float* P, const float* Y, void* dY, float* loss) {
    return guarded([&]() -> int32_t {
        if (M < 0 || nout < 0 || ld < nout || !P || !Y || !dY || !loss) throw std::runtime_error("mse: bad arguments");
        ck(launchMseGrad(M, nout, ld, P, Y, (__nv_bfloat16*)dY, loss, g_nnStream), "mse launch");
        nnFinish("mse");
        return 0;
    });
}

int32_t gb_nn_features(int32_t h, int32_t n, const double* T, const double* P, const double* Y, const float* mu,
                       const float* sd, void* X, int32_t ldx) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        requireMechDevice(e);
        if (n < 0 || ldx < e.m.K + 2 || !T || !P || !Y || !mu || !sd || !X) throw std::runtime_error("features: bad arguments");
        ck(launchFeatures(n, e.m.K, T, P, Y, mu, sd, (__nv_bfloat16*)X, ldx, g_nnStream), "features launch");
        nnFinish("features");
        return 0;
    });
}

int32_t gb_nn_apply(int32_t h, int32_t n, const float* O, int32_t ldo, const float* mu, const float* sd,
                    const double* T, const double* Y, double dt, const double* f0T, const double* f0Y, double* Tn,
                    double* Yn) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        requireMechDevice(e);
        if (n < 0 || ldo < e.m.K + 1 || !O || !mu || !sd || !T || !Y || !Tn || !Yn) throw std::runtime_error("apply: bad arguments");
        if ((f0T == nullptr) != (f0Y == nullptr)) throw std::runtime_error("apply: give both f0T and f0Y or neither");
        ck(launchApplyDelta(n, e.m.K, O, ldo, mu, sd, T, Y, dt, f0T, f0Y, Tn, Yn, g_nnStream), "apply launch");
        nnFinish("apply");
        return 0;
    });
}

int32_t gb_nn_gate(int32_t h, int32_t n, double dt, const double* T0, const double* Y0, const double* T1,
                   const double* Y1, const double* f0T, const double* f0Y, const double* f1T, const double* f1Y,
                   const double* elem_mass, double tol_elem, double tol_h, double tol_trap_t, double tol_trap_y,
                   int32_t* accept, double* score) {
    return guarded([&]() -> int32_t {
        MechEntry& e = mech(h);
        requireMechDevice(e);
        if (n < 0 || !T0 || !Y0 || !T1 || !Y1 || !f0T || !f0Y || !f1T || !f1Y || !elem_mass || !accept || !score)
            throw std::runtime_error("gate: bad arguments");
        GateArgs a{};
        a.n = n; a.K = e.m.K; a.E = (int)e.m.elementNames.size(); a.dt = dt;
        a.T0 = T0; a.Y0 = Y0; a.T1 = T1; a.Y1 = Y1; a.f0T = f0T; a.f0Y = f0Y; a.f1T = f1T; a.f1Y = f1Y;
        a.elemW = elem_mass; a.nasa = e.dm.nasa; a.Rgas = e.dm.Rgas; a.rmw = e.dm.rmw;
        a.tolElem = tol_elem; a.tolH = tol_h; a.tolTrapT = tol_trap_t; a.tolTrapY = tol_trap_y;
        a.accept = accept; a.score = score;
        ck(launchGate(a, 0), "gate launch");
        ck(cudaStreamSynchronize(0), "gate");
        return 0;
    });
}

}  // extern "C"
