// kinetics.cuh - warp-cooperative FP64 kinetics for one gas state per warp.
//
// One warp owns one state (T, P, Y[K]): lanes stride over species for thermo and the
// production-rate gather, over reactions for the rate constants and rates of progress,
// and over Jacobian columns for d(wdot)/dc.  Per-state scratch lives in the warp's slice
// of shared memory.  Operation semantics follow the reference:
//   NASA7                     include/cantera/thermo/NasaPoly1.h:103-122, NasaPoly2.h:105-112
//   state (no normalisation)  src/thermo/Phase.cpp:362-372,501-505; IdealGasPhase.h:338-354
//   chemical potentials       src/thermo/IdealGasPhase.cpp:59-66
//   Kc and reverse rates      src/kinetics/BulkKinetics.cpp:465-484,562-569
//   third bodies              include/cantera/kinetics/ThirdBodyCalc.h:75-92
//   Arrhenius                 include/cantera/kinetics/Arrhenius.h:196-198
//   falloff                   include/cantera/kinetics/Falloff.h:154-176; src/kinetics/Falloff.cpp:283-494
//   pressure-dependent Arrh.  include/cantera/kinetics/PlogRate.h:110-164
//   Chebyshev                 include/cantera/kinetics/ChebyshevRate.h:133-171
//   mass action + sign rules  include/cantera/kinetics/StoichManager.h:131-480
//   d(wdot)/dc                src/kinetics/BulkKinetics.cpp:712-811; StoichManager.h:164-168,227-236,300-312,406-430
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "devmech.h"
#include "fastexp.h"

namespace gbchem {

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warpMax(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// m * 2^e by an exponent-field add; the caller guarantees a normal result
__device__ __forceinline__ double scale2(double m, int e) {
    return __longlong_as_double(__double_as_longlong(m) + ((long long)e << 52));
}
__device__ __forceinline__ double fexp(double x, const uint64_t* tab) { return gbx_exp(x, tab); }

// a < 0 and b < 0 (IEEE comparison semantics, -0 is not negative) on the integer pipe
__device__ __forceinline__ bool bothNeg(double a, double b) {
    const long long la = __double_as_longlong(a), lb = __double_as_longlong(b);
    const long long nz = (long long)0x8000000000000000ULL;
    return (la & lb) < 0 && la != nz && lb != nz;
}

// Per-state scratch in shared memory (sizes in doubles: K, K, K, K, K, R, R, R, NTB, NTB, NF).
struct KinScratch {
    double* c;      // concentrations [K]
    double* cpR;    // cp/R [K]
    double* hRT;    // h/RT [K]
    double* g;      // g/RT + ln(P/Pref) [K]
    double* wdot;   // [K]
    double* rop;    // net rate of progress [R]
    double* kfe;    // forward coefficient times [M] for mass-action three-body reactions [R]
    double* rkc;    // 1/Kc (0 for irreversible) [R]
    double* Mtb;    // third-body concentrations [NTB]
    double* Qtb;    // d(rop)/d[M] per third-body reaction [NTB]
    double* dlk;    // d ln k / d[M] of falloff reactions [NF]
    uint64_t* xu;   // exp(g) = xu / 2^63 * 2^xe  [K]
    uint64_t* xiu;  // exp(-g) = xiu / 2^63 * 2^xie  [K]
    int* xe;        // [K]
    int* xie;       // [K]
    double* pw;     // (RT/P)^dn for dn = -3..3 [8]
    const uint64_t* tab;   // 2^(j/64) table (block shared)
    int* flags;     // [2] per-state flags (bit 0: some |g| >= 700)
    double* part;   // partial sums of the gather tasks [NT]
    // (xu, xiu need 8-byte alignment: they follow doubles)
    // ext: kfe and rkc live elsewhere (they are only written before a Jacobian evaluation)
    __host__ __device__ static int doubles(int K, int R, int NTB, int NF, int NT, bool ext = false) {
        return 5 * K + (ext ? 1 : 3) * R + 2 * NTB + NF + 2 * K + K + 8 + 2 + NT;
    }
    __device__ void carve(double* p, int K, int R, int NTB, int NF, int NT, double* ext = nullptr) {
        c = p; p += K; cpR = p; p += K; hRT = p; p += K; g = p; p += K; wdot = p; p += K;
        rop = p; p += R;
        if (ext) { kfe = ext; rkc = ext + R; }
        else { kfe = p; p += R; rkc = p; p += R; }
        Mtb = p; p += NTB; Qtb = p; p += NTB; dlk = p; p += NF;
        xu = (uint64_t*)p; p += K; xiu = (uint64_t*)p; p += K;
        xe = (int*)p; xie = xe + K; p += K;
        pw = p; p += 8;
        flags = (int*)p; p += 2;
        part = p;
    }
};

// Scalars of the current state, identical in every lane.
struct KinState {
    double T, P, RT, rho, mmw, ctot, lnT, recipT;
    double rrho;       // 1/rho
    double lnPP;       // ln(P/Pref)
    double lnC0;       // ln(P/RT), the log of the standard concentration
    double RTP, PRT;   // RT/P and P/RT
};
constexpr int kKinStateDoubles = 13;

// mass-action product of one side (expanded species list e, count n = e.w) with the
// StoichManager sign rules; `gen` selects the general power-law list (CN bucket).
__device__ __forceinline__ double massAction(const DevMech& m, int bucket, int4 e, int side,
                                             const double* c) {
    if (bucket == 1) return c[e.x];
    if (bucket == 2) {
        double a = c[e.x], b = c[e.y];
        return bothNeg(a, b) ? 0.0 : a * b;
    }
    if (bucket == 3) {
        double a = c[e.x], b = c[e.y], d = c[e.z];
        if (bothNeg(a, b) || bothNeg(a, d) || bothNeg(b, d)) return 0.0;
        return a * b * d;
    }
    double r = 1.0;
#pragma unroll 1
    for (int q = m.sidePtr[side]; q < m.sidePtr[side + 1]; q++) {
        double o = m.sideOrd[q];
        if (o != 0.0) {
            double x = c[GB_IX(m, m.sideK[q], m.K, GB_SITE_SIDE)];
            if (!(x > 0.0)) return 0.0;
            // pow(x, 1) = x and pow(x, 2) = x*x up to rounding
            r *= (o == 1.0) ? x : ((o == 2.0) ? x * x : pow(x, o));
        }
    }
    return r;
}

// d(mass-action product)/dc_j with the StoichManager derivative rules.
__device__ __forceinline__ double massActionDeriv(const DevMech& m, int bucket, int4 e, int side,
                                                  const double* c, int j) {
    if (bucket == 1) return (e.x == j) ? 1.0 : 0.0;
    if (bucket == 2) {
        double d = 0.0;
        if (e.x == j && c[e.y] > 0) d += c[e.y];
        if (e.y == j && c[e.x] > 0) d += c[e.x];
        return d;
    }
    if (bucket == 3) {
        double a = c[e.x], b = c[e.y], f = c[e.z], d = 0.0;
        if (e.x == j && b > 0 && f > 0) d += b * f;
        if (e.y == j && a > 0 && f > 0) d += a * f;
        if (e.z == j && a > 0 && b > 0) d += a * b;
        return d;
    }
    double d = 0.0;
    int q0 = m.sidePtr[side], q1 = m.sidePtr[side + 1];
#pragma unroll 1
    for (int q = q0; q < q1; q++) {
        if (m.sideK[q] != j) continue;
        double oi = m.sideOrd[q];
        double x = c[j];
        if (!(x > 0.0) || oi == 0.0) continue;
        double prod = oi * pow(x, oi - 1.0);
#pragma unroll 1
        for (int p = q0; p < q1; p++) {
            if (p == q) continue;
            double y = c[GB_IX(m, m.sideK[p], m.K, GB_SITE_SIDE)];
            if (y > 0) prod *= pow(y, m.sideOrd[p]);
            else { prod = 0.0; break; }
        }
        d += prod;
    }
    return d;
}

__device__ __forceinline__ double arrhenius(double A, double b, double EaR, double lnT, double recipT,
                                            const uint64_t* tab) {
    return A * fexp(b * lnT - EaR * recipT, tab);
}

// Falloff rate k(T, M) and, optionally, d ln k / d M (analytic).
//   k = khigh Pr/(1 + Pr) F,  Pr = [M] klow/(khigh + 1e-300)
//   Troe: log10 F = log10 Fcent / (1 + f^2), f = u/d, u = log10 Pr + c, d = n - 0.14 u
// The three quotients of the Troe form share one reciprocal, 1/((1 + Pr)(d^2 + u^2)).
//   d ln k/d[M] = (1/[M]) (1/(1 + Pr) + d ln F/d ln Pr),  d ln F/d ln Pr = -2 log10(Fcent) u n d/(d^2 + u^2)^2
__device__ __forceinline__ double falloff(D4 f1, D4 f2, double A, double b, double EaR,
                                          const KinState& st, double M, double* dlnk_dM, const uint64_t* tab) {
    const bool troe = f2.w != 0.0;
    double logFc = 0.0;
    if (troe) {
        double Fcent = (1.0 - f1.w) * fexp(-st.T * f2.x, tab) + f1.w * fexp(-st.T * f2.y, tab);
        if (f2.z != 0.0) Fcent += fexp(-f2.z * st.recipT, tab);
        logFc = gbx_log10(fmax(Fcent, 1e-300), tab);
    }
    const double klow = arrhenius(f1.x, f1.y, f1.z, st.lnT, st.recipT, tab);
    const double khigh = arrhenius(A, b, EaR, st.lnT, st.recipT, tab);
    const double pr = M * (klow / (khigh + 1e-300));
    const double onep = 1.0 + pr;
    double k;
    if (troe) {
        const double lpr = gbx_log10(fmax(pr, 1e-300), tab);
        const double nn = 0.75 - 1.27 * logFc;
        const double u = lpr + (-0.4 - 0.67 * logFc);
        const double d = nn - 0.14 * u;
        const double q = fma(d, d, u * u);
        const double inv = 1.0 / (onep * q);
        const double rq = inv * onep;          // 1/(d^2 + u^2)
        const double rop = inv * q;            // 1/(1 + Pr)
        const double lgF = logFc * (d * d) * rq;
        const double F = fexp(lgF * 2.302585092994046, tab);
        k = pr * (F * rop) * khigh;
        if (dlnk_dM) {
            double t = rop;
            if (pr > 1e-300) t -= 2.0 * logFc * u * nn * d * (rq * rq);
            *dlnk_dM = t / M;
        }
    } else {
        const double rop = 1.0 / onep;
        k = pr * rop * khigh;
        if (dlnk_dM) *dlnk_dM = rop / M;
    }
    return k;
}

// Rate constants of the less common forms, out of line so that the common reactions'
// instruction stream stays small: pressure-dependent Arrhenius (PLOG), Chebyshev, and the
// falloff forms SRI, Tsang and chemically activated reactions (with any falloff function).
// These use the integer-pipe exp / log of fastexp.h (powers as exp(y ln x)).  For falloff
// forms, *dlnk_dM
// receives d ln k / d[M] (analytic):
//   falloff               k = khigh Pr/(1 + Pr) F,  d ln k/d ln Pr = 1/(1 + Pr) + d ln F/d ln Pr
//   chemically activated  k = klow F/(1 + Pr),      d ln k/d ln Pr = -Pr/(1 + Pr) + d ln F/d ln Pr
//   Troe / Tsang          d ln F/d ln Pr = -2 log10(Fcent) f/(1 + f^2)^2 n/d^2,  f = u/d
//   SRI                   d ln F/d ln Pr = -2 ln(X) log10(Pr) x^2 / ln 10,  x = 1/(1 + log10(Pr)^2)
// (0 where Pr <= 1e-300, where log10 Pr is clamped).
GB_TU_LOCAL __device__ __noinline__ double rateExtra(const DevMech& m, int4 info, D4 ar, const KinState& st,
                                         double M, double* dlnk_dM, const uint64_t* tab) {
    constexpr double kLn10 = 2.302585092994046;
    const int kind = info.x & kKindMask;
    if (kind == kKindPlog) {
        const double* t = m.pdep + info.w;
        const int nl = (int)t[0];
        const double lnP = gbx_log(st.P, tab);
        // upper_bound over the levels: the first one above ln P
        int hi = 0;
#pragma unroll 1
        while (hi < nl && !(t[1 + 3 * hi] > lnP)) hi++;
        if (hi == 0 || hi == nl) return __longlong_as_double(0x7ff8000000000000LL);
        const int lo = hi - 1;
        double lk[2];
#pragma unroll 1
        for (int side = 0; side < 2; side++) {
            const int l = side ? hi : lo;
            double k = 1e-300;
            const int q1 = (int)t[3 + 3 * l];
#pragma unroll 1
            for (int q = (int)t[2 + 3 * l]; q < q1; q += 3) k += t[q] * fexp(t[q + 1] * st.lnT - t[q + 2] * st.recipT, tab);
            lk[side] = gbx_log(k, tab);
        }
        const double lp1 = t[1 + 3 * lo];
        const double rDeltaP = 1.0 / (t[1 + 3 * hi] - lp1);
        return fexp(lk[0] + (lk[1] - lk[0]) * (lnP - lp1) * rDeltaP, tab);
    }
    if (kind == kKindCheb) {
        const double* t = m.pdep + info.w;
        const int nT = (int)t[0], nP = (int)t[1];
        const double* c = t + 6;
        const double Pr = (2 * gbx_log10(st.P, tab) + t[4]) * t[5];
        const double Tr = (2 * st.recipT + t[2]) * t[3];
        // per temperature row the pressure series, then the temperature series over rows
        double logk = 0.0, CTm1 = Tr, CT = 1.0;
#pragma unroll 1
        for (int r = 0; r < nT; r++) {
            double dot = c[r * nP], Cm1 = Pr, C = 1.0;
#pragma unroll 1
            for (int j = 1; j < nP; j++) {
                const double Cp1 = 2 * Pr * C - Cm1;
                dot += Cp1 * c[r * nP + j];
                Cm1 = C;
                C = Cp1;
            }
            if (r == 0) {
                logk = dot;
            } else {
                const double CTp1 = 2 * Tr * CT - CTm1;
                logk += CTp1 * dot;
                CTm1 = CT;
                CT = CTp1;
            }
        }
        return fexp(logk * kLn10, tab);
    }
    // falloff forms
    const D4 f1 = m.fo1[info.z], f2 = m.fo2[info.z];
    const double T = st.T;
    const double klow = f1.x * fexp(f1.y * st.lnT - f1.z * st.recipT, tab);
    const double khigh = ar.x * fexp(ar.y * st.lnT - ar.z * st.recipT, tab);
    const double pr = M * (klow / (khigh + 1e-300));
    const bool live = pr > 1e-300;
    const double lpr = gbx_log10(fmax(pr, 1e-300), tab);
    double F = 1.0, dlnF = 0.0;
    if (kind == kKindTroe || kind == kKindTsang) {
        double Fcent;
        if (kind == kKindTroe) {
            Fcent = (1.0 - f1.w) * fexp(-T * f2.x, tab) + f1.w * fexp(-T * f2.y, tab);
            if (f2.z != 0.0) Fcent += fexp(-f2.z / T, tab);
        } else {
            Fcent = f1.w + (f2.x * T);
        }
        const double lfc = gbx_log10(fmax(Fcent, 1e-300), tab);
        const double cc = -0.4 - 0.67 * lfc, nn = 0.75 - 1.27 * lfc;
        const double u = lpr + cc, d = nn - 0.14 * u;
        const double f = u / d, q = 1.0 + f * f;
        F = fexp(lfc / q * kLn10, tab);
        if (live) dlnF = -lfc * 2.0 * f / (q * q) * (nn / (d * d));
    } else if (kind == kKindSri) {
        double X = f1.w * fexp(-f2.x / T, tab);
        if (f2.y != 0.0) X += fexp(-T / f2.y, tab);
        const double xx = 1.0 / (1.0 + lpr * lpr);
        // X^xx (X > 0; 0 for X = 0) times d T^e
        const double lnX = X > 0.0 ? gbx_log(X, tab) : -INFINITY;
        F = (X > 0.0 ? fexp(xx * lnX, tab) : (X == 0.0 ? 0.0 : __longlong_as_double(0x7ff8000000000000LL))) *
            (f2.z * fexp(f2.w * st.lnT, tab));
        if (live) dlnF = lnX * (-2.0 * lpr * xx * xx) / kLn10;
    }
    const double s1 = 1.0 / (1.0 + pr);
    double k, dl;
    if (info.x & kChemActBit) {
        k = (F * s1) * klow;
        dl = -pr * s1 + dlnF;
    } else {
        k = (pr * (F * s1)) * khigh;
        dl = s1 + dlnF;
    }
    if (dlnk_dM) *dlnk_dM = dl / M;
    return k;
}

// Mixture state from (T, P, Y).  Y may alias any readable [K] array.
// The per-state reciprocals and logarithms are evaluated once for the whole warp, one
// argument per lane (1/T, 1/sum(Y/W), 1/RT, 1/P and ln T, ln P, ln RT, ln Pref), then
// broadcast: a double division costs the FP64 pipe the same whether one lane or all 32
// need it.  The logarithm runs on the integer pipe (fastexp.h).
// kMoles: the third argument holds species amounts n_k (kmol) instead of mass fractions, as
// the state of IdealGasConstPressureMoleReactor (src/zeroD/IdealGasConstPressureMoleReactor.cpp:
// 34-51: the mass from the amounts, then the mixture at T, P); Y_k/W_k = n_k / mass.
template <bool kMoles = false>
__device__ __forceinline__ void warpState(const DevMech& m, double T, double P, const double* Y,
                                          KinScratch& s, KinState& st, int lane) {
    double part = 0.0;
    if (kMoles) {
        double pm = 0.0;
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) pm += Y[k] * m.mw[k];
        const double rmass = 1.0 / warpSum(pm);
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) {
            const double ym = Y[k] * rmass;
            s.c[k] = ym;
            part += ym;
        }
    } else {
#pragma unroll 1
        for (int k = lane; k < m.K; k += 32) {
            double ym = Y[k] * m.rmw[k];
            s.c[k] = ym;
            part += ym;
        }
    }
    const double sum = warpSum(part);
    const double RT = T * m.Rgas;
    const int l4 = lane & 3;
    const double xr = l4 == 0 ? T : (l4 == 1 ? sum : (l4 == 2 ? RT : P));
    const double xl = l4 == 0 ? T : (l4 == 1 ? P : (l4 == 2 ? RT : m.Pref));
    const double r = 1.0 / xr;
    const double lg = gbx_log(xl, s.tab);
    st.T = T;
    st.P = P;
    st.RT = RT;
    st.recipT = __shfl_sync(0xffffffffu, r, 0);
    st.mmw = __shfl_sync(0xffffffffu, r, 1);
    const double rRT = __shfl_sync(0xffffffffu, r, 2);
    const double rP = __shfl_sync(0xffffffffu, r, 3);
    st.lnT = __shfl_sync(0xffffffffu, lg, 0);
    const double lnP = __shfl_sync(0xffffffffu, lg, 1);
    const double lnRT = __shfl_sync(0xffffffffu, lg, 2);
    const double lnPref = __shfl_sync(0xffffffffu, lg, 3);
    st.PRT = P * rRT;
    st.RTP = RT * rP;
    st.ctot = st.PRT;                 // rho / mmw
    st.rho = st.PRT * st.mmw;
    st.rrho = st.RTP * sum;
    st.lnPP = lnP - lnPref;
    st.lnC0 = lnP - lnRT;
    __syncwarp();
#pragma unroll 1
    for (int k = lane; k < m.K; k += 32) s.c[k] *= st.rho;   // c_k = rho Y_k / W_k
}

// Species thermo + rates of progress + net production rates.  With `forJac`, also the
// per-reaction data d(wdot)/dc needs (Qtb, dlk).  kX: the mechanism has reactions of the
// less common forms (rateExtra); without it, such reactions must not occur.  forJac is a
// run-time flag: one copy of this large routine serves both the Newton iterations and the
// Jacobian evaluations, which keeps the integrator's instruction footprint small.
template <bool kX = false>
__device__ __noinline__ void warpRates(const DevMech& m, KinScratch& s, const KinState& st, int lane, bool forJac) {
    const double lnPP = st.lnPP;
    if (lane == 0) s.flags[0] = 0;
    __syncwarp();
#pragma unroll 1
    for (int k = lane; k < m.K; k += 32) {
        // Horner forms with the coefficients scaled on the host (kNasaStride layout)
        const double* a = m.nasa + (size_t)k * kNasaStride;
        const double* p = (st.T <= a[0]) ? a + 1 : a + 1 + kNasaRange;
        const double T = st.T;
        const double cp = fma(fma(fma(fma(p[4], T, p[3]), T, p[2]), T, p[1]), T, p[0]);
        const double h = fma(p[5], st.recipT, fma(fma(fma(fma(p[10], T, p[9]), T, p[8]), T, p[7]), T, p[0]));
        const double sR = fma(p[0], st.lnT, fma(fma(fma(fma(p[13], T, p[12]), T, p[11]), T, p[1]), T, p[6]));
        s.cpR[k] = cp;
        s.hRT[k] = h;
        const double gk = (h - sR) + lnPP;
        s.g[k] = gk;
        // exp(+-g) with split exponents: Kc of each reaction is then a product over its
        // species instead of one exponential per reaction
        if (!gbx_big(gk)) {
            XVal a, b;
            gbx_exp_pm(gk, a, b, s.tab);
            s.xu[k] = a.u;
            s.xe[k] = a.e;
            s.xiu[k] = b.u;
            s.xie[k] = b.e;
        } else {
            s.flags[0] = 1;
        }
    }
    if (lane < 7) {
        // (RT/P)^dn for dn = lane - 3  (= exp(-dn * ln(P/RT)))
        const double a = st.RTP, b = st.PRT;
        const int dn = lane - 3;
        double v = 1.0;
        if (dn > 0) { v = a; if (dn > 1) v *= a; if (dn > 2) v *= a; }
        if (dn < 0) { v = b; if (dn < -1) v *= b; if (dn < -2) v *= b; }
        s.pw[lane] = v;
    }
    __syncwarp();
#pragma unroll 1
    for (int t = lane; t < m.NTB; t += 32) {
        double sum = 0.0;
#pragma unroll 1
        for (int q = m.tbPtr[t]; q < m.tbPtr[t + 1]; q++) sum += m.tbE[q] * s.c[GB_IX(m, m.tbK[q], m.K, GB_SITE_TB_SPECIES)];
        s.Mtb[t] = m.tbDef[t] * st.ctot + sum;
    }
    __syncwarp();
    const double logStandConc = st.lnC0;
    const bool bigG = s.flags[0] != 0;
    // the next reaction's descriptors are loaded one iteration ahead
    int4 nInfo = make_int4(0, 0, 0, 0), nRe = nInfo, nPe = nInfo;
    D4 nAr{};
    if (lane < m.R) { nInfo = m.rinfo[lane]; nAr = m.rarr[lane]; nRe = m.rk[lane]; nPe = m.pk[lane]; }
#pragma unroll 1
    for (int i = lane; i < m.R; i += 32) {
#ifdef GBCHEM_CHECKED
        int4 info = nInfo;
        if (info.y >= 0) info.y = GB_IX(m, info.y, m.NTB, GB_SITE_TB);
        if (info.z >= 0) info.z = GB_IX(m, info.z, m.NF, GB_SITE_FALLOFF);
#else
        const int4 info = nInfo;
#endif
        const D4 ar = nAr;
        const int4 re = GB_IX4(m, nRe, m.K, GB_SITE_SPECIES), pe = GB_IX4(m, nPe, m.K, GB_SITE_SPECIES);
        if (i + 32 < m.R) {
            nInfo = m.rinfo[i + 32]; nAr = m.rarr[i + 32]; nRe = m.rk[i + 32]; nPe = m.pk[i + 32];
        }
        int kind = info.x & kKindMask;
        double kf;
        double dlnk = 0.0;
        if (kind <= 1) {
            kf = (info.x & kNoExpBit) ? ar.x : arrhenius(ar.x, ar.y, ar.z, st.lnT, st.recipT, s.tab);
        } else if (!kX) {
            // Lindemann / Troe falloff (the only other forms without kX)
            D4 f1 = m.fo1[info.z];
            D4 f2 = m.fo2[info.z];
            double M = s.Mtb[info.y];
            kf = falloff(f1, f2, ar.x, ar.y, ar.z, st, M, forJac ? &dlnk : nullptr, s.tab);
            // the reference sets this derivative to zero unless k != 0 and [M] > 0
            if (!(M > 0.0) || kf == 0.0) dlnk = 0.0;
            if (forJac) s.dlk[info.z] = dlnk;
        } else {
            const double M = info.y >= 0 ? s.Mtb[info.y] : 0.0;
            if (kind <= kKindTroe && !(info.x & kChemActBit)) {
                D4 f1 = m.fo1[info.z];
                D4 f2 = m.fo2[info.z];
                kf = falloff(f1, f2, ar.x, ar.y, ar.z, st, M, forJac ? &dlnk : nullptr, s.tab);
            } else {
                kf = rateExtra(m, info, ar, st, M, forJac ? &dlnk : nullptr, s.tab);
            }
            if (info.z >= 0) {
                if (!(M > 0.0) || kf == 0.0) dlnk = 0.0;
                if (forJac) s.dlk[info.z] = dlnk;
            }
        }
        double kfe = (kind == 1) ? kf * s.Mtb[info.y] : kf;
        int rb = (info.x >> kRBucketShift) & 7, pb = (info.x >> kPBucketShift) & 7;
        double rkc = 0.0;
        double fwd = massAction(m, rb, re, 2 * i, s.c);
        double rev = 0.0;
        if (info.x & kRevBit) {
            bool done = false;
            if (!bigG && pb != 0 && rb != 0 && (info.x & kDnIntBit)) {
                // 1/Kc = prod_p exp(g_p) * prod_r exp(-g_r) * (RT/P)^dn, multiplied in Q63
                // fixed point on the integer pipe and converted to double once
                XVal v{s.xu[pe.x], s.xe[pe.x]};
                if (pe.w > 1) v = gbx_mul(v, XVal{s.xu[pe.y], s.xe[pe.y]});
                if (pe.w > 2) v = gbx_mul(v, XVal{s.xu[pe.z], s.xe[pe.z]});
                v = gbx_mul(v, XVal{s.xiu[re.x], s.xie[re.x]});
                if (re.w > 1) v = gbx_mul(v, XVal{s.xiu[re.y], s.xie[re.y]});
                if (re.w > 2) v = gbx_mul(v, XVal{s.xiu[re.z], s.xie[re.z]});
                if (v.e > -980 && v.e < 960) {
                    int c;
                    const double mant = gbx_mant(v.u, c);
                    rkc = scale2(mant * s.pw[(int)ar.w + 3], v.e + c);
                    done = true;
                }
            }
            if (!done) {
            // Delta G / RT over the expanded species lists (products minus reactants)
            double dG = 0.0;
            if (pb != 0) {
                dG = s.g[pe.x];
                if (pe.w > 1) dG += s.g[pe.y];
                if (pe.w > 2) dG += s.g[pe.z];
            } else {
#pragma unroll 1
                for (int q = m.sidePtr[2 * i + 1]; q < m.sidePtr[2 * i + 2]; q++) dG += m.sideNu[q] * s.g[GB_IX(m, m.sideK[q], m.K, GB_SITE_SIDE)];
            }
            double dr = 0.0;
            if (rb != 0) {
                dr = s.g[re.x];
                if (re.w > 1) dr += s.g[re.y];
                if (re.w > 2) dr += s.g[re.z];
            } else {
#pragma unroll 1
                for (int q = m.sidePtr[2 * i]; q < m.sidePtr[2 * i + 1]; q++) dr += m.sideNu[q] * s.g[GB_IX(m, m.sideK[q], m.K, GB_SITE_SIDE)];
            }
            dG -= dr;
            rkc = fmin(fexp(dG - ar.w * logStandConc, s.tab), 1e300);
            }
            rev = massAction(m, pb, pe, 2 * i + 1, s.c);
        }
        double ropf = kfe * fwd;
        double ropr = (kfe * rkc) * rev;
        s.rop[i] = ropf - ropr;
        if (forJac) {
            s.kfe[i] = kfe;
            s.rkc[i] = rkc;
            if (kind == 1) s.Qtb[info.y] = kf * (fwd - rkc * rev);
            else if (kX ? info.z >= 0 : kind >= 2) s.Qtb[info.y] = kf * dlnk * (fwd - rkc * rev);
        }
    }
    __syncwarp();
    // wdot_k = sum_i nu_ki rop_i: balanced tasks, then a fixed-order sum per species
#pragma unroll 1
    for (int q = m.laneTaskPtr[lane]; q < m.laneTaskPtr[lane + 1]; q++) {
        const int t = GB_IX(m, m.laneTasks[q], m.NT, GB_SITE_TASK);
        double w = 0.0;
#pragma unroll 1
        for (int e = m.taskPtr[t]; e < m.taskPtr[t + 1]; e++) w = fma(m.spNu[e], s.rop[GB_IX(m, m.spRxn[e], m.R, GB_SITE_GATHER_RXN)], w);
        s.part[t] = w;
    }
    __syncwarp();
#pragma unroll 1
    for (int k = lane; k < m.K; k += 32) {
        double w = 0.0;
#pragma unroll 1
        for (int q = m.spTaskPtr[k]; q < m.spTaskPtr[k + 1]; q++) w += s.part[GB_IX(m, m.spTasks[q], m.NT, GB_SITE_TASK)];
        s.wdot[k] = w;
    }
    __syncwarp();
}

// d(wdot)/dc without the dense default-efficiency part: Jc[k*ld + j] (+)= ... for
// k, j < K (kT: the transpose, at Jc[j*ld + k]).  The dense part is g_k * (1 for every
// column); warpDenseG returns g in gout.  The caller zeroes Jc.  MT is the matrix element
// type (double or float).
template <typename MT, bool kT>
__device__ __noinline__ void warpJacC(const DevMech& m, const KinScratch& s, MT* Jc, int ld, int lane) {
#pragma unroll 1
    for (int q = m.laneColPtr[lane]; q < m.laneColPtr[lane + 1]; q++) {
        const int j = GB_IX(m, m.laneCols[q], m.K, GB_SITE_COLUMN);
        const int e0 = m.colPtr[j], e1 = m.colPtr[j + 1];
        // the next entry's reaction data are loaded one iteration ahead
        int iN = 0, rs0N = 0, rs1N = 0;
        int4 infoN = make_int4(0, 0, 0, 0), rkN = infoN, pkN = infoN;
        double epN = 0.0;
        if (e0 < e1) {
            iN = GB_IX(m, m.colRxn[e0], m.R, GB_SITE_COL_RXN);
            infoN = m.rinfo[iN]; rkN = GB_IX4(m, m.rk[iN], m.K, GB_SITE_SPECIES); pkN = GB_IX4(m, m.pk[iN], m.K, GB_SITE_SPECIES); epN = m.colE[e0];
            rs0N = m.rsPtr[iN]; rs1N = m.rsPtr[iN + 1];
        }
#pragma unroll 1
        for (int e = e0; e < e1; e++) {
            const int i = iN, rs0 = rs0N, rs1 = rs1N;
            const int4 info = infoN, rki = rkN, pki = pkN;
            const double ep = epN;
            if (e + 1 < e1) {
                iN = GB_IX(m, m.colRxn[e + 1], m.R, GB_SITE_COL_RXN);
                infoN = m.rinfo[iN]; rkN = GB_IX4(m, m.rk[iN], m.K, GB_SITE_SPECIES); pkN = GB_IX4(m, m.pk[iN], m.K, GB_SITE_SPECIES); epN = m.colE[e + 1];
                rs0N = m.rsPtr[iN]; rs1N = m.rsPtr[iN + 1];
            }
            const int rb = (info.x >> kRBucketShift) & 7, pb = (info.x >> kPBucketShift) & 7;
            const double kfe = s.kfe[i];
            double dF = kfe * massActionDeriv(m, rb, rki, 2 * i, s.c, j);
            if (info.x & kRevBit) dF -= (kfe * s.rkc[i]) * massActionDeriv(m, pb, pki, 2 * i + 1, s.c, j);
            if (ep != 0.0) dF += ep * s.Qtb[GB_IX(m, info.y, m.NTB, GB_SITE_TB)];
            if (dF == 0.0) continue;
#pragma unroll 1
            for (int r = rs0; r < rs1; r++) {
                const int kr = GB_IX(m, m.rsK[r], m.K, GB_SITE_NET_SPECIES);
                MT* p = kT ? Jc + (size_t)j * ld + kr : Jc + (size_t)kr * ld + j;
                *p = (MT)((double)*p + m.rsNu[r] * dF);
            }
        }
    }
    __syncwarp();
}

// d(wdot)/dc without the dense default-efficiency part, accumulated directly on the
// output pattern: Js[slot] (+)= ..., slots from DevMech::colSlot (same entries, same order
// of accumulation per element as warpJacC).  The caller zeroes Js[nnz].
GB_TU_LOCAL __device__ __noinline__ void warpJacSparse(const DevMech& m, const KinScratch& s, double* Js, int lane) {
#pragma unroll 1
    for (int q = m.laneColPtr[lane]; q < m.laneColPtr[lane + 1]; q++) {
        const int j = GB_IX(m, m.laneCols[q], m.K, GB_SITE_COLUMN);
        const int e0 = m.colPtr[j], e1 = m.colPtr[j + 1];
        int slot = m.colSlotStart[j];
        int iN = 0, rs0N = 0, rs1N = 0;
        int4 infoN = make_int4(0, 0, 0, 0), rkN = infoN, pkN = infoN;
        double epN = 0.0;
        if (e0 < e1) {
            iN = GB_IX(m, m.colRxn[e0], m.R, GB_SITE_COL_RXN);
            infoN = m.rinfo[iN]; rkN = GB_IX4(m, m.rk[iN], m.K, GB_SITE_SPECIES); pkN = GB_IX4(m, m.pk[iN], m.K, GB_SITE_SPECIES); epN = m.colE[e0];
            rs0N = m.rsPtr[iN]; rs1N = m.rsPtr[iN + 1];
        }
#pragma unroll 1
        for (int e = e0; e < e1; e++) {
            const int i = iN, rs0 = rs0N, rs1 = rs1N;
            const int4 info = infoN, rki = rkN, pki = pkN;
            const double ep = epN;
            if (e + 1 < e1) {
                iN = GB_IX(m, m.colRxn[e + 1], m.R, GB_SITE_COL_RXN);
                infoN = m.rinfo[iN]; rkN = GB_IX4(m, m.rk[iN], m.K, GB_SITE_SPECIES); pkN = GB_IX4(m, m.pk[iN], m.K, GB_SITE_SPECIES); epN = m.colE[e + 1];
                rs0N = m.rsPtr[iN]; rs1N = m.rsPtr[iN + 1];
            }
            const int rb = (info.x >> kRBucketShift) & 7, pb = (info.x >> kPBucketShift) & 7;
            const double kfe = s.kfe[i];
            double dF = kfe * massActionDeriv(m, rb, rki, 2 * i, s.c, j);
            if (info.x & kRevBit) dF -= (kfe * s.rkc[i]) * massActionDeriv(m, pb, pki, 2 * i + 1, s.c, j);
            if (ep != 0.0) dF += ep * s.Qtb[GB_IX(m, info.y, m.NTB, GB_SITE_TB)];
            if (dF == 0.0) {
                slot += rs1 - rs0;
                continue;
            }
#pragma unroll 1
            for (int r = rs0; r < rs1; r++, slot++) {
                const int t = m.colSlot[slot];
                if (t >= 0) {
                    const int tt = GB_IX(m, t, m.nnz, GB_SITE_SLOT);
                    Js[tt] = Js[tt] + m.rsNu[r] * dF;
                }
            }
        }
    }
    __syncwarp();
}

// g_k = sum over third-body reactions i with default efficiency d_i of S_net[k][i]*d_i*Q_i:
// the part of d(wdot_k)/dc_j that is the same for every column j.
__device__ __forceinline__ void warpDenseG(const DevMech& m, const KinScratch& s, double* gout, int lane) {
#pragma unroll 1
    for (int k = lane; k < m.K; k += 32) {
        double g = 0.0;
#pragma unroll 1
        for (int q = m.gsPtr[k]; q < m.gsPtr[k + 1]; q++) g += m.gsCoef[q] * s.Qtb[GB_IX(m, m.gsTb[q], m.NTB, GB_SITE_DENSE_TB)];
        gout[k] = g;
    }
    __syncwarp();
}

}  // namespace gbchem
