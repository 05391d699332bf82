// oracle.cpp - CPU restatement of the reference hot path.  TEST INFRASTRUCTURE ONLY.
// See oracle.h for the reference files each part follows.  Compiled with
// -ffp-contract=off so that x86 and Arm hosts give identical results.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../cantera_gb300/csrc/mechanism.h"

using namespace gbchem;

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Stoichiometry manager (include/cantera/kinetics/StoichManager.h:131-480, 676-797)
// ---------------------------------------------------------------------------
struct C1 { int rxn, k0; };
struct C2 { int rxn, k0, k1; };
struct C3 { int rxn, k0, k1, k2; };
struct CN { int rxn; std::vector<int> k; std::vector<double> order, nu; };

struct StoichMgr {
    std::vector<C1> c1;
    std::vector<C2> c2;
    std::vector<C3> c3;
    std::vector<CN> cn;

    void add(int rxn, const std::vector<int>& k, const std::vector<double>& order, const std::vector<double>& nu) {
        bool frac = false;
        for (size_t n = 0; n < nu.size(); n++)
            if (std::fmod(nu[n], 1.0) != 0.0 || nu[n] != order[n]) frac = true;
        if (frac || k.size() > 3) { cn.push_back(CN{rxn, k, order, nu}); return; }
        std::vector<int> rep;
        for (size_t n = 0; n < k.size(); n++)
            for (size_t i = 0; i < nu[n]; i++) rep.push_back(k[n]);
        switch (rep.size()) {
            case 1: c1.push_back(C1{rxn, rep[0]}); break;
            case 2: c2.push_back(C2{rxn, rep[0], rep[1]}); break;
            case 3: c3.push_back(C3{rxn, rep[0], rep[1], rep[2]}); break;
            default: cn.push_back(CN{rxn, k, order, nu});
        }
    }
    void multiply(const double* S, double* R) const {
        for (auto& c : c1) R[c.rxn] *= S[c.k0];
        for (auto& c : c2) {
            if (S[c.k0] < 0 && S[c.k1] < 0) R[c.rxn] = 0;
            else R[c.rxn] *= S[c.k0] * S[c.k1];
        }
        for (auto& c : c3) {
            if ((S[c.k0] < 0 && (S[c.k1] < 0 || S[c.k2] < 0)) || (S[c.k1] < 0 && S[c.k2] < 0)) R[c.rxn] = 0;
            else R[c.rxn] *= S[c.k0] * S[c.k1] * S[c.k2];
        }
        for (auto& c : cn) {
            for (size_t n = 0; n < c.k.size(); n++) {
                double order = c.order[n];
                if (order != 0.0) {
                    double x = S[c.k[n]];
                    if (x > 0.0) R[c.rxn] *= std::pow(x, order);
                    else R[c.rxn] = 0.0;
                }
            }
        }
    }
    void incrementSpecies(const double* R, double* S) const {
        for (auto& c : c1) S[c.k0] += R[c.rxn];
        for (auto& c : c2) { S[c.k0] += R[c.rxn]; S[c.k1] += R[c.rxn]; }
        for (auto& c : c3) { S[c.k0] += R[c.rxn]; S[c.k1] += R[c.rxn]; S[c.k2] += R[c.rxn]; }
        for (auto& c : cn) for (size_t n = 0; n < c.k.size(); n++) S[c.k[n]] += c.nu[n] * R[c.rxn];
    }
    void decrementSpecies(const double* R, double* S) const {
        for (auto& c : c1) S[c.k0] -= R[c.rxn];
        for (auto& c : c2) { S[c.k0] -= R[c.rxn]; S[c.k1] -= R[c.rxn]; }
        for (auto& c : c3) { S[c.k0] -= R[c.rxn]; S[c.k1] -= R[c.rxn]; S[c.k2] -= R[c.rxn]; }
        for (auto& c : cn) for (size_t n = 0; n < c.k.size(); n++) S[c.k[n]] -= c.nu[n] * R[c.rxn];
    }
    void incrementReactions(const double* S, double* R) const {
        for (auto& c : c1) R[c.rxn] += S[c.k0];
        for (auto& c : c2) R[c.rxn] += S[c.k0] + S[c.k1];
        for (auto& c : c3) R[c.rxn] += S[c.k0] + S[c.k1] + S[c.k2];
        for (auto& c : cn) for (size_t n = 0; n < c.k.size(); n++) R[c.rxn] += c.nu[n] * S[c.k[n]];
    }
    void decrementReactions(const double* S, double* R) const {
        for (auto& c : c1) R[c.rxn] -= S[c.k0];
        for (auto& c : c2) R[c.rxn] -= (S[c.k0] + S[c.k1]);
        for (auto& c : c3) R[c.rxn] -= (S[c.k0] + S[c.k1] + S[c.k2]);
        for (auto& c : cn) for (size_t n = 0; n < c.k.size(); n++) R[c.rxn] -= c.nu[n] * S[c.k[n]];
    }
    // derivatives(): entries (reaction, species) of d(rate * prod c^order)/dc; written
    // into a dense [R][K] array D (accumulated).
    void derivatives(const double* S, const double* R, double* D, int K) const {
        for (auto& c : c1) D[(size_t)c.rxn * K + c.k0] += R[c.rxn];
        for (auto& c : c2) {
            if (S[c.k1] > 0) D[(size_t)c.rxn * K + c.k0] += R[c.rxn] * S[c.k1];
            if (S[c.k0] > 0) D[(size_t)c.rxn * K + c.k1] += R[c.rxn] * S[c.k0];
        }
        for (auto& c : c3) {
            if (S[c.k1] > 0 && S[c.k2] > 0) D[(size_t)c.rxn * K + c.k0] += R[c.rxn] * S[c.k1] * S[c.k2];
            if (S[c.k0] > 0 && S[c.k2] > 0) D[(size_t)c.rxn * K + c.k1] += R[c.rxn] * S[c.k0] * S[c.k2];
            if (S[c.k0] > 0 && S[c.k1] > 0) D[(size_t)c.rxn * K + c.k2] += R[c.rxn] * S[c.k0] * S[c.k1];
        }
        for (auto& c : cn) {
            size_t m = c.k.size();
            for (size_t i = 0; i < m; i++) {
                double prod = R[c.rxn];
                double oi = c.order[i];
                if (S[c.k[i]] > 0. && oi != 0.) {
                    prod *= oi * std::pow(S[c.k[i]], oi - 1);
                    for (size_t j = 0; j < m; j++) {
                        if (i != j) {
                            if (S[c.k[j]] > 0) prod *= std::pow(S[c.k[j]], c.order[j]);
                            else { prod = 0.; break; }
                        }
                    }
                } else {
                    prod = 0.;
                }
                D[(size_t)c.rxn * K + c.k[i]] += prod;
            }
        }
    }
};

// ---------------------------------------------------------------------------
// Kinetics object: a mechanism plus its stoichiometry managers
// ---------------------------------------------------------------------------
struct Kin {
    Mechanism m;
    StoichMgr reac, prod, revProd;
    std::vector<double> Snet;   // [K][R] net stoichiometric matrix
    std::vector<double> rmw;    // 1/mw
    std::vector<int> revIndex, irrev;
    double R_gas;
    std::vector<int32_t> precOrder;   // fill-reducing ordering of the Krylov path's preconditioner
};

struct Work {  // per-thread scratch for one state
    std::vector<double> tpoly, cp_R, h_RT, s_R, g_RT, mu0, dG, rkcn, concm, kf0, rfn,
        ropf, ropr, ropnet, ym, c, wdot, outV, D;
    void init(int K, int R) {
        tpoly.assign(6, 0); cp_R.assign(K, 0); h_RT.assign(K, 0); s_R.assign(K, 0); g_RT.assign(K, 0);
        mu0.assign(K, 0); dG.assign(R, 0); rkcn.assign(R, 0); concm.assign(R, NAN); kf0.assign(R, 0);
        rfn.assign(R, 0); ropf.assign(R, 0); ropr.assign(R, 0); ropnet.assign(R, 0); ym.assign(K, 0);
        c.assign(K, 0); wdot.assign(K, 0); outV.assign(R, 0); D.clear();
    }
    double T = 0, P = 0, RT = 0, density = 0, mmw = 0, ctot = 0, logT = 0, recipT = 0;
};

std::mutex g_reg_mu;
std::vector<std::unique_ptr<Kin>> g_kins;

Kin* getKin(int32_t h) {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    if (h < 0 || h >= (int32_t)g_kins.size() || !g_kins[h]) return nullptr;
    return g_kins[h].get();
}

// NASA7 (NasaPoly1::updateProperties, NasaPoly2 range selection)
void speciesThermo(const Mechanism& m, double T, Work& w) {
    double* tt = w.tpoly.data();
    tt[0] = T;
    tt[1] = T * T;
    tt[2] = tt[1] * T;
    tt[3] = tt[2] * T;
    tt[4] = 1.0 / T;
    tt[5] = std::log(T);
    for (int k = 0; k < m.K; k++) {
        const double* a = (T <= m.nasaTmid[k]) ? &m.nasaLow[7 * k] : &m.nasaHigh[7 * k];
        double ct0 = a[0];
        double ct1 = a[1] * tt[0];
        double ct2 = a[2] * tt[1];
        double ct3 = a[3] * tt[2];
        double ct4 = a[4] * tt[3];
        w.cp_R[k] = ct0 + ct1 + ct2 + ct3 + ct4;
        w.h_RT[k] = ct0 + 0.5 * ct1 + 1.0 / 3.0 * ct2 + 0.25 * ct3 + 0.2 * ct4 + a[5] * tt[4];
        w.s_R[k] = ct0 * tt[5] + ct1 + 0.5 * ct2 + 1.0 / 3.0 * ct3 + 0.25 * ct4 + a[6];
        w.g_RT[k] = w.h_RT[k] - w.s_R[k];
    }
}

// Phase state from (T, P, Y) without normalising Y (Phase::setMassFractions_NoNorm,
// IdealGasPhase::setPressure).
void setState(const Kin& kn, double T, double P, const double* Y, Work& w) {
    const Mechanism& m = kn.m;
    w.T = T;
    w.P = P;
    w.RT = T * kn.R_gas;
    double sum = 0.0;
    for (int k = 0; k < m.K; k++) w.ym[k] = Y[k] * kn.rmw[k];
    for (int k = 0; k < m.K; k++) sum += w.ym[k];
    w.mmw = 1.0 / sum;
    w.density = P * w.mmw / w.RT;
    for (int k = 0; k < m.K; k++) w.c[k] = w.ym[k] * w.density;
    w.ctot = w.density / w.mmw;
}

double arrhenius(double A, double b, double EaR, double logT, double recipT) {
    return A * std::exp(b * logT - EaR * recipT);
}

// Temperature-dependent part of a falloff function (the updateTemp methods):
// Troe (reference src/kinetics/Falloff.cpp:283-290), SRI (:392-399), Tsang (:479-483).
void falloffWork(const Mechanism& m, int i, double T, double* work) {
    work[0] = 0.0;
    work[1] = 1.0;
    if (m.kind[i] == kTroe) {
        const double* tr = &m.troe[4 * i];
        double Fcent = (1.0 - tr[0]) * std::exp(-T * tr[1]) + tr[0] * std::exp(-T * tr[2]);
        if (tr[3] != 0.0) Fcent += std::exp(-tr[3] / T);
        work[0] = std::log10(std::max(Fcent, kSmallNumber));
    } else if (m.kind[i] == kSri) {
        const double* x = &m.falloffX[5 * i];
        work[0] = x[0] * std::exp(-x[1] / T);
        if (x[2] != 0.0) work[0] += std::exp(-T / x[2]);
        work[1] = x[3] * std::pow(T, x[4]);
    } else if (m.kind[i] == kTsang) {
        const double* x = &m.falloffX[5 * i];
        double Fcent = x[0] + (x[1] * T);
        work[0] = std::log10(std::max(Fcent, kSmallNumber));
    }
}

// Falloff function F(Pr) (the F methods: Troe Falloff.cpp:292-300, SRI :401-406, Tsang
// :485-494) and, if dlnF is given, d ln F / d ln Pr (analytic; 0 where Pr <= 1e-300, where
// the reference clamps log10 Pr).
double falloffF(const Mechanism& m, int i, double pr, const double* work, double* dlnF) {
    if (dlnF) *dlnF = 0.0;
    const int kind = m.kind[i];
    if (kind == kTroe || kind == kTsang) {
        double lpr = std::log10(std::max(pr, kSmallNumber));
        double cc = -0.4 - 0.67 * work[0];
        double nn = 0.75 - 1.27 * work[0];
        double f1 = (lpr + cc) / (nn - 0.14 * (lpr + cc));
        double lgf = work[0] / (1.0 + f1 * f1);
        if (dlnF && pr > kSmallNumber) {
            double u = lpr + cc, den = nn - 0.14 * u, q = 1.0 + f1 * f1;
            *dlnF = -work[0] * 2.0 * f1 / (q * q) * (nn / (den * den));   // ln 10 factors cancel
        }
        return std::pow(10.0, lgf);
    }
    if (kind == kSri) {
        double lpr = std::log10(std::max(pr, kSmallNumber));
        double xx = 1.0 / (1.0 + lpr * lpr);
        if (dlnF && pr > kSmallNumber) *dlnF = std::log(work[0]) * (-2.0 * lpr * xx * xx) / std::log(10.0);
        return std::pow(work[0], xx) * work[1];
    }
    return 1.0;
}

// FalloffRate::evalFromStruct with an explicit third-body concentration (reference
// include/cantera/kinetics/Falloff.h:154-176): falloff k = khigh Pr/(1+Pr) F, chemically
// activated k = klow F/(1+Pr).
double falloffRate(const Mechanism& m, int i, double T, double logT, double recipT, double M) {
    double work[2];
    falloffWork(m, i, T, work);
    double klow = arrhenius(m.A0[i], m.b0[i], m.Ea0R[i], logT, recipT);
    double khigh = arrhenius(m.A[i], m.b[i], m.EaR[i], logT, recipT);
    double pr = M * klow / (khigh + kSmallNumber);
    if (m.chemAct[i]) {
        pr = falloffF(m, i, pr, work, nullptr) / (1.0 + pr);
        return pr * klow;
    }
    pr *= falloffF(m, i, pr, work, nullptr) / (1.0 + pr);
    return pr * khigh;
}

// Analytic d k / d[M] of a falloff rate (k as above).
double falloffRate_dM(const Mechanism& m, int i, double T, double logT, double recipT, double M) {
    double work[2];
    falloffWork(m, i, T, work);
    double klow = arrhenius(m.A0[i], m.b0[i], m.Ea0R[i], logT, recipT);
    double khigh = arrhenius(m.A[i], m.b[i], m.EaR[i], logT, recipT);
    double dPr_dM = klow / (khigh + kSmallNumber);
    double pr = M * dPr_dM;
    double dlnF = 0.0;
    double F = falloffF(m, i, pr, work, &dlnF);
    double dF_dPr = pr > kSmallNumber ? F * dlnF / pr : 0.0;
    double s = 1.0 / (1.0 + pr);
    if (m.chemAct[i]) return klow * (dF_dPr * s - F * s * s) * dPr_dM;
    return khigh * (s * s * F + pr * s * dF_dPr) * dPr_dM;
}

// PlogRate::updateFromStruct / evalFromStruct (reference include/cantera/kinetics/
// PlogRate.h:110-164): the pressure interval by upper_bound over the levels (with the
// +-1000 sentinels), ln k of each bracketing level from its summed Arrhenius expressions
// (plus 1e-300), interpolated linearly in ln P.
double plogRate(const Mechanism& m, int i, double logP, double logT, double recipT) {
    const int l0 = m.plogPtr[i], l1 = m.plogPtr[i + 1];
    int hi = l0;
    while (hi < l1 && !(m.plogLogP[hi] > logP)) hi++;
    if (hi == l0 || hi == l1) return NAN;   // outside (-1000, 1000): the reference throws
    const int lo = hi - 1;
    auto logk = [&](int l) {
        double k = 1e-300;
        for (int q = m.plogFirst[l]; q < m.plogLast[l]; q++)
            k += m.plogA[q] * std::exp(m.plogB[q] * logT - m.plogEaR[q] * recipT);
        return std::log(k);
    };
    const double lk1 = logk(lo), lk2 = logk(hi);
    const double rDeltaP = 1.0 / (m.plogLogP[hi] - m.plogLogP[lo]);
    return std::exp(lk1 + (lk2 - lk1) * (logP - m.plogLogP[lo]) * rDeltaP);
}

// ChebyshevRate::updateFromStruct / evalFromStruct (reference include/cantera/kinetics/
// ChebyshevRate.h:133-171): the pressure series first (one dot product per temperature
// row), then the temperature series; k = 10^(log10 k).
double chebRate(const Mechanism& m, int i, double log10P, double recipT) {
    const int nT = m.chebNT[i], nP = m.chebNP[i];
    const double* c = &m.chebCoef[m.chebPtr[i]];
    const double* lim = &m.chebLim[4 * i];
    std::vector<double> dot(nT);
    const double Pr = (2 * log10P + lim[2]) * lim[3];
    double Cnm1 = Pr, Cn = 1, Cnp1;
    for (int t = 0; t < nT; t++) dot[t] = c[t * nP];
    for (int j = 1; j < nP; j++) {
        Cnp1 = 2 * Pr * Cn - Cnm1;
        for (int t = 0; t < nT; t++) dot[t] += Cnp1 * c[t * nP + j];
        Cnm1 = Cn;
        Cn = Cnp1;
    }
    const double Tr = (2 * recipT + lim[0]) * lim[1];
    Cnm1 = Tr;
    Cn = 1;
    double logk = dot[0];
    for (int t = 1; t < nT; t++) {
        Cnp1 = 2 * Tr * Cn - Cnm1;
        logk += Cnp1 * dot[t];
        Cnm1 = Cn;
        Cn = Cnp1;
    }
    return std::pow(10, logk);
}

// BulkKinetics::updateROP + Kinetics::getNetProductionRates
void updateROP(const Kin& kn, Work& w) {
    const Mechanism& m = kn.m;
    const int K = m.K, R = m.R;
    speciesThermo(m, w.T, w);
    // getStandardChemPotentials: mu0 = RT*g/RT + RT ln(P/P0)
    double tmp = std::log(w.P / m.Pref) * w.RT;
    for (int k = 0; k < K; k++) { w.mu0[k] = w.g_RT[k] * w.RT; w.mu0[k] += tmp; }
    std::fill(w.dG.begin(), w.dG.end(), 0.0);
    double logStandConc = std::log(w.P / w.RT);
    kn.revProd.incrementReactions(w.mu0.data(), w.dG.data());
    kn.reac.decrementReactions(w.mu0.data(), w.dG.data());
    double rrt = 1.0 / w.RT;
    for (int irxn : kn.revIndex)
        w.rkcn[irxn] = std::min(std::exp(w.dG[irxn] * rrt - m.dn[irxn] * logStandConc), kBigNumber);
    for (int irxn : kn.irrev) w.rkcn[irxn] = 0.0;
    // third-body concentrations (ThirdBodyCalc::update)
    for (int t = 0; t < m.nThirdBody(); t++) {
        double sum = 0.0;
        for (int j = m.tbPtr[t]; j < m.tbPtr[t + 1]; j++) sum += m.tbEffMinusDefault[j] * w.c[m.tbSpecies[j]];
        w.concm[m.tbRxn[t]] = m.tbDefault[t] * w.ctot + sum;
    }
    // rate constants
    w.logT = std::log(w.T);
    w.recipT = 1. / w.T;
    for (int i = 0; i < R; i++) {
        if (m.kind[i] == kArrhenius || m.kind[i] == kThreeBody)
            w.kf0[i] = arrhenius(m.A[i], m.b[i], m.EaR[i], w.logT, w.recipT);
        else if (m.kind[i] == kPlog)
            w.kf0[i] = plogRate(m, i, std::log(w.P), w.logT, w.recipT);
        else if (m.kind[i] == kChebyshev)
            w.kf0[i] = chebRate(m, i, std::log10(w.P), w.recipT);
        else
            w.kf0[i] = falloffRate(m, i, w.T, w.logT, w.recipT, w.concm[i]);
    }
    for (int i = 0; i < R; i++) w.rfn[i] = w.kf0[i] * 1.0;  // perturbation multiplier 1
    w.ropf = w.rfn;
    for (int t = 0; t < m.nThirdBody(); t++)
        if (m.tbMassAction[t]) w.ropf[m.tbRxn[t]] *= w.concm[m.tbRxn[t]];
    w.ropr = w.ropf;
    for (int i = 0; i < R; i++) w.ropr[i] *= w.rkcn[i];
    kn.reac.multiply(w.c.data(), w.ropf.data());
    kn.revProd.multiply(w.c.data(), w.ropr.data());
    for (int j = 0; j < R; j++) w.ropnet[j] = w.ropf[j] - w.ropr[j];
    std::fill(w.wdot.begin(), w.wdot.end(), 0.0);
    kn.prod.incrementSpecies(w.ropnet.data(), w.wdot.data());
    kn.reac.decrementSpecies(w.ropnet.data(), w.wdot.data());
}

// jac[k*K+j] += sign * sum_i Snet[k][i] * D[i][j]
void accumulateStoichProduct(const Kin& kn, const double* D, double sign, double* jac) {
    const int K = kn.m.K, R = kn.m.R;
    for (int i = 0; i < R; i++) {
        for (int k = 0; k < K; k++) {
            double s = kn.Snet[(size_t)k * R + i];
            if (s == 0.0) continue;
            const double* Di = D + (size_t)i * K;
            double* Jk = jac + (size_t)k * K;
            for (int j = 0; j < K; j++)
                if (Di[j] != 0.0) Jk[j] += s * (sign * Di[j]);
        }
    }
}

// BulkKinetics::accumulateCompositionDerivatives (mode 0: FD in [M] for falloff with
// delta 1e-8 (MultiRate::processRateConstants_ddM); mode 1: analytic).
void accumulateCompDeriv(const Kin& kn, Work& w, const StoichMgr& sm, const std::vector<double>& in,
                         double sign, int mode, double* jac) {
    const Mechanism& m = kn.m;
    const int K = m.K, R = m.R;
    std::vector<double> outV(in);
    for (int t = 0; t < m.nThirdBody(); t++)
        if (m.tbMassAction[t]) outV[m.tbRxn[t]] *= w.concm[m.tbRxn[t]];
    w.D.assign((size_t)R * K, 0.0);
    sm.derivatives(w.c.data(), outV.data(), w.D.data(), K);
    accumulateStoichProduct(kn, w.D.data(), sign, jac);
    if (m.nThirdBody() == 0) return;
    outV = in;
    sm.multiply(w.c.data(), outV.data());
    const double deltaM = 1e-8;
    for (int i = 0; i < R; i++) {
        if (!isFalloffKind(m.kind[i])) continue;
        double M = w.concm[i];
        if (mode == 0) {
            double Mp = M * (1. + deltaM);
            if (w.kf0[i] != 0. && Mp > 0.) {
                double k1 = falloffRate(m, i, w.T, w.logT, w.recipT, Mp);
                outV[i] *= (1. / deltaM) * (k1 / w.kf0[i] - 1.);
                outV[i] /= Mp;
            } else {
                outV[i] = 0.;
            }
        } else {
            if (w.kf0[i] != 0. && M > 0.) {
                outV[i] *= falloffRate_dM(m, i, w.T, w.logT, w.recipT, M) / w.kf0[i];
            } else {
                outV[i] = 0.;
            }
        }
    }
    // ThirdBodyCalc::derivatives: diag(outV) * (efficiency matrix + default fill)
    w.D.assign((size_t)R * K, 0.0);
    for (int t = 0; t < m.nThirdBody(); t++) {
        int i = m.tbRxn[t];
        double d = m.tbDefault[t];
        double* Di = &w.D[(size_t)i * K];
        if (d != 0.0)
            for (int j = 0; j < K; j++) Di[j] = d;
        for (int j = m.tbPtr[t]; j < m.tbPtr[t + 1]; j++) Di[m.tbSpecies[j]] = m.tbEffMinusDefault[j] + d;
        for (int j = 0; j < K; j++) Di[j] *= outV[i];
    }
    accumulateStoichProduct(kn, w.D.data(), sign, jac);
}

void ddCi(const Kin& kn, Work& w, int mode, double* jac) {
    const int K = kn.m.K;
    std::fill(jac, jac + (size_t)K * K, 0.0);
    std::vector<double> r0(w.rfn);
    accumulateCompDeriv(kn, w, kn.reac, r0, 1.0, mode, jac);
    for (int i = 0; i < kn.m.R; i++) r0[i] *= w.rkcn[i];
    accumulateCompDeriv(kn, w, kn.revProd, r0, -1.0, mode, jac);
}

struct Reactor;
int reactorJacobian(Reactor& r, const double* z, const double* fz, double* J);

// ---------------------------------------------------------------------------
// Constant-pressure ideal-gas reactor (IdealGasConstPressureReactor::eval,
// ReactorNet::eval).  The integrated state is z = [T, Y1..YK]; the constant mass
// m = y[0] has dm/dt = 0 and never enters the other equations.
// ---------------------------------------------------------------------------
// Right-hand side interface used by the integrator.
struct System {
    virtual ~System() = default;
    virtual int size() const = 0;                       // integrated components
    virtual int normSize() const = 0;                   // WRMS-norm divisor
    virtual int rhs(const double* z, double* zdot) = 0; // 0 ok, 1 recoverable failure
    virtual int jac(const double* z, const double* fz, double* J) = 0;
    // Approximate Jacobian for a preconditioner (dense storage); -1: not available
    virtual int precJac(const double* z, double atol, double* J) { (void)z; (void)atol; (void)J; return -1; }
    int nrhs = 0;
};

struct Reactor : System {
    Reactor(const Kin* k, double p) : kn(k), P(p) { w.init(k->m.K, k->m.R); }
    const Kin* kn;
    double P;
    Work w;
    int size() const override { return kn->m.K + 1; }
    int normSize() const override { return kn->m.K + 2; }
    int jac(const double* z, const double* fz, double* J) override;
    // returns 0, or 1 (recoverable) when the derivative is not finite
    int rhs(const double* z, double* zdot) override {
        const Mechanism& m = kn->m;
        const int K = m.K;
        nrhs++;
        setState(*kn, z[0], P, z + 1, w);
        updateROP(*kn, w);
        // getPartialMolarEnthalpies: h_k = RT * h/RT
        double mcpdTdt = 0.0;
        double mass = 1.0;                 // any positive mass: the ratios below do not depend on it
        double vol = mass / w.density;
        for (int n = 0; n < K; n++) {
            double hk = w.h_RT[n] * w.RT;
            mcpdTdt -= w.wdot[n] * hk * vol;
            zdot[1 + n] = (w.wdot[n] * vol) * m.mw[n];
        }
        // cp_mass = cp_mole / mmw; cp_mole = R * mmw * sum(ym * cp_R)
        double s = 0.0;
        for (int k = 0; k < K; k++) s += w.ym[k] * w.cp_R[k];
        double cp_mole = kn->R_gas * (w.mmw * s);
        double cp_mass = cp_mole / w.mmw;
        zdot[0] = mcpdTdt / (mass * cp_mass);
        for (int n = 0; n < K; n++) zdot[1 + n] /= mass;
        for (int i = 0; i <= K; i++)
            if (!std::isfinite(zdot[i])) return 1;
        return 0;
    }
};

// Constant-pressure ideal-gas reactor with moles as the state, z = [T, n_1..n_K] (kmol):
// IdealGasConstPressureMoleReactor::updateState / eval (reference src/zeroD/
// IdealGasConstPressureMoleReactor.cpp:34-104).  The mass follows from the moles, the volume
// from the mass and the density; dn_k/dt = wdot_k V, m cp dT/dt = -sum_k h_k wdot_k V.
struct MoleReactor : System {
    MoleReactor(const Kin* k, double p) : kn(k), P(p) { w.init(k->m.K, k->m.R); }
    const Kin* kn;
    double P;
    Work w;
    double mass = 0.0, vol = 0.0, mcp = 0.0;
    int size() const override { return kn->m.K + 1; }
    int normSize() const override { return kn->m.K + 1; }
    int jac(const double*, const double*, double*) override { return -1; }
    // thermo state from z (setMassFromMoles, setMolesNoTruncate, setState_TP)
    void update(const double* z) {
        const Mechanism& m = kn->m;
        const int K = m.K;
        mass = 0.0;
        for (int k = 0; k < K; k++) mass += z[1 + k] * m.mw[k];
        std::vector<double> Y(K);
        for (int k = 0; k < K; k++) Y[k] = z[1 + k] * m.mw[k] / mass;
        setState(*kn, z[0], P, Y.data(), w);
        vol = mass / w.density;
        updateROP(*kn, w);
        double s = 0.0;
        for (int k = 0; k < K; k++) s += w.ym[k] * w.cp_R[k];
        mcp = mass * kn->R_gas * s;        // m * cp_mass = m * R * sum(Y_k/W_k cp_k/R)
    }
    int rhs(const double* z, double* zdot) override {
        const int K = kn->m.K;
        nrhs++;
        update(z);
        double mcpdTdt = 0.0;
        for (int n = 0; n < K; n++) {
            mcpdTdt -= w.wdot[n] * (w.h_RT[n] * w.RT) * vol;
            zdot[1 + n] = w.wdot[n] * vol;
        }
        zdot[0] = mcpdTdt / mcp;
        for (int i = 0; i <= K; i++)
            if (!std::isfinite(zdot[i])) return 1;
        return 0;
    }
    // IdealGasConstPressureMoleReactor::getJacobianElements (reference
    // IdealGasConstPressureMoleReactor.cpp:106-221) at the state adjusted by
    // AdaptivePreconditioner::stateAdjustment (components clipped below at atol,
    // src/numerics/AdaptivePreconditioner.cpp:17-22): d(dn_k/dt)/dn_j = d(wdot_k)/dc_j (the
    // reference's ddCi; the -n_i/(V N) dc_i/dn_j terms are left out, as there), the T column by
    // a one-sided difference with dT = T sqrt(eps), and the T row
    // d(dT/dt)/dn_j = (cp_j qdot - m cp sum_k h_k d(dn_k/dt)/dn_j) / (m cp)^2, qdot = sum_k h_k wdot_k V.
    int precJac(const double* z0, double atol, double* J) override {
        const int K = kn->m.K, N = K + 1;
        std::vector<double> z(z0, z0 + N), fc(N), fp(N);
        for (int i = 0; i < N; i++) z[i] = std::max(z[i], atol);
        std::fill(J, J + (size_t)N * N, 0.0);
        // temperature column (perturbed first, then the current state, as the reference)
        const double dT = z[0] * std::sqrt(std::numeric_limits<double>::epsilon());
        std::vector<double> zp(z);
        zp[0] += dT;
        if (rhs(zp.data(), fp.data())) return 1;
        if (rhs(z.data(), fc.data())) return 1;
        for (int j = 0; j < N; j++) J[(size_t)j * N] = (fp[j] - fc[j]) / dT;
        // species block: ddCi at the current state (the work arrays hold it after rhs(z))
        std::vector<double> D((size_t)K * K);
        ddCi(*kn, w, 0, D.data());
        for (int k = 0; k < K; k++)
            for (int j = 0; j < K; j++) J[(size_t)(1 + k) * N + 1 + j] = D[(size_t)k * K + j];
        // temperature row
        double qdot = 0.0;
        std::vector<double> hk(K);
        for (int k = 0; k < K; k++) {
            hk[k] = w.h_RT[k] * w.RT;
            qdot += hk[k] * (w.wdot[k] * vol);
        }
        const double denom = 1.0 / (mcp * mcp);
        for (int j = 0; j < K; j++) {
            double hs = 0.0;
            for (int k = 0; k < K; k++) hs += D[(size_t)k * K + j] * hk[k];
            const double cpj = w.cp_R[j] * kn->R_gas;    // partial molar cp, J/kmol/K
            J[1 + j] = (cpj * qdot - mcp * hs) * denom;
        }
        return 0;
    }
};

// Analytic Jacobian of the reactor RHS over z = [T, Y]; the T column by a one-sided
// difference, the species columns by the chain rule through c = rho*Y/W.
int Reactor::jac(const double* z, const double* fz, double* J) { return reactorJacobian(*this, z, fz, J); }

int reactorJacobian(Reactor& r, const double* z, const double* fz, double* J /*[(K+1)^2] row-major*/) {
    const Mechanism& m = r.kn->m;
    const int K = m.K, N = K + 1;
    std::vector<double> zp(z, z + N), fp(N);
    double dT = std::sqrt(std::numeric_limits<double>::epsilon()) * std::max(1.0, std::fabs(z[0]));
    zp[0] = z[0] + dT;
    int st = r.rhs(zp.data(), fp.data());
    if (st) return st;
    for (int i = 0; i < N; i++) J[(size_t)i * N] = (fp[i] - fz[i]) / dT;
    // state at z (rhs above changed the work arrays)
    r.rhs(z, fp.data());
    Work& w = r.w;
    std::vector<double> Jc((size_t)K * K);
    ddCi(*r.kn, w, 1, Jc.data());
    std::vector<double> X(K), JX(K, 0.0), hJ(K, 0.0), hk(K);
    for (int k = 0; k < K; k++) X[k] = w.ym[k] * w.mmw;
    for (int k = 0; k < K; k++) {
        double s = 0.0;
        for (int l = 0; l < K; l++) s += Jc[(size_t)k * K + l] * X[l];
        JX[k] = s;
        hk[k] = w.h_RT[k] * w.RT;
    }
    for (int j = 0; j < K; j++) {
        double s = 0.0;
        for (int k = 0; k < K; k++) s += hk[k] * Jc[(size_t)k * K + j];
        hJ[j] = s;
    }
    double hJX = 0.0;
    for (int k = 0; k < K; k++) hJX += hJ[k] * X[k];
    double rho = w.density, mmw = w.mmw;
    double cpmix = 0.0;
    for (int k = 0; k < K; k++) cpmix += X[k] * w.cp_R[k];
    double D = rho * r.kn->R_gas * (cpmix / mmw);   // rho * cp_mass
    double G = fz[0];
    for (int j = 0; j < K; j++) {
        double Wj = m.mw[j];
        for (int k = 0; k < K; k++) {
            double Wk = m.mw[k];
            J[(size_t)(1 + k) * N + 1 + j] = (Wk / Wj) * (Jc[(size_t)k * K + j] - JX[k]) + w.wdot[k] * Wk * mmw / (rho * Wj);
        }
        double dH = (rho / Wj) * (hJ[j] - hJX);
        double dD = (rho * r.kn->R_gas / Wj) * (w.cp_R[j] - cpmix);
        J[(size_t)0 * N + 1 + j] = -(dH + G * dD) / D;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Variable-order BDF integrator in Nordsieck form (the CVODES algorithm restated)
// ---------------------------------------------------------------------------
constexpr int QMAX = 5;
constexpr double BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, ADDON = 1e-6;
constexpr double ETA_FIX_MAX = 1.5;     // keep h when the suggested ratio is below this
constexpr double ETA_MAX_FIRST = 1e4, ETA_MAX_EARLY = 10.0, ETA_MAX_GENERAL = 10.0;
constexpr int SMALL_NST = 10;
constexpr double ETA_MIN_EF = 0.1, ETA_MAX_EF = 0.2, ETA_CF = 0.25;
constexpr int SMALL_NEF = 2, MXNEF1 = 3, MXNEF = 7, MXNCF = 10;
constexpr int MAXCOR = 3;
constexpr double NLSCOEF = 0.1, CRDOWN = 0.3, RDIV = 2.0;
constexpr int MSBP = 20;
constexpr double DGMAX = 0.3;
constexpr int MSBJ = 51;
constexpr double DGMAX_JBAD = 0.2;

enum { ST_OK = 0, ST_MAX_STEPS = 1, ST_ERR_FAIL = 2, ST_CONV_FAIL = 3, ST_NONFINITE = 4, ST_H_TOO_SMALL = 5 };

// ILUT(p, tau), the dual-threshold incomplete LU of Saad (1994), row by row, with the
// parameters the reference's AdaptivePreconditioner leaves Eigen's IncompleteLUT
// (AdaptivePreconditioner.cpp:24-38: drop tolerance 1e-12; its fill factor is set only when
// no drop tolerance was, so Eigen's default of 10 holds): a multiplier at or below tau is
// dropped, then the entries of the row below tau times its 2-norm, then all but the p
// largest of its L and of its U part, p = 10 nnz(P) / N + 1.  A zero pivot becomes a small
// multiple of the row norm.  The integrator factors its preconditioner in a fill-reducing
// order, as Eigen's IncompleteLUT orders the matrix first (there AMD; here the greedy minimum
// degree of preconditionerOrdering, which the engine uses too): the drops are below 1e-12 of a
// row's norm, so the order changes the factorisation's cost, not the preconditioner.
void ilutFactor(int N, double* a) {
    const double tau = 1e-12;
    long nnz = 0;
    for (size_t i = 0; i < (size_t)N * N; i++) nnz += a[i] != 0.0;
    const int fill = (int)(nnz * 10 / N) + 1;
    std::vector<double> w(N);
    std::vector<std::pair<double, int>> e;
    for (int i = 0; i < N; i++) {
        double rn = 0.0;
        for (int j = 0; j < N; j++) { w[j] = a[(size_t)i * N + j]; rn += w[j] * w[j]; }
        rn = std::sqrt(rn);
        for (int k = 0; k < i; k++) {
            if (w[k] == 0.0) continue;
            const double f = w[k] / a[(size_t)k * N + k];
            if (std::fabs(f) <= tau) { w[k] = 0.0; continue; }
            w[k] = f;
            for (int j = k + 1; j < N; j++) {
                const double u = a[(size_t)k * N + j];
                if (u != 0.0) w[j] -= f * u;
            }
        }
        auto keep = [&](int j0, int j1) {
            e.clear();
            for (int j = j0; j < j1; j++) {
                if (std::fabs(w[j]) > tau * rn) e.push_back({std::fabs(w[j]), j});
                else w[j] = 0.0;
            }
            if ((int)e.size() > fill) {
                std::nth_element(e.begin(), e.begin() + fill, e.end(),
                                 [](const std::pair<double, int>& x, const std::pair<double, int>& y) { return x.first > y.first; });
                for (size_t q = fill; q < e.size(); q++) w[e[q].second] = 0.0;
            }
        };
        keep(0, i);
        keep(i + 1, N);
        if (w[i] == 0.0) w[i] = std::sqrt(tau) * rn;
        for (int j = 0; j < N; j++) a[(size_t)i * N + j] = w[j];
    }
}

struct Bdf {
    System* r = nullptr;
    int N = 0;            // integrated components (K+1)
    int Nnorm = 0;        // norm divisor: components of the reference state [m, T, Y] (K+2)
    or_bdf_opts o{};
    double uround = std::numeric_limits<double>::epsilon();
    std::vector<std::vector<double>> zn;   // [QMAX+1][N]
    std::vector<double> ewt, acor, y, ftemp, tempv, Jm, Mlu;
    std::vector<float> Mlu32;
    std::vector<int> piv;
    double tn = 0, h = 0, hscale = 0, hprime = 0, eta = 1, etamax = ETA_MAX_FIRST;
    double tau[QMAX + 2] = {0}, tq[6] = {0}, l[QMAX + 1] = {0};
    int q = 1, qprime = 1, qwait = 2, L = 2;
    double gamma = 0, gammap = 0, gamrat = 1, crate = 1, acnrm = 0, saved_tq5 = 0;
    long nst = 0, nstlp = 0, nstlj = 0, nsetups = 0, nje = 0, nni = 0, netf = 0, ncfn = 0;
    std::vector<double> Jsaved;
    bool haveJ = false;
    // GMRES with the adaptive preconditioner (linear_solver = 1)
    std::vector<double> Jp, Pf;        // preconditioner Jacobian (kept between setups), factors of I - gamma Jp
    const int32_t* qord = nullptr;     // the preconditioner's ordering (order[new] = old), or null
    long nli = 0, nps = 0, njtv = 0;    // linear iterations, preconditioner solves, J v products
    bool jcur = false, haveLU = false;
    // ignition tracking (see recordSample)
    long nsamp = 0;
    double ls_t = 0, ls_v = 0, pv_t = 0, pv_v = 0, bs_t = 0, bs_v = 0, nx_t = 0, nx_v = 0;
    bool hasPrev = false, hasRight = false, awaitRight = false;

    double wrms(const double* v) const {
        double s = 0.0;
        for (int i = 0; i < N; i++) { double x = v[i] * ewt[i]; s += x * x; }
        return std::sqrt(s / Nnorm);
    }
    void setEwt(const double* yv) {
        for (int i = 0; i < N; i++) ewt[i] = 1.0 / (o.rtol * std::fabs(yv[i]) + o.atol);
    }

    void init(System* rr, const double* z0, const or_bdf_opts& opts, double tout) {
        r = rr;
        o = opts;
        N = rr->size();
        Nnorm = rr->normSize();
        zn.assign(QMAX + 1, std::vector<double>(N, 0.0));
        ewt.assign(N, 0); acor.assign(N, 0); y.assign(N, 0); ftemp.assign(N, 0); tempv.assign(N, 0);
        Jm.assign((size_t)N * N, 0); Mlu.assign((size_t)N * N, 0); Mlu32.assign((size_t)N * N, 0); piv.assign(N, 0);
        if (o.linear_solver == 1) { Jp.assign((size_t)N * N, 0); Pf.assign((size_t)N * N, 0); }
        for (int i = 0; i < N; i++) zn[0][i] = z0[i];
        tn = 0.0;
        setEwt(z0);
        r->rhs(z0, zn[1].data());
        h = initialStep(tout);
        for (int i = 0; i < N; i++) zn[1][i] *= h;
        hscale = h; hprime = h; q = 1; qprime = 1; L = 2; qwait = L; etamax = ETA_MAX_FIRST;
        tau[1] = h;  // not used before the first step completes
        nst = 0;
        recordSample(0.0, zn[1][0] / h);
    }

    // Initial step (the CVODE user guide's algorithm: bound by 0.1*|tout-t0| and by the
    // ratio |y|/|y'|, estimate ||y''|| by a difference, h0 = 0.5 * sqrt(2/||y''||)).
    double initialStep(double tout) {
        double tdist = std::fabs(tout - tn);
        double tround = uround * std::max(std::fabs(tn), std::fabs(tout));
        double hlb = 100.0 * tround;
        // upper bound
        double hub_inv = 0.0;
        for (int i = 0; i < N; i++) {
            double denom = 0.1 * std::fabs(zn[0][i]) + o.atol;
            hub_inv = std::max(hub_inv, std::fabs(zn[1][i]) / denom);
        }
        double hub = 0.1 * tdist;
        if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
        if (hub < hlb) return std::sqrt(hlb * hub);
        double hg = std::sqrt(hlb * hub);
        double hnew = hg;
        for (int count = 1; count <= 4; count++) {
            // y'' estimate
            for (int i = 0; i < N; i++) y[i] = zn[0][i] + hg * zn[1][i];
            int st = r->rhs(y.data(), tempv.data());
            if (st) { hg *= 0.2; continue; }
            for (int i = 0; i < N; i++) tempv[i] = (tempv[i] - zn[1][i]) / hg;
            double yddnrm = wrms(tempv.data());
            hnew = (yddnrm * hub * hub > 2.0) ? std::sqrt(2.0 / yddnrm) : std::sqrt(hg * hub);
            if (count == 4) break;
            double hrat = hnew / hg;
            if (hrat > 0.5 && hrat < 2.0) break;
            if (count > 1 && hrat > 2.0) { hnew = hg; break; }
            hg = hnew;
        }
        double h0 = 0.5 * hnew;
        h0 = std::min(std::max(h0, hlb), hub);
        if (o.max_time_step > 0) h0 = std::min(h0, o.max_time_step);
        return h0;
    }

    void predict() {
        tn += h;
        for (int k = 1; k <= q; k++)
            for (int j = q; j >= k; j--)
                for (int i = 0; i < N; i++) zn[j - 1][i] += zn[j][i];
    }
    void restore(double saved_t) {
        tn = saved_t;
        for (int k = 1; k <= q; k++)
            for (int j = q; j >= k; j--)
                for (int i = 0; i < N; i++) zn[j - 1][i] -= zn[j][i];
    }
    void rescale() {
        double f = eta;
        for (int j = 1; j <= q; j++) {
            for (int i = 0; i < N; i++) zn[j][i] *= f;
            f *= eta;
        }
        h = hscale * eta;
        hscale = h;
    }

    // Coefficients of Lambda(x) = (1 + x/xi*) prod_{i<q} (1 + x/xi_i) (fixed leading
    // coefficient BDF) and the error-test constants.
    void setCoefficients() {
        for (int i = 0; i <= QMAX; i++) l[i] = 0.0;
        l[0] = l[1] = 1.0;
        double xi_inv = 1.0, xistar_inv = 1.0, alpha0 = -1.0, alpha0_hat = -1.0, hsum = h;
        if (q > 1) {
            for (int j = 2; j < q; j++) {
                hsum += tau[j - 1];
                xi_inv = h / hsum;
                alpha0 -= 1.0 / j;
                for (int i = j; i >= 1; i--) l[i] += l[i - 1] * xi_inv;
            }
            alpha0 -= 1.0 / q;
            xistar_inv = -l[1] - alpha0;
            hsum += tau[q - 1];
            xi_inv = h / hsum;
            alpha0_hat = -l[1] - xi_inv;
            for (int i = q; i >= 1; i--) l[i] += l[i - 1] * xistar_inv;
        }
        double A1 = 1.0 - alpha0_hat + alpha0;
        double A2 = 1.0 + q * A1;
        tq[2] = std::fabs(A1 / (alpha0 * A2));
        tq[5] = std::fabs(A2 * xistar_inv / (l[q] * xi_inv));
        if (qwait == 1) {
            if (q > 1) {
                double C = xistar_inv / l[q];
                double A3 = alpha0 + 1.0 / q;
                double A4 = alpha0_hat + xi_inv;
                double Cpinv = (1.0 - A4 + A3) / A3;
                tq[1] = std::fabs(C * Cpinv);
            } else {
                tq[1] = 1.0;
            }
            double hs = hsum + tau[q];
            double xi2 = h / hs;
            double A5 = alpha0 - 1.0 / (q + 1);
            double A6 = alpha0_hat - xi2;
            double Cppinv = (1.0 - A6 + A5) / A2;
            tq[3] = std::fabs(Cppinv / (xi2 * (q + 2) * A5));
        }
        tq[4] = NLSCOEF / tq[2];
    }

    // M = I - gamma*J, LU with partial pivoting (row-major, in place).
    // convfail: 0 none, 1 retry after a failed solve with a stale J, 2 previous attempt failed
    int setupLinear(int convfail) {
        if (o.linear_solver == 1) return setupPreconditioner(convfail);
        int st = 0;
        double dgamma = std::fabs(gamma / gammap - 1.0);
        bool jbad = !o.jac_reuse || !haveJ || (nst == 0) || (nst >= nstlj + MSBJ) ||
                    (convfail == 1 && dgamma < DGMAX_JBAD) || (convfail == 2);
        if (jbad) {
            if (o.analytic_jacobian) {
                st = r->jac(y.data(), ftemp.data(), Jm.data());
            } else {
                st = dqJacobian();
            }
            if (st) return st;
            nje++;
            nstlj = nst;
            Jsaved = Jm;
            haveJ = true;
            jcur = true;
        } else {
            Jm = Jsaved;
            jcur = false;
        }
        nsetups++;
        for (size_t i = 0; i < (size_t)N * N; i++) Mlu[i] = -gamma * Jm[i];
        for (int i = 0; i < N; i++) Mlu[(size_t)i * N + i] += 1.0;
        int fail = o.lu_fp32 ? luFactor32() : luFactor();
        gammap = gamma;
        gamrat = 1.0;
        crate = 1.0;
        nstlp = nst;
        haveLU = true;
        return fail ? 1 : 0;
    }
    // Preconditioner setup, as CVODE's linear-solver interface drives it for a matrix-free
    // solver (cvLsSetup: the preconditioner's Jacobian is re-evaluated on the first step, every
    // MSBJ = 51 steps, after a convergence failure with a stale one and a small change of
    // gamma, or after a failed step; otherwise only gamma changes) and as the reference's
    // callback answers it (CVodesIntegrator.cpp:67-80: a new Jacobian through
    // ReactorNet::preconditionerSetup, or EigenSparseJacobian::updatePreconditioner with the
    // kept elements): P = I - gamma Jp, factored incompletely.
    int setupPreconditioner(int convfail) {
        const double dgamma = std::fabs(gamma / gammap - 1.0);
        const bool jbad = !haveJ || (nst == 0) || (nst >= nstlj + MSBJ) ||
                          (convfail == 1 && dgamma < DGMAX_JBAD) || (convfail == 2);
        if (jbad) {
            int st = r->precJac(y.data(), o.atol, Jp.data());
            if (st) return st;
            nje++;
            nstlj = nst;
            haveJ = true;
            jcur = true;
        } else {
            jcur = false;
        }
        nsetups++;
        // P' = Q P Q^T in the fill-reducing order (Eigen's IncompleteLUT, which the reference's
        // preconditioner uses, orders the matrix before the factorisation)
        for (int a = 0; a < N; a++)
            for (int b = 0; b < N; b++) {
                const int i = qord ? qord[a] : a, j = qord ? qord[b] : b;
                Pf[(size_t)a * N + b] = -gamma * Jp[(size_t)i * N + j] + (i == j ? 1.0 : 0.0);
            }
        ilut(Pf.data());
        gammap = gamma;
        gamrat = 1.0;
        crate = 1.0;
        nstlp = nst;
        haveLU = true;
        return 0;
    }

    void ilut(double* a) const { ilutFactor(N, a); }
    void precSolve(double* xo) {
        nps++;
        const double* a = Pf.data();
        std::vector<double> xv(N);
        for (int i = 0; i < N; i++) xv[i] = xo[qord ? qord[i] : i];
        double* x = xv.data();
        for (int i = 0; i < N; i++) {
            double s = x[i];
            for (int k = 0; k < i; k++) s -= a[(size_t)i * N + k] * x[k];
            x[i] = s;
        }
        for (int i = N - 1; i >= 0; i--) {
            double s = x[i];
            for (int j = i + 1; j < N; j++) s -= a[(size_t)i * N + j] * x[j];
            x[i] = s / a[(size_t)i * N + i];
        }
        for (int i = 0; i < N; i++) xo[qord ? qord[i] : i] = x[i];
    }
    // J v by the difference quotient (f(y + sig v) - f(y)) / sig, sig = 1 / ||v||_wrms, sig
    // shrunk by 1/4 (at most three tries) when f fails recoverably (CVODE's default
    // Jacobian-times-vector product); y and f(y) are the current Newton iterate.
    int jtimes(const double* v, double* Jv) {
        double sig = 1.0 / wrms(v);
        std::vector<double> work(N);
        int st = 1;
        for (int it = 0; it < 3; it++) {
            for (int i = 0; i < N; i++) work[i] = y[i] + sig * v[i];
            st = r->rhs(work.data(), Jv);
            njtv++;
            if (st == 0) break;
            sig *= 0.25;
        }
        if (st) return st;
        const double siginv = 1.0 / sig;
        for (int i = 0; i < N; i++) Jv[i] = (Jv[i] - ftemp[i]) * siginv;
        return 0;
    }
    // (I - gamma J) x = b by right-preconditioned GMRES, as CVODE's iterative linear-solver
    // interface runs SUNDIALS' SPGMR (cvLsSolve): tolerance eplifac = 0.05 times the Newton
    // test constant tq[4] in the weighted RMS norm (sqrt(N) times it in the scaled 2-norm),
    // both scaling vectors the error weights, zero initial guess, at most MAXL = 5 Krylov
    // vectors, no restarts, modified Gram-Schmidt with one reorthogonalisation when the new
    // vector's norm collapses by the factor 1000, Givens rotations for the least-squares
    // problem.  A right-hand side already below the tolerance is returned as the solution on
    // the first Newton iteration and as zero afterwards.  Returns 0, or 1 (recoverable: not
    // converged and, after the first Newton iteration, only reduced).
    int gmresSolve(double* b, int mnewt) {
        constexpr int MAXL = 5;
        constexpr double EPLIFAC = 0.05;
        const double deltar = EPLIFAC * tq[4];
        if (wrms(b) <= deltar) {
            if (mnewt > 0) std::fill(b, b + N, 0.0);
            return 0;
        }
        const double delta = deltar * std::sqrt((double)N);
        auto dot = [&](const std::vector<double>& x, const std::vector<double>& z) {
            double s = 0.0;
            for (int i = 0; i < N; i++) s += x[i] * z[i];
            return s;
        };
        std::vector<std::vector<double>> V(MAXL + 1, std::vector<double>(N, 0.0));
        double H[MAXL + 1][MAXL] = {{0}};
        double cs[MAXL] = {0}, sn[MAXL] = {0}, g[MAXL + 1] = {0};
        for (int i = 0; i < N; i++) V[0][i] = ewt[i] * b[i];
        const double beta = std::sqrt(dot(V[0], V[0]));
        for (int i = 0; i < N; i++) V[0][i] /= beta;
        g[0] = beta;
        double rho = beta;
        bool converged = false;
        int m = 0;
        std::vector<double> z(N), Az(N);
        while (m < MAXL) {
            const int l = m;
            for (int i = 0; i < N; i++) z[i] = V[l][i] / ewt[i];
            precSolve(z.data());
            if (jtimes(z.data(), Az.data())) return 1;
            std::vector<double>& vn = V[l + 1];
            for (int i = 0; i < N; i++) vn[i] = ewt[i] * (z[i] - gamma * Az[i]);
            const double vk = std::sqrt(dot(vn, vn));
            for (int i = 0; i <= l; i++) {
                H[i][l] = dot(V[i], vn);
                for (int q = 0; q < N; q++) vn[q] -= H[i][l] * V[i][q];
            }
            double vnorm = std::sqrt(dot(vn, vn));
            const double fac = 1000.0 * vk;
            if (fac + vnorm == fac) {
                for (int i = 0; i <= l; i++) {
                    const double p = dot(V[i], vn);
                    for (int q = 0; q < N; q++) vn[q] -= p * V[i][q];
                    H[i][l] += p;
                }
                vnorm = std::sqrt(dot(vn, vn));
            }
            H[l + 1][l] = vnorm;
            for (int i = 0; i < l; i++) {
                const double t1 = H[i][l], t2 = H[i + 1][l];
                H[i][l] = cs[i] * t1 + sn[i] * t2;
                H[i + 1][l] = -sn[i] * t1 + cs[i] * t2;
            }
            const double d = std::hypot(H[l][l], H[l + 1][l]);
            cs[l] = H[l][l] / d;
            sn[l] = H[l + 1][l] / d;
            H[l][l] = d;
            H[l + 1][l] = 0.0;
            g[l + 1] = -sn[l] * g[l];
            g[l] = cs[l] * g[l];
            rho = std::fabs(g[l + 1]);
            m++;
            if (rho <= delta) { converged = true; break; }
            if (vnorm == 0.0) break;
            for (int q = 0; q < N; q++) vn[q] /= vnorm;
        }
        nli += m;
        double yv[MAXL] = {0};
        for (int i = m - 1; i >= 0; i--) {
            double s = g[i];
            for (int j = i + 1; j < m; j++) s -= H[i][j] * yv[j];
            yv[i] = s / H[i][i];
        }
        for (int q = 0; q < N; q++) {
            double s = 0.0;
            for (int j = 0; j < m; j++) s += yv[j] * V[j][q];
            z[q] = s / ewt[q];
        }
        precSolve(z.data());
        for (int q = 0; q < N; q++) b[q] = z[q];
        if (converged) return 0;
        if (rho < beta && mnewt == 0) return 0;
        return 1;
    }

    int dqJacobian() {
        // difference-quotient Jacobian as in the dense CVODE linear solver
        double fnorm = wrms(ftemp.data());
        double srur = std::sqrt(uround);
        double minInc = (fnorm != 0.0) ? (1000.0 * std::fabs(h) * uround * Nnorm * fnorm) : 1.0;
        std::vector<double> yj(y), fj(N);
        for (int j = 0; j < N; j++) {
            double ys = yj[j];
            double inc = std::max(srur * std::fabs(ys), minInc / ewt[j]);
            yj[j] += inc;
            int st = r->rhs(yj.data(), fj.data());
            if (st) return st;
            inc = yj[j] - ys;
            for (int i = 0; i < N; i++) Jm[(size_t)i * N + j] = (fj[i] - ftemp[i]) / inc;
            yj[j] = ys;
        }
        return 0;
    }
    int luFactor() {
        double* a = Mlu.data();
        for (int k = 0; k < N; k++) {
            int p = k;
            double mx = std::fabs(a[(size_t)k * N + k]);
            for (int i = k + 1; i < N; i++) {
                double v = std::fabs(a[(size_t)i * N + k]);
                if (v > mx) { mx = v; p = i; }
            }
            piv[k] = p;
            if (mx == 0.0) return 1;
            if (p != k)
                for (int j = 0; j < N; j++) std::swap(a[(size_t)k * N + j], a[(size_t)p * N + j]);
            double inv = 1.0 / a[(size_t)k * N + k];
            for (int i = k + 1; i < N; i++) {
                double f = a[(size_t)i * N + k] * inv;
                a[(size_t)i * N + k] = f;
                if (f != 0.0)
                    for (int j = k + 1; j < N; j++) a[(size_t)i * N + j] -= f * a[(size_t)k * N + j];
            }
        }
        return 0;
    }
    int luFactor32() {
        for (size_t i = 0; i < (size_t)N * N; i++) Mlu32[i] = (float)Mlu[i];
        float* a = Mlu32.data();
        for (int k = 0; k < N; k++) {
            int p = k;
            float mx = std::fabs(a[(size_t)k * N + k]);
            for (int i = k + 1; i < N; i++) {
                float v = std::fabs(a[(size_t)i * N + k]);
                if (v > mx) { mx = v; p = i; }
            }
            piv[k] = p;
            if (mx == 0.0f) return 1;
            if (p != k)
                for (int j = 0; j < N; j++) std::swap(a[(size_t)k * N + j], a[(size_t)p * N + j]);
            float inv = 1.0f / a[(size_t)k * N + k];
            for (int i = k + 1; i < N; i++) {
                float f = a[(size_t)i * N + k] * inv;
                a[(size_t)i * N + k] = f;
                if (f != 0.0f)
                    for (int j = k + 1; j < N; j++) a[(size_t)i * N + j] -= f * a[(size_t)k * N + j];
            }
        }
        return 0;
    }
    void luSolve(double* b) {
        if (o.lu_fp32) {
            std::vector<float> x(N);
            for (int i = 0; i < N; i++) x[i] = (float)b[i];
            const float* a = Mlu32.data();
            // the factorisation swapped whole rows, so L is in final pivot order:
            // apply every interchange before the forward substitution
            for (int k = 0; k < N; k++)
                if (piv[k] != k) std::swap(x[k], x[piv[k]]);
            for (int k = 0; k < N; k++)
                for (int i = k + 1; i < N; i++) x[i] -= a[(size_t)i * N + k] * x[k];
            for (int k = N - 1; k >= 0; k--) {
                float s = x[k];
                for (int j = k + 1; j < N; j++) s -= a[(size_t)k * N + j] * x[j];
                x[k] = s / a[(size_t)k * N + k];
            }
            for (int i = 0; i < N; i++) b[i] = x[i];
            return;
        }
        const double* a = Mlu.data();
        for (int k = 0; k < N; k++)
            if (piv[k] != k) std::swap(b[k], b[piv[k]]);
        for (int k = 0; k < N; k++)
            for (int i = k + 1; i < N; i++) b[i] -= a[(size_t)i * N + k] * b[k];
        for (int k = N - 1; k >= 0; k--) {
            double s = b[k];
            for (int j = k + 1; j < N; j++) s -= a[(size_t)k * N + j] * b[j];
            b[k] = s / a[(size_t)k * N + k];
        }
    }

    enum { NLS_OK = 0, NLS_RECOVER = 1, NLS_FAIL = 2 };
    // Modified Newton on G(acor) = acor - gamma*f(zn0 + acor) + zn1/l1 = 0
    int newton(bool& callSetup, bool convFailedBefore) {
        double rl1 = 1.0 / l[1];
        int convfail = convFailedBefore ? 2 : 0;
        for (;;) {
            for (int i = 0; i < N; i++) { y[i] = zn[0][i]; acor[i] = 0.0; }
            if (r->rhs(y.data(), ftemp.data())) return NLS_RECOVER;
            if (callSetup) {
                int st = setupLinear(convfail);
                callSetup = false;
                if (st) return NLS_RECOVER;
            }
            double delp = 0.0, del = 0.0;
            int m = 0;
            bool retryWithJ = false;
            for (;;) {
                nni++;
                for (int i = 0; i < N; i++) tempv[i] = gamma * ftemp[i] - (rl1 * zn[1][i] + acor[i]);
                if (o.linear_solver == 1) {
                    // an iterative solve uses the current gamma: no correction for its change
                    if (gmresSolve(tempv.data(), m)) { retryWithJ = !jcur; break; }
                } else {
                    luSolve(tempv.data());
                    if (gamrat != 1.0) {
                        double f = 2.0 / (1.0 + gamrat);
                        for (int i = 0; i < N; i++) tempv[i] *= f;
                    }
                }
                del = wrms(tempv.data());
                for (int i = 0; i < N; i++) { acor[i] += tempv[i]; y[i] = zn[0][i] + acor[i]; }
                if (!std::isfinite(del)) { retryWithJ = !jcur; break; }
                if (m > 0) crate = std::max(CRDOWN * crate, del / delp);
                double dcon = del * std::min(1.0, crate) / tq[4];
                if (dcon <= 1.0) {
                    acnrm = (m == 0) ? del : wrms(acor.data());
                    jcur = false;   // later steps see this Jacobian as stale
                    return NLS_OK;
                }
                m++;
                if (m == MAXCOR || (m >= 2 && del > RDIV * delp)) { retryWithJ = !jcur; break; }
                delp = del;
                if (r->rhs(y.data(), ftemp.data())) { retryWithJ = !jcur; break; }
            }
            (void)convFailedBefore;
            if (retryWithJ && haveLU) {   // stale Jacobian: refresh it and try again at the same h
                callSetup = true;
                convfail = 1;
                continue;
            }
            return NLS_RECOVER;
        }
    }

    // Order change of the Nordsieck history.  Decrease: subtract z_q * W(x),
    // W = x^2 prod_{j=1}^{q-2}(x + xi_j) (keeps value and slope at t_n and the past
    // values at t_{n-1..n-q+2}).  Increase: add c * x^2 prod_{j=1}^{q-1}(x + xi_j) with
    // c = l_q * e / (q+1) the new top coefficient estimated from the saved correction e.
    void decreaseOrder() {
        double w[QMAX + 2] = {0};
        w[2] = 1.0;
        double hsum = 0.0;
        for (int j = 1; j <= q - 2; j++) {
            hsum += tau[j];
            double xi = hsum / hscale;
            for (int i = j + 2; i >= 2; i--) w[i] = w[i] * xi + w[i - 1];
        }
        for (int j = 2; j < q; j++)
            for (int i = 0; i < N; i++) zn[j][i] -= w[j] * zn[q][i];
        for (int i = 0; i < N; i++) zn[q][i] = 0.0;
    }
    void increaseOrder(double lq_prev) {
        double w[QMAX + 2] = {0};
        w[2] = 1.0;
        double hsum = 0.0;
        for (int j = 1; j <= q - 1; j++) {
            hsum += tau[j];
            double xi = hsum / hscale;
            for (int i = j + 2; i >= 2; i--) w[i] = w[i] * xi + w[i - 1];
        }
        double c = lq_prev / (q + 1);
        std::vector<double> top(N);
        for (int i = 0; i < N; i++) top[i] = c * zn[QMAX][i];
        for (int j = 2; j <= q; j++)
            for (int i = 0; i < N; i++) zn[j][i] += w[j] * top[i];
        for (int i = 0; i < N; i++) zn[q + 1][i] = top[i];
    }

    // Ignition marker: the accepted step with the largest dT/dt, refined by the vertex of
    // the parabola through it and its accepted neighbours.
    void recordSample(double t, double v) {
        if (awaitRight) { nx_t = t; nx_v = v; awaitRight = false; hasRight = true; }
        if (nsamp == 0 || v > bs_v) {
            pv_t = ls_t; pv_v = ls_v; hasPrev = nsamp > 0;
            bs_t = t; bs_v = v;
            awaitRight = true; hasRight = false;
        }
        ls_t = t; ls_v = v;
        nsamp++;
    }
    double ignitionTime() const {
        if (!hasPrev || !hasRight) return bs_t;
        double t0 = pv_t, t1 = bs_t, t2 = nx_t;
        double s0 = (bs_v - pv_v) / (t1 - t0), s1 = (nx_v - bs_v) / (t2 - t1);
        double curv = (s1 - s0) / (t2 - t0);
        if (!(curv < 0)) return t1;
        double tv = 0.5 * (t0 + t1) - s0 / (2.0 * curv);
        return std::min(std::max(tv, t0), t2);
    }

    // One internal step (CVode in CV_ONE_STEP mode); returns a status code.
    int step() {
        double saved_t = tn;
        int ncf = 0, nef = 0;
        bool prevConvFail = false;
        if (nst > 0) {
            if (qprime != q) {
                // increase uses l_q of the last completed step, captured before set
                if (qprime == q + 1) increaseOrder(l[q]);
                else decreaseOrder();
                q = qprime;
                L = q + 1;
                qwait = L;
            }
            if (hprime != h) {
                eta = hprime / h;
                rescale();
            }
        }
        setEwt(zn[0].data());
        for (;;) {
            predict();
            setCoefficients();
            double rl1 = 1.0 / l[1];
            gamma = h * rl1;
            if (nst == 0) gammap = gamma;
            gamrat = (nst > 0) ? gamma / gammap : 1.0;
            bool callSetup = (nst == 0) || prevConvFail || (nst >= nstlp + MSBP) ||
                             (std::fabs(gamrat - 1.0) > DGMAX) || !haveLU;
            int nls = newton(callSetup, prevConvFail);
            if (nls != NLS_OK) {
                ncfn++;
                ncf++;
                restore(saved_t);
                if (ncf == MXNCF) return ST_CONV_FAIL;
                eta = ETA_CF;
                rescale();
                prevConvFail = true;
                etamax = 1.0;
                if (std::fabs(h) < 10.0 * uround * std::max(1.0, std::fabs(tn))) return ST_H_TOO_SMALL;
                continue;
            }
            // local error test
            double dsm = acnrm * tq[2];
            if (dsm > 1.0) {
                netf++;
                nef++;
                restore(saved_t);
                if (nef == MXNEF) return ST_ERR_FAIL;
                etamax = 1.0;
                if (nef <= MXNEF1) {
                    eta = 1.0 / (std::pow(BIAS2 * dsm, 1.0 / L) + ADDON);
                    eta = std::max(ETA_MIN_EF, eta);
                    if (nef >= SMALL_NEF) eta = std::min(eta, ETA_MAX_EF);
                    rescale();
                } else {
                    // repeated failures: restart at order 1 with h reduced by ETA_MIN_EF
                    eta = ETA_MIN_EF;
                    h *= eta;
                    hscale = h;
                    qwait = 10;
                    if (q > 1) {
                        q = 1;
                        L = 2;
                    }
                    if (r->rhs(zn[0].data(), tempv.data())) return ST_NONFINITE;
                    for (int i = 0; i < N; i++) zn[1][i] = h * tempv[i];
                    for (int j = 2; j <= QMAX; j++) std::fill(zn[j].begin(), zn[j].end(), 0.0);
                }
                if (std::fabs(h) < 10.0 * uround * std::max(1.0, std::fabs(tn))) return ST_H_TOO_SMALL;
                continue;
            }
            // ---- step accepted: complete it ----
            nst++;
            for (int i = q; i >= 2; i--) tau[i] = tau[i - 1];
            if (q == 1 && nst > 1) tau[2] = tau[1];
            tau[1] = h;
            for (int j = 0; j <= q; j++)
                for (int i = 0; i < N; i++) zn[j][i] += l[j] * acor[i];
            qwait--;
            if (qwait == 1 && q != QMAX) {
                for (int i = 0; i < N; i++) zn[QMAX][i] = acor[i];
                saved_tq5 = tq[5];
            }
            recordSample(tn, zn[1][0] / h);
            prepareNext(dsm);
            return ST_OK;
        }
    }

    void prepareNext(double dsm) {
        if (etamax == 1.0) {  // no growth right after a failure
            qwait = std::max(qwait, 2);
            qprime = q;
            hprime = h;
            eta = 1.0;
            etamax = (nst <= SMALL_NST) ? ETA_MAX_EARLY : ETA_MAX_GENERAL;
            return;
        }
        double etaq = 1.0 / (std::pow(BIAS2 * dsm, 1.0 / L) + ADDON);
        if (qwait != 0) {
            eta = etaq;
            qprime = q;
        } else {
            qwait = 2;
            double etaqm1 = 0.0, etaqp1 = 0.0;
            if (q > 1) {
                double ddn = wrms(zn[q].data()) * tq[1];
                etaqm1 = 1.0 / (std::pow(BIAS1 * ddn, 1.0 / q) + ADDON);
            }
            if (q != o.max_order && saved_tq5 != 0.0) {
                double cquot = (tq[5] / saved_tq5) * std::pow(h / tau[2], (double)L);
                for (int i = 0; i < N; i++) tempv[i] = acor[i] - cquot * zn[QMAX][i];
                double dup = wrms(tempv.data()) * tq[3];
                etaqp1 = 1.0 / (std::pow(BIAS3 * dup, 1.0 / (L + 1)) + ADDON);
            }
            double etam = std::max(etaqm1, std::max(etaq, etaqp1));
            if (etam < ETA_FIX_MAX) {
                eta = 1.0;
                qprime = q;
            } else if (etam == etaq) {
                eta = etaq;
                qprime = q;
            } else if (etam == etaqm1) {
                eta = etaqm1;
                qprime = q - 1;
            } else {
                eta = etaqp1;
                qprime = q + 1;
                for (int i = 0; i < N; i++) zn[QMAX][i] = acor[i];
            }
        }
        if (eta < ETA_FIX_MAX) {
            eta = 1.0;
            qprime = q;  // keep the order when the step is kept
        } else {
            eta = std::min(eta, etamax);
            if (o.max_time_step > 0) eta /= std::max(1.0, std::fabs(h) * eta / o.max_time_step);
        }
        hprime = h * eta;
        etamax = (nst <= SMALL_NST) ? ETA_MAX_EARLY : ETA_MAX_GENERAL;
    }

    // value of the solution at time t inside the last step: sum_j zn[j] * ((t - tn)/h)^j
    void interpolate(double t, double* out) const {
        double s = (t - tn) / h;
        for (int i = 0; i < N; i++) out[i] = zn[q][i];
        for (int j = q - 1; j >= 0; j--)
            for (int i = 0; i < N; i++) out[i] = zn[j][i] + s * out[i];
    }

    // ReactorNet::advance(tout): step past tout, then interpolate.
    int advance(double tout, double* out, long& stepsTaken) {
        long count = 0;
        while (tn < tout) {
            if (count >= o.max_steps) return ST_MAX_STEPS;
            int st = step();
            if (st != ST_OK) return st;
            count++;
        }
        stepsTaken += count;
        interpolate(tout, out);
        return ST_OK;
    }
};

void fillStats(const Bdf& b, int status, int64_t* st) {
    if (!st) return;
    st[OR_ST_STEPS] = b.nst;
    st[OR_ST_RHS] = b.r->nrhs;
    st[OR_ST_NEWTON] = b.nni;
    st[OR_ST_SETUPS] = b.nsetups;
    st[OR_ST_JACS] = b.nje;
    st[OR_ST_ERRFAIL] = b.netf;
    st[OR_ST_CONVFAIL] = b.ncfn;
    st[OR_ST_ORDER] = b.q;
    st[OR_ST_STATUS] = status;
    st[OR_ST_LIN_ITERS] = b.nli;
    st[OR_ST_PREC_SOLVES] = b.nps;
    st[OR_ST_JTIMES] = b.njtv;
}

Kin* buildKin(const std::string& path, const std::string& phase) {
    auto kn = std::make_unique<Kin>();
    kn->m = loadMechanism(path, phase);
    const Mechanism& m = kn->m;
    kn->R_gas = gasConstant();
    for (int k = 0; k < m.K; k++) kn->rmw.push_back(1.0 / m.mw[k]);
    kn->Snet.assign((size_t)m.K * m.R, 0.0);
    for (int i = 0; i < m.R; i++) {
        std::vector<int> rk, pk;
        std::vector<double> rord, rnu, pnu;
        for (int j = m.reacPtr[i]; j < m.reacPtr[i + 1]; j++) {
            rk.push_back(m.reacK[j]); rord.push_back(m.reacOrder[j]); rnu.push_back(m.reacNu[j]);
            kn->Snet[(size_t)m.reacK[j] * m.R + i] -= m.reacNu[j];
        }
        for (int j = m.prodPtr[i]; j < m.prodPtr[i + 1]; j++) {
            pk.push_back(m.prodK[j]); pnu.push_back(m.prodNu[j]);
            kn->Snet[(size_t)m.prodK[j] * m.R + i] += m.prodNu[j];
        }
        kn->reac.add(i, rk, rord, rnu);
        kn->prod.add(i, pk, pnu, pnu);
        if (m.reversible[i]) { kn->revIndex.push_back(i); kn->revProd.add(i, pk, pnu, pnu); }
        else kn->irrev.push_back(i);
    }
    kn->precOrder = preconditionerOrdering(m);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    g_kins.push_back(std::move(kn));
    return g_kins.back().get();
}

int32_t handleOf(Kin* k) {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    for (size_t i = 0; i < g_kins.size(); i++)
        if (g_kins[i].get() == k) return (int32_t)i;
    return -1;
}

template <class F>
void parallelFor(int n, int threads, F&& f) {
    if (threads <= 1 || n <= 1) {
        for (int i = 0; i < n; i++) f(i, 0);
        return;
    }
    threads = std::min(threads, n);
    std::vector<std::thread> pool;
    // static schedule with chunk 1 (openmp_ignition.cpp:59: schedule(static, 1))
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&, t]() {
            for (int i = t; i < n; i += threads) f(i, t);
        });
    for (auto& th : pool) th.join();
}

int runReactor(const Kin* kn, double T0, double P, const double* Y0, double t_end, const or_bdf_opts& o,
               double* Tout, double* Yout, int64_t* stats, double* tign) {
    const int K = kn->m.K;
    if (o.linear_solver == 1 && !o.mole_reactor) {
        if (stats) stats[OR_ST_STATUS] = ST_NONFINITE;
        return ST_NONFINITE;   // GMRES with the preconditioner needs the mole reactor (as the reference)
    }
    Reactor r(kn, P);
    MoleReactor mr(kn, P);
    std::vector<double> z0(K + 1), zout(K + 1);
    z0[0] = T0;
    if (o.mole_reactor) {
        // moles in an initial volume of 1 m^3: n_k = rho Y_k / W_k
        Work w0;
        w0.init(K, kn->m.R);
        setState(*kn, T0, P, Y0, w0);
        for (int k = 0; k < K; k++) z0[1 + k] = w0.density * Y0[k] / kn->m.mw[k];
    } else {
        for (int k = 0; k < K; k++) z0[1 + k] = Y0[k];
    }
    Bdf b;
    if (o.linear_solver == 1) b.qord = kn->precOrder.data();
    b.init(o.mole_reactor ? (System*)&mr : (System*)&r, z0.data(), o, t_end);
    long steps = 0;
    int st = b.advance(t_end, zout.data(), steps);
    if (st != ST_OK) for (int i = 0; i <= K; i++) zout[i] = b.zn[0][i];
    if (o.mole_reactor) {
        // mass fractions from the moles
        double m = 0.0;
        for (int k = 0; k < K; k++) m += zout[1 + k] * kn->m.mw[k];
        for (int k = 0; k < K; k++) zout[1 + k] = zout[1 + k] * kn->m.mw[k] / m;
    }
    if (Tout) *Tout = zout[0];
    if (Yout) for (int k = 0; k < K; k++) Yout[k] = zout[1 + k];
    fillStats(b, st, stats);
    if (tign) *tign = b.ignitionTime();
    return st;
}

}  // namespace

extern "C" {

const char* or_last_error(void) { return g_err.c_str(); }

void or_add_data_directory(const char* dir) {
    if (dir) addDataDirectory(dir);
}

int32_t or_mech_load(const char* path, const char* phase) {
    try {
        Kin* k = buildKin(path, phase ? phase : "");
        return handleOf(k);
    } catch (std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

int32_t or_mech_sizes(int32_t h, int32_t* K, int32_t* R) {
    Kin* k = getKin(h);
    if (!k) { g_err = "bad handle"; return -1; }
    *K = k->m.K;
    *R = k->m.R;
    return 0;
}

int32_t or_species_index(int32_t h, const char* name) {
    Kin* k = getKin(h);
    if (!k) return -1;
    return k->m.speciesIndex(name);
}

int32_t or_molecular_weights(int32_t h, double* mw) {
    Kin* k = getKin(h);
    if (!k) return -1;
    for (int i = 0; i < k->m.K; i++) mw[i] = k->m.mw[i];
    return 0;
}

int32_t or_thermo(int32_t h, double T, double* cp_R, double* h_RT, double* s_R) {
    Kin* k = getKin(h);
    if (!k) return -1;
    Work w;
    w.init(k->m.K, k->m.R);
    speciesThermo(k->m, T, w);
    for (int i = 0; i < k->m.K; i++) {
        if (cp_R) cp_R[i] = w.cp_R[i];
        if (h_RT) h_RT[i] = w.h_RT[i];
        if (s_R) s_R[i] = w.s_R[i];
    }
    return 0;
}

int32_t or_rates(int32_t h, double T, double P, const double* Y, double* kf, double* rkc,
                 double* ropf, double* ropr, double* ropnet, double* wdot) {
    Kin* k = getKin(h);
    if (!k) return -1;
    Work w;
    w.init(k->m.K, k->m.R);
    setState(*k, T, P, Y, w);
    updateROP(*k, w);
    for (int i = 0; i < k->m.R; i++) {
        if (kf) kf[i] = w.rfn[i];
        if (rkc) rkc[i] = w.rkcn[i];
        if (ropf) ropf[i] = w.ropf[i];
        if (ropr) ropr[i] = w.ropr[i];
        if (ropnet) ropnet[i] = w.ropnet[i];
    }
    if (wdot) for (int i = 0; i < k->m.K; i++) wdot[i] = w.wdot[i];
    return 0;
}

int32_t or_ddci(int32_t h, double T, double P, const double* Y, int32_t mode, double* jac) {
    Kin* k = getKin(h);
    if (!k) return -1;
    Work w;
    w.init(k->m.K, k->m.R);
    setState(*k, T, P, Y, w);
    updateROP(*k, w);
    ddCi(*k, w, mode, jac);
    return 0;
}

int32_t or_rates_batch(int32_t h, int32_t n, const double* T, const double* P, const double* Y,
                       double* wdot, int32_t mode, const int32_t* colPtr, const int32_t* rowIdx,
                       double* jacVals, double* gross, int32_t threads) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const int K = k->m.K, R = k->m.R;
    std::vector<Work> ws(std::max(1, (int)threads));
    for (auto& w : ws) w.init(K, R);
    std::vector<std::vector<double>> ybuf(ws.size(), std::vector<double>(K)), jbuf(ws.size());
    parallelFor(n, threads, [&](int s, int t) {
        Work& w = ws[t];
        std::vector<double>& y = ybuf[t];
        for (int j = 0; j < K; j++) y[j] = Y[(size_t)j * n + s];
        setState(*k, T[s], P[s], y.data(), w);
        updateROP(*k, w);
        if (wdot) for (int j = 0; j < K; j++) wdot[(size_t)j * n + s] = w.wdot[j];
        if (gross) {
            const Mechanism& m = k->m;
            for (int j = 0; j < K; j++) gross[(size_t)j * n + s] = 0.0;
            for (int i = 0; i < R; i++) {
                double a = std::fabs(w.ropf[i]) + std::fabs(w.ropr[i]);
                for (int q = m.reacPtr[i]; q < m.reacPtr[i + 1]; q++) gross[(size_t)m.reacK[q] * n + s] += std::fabs(m.reacNu[q]) * a;
                for (int q = m.prodPtr[i]; q < m.prodPtr[i + 1]; q++) gross[(size_t)m.prodK[q] * n + s] += std::fabs(m.prodNu[q]) * a;
            }
        }
        if (jacVals && colPtr && rowIdx) {
            jbuf[t].resize((size_t)K * K);
            ddCi(*k, w, mode, jbuf[t].data());
            for (int c = 0; c < K; c++)
                for (int p = colPtr[c]; p < colPtr[c + 1]; p++)
                    jacVals[(size_t)p * n + s] = jbuf[t][(size_t)rowIdx[p] * K + c];
        }
    });
    return 0;
}

int32_t or_reactor_rhs(int32_t h, double P, const double* y, double* ydot) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const int K = k->m.K;
    Reactor r(k, P);
    std::vector<double> zd(K + 1);
    int st = r.rhs(y + 1, zd.data());
    ydot[0] = 0.0;
    for (int i = 0; i <= K; i++) ydot[1 + i] = zd[i];
    return st;
}

int32_t or_mole_reactor_rhs(int32_t h, double P, const double* z, double* zdot) {
    Kin* k = getKin(h);
    if (!k) return -1;
    MoleReactor r(k, P);
    return r.rhs(z, zdot);
}

int32_t or_ilut(int32_t N, double* a) {
    if (N <= 0 || !a) return -1;
    ilutFactor(N, a);
    return 0;
}

// The fill-reducing order the Krylov path factors its preconditioner in (K + 1 entries over
// z = [T, n_1..n_K], order[new] = old), and the structural pattern of d(wdot)/dc it is built
// on (CSC: colptr K + 1 entries, rowidx up to cap; returns nnz, or -1 when cap is too small).
int32_t or_prec_order(int32_t h, int32_t* order) {
    Kin* k = getKin(h);
    if (!k || !order) return -1;
    std::copy(k->precOrder.begin(), k->precOrder.end(), order);
    return (int32_t)k->precOrder.size();
}

int32_t or_jac_pattern(int32_t h, int32_t cap, int32_t* colptr, int32_t* rowidx) {
    Kin* k = getKin(h);
    if (!k) return -1;
    std::vector<int32_t> cp, ri;
    jacobianPattern(k->m, cp, ri);
    if ((int32_t)ri.size() > cap || !colptr || !rowidx) { g_err = "pattern buffer too small"; return -1; }
    std::copy(cp.begin(), cp.end(), colptr);
    std::copy(ri.begin(), ri.end(), rowidx);
    return (int32_t)ri.size();
}

int32_t or_mole_precond_jacobian(int32_t h, double P, const double* z, double atol, double* J) {
    Kin* k = getKin(h);
    if (!k) return -1;
    MoleReactor r(k, P);
    return r.precJac(z, atol, J);
}

int32_t or_advance_batch(int32_t h, int32_t n, const double* T0, const double* P, const double* Y0,
                         double t_end, const or_bdf_opts* opts, double* T, double* Y,
                         int64_t* stats, double* tign, int32_t threads) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const int K = k->m.K;
    parallelFor(n, threads, [&](int s, int) {
        runReactor(k, T0[s], P[s], Y0 + (size_t)s * K, t_end, *opts, T ? T + s : nullptr,
                   Y ? Y + (size_t)s * K : nullptr, stats ? stats + (size_t)s * OR_NSTAT : nullptr,
                   tign ? tign + s : nullptr);
    });
    return 0;
}

int32_t or_advance_trajectory(int32_t h, double T0, double P, const double* Y0, int32_t nt,
                              const double* times, const or_bdf_opts* opts, double* out, int64_t* stats) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const int K = k->m.K;
    if (opts->linear_solver == 1 && !opts->mole_reactor) return -1;
    Reactor r(k, P);
    MoleReactor mr(k, P);
    std::vector<double> z0(K + 1), zo(K + 1);
    z0[0] = T0;
    if (opts->mole_reactor) {
        Work w0;
        w0.init(K, k->m.R);
        setState(*k, T0, P, Y0, w0);
        for (int i = 0; i < K; i++) z0[1 + i] = w0.density * Y0[i] / k->m.mw[i];
    } else {
        for (int i = 0; i < K; i++) z0[1 + i] = Y0[i];
    }
    Bdf b;
    if (opts->linear_solver == 1) b.qord = k->precOrder.data();
    b.init(opts->mole_reactor ? (System*)&mr : (System*)&r, z0.data(), *opts, times[nt - 1]);
    long steps = 0;
    int st = ST_OK;
    for (int i = 0; i < nt; i++) {
        st = b.advance(times[i], zo.data(), steps);
        if (st != ST_OK) break;
        if (opts->mole_reactor) {
            double m = 0.0;
            for (int j = 0; j < K; j++) m += zo[1 + j] * k->m.mw[j];
            for (int j = 0; j < K; j++) zo[1 + j] = zo[1 + j] * k->m.mw[j] / m;
        }
        for (int j = 0; j <= K; j++) out[(size_t)i * (K + 1) + j] = zo[j];
    }
    fillStats(b, st, stats);
    return st;
}

int32_t or_ignition_by_steps(int32_t h, double T0, double P, const double* Y0, double dT_ign,
                             const or_bdf_opts* opts, double* t_ign, int64_t* stats) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const int K = k->m.K;
    Reactor r(k, P);
    std::vector<double> z0(K + 1);
    z0[0] = T0;
    for (int i = 0; i < K; i++) z0[1 + i] = Y0[i];
    Bdf b;
    // ReactorNet::step() integrates toward t + 1.0
    b.init(&r, z0.data(), *opts, 1.0);
    int st = ST_OK;
    long count = 0;
    // each ReactorNet::step() is one CVode(CV_ONE_STEP) call: the per-call step limit never binds
    while (b.zn[0][0] < T0 + dT_ign) {
        if (count >= 50L * opts->max_steps) { st = ST_MAX_STEPS; break; }
        st = b.step();
        if (st != ST_OK) break;
        count++;
    }
    *t_ign = b.tn;
    fillStats(b, st, stats);
    return st;
}

int32_t or_mole_to_mass(int32_t h, const double* X, double* Y) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const Mechanism& m = k->m;
    double sum = 0.0;
    for (int i = 0; i < m.K; i++) sum += X[i] * m.mw[i];
    for (int i = 0; i < m.K; i++) Y[i] = X[i] * m.mw[i] / sum;
    return 0;
}

int32_t or_equivalence_ratio(int32_t h, double phi, const double* fuelX, const double* oxX, double* Y) {
    Kin* k = getKin(h);
    if (!k) return -1;
    const Mechanism& m = k->m;
    const int K = m.K, E = (int)m.elementNames.size();
    std::vector<double> fuel(K), ox(K);
    or_mole_to_mass(h, fuelX, fuel.data());
    or_mole_to_mass(h, oxX, ox.data());
    auto eidx = [&](const char* e) {
        for (int i = 0; i < E; i++) if (m.elementNames[i] == e) return i;
        return -1;
    };
    int iC = eidx("C"), iS = eidx("S"), iH = eidx("H"), iO = eidx("O");
    auto o2req = [&](const std::vector<double>& y) {
        double r = 0, s = 0;
        for (int q = 0; q < K; q++) {
            s += y[q];
            double x = y[q] / m.mw[q];
            if (iC >= 0) r += x * m.atoms[(size_t)q * E + iC];
            if (iS >= 0) r += x * m.atoms[(size_t)q * E + iS];
            if (iH >= 0) r += x * 0.25 * m.atoms[(size_t)q * E + iH];
        }
        return r / s;
    };
    auto o2pres = [&](const std::vector<double>& y) {
        double r = 0, s = 0;
        for (int q = 0; q < K; q++) { s += y[q]; r += y[q] / m.mw[q] * m.atoms[(size_t)q * E + iO]; }
        return 0.5 * r / s;
    };
    double of = o2req(fuel) - o2pres(fuel), oo = o2req(ox) - o2pres(ox);
    double afr = of / (-oo);
    double sf = 0, so = 0;
    for (int q = 0; q < K; q++) { sf += fuel[q]; so += ox[q]; }
    double tot = 0;
    for (int q = 0; q < K; q++) { Y[q] = phi * fuel[q] / sf + afr * ox[q] / so; tot += Y[q]; }
    for (int q = 0; q < K; q++) Y[q] /= tot;   // setMassFractions normalises
    return 0;
}

}  // extern "C"
