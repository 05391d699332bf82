// mechanism.h - flat, species-major description of an ideal-gas reaction mechanism.
//
// Built once on the host from a Cantera YAML file (the semantics of Cantera's
// loader: reference src/base/Solution.cpp:242-330, src/kinetics/KineticsFactory.cpp:
// 108-218, src/kinetics/Reaction.cpp:93-135,284-320,389-555,576-617,777-956,
// src/base/Units.cpp:44,53,562-571,634-741) and then copied to the GPU as-is.
// Every array is plain data: no pointers into YAML, no virtual dispatch.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gbchem {

// Physical constants (reference include/cantera/base/ct_defs.h:84-163).
constexpr double kAvogadro = 6.02214076e26;       // 1/kmol
constexpr double kBoltzmann = 1.380649e-23;       // J/K
constexpr double kOneAtm = 1.01325e5;             // Pa
constexpr double kSmallNumber = 1.e-300;
constexpr double kBigNumber = 1.e300;
inline double gasConstant() { return kAvogadro * kBoltzmann; }  // J/kmol/K

// Rate-constant form of a reaction.
enum RateKind : int32_t {
    kArrhenius = 0,        // k = A T^b exp(-Ea/RT)
    kThreeBody = 1,        // Arrhenius, rate of progress multiplied by [M]
    kLindemann = 2,        // falloff, F = 1
    kTroe = 3,             // falloff, Troe F(Pr, T)
    kPlog = 4,             // pressure-dependent Arrhenius: ln k interpolated linearly in ln P
    kChebyshev = 5,        // log10 k = Chebyshev series in reduced 1/T and log10 P
    kSri = 6,              // falloff, SRI F(Pr, T)
    kTsang = 7,            // falloff, Tsang F(Pr, T) (the Troe form with Fcent = a + b T)
};
inline bool isFalloffKind(int k) { return k == kLindemann || k == kTroe || k == kSri || k == kTsang; }

// Stoichiometry bucket of one side of a reaction (reference StoichManager.h:676-722):
// C1/C2/C3 when every coefficient equals its order, is integral and at most three
// molecules take part (repeated species are expanded); otherwise CN (general power law).
enum StoichBucket : int32_t { kC1 = 1, kC2 = 2, kC3 = 3, kCN = 0 };

struct Mechanism {
    std::string source;      // file path
    std::string phase;       // phase name
    int K = 0;               // species
    int R = 0;               // reactions
    double Pref = kOneAtm;   // reference pressure of the NASA7 data

    // ---- species ----
    std::vector<std::string> speciesNames;   // [K]
    std::vector<double> mw;                  // [K] kg/kmol
    std::vector<double> nasaTmid;            // [K]
    std::vector<double> nasaLow;             // [K][7]  a0..a6, T <= Tmid
    std::vector<double> nasaHigh;            // [K][7]  a0..a6, T >  Tmid
    std::vector<double> Tmin, Tmax;          // [K]
    std::vector<std::string> elementNames;   // [E]
    std::vector<double> elementWeights;      // [E]
    std::vector<double> atoms;               // [K][E]

    // ---- reactions ----
    std::vector<std::string> equations;      // [R] (as written in the file)
    std::vector<int32_t> kind;               // [R] RateKind
    std::vector<int32_t> reversible;         // [R] 0/1
    std::vector<int32_t> duplicate;          // [R] 0/1
    std::vector<double> dn;                  // [R] sum(nu_prod) - sum(nu_reac)
    std::vector<double> A, b, EaR;           // [R] high-pressure (or only) Arrhenius
    std::vector<double> A0, b0, Ea0R;        // [R] low-pressure Arrhenius (falloff only)
    std::vector<double> troe;                // [R][4] a, 1/T3, 1/T1, T2 (Troe only)
    std::vector<double> falloffX;            // [R][5] SRI a, b, c, d, e; Tsang a, b
    std::vector<int32_t> chemAct;            // [R] 1: chemically-activated falloff, k = klow F / (1 + Pr)

    // Pressure-dependent Arrhenius (PlogRate::setRates, reference src/kinetics/PlogRate.cpp:
    // 91-120): reaction i has pressure levels plogPtr[i] .. plogPtr[i+1], ascending in ln P
    // and bracketed by the reference's sentinels at ln P = -1000 and +1000 (copies of the
    // first and last level); level l holds the Arrhenius expressions plogFirst[l] ..
    // plogLast[l] of the rate tables, summed at evaluation.
    std::vector<int32_t> plogPtr;            // [R+1]
    std::vector<double> plogLogP;            // [levels]
    std::vector<int32_t> plogFirst, plogLast;   // [levels]
    std::vector<double> plogA, plogB, plogEaR;  // [rates]

    // Chebyshev (ChebyshevRate::setLimits / setData, reference src/kinetics/ChebyshevRate.cpp:
    // 64-118): nT x nP coefficients, row-major (temperature index first), with the unit
    // offset log10(conversion factor) already added to the (0, 0) coefficient.
    std::vector<int32_t> chebPtr;            // [R+1] into chebCoef
    std::vector<int32_t> chebNT, chebNP;     // [R]
    std::vector<double> chebLim;             // [R][4] TrNum, TrDen, PrNum, PrDen
    std::vector<double> chebCoef;

    // Third bodies, in installation order (reference ThirdBodyCalc.h:23-45).
    std::vector<int32_t> tbOfRxn;            // [R] index into the tables below or -1
    std::vector<int32_t> tbRxn;              // [NTB] reaction index
    std::vector<double> tbDefault;           // [NTB] default efficiency
    std::vector<int32_t> tbMassAction;       // [NTB] 1: ropf *= [M]; 0: falloff
    std::vector<int32_t> tbPtr;              // [NTB+1] CSR over the species lists
    std::vector<int32_t> tbSpecies;          // [nnz] species index (ascending)
    std::vector<double> tbEffMinusDefault;   // [nnz] efficiency - default

    // Reactant side: species, order and stoichiometric coefficient, in the order the
    // reference stoichiometry manager receives them (species-name order of the
    // reaction's composition map, then any non-reactant orders).
    std::vector<int32_t> reacPtr;            // [R+1]
    std::vector<int32_t> reacK;
    std::vector<double> reacOrder, reacNu;
    std::vector<int32_t> reacBucket;         // [R] StoichBucket
    // Product side (orders equal coefficients).
    std::vector<int32_t> prodPtr;            // [R+1]
    std::vector<int32_t> prodK;
    std::vector<double> prodNu;
    std::vector<int32_t> prodBucket;         // [R]

    int speciesIndex(const std::string& name) const;  // -1 if absent
    int nThirdBody() const { return (int)tbRxn.size(); }
};

// Load phase `phase` (empty: the first phase) of a Cantera YAML mechanism.
// Throws std::runtime_error with a message naming the file and line on failure.
// Sections named "file.yaml/section" are looked up next to the including file, then in
// the working directory, then in the data directories (addDataDirectory).
Mechanism loadMechanism(const std::string& path, const std::string& phase);

// Add a directory to the search path for mechanism files referenced by other files
// (Application::addDataDirectory, reference src/base/application.cpp:286).
void addDataDirectory(const std::string& dir);

// Mass fractions of the mixture with equivalence ratio phi of fuel and oxidizer given
// as mole fractions [K] (ThermoPhase::setEquivalenceRatio with the molar basis,
// reference src/thermo/ThermoPhase.cpp:783-910); the result is normalised.
void equivalenceRatioMassFractions(const Mechanism& m, double phi, const double* fuelX,
                                   const double* oxX, double* Y);

// Structural nonzeros of d(wdot)/d(c) (the union of every reaction's species
// couplings and its third-body efficiencies, including default efficiencies),
// returned as compressed sparse columns: colPtr[K+1], rowIdx[nnz], rows ascending.
void jacobianPattern(const Mechanism& m, std::vector<int32_t>& colPtr, std::vector<int32_t>& rowIdx);

// Fill-reducing ordering of the Krylov path's preconditioner I - gamma Jp over z = [T, n_1..n_K]
// (the reference factors it with Eigen's IncompleteLUT, which orders the matrix first): a
// greedy minimum-degree ordering of the symmetric structure of Jp + Jp^T (species block from
// jacobianPattern, dense T row and column), ties to the lowest index.  order[new] = old.
std::vector<int32_t> preconditionerOrdering(const Mechanism& m);

}  // namespace gbchem
