// oracle.h - CPU restatement of the reference hot path.  TEST INFRASTRUCTURE ONLY.
//
// This library is the checker for the GPU engine: only tests, the smoke check and
// the CPU-baseline leg of the benchmark load it.  The product never calls it.
//
// It restates, in scalar FP64 C++ and in the reference's operation order:
//   * NASA7 species thermo           include/cantera/thermo/NasaPoly1.h:83-122, NasaPoly2.h:105-112
//   * ideal-gas state / chem. pot.   src/thermo/IdealGasPhase.cpp:59-66,289-306; src/thermo/Phase.cpp:362-372,501-505
//   * rates of progress + wdot       src/kinetics/BulkKinetics.cpp:457-545; src/kinetics/Kinetics.cpp:408-418,447-457
//   * stoichiometry managers         include/cantera/kinetics/StoichManager.h:131-480,725-797
//   * third bodies                   include/cantera/kinetics/ThirdBodyCalc.h:47-100
//   * falloff (Lindemann / Troe / SRI / Tsang, falloff and chemically activated)
//                                    include/cantera/kinetics/Falloff.h:154-176; src/kinetics/Falloff.cpp:283-494
//   * pressure-dependent Arrhenius   include/cantera/kinetics/PlogRate.h:110-164
//   * Chebyshev                       include/cantera/kinetics/ChebyshevRate.h:133-171
//   * d(wdot)/d(c)                   src/kinetics/BulkKinetics.cpp:712-811; include/cantera/kinetics/MultiRate.h:135-165
//   * const-pressure reactor RHS     src/zeroD/IdealGasConstPressureReactor.cpp:34-110; src/zeroD/ReactorNet.cpp:617-635
//   * integrator                      SUNDIALS CVODES 7.5 (not vendored in the reference: ext/sundials is an
//                                    empty submodule) as configured by src/numerics/CVodesIntegrator.cpp:281-529
//                                    and src/zeroD/ReactorNet.cpp:164-169: variable-order (1-5) BDF in Nordsieck
//                                    form, fixed-leading-coefficient variable-step coefficients, modified Newton
//                                    with a dense LU and a difference-quotient Jacobian, or (mole
//                                    reactor) with right-preconditioned GMRES: CVODE's SPGMR
//                                    iterative linear solver with the reference's adaptive
//                                    preconditioner (src/zeroD/IdealGasConstPressureMoleReactor.cpp:
//                                    16-229, src/zeroD/ReactorNet.cpp:881-903,
//                                    src/numerics/AdaptivePreconditioner.cpp:24-81,
//                                    src/numerics/EigenSparseJacobian.cpp:41-49,
//                                    src/numerics/CVodesIntegrator.cpp:67-88,424-434).  Restated from the
//                                    published algorithm (Cohen & Hindmarsh 1996; Hindmarsh et al., ACM TOMS
//                                    31(3) 2005; Brown, Byrne & Hindmarsh, SIAM J. Sci. Stat. Comput. 10(5) 1989;
//                                    Jackson & Sacks-Davis 1980) and the documented CVODE default parameters.
//
// The reference itself cannot be built in this environment (SUNDIALS, Eigen, yaml-cpp and
// fmt submodules are empty), so parity is pinned by the reference's blessed outputs
// (test_problems/cxx_samples/kin1_blessed.csv, opmenmp_ignition_blessed.txt) and the
// known-answer tests in test/thermo/nasapoly.cpp, test/kinetics/pdep.cpp (PLOG and Chebyshev
// rate constants and rates of progress) and test/python/test_kinetics.py (chemically
// activated rates of progress).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Options of the CPU BDF integrator.
typedef struct {
    double rtol, atol;
    int32_t max_steps;          // per advance() call, as CVodesIntegrator::integrate
    int32_t max_order;          // 1..5
    int32_t analytic_jacobian;  // 0: CVODES-style difference-quotient Jacobian (reference default)
                                // 1: analytic Jacobian (what the GPU engine uses)
    int32_t lu_fp32;            // 1: factor I - gamma*J in single precision (mixed-precision form)
    double max_time_step;       // 0: unlimited
    int32_t jac_reuse;          // 1: keep the last Jacobian between linear-solver setups and
                                //    re-evaluate it only on the first step, every 51 steps and after
                                //    convergence failures (CVODE's documented msbj policy);
                                // 0: evaluate it at every setup (the GPU engine's policy)
    int32_t mole_reactor;       // 1: IdealGasConstPressureMoleReactor, state [T, n_1..n_K] (kmol, initial
                                //    volume 1 m^3); 0: IdealGasConstPressureReactor, state [T, Y]
    int32_t linear_solver;      // 0: dense direct LU; 1: GMRES with the adaptive preconditioner
                                //    (needs mole_reactor = 1)
} or_bdf_opts;

// Per-reactor counters, mirroring CVodesIntegrator::solverStats.
enum { OR_ST_STEPS = 0, OR_ST_RHS, OR_ST_NEWTON, OR_ST_SETUPS, OR_ST_JACS, OR_ST_ERRFAIL,
       OR_ST_CONVFAIL, OR_ST_ORDER, OR_ST_STATUS, OR_ST_LIN_ITERS, OR_ST_PREC_SOLVES, OR_ST_JTIMES,
       OR_NSTAT };

int32_t or_mech_load(const char* path, const char* phase);      // handle >= 0, or -1
void or_add_data_directory(const char* dir);                     // search path of referenced files
int32_t or_mech_sizes(int32_t h, int32_t* K, int32_t* R);
const char* or_last_error(void);
int32_t or_species_index(int32_t h, const char* name);
int32_t or_molecular_weights(int32_t h, double* mw);

// Species thermo at T: cp/R, h/RT, s/R  [K each]
int32_t or_thermo(int32_t h, double T, double* cp_R, double* h_RT, double* s_R);

// One state (T, P, unnormalised mass fractions Y[K]).  Any output pointer may be NULL.
int32_t or_rates(int32_t h, double T, double P, const double* Y, double* kf, double* rkc,
                 double* ropf, double* ropr, double* ropnet, double* wdot);

// Dense d(wdot)/d(c) [K*K row-major, jac[k*K+j] = d wdot_k / d c_j] at const T and
// other c.  mode 0: the reference's own scheme (falloff [M] derivative by one-sided
// difference, delta 1e-8); mode 1: fully analytic.
int32_t or_ddci(int32_t h, double T, double P, const double* Y, int32_t mode, double* jac);

// Batch over n states in species-major layout Y[K][n] (the GPU API layout), using
// `threads` host threads.  wdot [K][n]; jac [nnz][n] on the pattern colPtr/rowIdx (may be NULL);
// gross [K][n] = sum_i |nu_ki| (|ropf_i| + |ropr_i|), the scale of wdot_k's cancellation (may be NULL).
int32_t or_rates_batch(int32_t h, int32_t n, const double* T, const double* P, const double* Y,
                       double* wdot, int32_t mode, const int32_t* colPtr, const int32_t* rowIdx,
                       double* jacVals, double* gross, int32_t threads);

// Reactor right-hand side for y = [m, T, Y1..YK] at pressure P: ydot[K+2].
int32_t or_reactor_rhs(int32_t h, double P, const double* y, double* ydot);

// Mole reactor (z = [T, n_1..n_K], kmol) at pressure P: right-hand side zdot[K+1], and the
// preconditioner's Jacobian elements J[(K+1)^2] (row-major) at z clipped below at atol.
int32_t or_mole_reactor_rhs(int32_t h, double P, const double* z, double* zdot);
int32_t or_mole_precond_jacobian(int32_t h, double P, const double* z, double atol, double* J);
/* The adaptive preconditioner's ILUT (the factorisation the Krylov path uses) of one N x N
 * row-major matrix, in place: L (unit diagonal, strictly lower) and U. */
int32_t or_ilut(int32_t N, double* a);
int32_t or_prec_order(int32_t h, int32_t* order);
int32_t or_jac_pattern(int32_t h, int32_t cap, int32_t* colptr, int32_t* rowidx);

// Advance n independent constant-pressure reactors from t=0 to t_end.
//  T0[n], P[n], Y0[n][K] (reactor-major); outputs T[n], Y[n][K], stats[n][OR_NSTAT],
//  tign[n] (time of maximum dT/dt, refined by a parabola through the accepted steps).
int32_t or_advance_batch(int32_t h, int32_t n, const double* T0, const double* P, const double* Y0,
                         double t_end, const or_bdf_opts* opts, double* T, double* Y,
                         int64_t* stats, double* tign, int32_t threads);

// Trajectory of one reactor: advance to each of times[nt] in turn (like repeated
// ReactorNet::advance), writing T and Y at each output time: out[nt][1+K].
int32_t or_advance_trajectory(int32_t h, double T0, double P, const double* Y0, int32_t nt,
                              const double* times, const or_bdf_opts* opts, double* out, int64_t* stats);

// Ignition by single internal steps (ReactorNet::step): step until T >= T0 + dT_ign,
// returning the time reached (the reference openmp_ignition sample's definition).
int32_t or_ignition_by_steps(int32_t h, double T0, double P, const double* Y0, double dT_ign,
                             const or_bdf_opts* opts, double* t_ign, int64_t* stats);

// Mixture helpers: mole fractions -> mass fractions; equivalence-ratio mixture
// (ThermoPhase::setEquivalenceRatio, molar basis; src/thermo/ThermoPhase.cpp:879-910).
int32_t or_mole_to_mass(int32_t h, const double* X, double* Y);
int32_t or_equivalence_ratio(int32_t h, double phi, const double* fuelX, const double* oxX, double* Y);

#ifdef __cplusplus
}
#endif
