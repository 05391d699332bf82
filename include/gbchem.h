/* gbchem.h - C ABI of the GB300 batched chemistry engine.
 *
 * A batched drop-in behind Cantera's hot path for many independent, constant-pressure,
 * ideal-gas reactors.  The verbs and conventions mirror Cantera's generated C interface
 * (CLib): int32 handles, an int32 status where 0 means success and GB_ERR (-999) an
 * error whose message gb_get_error() returns, and no exception crossing the ABI
 * (reference: interfaces/clib/include/cantera_clib/clib_defs.h ERR = -999;
 * interfaces/clib/src/clib_utils.h:32-52 handleAllExceptions).
 *
 * Array layout: state batches are species-major, Y[k*n + s] for species k of state s
 * (T[s], P[s] one value per state).  Pointers are host pointers unless `flags` has
 * GB_DEVICE_POINTERS, in which case they are CUDA device pointers on the engine's
 * device; the engine reads them after the work already issued to the legacy and the
 * per-thread default streams (arrays written on another stream must be synchronised by the
 * caller first).  Every call returns after the GPU work it starts has finished.
 *
 * Threading: a handle is used by one host thread at a time; distinct handles may be
 * used from distinct threads.  The last error message is kept per host thread.
 */
#ifndef GBCHEM_H
#define GBCHEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_ERR (-999)
#define GB_DEVICE_POINTERS 1

/* ---- mechanisms -------------------------------------------------------------------
 * gb_mech_load replaces newSolution(yaml, phase, "none") (src/base/Solution.cpp:242-330)
 * for ideal-gas phases with NASA7 thermo and elementary, three-body, falloff (Lindemann,
 * Troe, SRI, Tsang; falloff or chemically activated), pressure-dependent Arrhenius (PLOG)
 * and Chebyshev reactions.  Returns a handle >= 0 or GB_ERR. */
int32_t gb_mech_load(const char* yaml_path, const char* phase_name);
/* Adds a directory to the search path of files that a mechanism references
 * ("gri30.yaml/species"): CLib ct_addDataDirectory (interfaces/sourcegen/src/sourcegen/
 * headers/ct.yaml:12, Application::addDataDirectory, src/base/application.cpp:286).
 * Returns 0. */
int32_t gb_add_data_directory(const char* dir);
int32_t gb_mech_del(int32_t mech);
int32_t gb_mech_n_species(int32_t mech);                  /* Kinetics::nTotalSpecies */
int32_t gb_mech_n_reactions(int32_t mech);                /* Kinetics::nReactions */
int32_t gb_mech_species_name(int32_t mech, int32_t k, int32_t buflen, char* buf);
int32_t gb_mech_species_index(int32_t mech, const char* name);  /* -1 if absent */
int32_t gb_mech_molecular_weights(int32_t mech, int32_t buflen, double* mw);
/* Mass fractions Y[K] of the mixture with equivalence ratio phi of a fuel and an
 * oxidizer given as mole fractions [K] (ThermoPhase::setEquivalenceRatio, molar basis;
 * src/thermo/ThermoPhase.cpp:879-910). */
int32_t gb_mech_equivalence_ratio(int32_t mech, double phi, const double* fuelX, const double* oxX,
                                  int32_t buflen, double* Y);
/* Reference-state species properties at n temperatures, host arrays [K][n] (species-major):
 * cp/R, h/RT and s/R of the NASA7 polynomials, the low range up to and including the midpoint
 * temperature (NasaPoly1::updateProperties, include/cantera/thermo/NasaPoly1.h:83-122;
 * NasaPoly2::updateProperties, NasaPoly2.h:105-112; MultiSpeciesThermo::update,
 * src/thermo/MultiSpeciesThermo.cpp:94-107).  Evaluated on the host, for single states and
 * setup (the kernels evaluate their own); every temperature must be positive. */
int32_t gb_mech_species_thermo(int32_t mech, int32_t n, const double* T, double* cp_R, double* h_RT,
                               double* s_R);
/* The reference pressure of the species' thermodynamic data in Pa (ThermoPhase::refPressure),
 * or -999.999 with an invalid handle. */
double gb_mech_reference_pressure(int32_t mech);

/* ---- kinetics ----------------------------------------------------------------------
 * Batched Kinetics::getNetProductionRates (src/kinetics/Kinetics.cpp:447-457; CLib
 * kin_getNetProductionRates, interfaces/sourcegen/src/sourcegen/headers/ctkin.yaml:46).
 * n states (T [K], P [Pa], unnormalised mass fractions Y[K][n]) -> wdot[K][n] kmol/m^3/s.
 * bufLen must be >= K*n. */
int32_t gb_kin_net_production_rates(int32_t mech, int32_t n, const double* T, const double* P,
                                    const double* Y, int32_t bufLen, double* wdot, int32_t flags);

/* Structural nonzeros of d(wdot)/d(c) as compressed sparse columns (colptr[K+1],
 * rowidx[nnz], rows ascending in each column).  gb_kin_jac_nnz returns nnz. */
int32_t gb_kin_jac_nnz(int32_t mech);
int32_t gb_kin_jac_pattern(int32_t mech, int32_t ncolptr, int32_t* colptr, int32_t nnz, int32_t* rowidx);

/* Batched Kinetics::netProductionRates_ddCi (src/kinetics/BulkKinetics.cpp:794-811;
 * include/cantera/kinetics/Kinetics.h:1148): d(wdot_k)/d(c_j) at constant T and other
 * concentrations, values vals[p*n + s] on the pattern above (p = slot).  The falloff
 * [M]-dependence is differentiated analytically (the reference uses a one-sided
 * difference with delta 1e-8).  wdot may be NULL; if not, wdot[K][n] is written too. */
int32_t gb_kin_net_production_rates_ddCi(int32_t mech, int32_t n, const double* T, const double* P,
                                         const double* Y, int32_t nnz, double* vals, double* wdot,
                                         int32_t flags);

/* Device time in ms of the kernel launch of the last rates or ddCi call on this mechanism
 * (CUDA events on the engine's stream around the launch; no counterpart in the
 * reference), or -999.999 with an invalid handle. */
double gb_kin_last_kernel_ms(int32_t mech);

/* ---- batched reactor network ------------------------------------------------------------
 * gb_net_* replace ReactorNet over IdealGasConstPressureReactor (src/zeroD/ReactorNet.cpp:
 * 37-357; CLib reactornet_advance, headers/ctreactornet.yaml:19-20): n independent reactors,
 * each integrated by a variable-order (1..5) BDF method with modified Newton and a dense LU
 * of I - gamma*J, per-reactor step and order control. */
typedef struct {
    double rtol;            /* ReactorNet::setRelativeTolerance; default 1e-9 */
    double atol;            /* ReactorNet::setAbsoluteTolerance; default 1e-15 */
    int32_t max_steps;      /* ReactorNet::setMaxSteps (per advance call); default 20000 */
    int32_t max_order;      /* 1..5; default 5 */
    double max_time_step;   /* ReactorNet::setMaxTimeStep; 0 = unlimited */
    int32_t lu_precision;   /* 64: factor I - gamma*J in FP64; 32: in FP32 (residual, RHS,
                               error norm and step control stay FP64) */
    int32_t warps_per_block;/* reactors per thread block; 0 = autotuned */
    int32_t use_graph;      /* 1: launch the advance through a captured CUDA graph */
    int32_t matrix_placement; /* Newton matrix: 0 = automatic, 1 = shared memory, 2 = an
                               L2-resident global slot per warp (frees shared memory for
                               more resident reactors) */
    int32_t mechanism_in_shared; /* mechanism data copied into each block's shared memory:
                               0 = automatic, 1 = none, 2 = what the right-hand side reads,
                               3 = also the Jacobian's data, 4 = everything but the rest */
    int32_t jacobian_reuse; /* 1: keep the Jacobian between linear-solver setups as CVODE
                               does (a new one on the first step, after 51 steps, after a
                               convergence failure with a stale one or a failed step); 0
                               (default): a new Jacobian at every setup - with the analytic
                               Jacobian this is faster (gri30: reuse raised the steps per
                               reactor from 867 to 1,128 and cost 19 % throughput) */
    int32_t lu_staging;     /* with the Newton matrices in global memory, factor them in
                               shared-memory buffers a block keeps for that (a warp that finds
                               none free factors in place): 0 = automatic (none: the buffers
                               take L1 capacity the global matrices need), k > 0 = at most k */
    int32_t linear_solver;  /* 0 (default): the mass-fraction reactor [T, Y] with the analytic
                               Jacobian and a dense LU of I - gamma*J.  1: the reference's
                               preconditioned Krylov path - IdealGasConstPressureMoleReactor
                               (state T and the species amounts in kmol, an initial volume of
                               1 m^3; src/zeroD/IdealGasConstPressureMoleReactor.cpp:34-104)
                               with ReactorNet's GMRES solver and the AdaptivePreconditioner
                               (src/zeroD/ReactorNet.cpp:881-908, src/numerics/
                               AdaptivePreconditioner.cpp:17-81; Python: net.preconditioner =
                               AdaptivePreconditioner()): an approximate Jacobian (ddCi species
                               block, difference T column, enthalpy T row) factored by ILUT,
                               J v by difference quotients.  With lu_precision 32 the ILUT
                               factors and their triangular solves are FP32 (J v, GMRES and step
                               control stay FP64).  The state handed in and out stays T and mass
                               fractions. */
} gb_net_options;

void gb_net_default_options(gb_net_options* opts);
int32_t gb_net_new(int32_t mech, int32_t n, const gb_net_options* opts);
int32_t gb_net_del(int32_t net);
/* Set the initial state of every reactor and restart the integrators at time 0
 * (IdealGasConstPressureReactor::getState; ReactorNet::reinitialize). */
int32_t gb_net_set_state(int32_t net, const double* T, const double* P, const double* Y, int32_t flags);
/* Integrator settings of a running network, applied from the next step on without restarting
 * the integration (ReactorNet::setTolerances / setMaxSteps / setMaxTimeStep,
 * src/zeroD/ReactorNet.cpp:179-183,218-231,341-344, which pass them to CVODES unchanged:
 * src/numerics/CVodesIntegrator.cpp:171-180,209-230).  A tolerance <= 0 keeps the current
 * value; max_steps must be positive; max_time_step 0 means unlimited.  Returns 0 or GB_ERR. */
int32_t gb_net_set_tolerances(int32_t net, double rtol, double atol);
int32_t gb_net_set_max_steps(int32_t net, int32_t max_steps);
int32_t gb_net_set_max_time_step(int32_t net, double max_time_step);
/* Advance every reactor to time t (ReactorNet::advance: step past t, interpolate back).
 * Returns the number of reactors whose integration failed (status != 0), or GB_ERR. */
int32_t gb_net_advance(int32_t net, double t);
/* One internal step of every reactor (ReactorNet::step, src/zeroD/ReactorNet.cpp:435-441,
 * which makes one CV_ONE_STEP call towards time + 1: CVodesIntegrator::step,
 * src/numerics/CVodesIntegrator.cpp:531-549; Python ReactorNet.step,
 * interfaces/cython/cantera/reactor.py:1822).  Each reactor's state becomes its state at its
 * new internal time, written to times[n] (host, or device with GB_DEVICE_POINTERS; may be
 * NULL).  The reactors are independent, so their times differ; the network's time
 * (gb_net_time) becomes the latest of them, and a later gb_net_advance(t) needs t >= that
 * time (reactors behind it step on, the others interpolate back within their last step).
 * Returns the number of reactors whose step failed, or GB_ERR. */
int32_t gb_net_step(int32_t net, double* times, int32_t flags);
double gb_net_time(int32_t net);
/* Device time of the integrator launch of the last gb_net_advance, in ms (CUDA events on
 * the engine's stream around the launch). */
double gb_net_last_advance_ms(int32_t net);
int32_t gb_net_get_state(int32_t net, double* T, double* Y, int32_t flags);
/* The k-th time derivative (0 <= k <= 5) of every reactor's integrator state at its output
 * time - the network's time after gb_net_advance, the reactor's own time after gb_net_step or
 * a failed step - from its Nordsieck history (ReactorNet::getDerivative,
 * src/zeroD/ReactorNet.cpp:721-726, through CVodesIntegrator::derivative and CVodeGetDky,
 * src/numerics/CVodesIntegrator.cpp:551-556).  out[N][n], species-major, N = K + 1: row 0 the
 * temperature, rows 1..K the mass fractions (linear_solver 0) or the species amounts in kmol
 * per m^3 of initial volume (linear_solver 1).  The interpolating polynomial of a reactor at
 * order q < k gives 0 (CVODES refuses k > q for its one system).  Host array, or device with
 * GB_DEVICE_POINTERS.  Returns 0, or GB_ERR before the first integration after a state was
 * set. */
int32_t gb_net_get_derivative(int32_t net, int32_t k, double* out, int32_t flags);

/* Checkpoint of a network (no counterpart in the reference, whose CVODES state cannot be
 * saved; the nearest is ReactorNet::reinitialize from the reactors' states,
 * src/zeroD/ReactorNet.cpp:306-322): its time, every reactor's integrator record (Nordsieck
 * array, step size, order, error-test history, ignition marker), counters, status and the
 * state at the network's time, into a host buffer of gb_net_checkpoint_bytes bytes.
 * gb_net_restore puts such a checkpoint into a network of the same size and mechanism;
 * advancing it then continues the saved integration exactly (bit for bit).  The returned size
 * is an int64, or GB_ERR. */
int64_t gb_net_checkpoint_bytes(int32_t net);
int32_t gb_net_checkpoint(int32_t net, void* buf, int64_t bytes);
int32_t gb_net_restore(int32_t net, const void* buf, int64_t bytes);

/* Launch shape of the integrator: info[0..5] = blocks, reactors (warps) per block, shared
 * bytes per warp, mechanism bytes in shared memory per block, Newton matrices in shared (1)
 * or global (2) memory, factorisation buffers per block.  (No counterpart in the reference.) */
int32_t gb_net_launch_info(int32_t net, int32_t* info);

/* Per-reactor status: 0 ok, 1 max steps, 2 repeated error-test failures, 3 repeated
 * convergence failures, 4 non-finite state, 5 step size too small. */
enum { GB_OK = 0, GB_MAX_STEPS = 1, GB_ERR_TEST_FAILS = 2, GB_CONV_FAILS = 3,
       GB_NONFINITE = 4, GB_H_TOO_SMALL = 5 };
int32_t gb_net_get_status(int32_t net, int32_t* status);

/* Counters per reactor, stats[s*GB_NSTAT + i] (CVodesIntegrator::solverStats names). */
enum { GB_STAT_STEPS = 0, GB_STAT_RHS, GB_STAT_NEWTON, GB_STAT_SETUPS, GB_STAT_JACS,
       GB_STAT_ERRFAIL, GB_STAT_CONVFAIL, GB_STAT_ORDER, GB_NSTAT };
int32_t gb_net_solver_stats(int32_t net, int64_t* stats);

/* Counters of the Krylov path per reactor, stats[s*3 + i]: linear (GMRES) iterations,
 * preconditioner solves, Jacobian-times-vector products (CVodesIntegrator::solverStats
 * lin_iters, prec_solves, jt_vec_prod_evals; src/numerics/CVodesIntegrator.cpp:572-621).
 * GB_ERR for a network with the dense solver. */
int32_t gb_net_krylov_stats(int32_t net, int64_t* stats);

/* Batched incomplete factorisation of the adaptive preconditioner (AdaptivePreconditioner::
 * factorize, src/numerics/AdaptivePreconditioner.cpp:42-55, with the ILUT parameters it sets,
 * :24-38): n matrices P[n][N][N] (row-major, host) are factored by ILUT(p, tau) with
 * tau = 1e-12 and p = 10 nnz(P)/N + 1, one warp per matrix on the current device; F[n][N][N]
 * (host) receives L (unit diagonal, strictly lower part) and U in place.  N <= 256. */
int32_t gb_precond_ilut(int32_t n, int32_t N, const double* P, double* F);

/* Time of the largest dT/dt seen at accepted steps since gb_net_set_state, refined by the
 * vertex of the parabola through that step and its accepted neighbours. */
int32_t gb_net_ignition_times(int32_t net, double* tign);

/* ---- allocation-free advance (no counterpart in the reference) -----------------------
 * For callers that cannot allocate device memory (their own allocator owns the device, or
 * the device memory is fully budgeted): advance n reactors from time 0 to t_end in one
 * call, with the same integrator as gb_net_advance, allocating nothing.  T[n] and Y[K][n]
 * (in place) and P[n] are device pointers on the current device; status[n] (device)
 * receives the per-reactor status codes below.  opts may be NULL (defaults; use_graph is
 * ignored; the Newton matrices stay in shared memory; a new Jacobian at every setup).  The integrator records live in a 16 MiB array in the library's device image,
 * so n is limited to what fits (about 5,500 reactors for GRI-Mech 3.0); a larger n fails
 * with GB_ERR and a message giving the limit.  The call is ordered on `stream` (a
 * cudaStream_t; NULL is the default stream) and synchronises it before returning.  Every
 * call on a device shares that one array: calls of this process are serialised by a lock,
 * and calls that overlap on one device from other code that bypasses it would race.  The
 * call queries its pointers and synchronises its stream, so it cannot be made while that
 * stream is being captured (it returns GB_ERR then); its first call on each device looks the
 * array up and may load the module.  The mechanism must have been loaded with the same
 * device current (GB_ERR otherwise), as for every call that launches work. */
int32_t gb_reactors_advance_noalloc(int32_t mech, int32_t n, double t_end, double* T, const double* P,
                                    double* Y, int32_t* status, const gb_net_options* opts,
                                    void* stream);

/* ---- batched reactor right-hand side -------------------------------------------------
 * IdealGasConstPressureReactor::eval (src/zeroD/IdealGasConstPressureReactor.cpp:53-110)
 * over n states: dT/dt [n] and dY/dt [K][n] of the state [T, Y] at pressure P. */
int32_t gb_reactor_rhs(int32_t mech, int32_t n, const double* T, const double* P, const double* Y,
                       double* dTdt, double* dYdt, int32_t flags);
int32_t gb_mech_n_elements(int32_t mech);
/* out[e*K + k] = atoms of element e in species k * W_e / W_k (element mass per species mass). */
int32_t gb_mech_element_mass(int32_t mech, int32_t buflen, double* out);

/* ---- learned surrogate (no counterpart in the reference) -------------------------------
 * Device-pointer operations of the MLP surrogate, on the calling thread's surrogate stream
 * (gb_nn_set_stream; the default stream until set) and finished on return unless that
 * thread asked for asynchronous calls.  gb_nn_gemm: C(m,n) = epilogue(alpha * sum_k A(m,k) B(n,k)) with BF16 A, B on
 * the tensor cores, FP32 accumulation; element (i,j) of X at X[i*s_i + j*s_j]; M, N multiples
 * of 128, K of 32; epilogue: + bias[n] (float, may be NULL), act 1 = GELU (tanh form) with the
 * pre-activation written to Z (unless Z is NULL), act 2 = multiply by GELU'(Z); C and Z float
 * (flag 1) or bf16. */
int32_t gb_nn_gemm(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, int64_t sak,
                   const void* B, int64_t sbn, int64_t sbk, void* C, int64_t scm, int64_t scn,
                   int32_t c_float, float alpha, const float* bias, int32_t act, void* Z, int64_t szm,
                   int64_t szn, int32_t z_float);
/* The same products on the 5th-generation tensor cores (tcgen05.mma, accumulators in tensor
 * memory, operands staged by TMA), the surrogate's GEMM: C(m,n) = epilogue(alpha * sum_k
 * A[m*lda + k] B[n*ldb + k]) with BF16 A [M][K] and B [N][K] both K-major (lda, ldb >= K,
 * multiples of 8), M and N multiples of 128, K a multiple of 64 * splits; epilogue as
 * gb_nn_gemm (bias, act 1 GELU keeping the pre-activation in Z, act 2 times GELU'(Z); Z float
 * or bf16 with row stride ldz); C float (c_float 1) or bf16, row stride ldc; CT (bf16, may be
 * NULL) receives C transposed, CT[n*ldct + m].  splits > 1 divides K among blocks that add
 * their partial products into FP32 C (the call clears C first; no bias, act or CT then).
 * Ordered on `stream` (a cudaStream_t, NULL the default stream), not synchronised: call
 * gb_nn_sync to wait and to collect errors. */
int32_t gb_nn_gemm_tc(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb,
                      void* C, int64_t ldc, int32_t c_float, float alpha, const float* bias, int32_t act, void* Z,
                      int64_t ldz, int32_t z_float, void* CT, int64_t ldct, int32_t splits, void* stream);
/* dst[n*ldd + m] = src[m*lds + n] for m < M, n < N (bf16), ordered on `stream`. */
int32_t gb_nn_transpose(int32_t M, int32_t N, const void* src, int64_t lds, void* dst, int64_t ldd, void* stream);
/* Stream of this host thread's gb_nn_* calls (NULL: the default stream); async = 1: they
 * return without waiting for their work (gb_nn_sync waits). */
int32_t gb_nn_set_stream(void* stream, int32_t async);
/* Wait for `stream`; GB_ERR if a tensor-core GEMM block gave up a bounded wait since the
 * last call (its tile is then not written). */
int32_t gb_nn_sync(void* stream);
/* Adam step on FP32 master weights w with moments m, v and gradient g; writes the bf16 copy. */
int32_t gb_nn_adam(int32_t n, float* w, float* m, float* v, const float* g, void* wb, float lr,
                   float beta1, float beta2, float eps, int32_t step);
/* out[j] = alpha * sum_i X[i*ld + j], j < N, X bf16 (bias gradients). */
int32_t gb_nn_colsum(int32_t M, int32_t N, const void* X, int32_t ld, float alpha, float* out);
/* Mean-squared-error gradient (bf16 dY [M][ld], zero beyond nout) and loss (added to *loss). */
int32_t gb_nn_mse(int32_t M, int32_t nout, int32_t ld, const float* P, const float* Y, void* dY, float* loss);
/* Network inputs (bf16 [n][ldx]): normalised T, ln P and Box-Cox(Y_k, lambda 0.1). */
int32_t gb_nn_features(int32_t mech, int32_t n, const double* T, const double* P, const double* Y,
                       const float* mu, const float* sd, void* X, int32_t ldx);
/* New state from the normalised network output O [n][ldo] (component k < K for Y_k, K for
 * T): v = O sd + mu; x1 = x0 + v, or, given the right-hand sides f0T, f0Y at the start,
 * x1 = x0 + dt f0 + v (dt |f0| + floor) with floor 1e-12 (Y) and 1e-6 K (T). */
int32_t gb_nn_apply(int32_t mech, int32_t n, const float* O, int32_t ldo, const float* mu, const float* sd,
                    const double* T, const double* Y, double dt, const double* f0T, const double* f0Y,
                    double* Tn, double* Yn);
/* Physics gate of a predicted step x0 -> x1 over dt: element mass fractions conserved to
 * tol_elem, enthalpy to tol_h (relative to cp T), and the trapezoidal rule with the reactor
 * right-hand sides f0, f1 satisfied to tol_trap_t (T, relative) and tol_trap_y (Y, absolute).
 * accept[r] = 1 when every check passes; score[r] = the largest normalised violation. */
int32_t gb_nn_gate(int32_t mech, int32_t n, double dt, const double* T0, const double* Y0,
                   const double* T1, const double* Y1, const double* f0T, const double* f0Y,
                   const double* f1T, const double* f1Y, const double* elem_mass, double tol_elem,
                   double tol_h, double tol_trap_t, double tol_trap_y, int32_t* accept, double* score);

/* ---- measurement helpers (no counterpart in the reference) ---------------------------
 * Structure counts of a mechanism for the benchmark's FP64 operation model:
 * counts[0..11] = K, R, reversible, falloff, Troe, three-body reactions, third-body
 * efficiency entries, species-gather entries, Jacobian column entries, Jacobian scatter
 * entries, reactant-side species slots, product-side species slots; with ncounts >= 16 also
 * counts[12..15] = bytes of the device arena a right-hand side reads, + what a Jacobian adds,
 * + the general side lists, and the whole arena. */
int32_t gb_mech_structure(int32_t mech, int32_t ncounts, int64_t* counts);
/* Sustained FP64 FMA rate of the device in GFLOP/s (2 flops per FMA), measured by a
 * dependent-chain kernel over every SM; also the per-call cost of exp and log in
 * FMA-equivalents (results[0] = GFLOP/s, [1] = exp, [2] = log). */
int32_t gb_measure_fp64(double* results);
/* Evaluate the engine's own FP64 exponential and the CUDA library exp on n device-resident
 * arguments x (device pointers): out_engine[i], out_library[i].  For accuracy tests. */
int32_t gb_check_exp(int32_t n, const double* x, double* out_engine, double* out_library);
/* The same for the engine's logarithm against the CUDA library log. */
int32_t gb_check_log(int32_t n, const double* x, double* out_engine, double* out_library);

/* Bounds checks (no counterpart in the reference): a library built with GBCHEM_CHECKED
 * (python -c "from cantera_gb300 import build; build.build(checked=True)", loaded with
 * GBCHEM_CHECKED=1) checks every index its kernels take from the mechanism's tables or
 * queues; an index out of range is recorded and replaced by 0, so the kernel stays in
 * bounds.  out[0..2] = the first failing check site (0: none), its index and its bound,
 * for the kernels run on this mechanism since the last call (the record is then cleared).
 * Returns 1 for a checked build, 0 for the normal one (whose kernels record nothing), or
 * GB_ERR. */
int32_t gb_check_status(int32_t mech, int32_t* out);

/* Copy the most recent error message (thread-local) into buf; returns its length. */
int32_t gb_get_error(int32_t buflen, char* buf);

#ifdef __cplusplus
}
#endif
#endif /* GBCHEM_H */
