/*
 * conicxx_gb300.h -- C-ABI of the GB300-native ConicXX interior-point path.
 *
 * Problem (identical to ConicXX, README.md:21-33):
 *     minimise    1/2 x'Px + q'x
 *     subject to  Ax + s = b,   s in K = Zero^p x R^l_+ x Q^k1 x ... x Q^kN
 *
 * Every entry point takes plain pointers and sizes; no C++ or torch type crosses this
 * boundary. Matrices are CSC with 32-bit indices (ConicXX's SparseMat, include/conicxx/types.h:18).
 * P is given as its upper triangle (entries below the diagonal are ignored, as in
 * src/conicxx/kkt/kkt_system.cpp:58-65 and the selfadjointView<Upper> product at
 * src/conicxx/solver_impl.cpp:102).
 *
 * Return codes: CXG_OK (0) on success, a negative CXG_E_* on a usage or runtime error.
 * The solver status of a solve is reported in cxg_info.status (never as a return code).
 * After any non-zero return, cxg_last_error() gives a message for the calling thread.
 * No C++ exception ever crosses this boundary.
 */
#ifndef CONICXX_GB300_H
#define CONICXX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------------------------ */
enum {
  CXG_OK = 0,
  CXG_E_INVALID = -1,      /* bad argument, dimension mismatch, invalid cone spec */
  CXG_E_PATTERN = -2,      /* updateData: sparsity pattern differs from setup() */
  CXG_E_NOT_SETUP = -3,    /* handle used before a successful setup */
  CXG_E_CUDA = -4,         /* CUDA runtime error (message in cxg_last_error) */
  CXG_E_NOMEM = -5,        /* host or device allocation failed */
  CXG_E_UNSUPPORTED = -6,  /* instance too large for the device path, or feature not built */
  CXG_E_INTERNAL = -7
};

/* ---- solver status: same values and meaning as conicxx::Status
 *      (include/conicxx/solution.h:9-16) -------------------------------------------------- */
enum {
  CXG_STATUS_UNSOLVED = 0,
  CXG_STATUS_SOLVED = 1,
  CXG_STATUS_PRIMAL_INFEASIBLE = 2,
  CXG_STATUS_DUAL_INFEASIBLE = 3,
  CXG_STATUS_MAX_ITERATIONS = 4,
  CXG_STATUS_NUMERICAL_ERROR = 5
};

/* conicxx::LinearSolverBackend (include/conicxx/settings.h:8-18). The device path has one
 * factorisation; the value selects its pivot rule: QDLDL = retry ladder only,
 * REGULARIZED = per-pivot correction plus the ladder. EIGEN behaves as QDLDL. */
enum { CXG_LINSOLVER_EIGEN = 0, CXG_LINSOLVER_QDLDL = 1, CXG_LINSOLVER_REGULARIZED = 2 };

/* Arithmetic of the KKT factorisation and triangular solves (new; no reference counterpart).
 * Residuals, refinement residuals, cone scaling, step lengths and termination are FP64 in
 * both modes. */
enum { CXG_PRECISION_FP64 = 0, CXG_PRECISION_MIXED = 1 };

/* Field-for-field the reference's Settings (include/conicxx/settings.h:21-62), same defaults
 * (cxg_default_settings), followed by the GB300 additions. */
typedef struct cxg_settings {
  double tol_feas;            /* 1e-8 */
  double tol_gap_abs;         /* 1e-8 */
  double tol_gap_rel;         /* 1e-8 */
  double tol_infeas;          /* 1e-7 */
  int max_iter;               /* 200 */
  double static_reg_P;        /* 1e-8 */
  double static_reg_A;        /* 1e-8 */
  double dynamic_reg_eps;     /* 1e-14 */
  double dynamic_reg_delta;   /* 1e-7 */
  int refine_max_iter;        /* 3 */
  double refine_tol;          /* 1e-12 */
  double max_step_fraction;   /* 0.99 */
  int equilibrate;            /* 1 */
  int equilibrate_max_iter;   /* 10 */
  double equilibrate_min_scale; /* 1e-4 */
  double equilibrate_max_scale; /* 1e4 */
  int warm_start;             /* 1 */
  int verbose;                /* 0 (declared, unused, as in the reference) */
  int record_timings;         /* 0 */
  int validate_inputs;        /* 1 */
  int linear_solver;          /* CXG_LINSOLVER_QDLDL */
  /* ---- GB300 additions ---- */
  int precision;              /* CXG_PRECISION_FP64 for cxg_solver, MIXED for cxg_batch */
  int mixed_refine_max_iter;  /* refinement steps allowed on an FP32 factor before the
                                 high-precision refactorisation fallback (default 4; a step
                                 contracting the residual by less than 4x falls back at once) */
  double mixed_fallback_tol;  /* relative KKT residual above which an FP32-factor solve is redone
                                 with the high-precision factor: double-float arithmetic (about
                                 48 bits) on the FP32 pipe (default 1e-10) */
  int threads_per_instance;   /* 0 = by root size (32 up to 32 rows, 64 up to 64, 128 up to 128,
                                 else 256); else 32, 64, 128 or 256 */
  int differentiable;         /* keep each instance's final factorisation, scaling and iterate on the
                                 device so backward() can reuse them (default 0; cxg_solver: 1);
                                 ignored for whole-GPU roots above 8192 rows */
  int whole_gpu_root;         /* one instance (cxg_solver, or a batch of count 1): 1 = spread the root
                                 over every SM (cooperative launch, roots up to 131072 rows); -1 =
                                 never (one CTA, roots up to 4096 rows); 0 = automatic: cxg_solver
                                 spreads roots of more than 512 rows, a batch of one only roots of
                                 more than 4096 */
  /* ---- fault injection for tests of the recovery paths (0 = off; counted per instance and
   *      per solve call, from the start of the solve) ---- */
  int fault_factor_failures;  /* the first k factorisation attempts report failure, so the x10
                                 regularisation ladder of factorizeWithRetry runs
                                 (src/conicxx/kkt/kkt_system.cpp:242-264) */
  int fault_nonfinite_solves; /* the first k solves with the factor return a non-finite vector, so
                                 escalateAndResolve's x1000 bumps run (kkt_system.cpp:266-294) */
  /* ---- GB300 addition ---- */
  int soc_reference_dense;    /* 1 (default): second-order blocks of up to 8 rows enter two decisions
                                 in the reference's dense FP64 form Hs = W W
                                 (second_order_cone.cpp:132-158): a factorisation attempt fails where
                                 the reference's dense block -(Hs + eps I) has a pivot at or below
                                 dynamic_reg_eps, as its sparse LDL' of K does near the cone boundary
                                 (kkt_system.cpp:242-264), and the step directions ds = -(Hs dz + ...)
                                 use the dense product (cone_set.cpp:70-75). The device's eigen-form
                                 scaling is otherwise exact to rounding there; the reference's
                                 convergence on problems with many near-boundary blocks relies on
                                 the dense form's rounding. 0: eigen-form throughout. The pivot test
                                 is off with CXG_LINSOLVER_REGULARIZED */
} cxg_settings;

/* conicxx::Info (include/conicxx/solution.h:18-26) plus Solution::objective/status and counters. */
typedef struct cxg_info {
  int status;                 /* CXG_STATUS_* */
  int iterations;
  double objective;
  double primal_residual;
  double dual_residual;
  double duality_gap;
  double mu;
  double setup_time_s;
  double solve_time_s;
  int fp64_fallbacks;         /* mixed precision: switches to the high-precision (double-float)
                                 factor after an FP32 factor fell short */
  int refine_steps;           /* total refinement steps taken */
  double max_relres;          /* worst final relative KKT residual over all solves */
  /* with settings.record_timings: device time split of this instance's solve, seconds */
  double time_factor_s;       /* KKT assembly + LDL' factorisations */
  double time_kkt_solve_s;    /* KKT solves incl. iterative refinement */
  double time_other_s;        /* residuals, cone algebra, step lengths */
  /* with settings.record_timings: parts of the above, seconds */
  double time_assemble_s;     /* reduced-KKT assembly (inside time_factor_s / fallback refactors) */
  double time_ldlt_s;         /* dense LDL' of the reduced root */
  double time_dense_solve_s;  /* triangular solves with the root factor */
  double time_residual_s;     /* KKT residuals of the refinement */
  int factor_attempts;        /* factorisations attempted (retry ladder and fallback included) */
  /* with settings.record_timings: when this instance started and finished on the device, in
     seconds after the earliest start in the batch (batches; 0 for cxg_solver) */
  double time_start_s;
  double time_end_s;
  int escalations;            /* refactorisations with x1000 bumps after a non-finite solve
                                 (escalateAndResolve, src/conicxx/kkt/kkt_system.cpp:266-294) */
} cxg_info;

/* One problem instance; all pointers are caller-owned host memory (copied, never retained). */
typedef struct cxg_problem {
  int n, m;
  const int* Pp; const int* Pi; const double* Px;   /* n x n, upper triangle, CSC */
  const double* q;                                  /* n */
  const int* Ap; const int* Ai; const double* Ax;   /* m x n, CSC */
  const double* b;                                  /* m */
  int zero_dim, nonneg_dim, n_soc;                  /* ConeSpec (include/conicxx/cone_spec.h) */
  const int* soc_dims;
} cxg_problem;

void cxg_default_settings(cxg_settings* settings);
const char* cxg_status_string(int status);
const char* cxg_version(void);
const char* cxg_last_error(void);
/* Number of CUDA devices visible to the library (0 without a GPU). Never fails. */
int cxg_device_count(void);

/* ---- single instance: replaces conicxx::Solver (include/conicxx/solver.h:33-95) ---------- */
typedef struct cxg_solver cxg_solver;

/* Solver::Solver() (include/conicxx/solver.h:35). */
int cxg_solver_create(cxg_solver** out);
void cxg_solver_destroy(cxg_solver* solver);
/* Solver::setup(P, q, A, b, cone_spec, settings) (include/conicxx/solver.h:46-47). settings may
 * be NULL (defaults). Returns CXG_E_INVALID where the reference returns false. */
int cxg_solver_setup(cxg_solver* solver, const cxg_problem* problem, const cxg_settings* settings);
/* Solver::updateData(P*, q*, A*, b*) (include/conicxx/solver.h:78). Any pointer may be NULL
 * (unchanged). A matrix is passed as its CSC arrays; CXG_E_PATTERN where the reference returns
 * false because the pattern changed. */
int cxg_solver_update_data(cxg_solver* solver, const int* Pp, const int* Pi, const double* Px,
                           const double* q, const int* Ap, const int* Ai, const double* Ax,
                           const double* b);
/* Solver::setWarmStart(x, s, z) (include/conicxx/solver.h:82). */
int cxg_solver_set_warm_start(cxg_solver* solver, const double* x, const double* s, const double* z);
/* Solver::setSettings / settings() (include/conicxx/solver.h:84-85). */
int cxg_solver_set_settings(cxg_solver* solver, const cxg_settings* settings);
int cxg_solver_get_settings(const cxg_solver* solver, cxg_settings* out);
/* Solver::solve() + Solution (include/conicxx/solver.h:90, solution.h:28-39). x (n), s (m),
 * z (m) and info may each be NULL. */
int cxg_solver_solve(cxg_solver* solver, double* x, double* s, double* z, cxg_info* info);
/* Solver::backward (new, no reference counterpart): given dL/dx (n) at the last Solved
 * solution, returns dL/dq (n), dL/db (m), dL/d(values of P upper, in setup CSC order) and
 * dL/d(values of A, in setup CSC order). Output pointers may be NULL. */
int cxg_solver_backward(cxg_solver* solver, const double* dL_dx, double* dq, double* db,
                        double* dPx, double* dAx);

/* ---- batch of independent instances (new; no reference counterpart) --------------------- */
typedef struct cxg_batch cxg_batch;

/* Symbolic set-up of `count` instances (patterns fixed from here on). */
int cxg_batch_create(cxg_batch** out, int count, const cxg_problem* problems,
                     const cxg_settings* settings);
void cxg_batch_destroy(cxg_batch* batch);
int cxg_batch_count(const cxg_batch* batch);
/* A new set-up of some instances of a batch (conicxx::Solver::setup of each,
 * include/conicxx/solver.h:33-56, src/conicxx/solver_impl.cpp:9-55): instance indices[j] becomes
 * problems[j], j < k, new sparsity patterns and sizes allowed (the per-timestep contact-pattern
 * change). Only the replaced instances are planned again (symbolic analysis and equilibration of
 * each, on host threads); the others keep their plans, their values as last set and their
 * device-resident warm starts, which move to the new layout on the device. The replaced
 * instances start cold. Offsets (cxg_batch_offsets) and sizes (cxg_batch_sizes) change; with
 * settings.differentiable, backward needs a solve first. Refused for the whole-GPU single
 * instance (CXG_E_UNSUPPORTED); errors as cxg_batch_create, the batch unchanged on a validation
 * error. Synchronises the device. */
int cxg_batch_replace(cxg_batch* batch, int k, const int* indices, const cxg_problem* problems);
/* Sizes of the concatenated value/solution arrays: sum of nnz(P upper), n, nnz(A), m. */
int cxg_batch_sizes(const cxg_batch* batch, int64_t* nnzP, int64_t* n_total, int64_t* nnzA,
                    int64_t* m_total);
/* Offsets of instance i inside the concatenated arrays (each may be NULL). */
int cxg_batch_offsets(const cxg_batch* batch, int i, int64_t* pOff, int64_t* nOff, int64_t* aOff,
                      int64_t* mOff);
/* updateData for every instance at once from HOST arrays (concatenated in instance order;
 * any may be NULL = unchanged). Values only: the patterns are those given at create time. */
int cxg_batch_update_values(cxg_batch* batch, const double* Px, const double* q, const double* Ax,
                            const double* b);
/* Solve every instance; HOST outputs (concatenated x, s, z; info[count]); any may be NULL. */
int cxg_batch_solve(cxg_batch* batch, double* x, double* s, double* z, cxg_info* info);
/* Device-pointer variants: inputs/outputs are device buffers; work is enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and the call returns without synchronising. */
int cxg_batch_update_values_device(cxg_batch* batch, const double* Px, const double* q,
                                   const double* Ax, const double* b, void* stream);
int cxg_batch_solve_device(cxg_batch* batch, double* x, double* s, double* z, cxg_info* info,
                           void* stream);
/* Adjoint of every instance at its last solution (see cxg_solver_backward); host arrays. */
int cxg_batch_backward(cxg_batch* batch, const double* dL_dx, double* dq, double* db, double* dPx,
                       double* dAx);
int cxg_batch_backward_device(cxg_batch* batch, const double* dL_dx, double* dq, double* db,
                              double* dPx, double* dAx, void* stream);
/* Allocation-free solve. No reference counterpart: ConicXX has no device path. It exists for
 * callers that must not allocate or free device memory while they solve. One example is a
 * simulator's per-timestep loop that reserves its device memory up front. There, an allocation
 * could fail in mid-step, and cudaFree would synchronise the whole device.
 *
 * Same contract as cxg_batch_solve_device, with three differences:
 * - The IPM kernel's per-CTA working memory comes from one fixed device array of
 *   CXG_NOALLOC_SCRATCH_BYTES per device, not from memory the batch owns.
 * - The size buckets run one after another on `stream`, with no captured graph and no stream or
 *   event creation.
 * - Each bucket's persistent grid is cut down to what the array holds.
 * Like the other solve entry points, it re-orders each bucket's work queue afterwards by the cost
 * each instance just had (a kernel with static shared memory only).
 *
 * The call allocates nothing. The first call on a device looks up that array's address with the
 * device current. Make that first call before any stream capture.
 *
 * Returns CXG_E_UNSUPPORTED with a message if one CTA's working memory for a bucket exceeds the
 * array, that is, if one instance's plan is too big.
 *
 * The work-queue counters live in the same array; each call clears them on `stream` before its
 * launches. Calls whose work overlaps in time share the array and race: two in flight at once
 * on one device, from any batch and on any stream, corrupt each other's results. Keep them
 * ordered on one stream or synchronise between them. */
#define CXG_NOALLOC_SCRATCH_BYTES (32ll << 20)
int cxg_batch_solve_device_noalloc(cxg_batch* batch, double* x, double* s, double* z, cxg_info* info,
                                   void* stream);
/* Autotuner (no reference counterpart), by timing whole concurrent solves of the batch (trials
 * timed solves after one warm-up each, median kept): (1) the size-bucket edges on the root size,
 * from five candidate sets (finer and coarser than the built-in one), each planned with its SM
 * shares and working memory; (2) then, one bucket at a time, 32 (roots of at most 64 rows), 64,
 * 128 or 256 threads per instance. The fastest choices are kept for later solves. The trials
 * solve the current values with warm start off and overwrite the last solution (solve again to
 * read one). Allocates device memory. report (may be NULL) receives one line per edge set and
 * one line per bucket with the measured times. */
int cxg_batch_autotune(cxg_batch* batch, int trials, char* report, int reportLen);
/* Kernel launches enqueued by the last solve/backward call of this batch. */
int cxg_batch_last_launches(const cxg_batch* batch);
/* Iteration trace of one instance of the last solve made with record_timings set (no reference
 * counterpart; the quantities SolverImpl::solve computes per iteration, solver_impl.cpp:367-466):
 * up to cap_rows rows of 12 doubles each -- mu, ||rx||/tau, ||rz||/tau, primal objective, dual
 * objective, affine step, sigma, step, tau, kappa, the iteration's largest relative KKT residual,
 * factorisation attempts. Returns the number of rows written (the instance's iterations, capped),
 * or a negative CXG_E_* code. */
int cxg_batch_trace(cxg_batch* batch, int instance, double* out, int cap_rows);
int cxg_solver_trace(cxg_solver* solver, double* out, int cap_rows);
/* Device footprint of the batch in bytes: index plans + equilibration (plan), problem values +
 * solutions + results (values), per-CTA working memory (scratch). Any pointer may be NULL. */
int cxg_batch_footprint(const cxg_batch* batch, int64_t* plan_bytes, int64_t* value_bytes, int64_t* scratch_bytes);
/* Human-readable launch configuration (one line per size bucket) into buf; returns the length. */
int cxg_batch_describe(const cxg_batch* batch, char* buf, int buflen);

/* ---- diagnostics (used by the parity tests) ---------------------------------------------- */
/* Runs the IPM kernel's device cone algebra on one cone set K = Zero^zero x R^nn_+ x Q^... of
 * total dimension m, after the Nesterov-Todd scaling of (s, z) (NonnegativeCone/SecondOrderCone
 * ::updateScaling, src/conicxx/cones/nonnegative_cone.cpp:22-26, second_order_cone.cpp:70-159).
 * op: 0 out = W u, 1 out = W^-1 u, 2 out = Hs u (ConeSet::applyW / applyWInv / mulHs,
 * cone_set.cpp:56-75), 7 out = (Hs + eps I)^-1 u with eps = alpha_or_eps; 3 out = u o v,
 * 4 out = u \ v (product / inverseProduct, cone_set.cpp:34-46); 5 scalars[0] = maxStep(u, v,
 * alpha_or_eps) (cone_set.cpp:108-115); 6 scalars[0..1] = margins(u) (cone_set.cpp:77-90).
 * soc_params (optional, 8 per SOC block): [kind, beta, lambda, q_c, q_s, ...] of the scaling. */
int cxg_cones_eval(int op, int zero_dim, int nonneg_dim, int n_soc, const int* soc_dims, const double* s,
                   const double* z, const double* u, const double* v, double alpha_or_eps, double* out,
                   double* scalars, double* soc_params);
/* Dense root factorisation of the IPM kernel (the reduced KKT root's LDL', QDLDL-style no
 * pivoting with the per-pivot rule of RegularizedLdlt::regularizePivot when linear_solver is
 * CXG_LINSOLVER_REGULARIZED, src/conicxx/kkt/regularized_ldlt.cpp:132-139) on one given dense
 * symmetric matrix K (nr x nr, column-major; pivots < nx expected positive, the rest negative),
 * run by one CTA of `threads` (32..256, a multiple of 32) threads in arith 0 = FP64, 1 = FP32, 2 = double-float; then the
 * triangular solves for K x = b. Outputs (each may be NULL): L (nr x nr unit lower, column-major),
 * D (nr), x (nr), cycles[2] = SM clock cycles of {factorisation, solve}, flags[2] = {exact zero /
 * too many corrections, wrong-signed pivot}. Allocates its own device buffers.
 * threads = -1: the whole-GPU root of a single large instance instead (every SM, cooperative
 * launch); cycles then hold nanoseconds and flags has a third entry, 1 if a grid barrier wait ran
 * out. */
int cxg_dense_ldlt(int nr, int nx, const double* K, const double* b, int arith, int threads, int linear_solver,
                   double* L, double* D, double* x, long long* cycles, int* flags);

/* Diagnostic, no reference counterpart: the bounded wait of the whole-GPU root's grid barrier.
 * One cooperative launch of one CTA per SM passes `rounds` grid barriers; when skip_cta >= 0 that
 * CTA returns without arriving, so the others' first wait runs out after timeout_s (1e-3..5 s),
 * the barrier's error flag is set and every CTA returns (a large instance whose barrier runs out
 * ends with NumericalError and error_code 1 the same way). Outputs: error_flag (1 when a wait ran
 * out), max_rounds_passed (most barriers any CTA got through), elapsed_s (launch time). */
int cxg_grid_barrier_selftest(int skip_cta, int rounds, double timeout_s, int* error_flag, int* max_rounds_passed,
                              double* elapsed_s);
/* Host equilibration of the set-up path (Equilibration::compute, src/conicxx/kkt/equilibration.cpp:8-100):
 * d (n), e (m), c. No GPU needed. */
int cxg_equilibration(const cxg_problem* problem, const cxg_settings* settings, double* d, double* e, double* c);
/* Host planning of one instance (the symbolic set-up of KktSystem::setup and SparsityMap,
 * src/conicxx/kkt/kkt_system.cpp:22-117, sparsity_map.cpp:8-56) without any device work, for
 * tests of the plan: counts[0..8] = nr, root entries, strictly-upper P scatter entries, Zero-row A
 * scatter entries, cone-unit target entries, full symmetric P entries, densified A-block entries,
 * contributions, and 1 when every 64-bit root offset map sits 8-byte aligned in the int pool.
 * The first `cap` root element offsets of each scatter map go to plow / az / tgt (each nullable).
 * CXG_E_UNSUPPORTED when a 32-bit plan count would overflow. No GPU needed. */
int cxg_plan_inspect(const cxg_problem* problem, const cxg_settings* settings, long long* counts, long long* plow,
                     long long* az, long long* tgt, int cap);

#ifdef __cplusplus
}
#endif

#endif /* CONICXX_GB300_H */
