/*
 * sfgpu.h - C ABI of the GB300-native Levenberg-Marquardt back end for SymForce's sym::Optimizer.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, never throws, and returns an
 * int32 status (SFG_OK == 0).  sfg_last_error() returns a thread-local message for the last
 * failure on the calling thread.  Device memory is owned by the handle; host arrays passed in are
 * borrowed for the duration of the call only (the reference Optimizer copies factors in and updates
 * Values in place: symforce/opt/optimizer.tcc:20-40, symforce/opt/internal/optimizer_utils.h:69).
 *
 * One handle = one CUDA stream; a handle is not thread safe, handles on different threads are
 * independent (symforce/opt/optimizer.h:23 "Not thread safe! Create one per thread.").
 */
#ifndef SFGPU_H_
#define SFGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFG_ABI_VERSION 3

/* ---------------------------------------------------------------------------------------------
 * Status codes.  Solver outcomes (SUCCESS / HIT_ITERATION_LIMIT / FAILED) are not errors: they are
 * reported in sfg_stats_t exactly like the reference reports them in OptimizationStats
 * (symforce/opt/internal/optimizer_utils.h:45-64).  Errors are what the reference raises with
 * SYM_ASSERT (symforce/opt/assert.h:41-47).
 * ------------------------------------------------------------------------------------------- */
enum {
  SFG_OK = 0,
  SFG_ERR_INVALID_ARGUMENT = 1, /* bad sizes, bad key/factor kinds, null pointers */
  SFG_ERR_CUDA = 2,             /* a CUDA runtime call failed (message in sfg_last_error) */
  SFG_ERR_NO_DEVICE = 3,        /* no CUDA device visible: there is no CPU fallback */
  SFG_ERR_STRUCTURE = 4,        /* structure not supported (e.g. Schur block C not block diagonal) */
  SFG_ERR_DEVICE_STATUS = 5,    /* a device loop hit its hard cap or saw non-finite values */
  SFG_ERR_OUT_OF_MEMORY = 6,
  SFG_ERR_CAPACITY = 7,         /* a caller-provided output buffer is too small */
  SFG_ERR_NUMERICAL = 8         /* sfg_dense_ldlt_solve_noalloc: a zero or non-finite pivot */
};

/* Optimization status and LM failure reasons: same integer values as the reference LCM enums
 * optimization_status_t / levenberg_marquardt_solver_failure_reason_t
 * (lcmtypes/symforce.lcm:279-300). */
enum { SFG_STATUS_INVALID = 0, SFG_STATUS_SUCCESS = 1, SFG_STATUS_HIT_ITERATION_LIMIT = 2,
       SFG_STATUS_FAILED = 3 };
enum { SFG_FAILURE_INVALID = 0, SFG_FAILURE_LAMBDA_OUT_OF_BOUNDS = 1,
       SFG_FAILURE_INITIAL_ERROR_NOT_FINITE = 2 };

/* lambda_update_type_t (lcmtypes/symforce.lcm:117-131). */
enum { SFG_LAMBDA_UPDATE_INVALID = 0, SFG_LAMBDA_UPDATE_STATIC = 1, SFG_LAMBDA_UPDATE_DYNAMIC = 2 };

/* ---------------------------------------------------------------------------------------------
 * Variable (key) types.  Storage / tangent layouts are the reference's:
 *   VEC1..VEC6: storage = tangent = n scalars, Retract is +=   (symforce/opt/values.cc:303-309,
 *               gen/cpp/sym/ops/matrix/lie_group_ops.h)
 *   POSE2: storage [re, im, x, y], tangent [theta, x, y]        (gen/cpp/sym/ops/pose2/lie_group_ops.cc:58-82)
 *   POSE3: storage [qx, qy, qz, qw, x, y, z], tangent [w(3), t(3)]
 *          Retract q <- q * exp(w) with eps-regularised norm, t <- t + dt
 *                                                               (gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102)
 *   ROT3:  storage [qx, qy, qz, qw], tangent [w(3)], Retract q <- q * exp(w) as POSE3's rotation
 *                                                               (gen/cpp/sym/ops/rot3/lie_group_ops.cc)
 * ------------------------------------------------------------------------------------------- */
enum { SFG_KEY_VEC1 = 1, SFG_KEY_VEC2 = 2, SFG_KEY_VEC3 = 3, SFG_KEY_POSE2 = 4, SFG_KEY_POSE3 = 5,
       SFG_KEY_ROT3 = 6, SFG_KEY_VEC4 = 7, SFG_KEY_VEC5 = 8, SFG_KEY_VEC6 = 9 };

/* ---------------------------------------------------------------------------------------------
 * Typed factor kinds.  The reference stores a factor as a type-erased std::function
 * (symforce/opt/factor.h:99-119) that a GPU cannot call, so each factor batch names one of these
 * kinds, its keys (indices into the key table) and its constants.  Residual conventions follow the
 * reference's generated factors; consts are laid out per factor, factor-major.
 *
 *  BEARING_POSE2      keys [pose2]                consts [lx, ly, angle, epsilon, sqrt_info]
 *      r = sqrt_info * wrap_angle(atan2(tb.y, tb.x + copysign(eps, tb.x)) - angle),
 *      tb = pose^-1 * landmark   (symforce/examples/robot_2d_localization/gen/bearing_factor.h:21-97)
 *  ODOMETRY_POSE2     keys [pose2 a, pose2 b]     consts [dist, epsilon, sqrt_info]
 *      r = sqrt_info * (sqrt(|tb - ta|^2 + eps) - dist)
 *                                (symforce/examples/robot_2d_localization/gen/odometry_factor.h:21-98)
 *  SNAVELY_REPROJECTION keys [pose3 cam_T_world, vec3 (f,k1,k2), vec3 point]
 *                     consts [px, py, epsilon, cauchy_delta]
 *      e = f*(1 + k1 |p|^2 + k2 |p|^4) * p - pixel, p = pc.xy / -pc.z, pc = cam_T_world * point
 *      (symforce/examples/bundle_adjustment_in_the_large/bundle_adjustment_in_the_large.py:18-63);
 *      cauchy_delta > 0 whitens the norm with the Cauchy loss (Barron alpha=0 limit,
 *      symforce/opt/noise_models.py:318-428 whiten_norm): r = sqrt(2 rho(n)) / n * e,
 *      n = sqrt(|e|^2 + eps), rho(n) = delta^2 log(1 + n^2 / (2 delta^2)).  0 = no loss.
 *  BETWEEN_POSE3      keys [pose3 a, pose3 b]     consts [a_T_b (7 storage), sqrt_info_diag (6), epsilon]
 *      r = diag(s) * local_coordinates(a_T_b, a^-1 * b)     (gen/cpp/sym/factors/between_factor_pose3.h)
 *  PRIOR_POSE3        keys [pose3]                consts [prior (7 storage), sqrt_info_diag (6), epsilon]
 *      r = diag(s) * local_coordinates(prior, value)        (gen/cpp/sym/factors/prior_factor_pose3.h)
 *  RANGE_POSE3        keys [pose3]                consts [lx, ly, lz, range, sqrt_info, epsilon]
 *      r = sqrt_info * (sqrt(|t - l|^2 + eps) - range)   (no reference counterpart; written in the
 *      same style as the odometry factor)
 *
 * Kinds generated from symbolic residuals (symforce_gb300/factor_defs.py, compiled from the
 * generated functors in symforce_gb300/csrc/generated_factors.cuh):
 *  PRIOR_ROT3         keys [rot3]                 consts [prior q (4), sqrt_info_diag (3), epsilon]
 *      r = diag(s) * local_coordinates(prior, value)  (symforce/codegen/geo_factors_codegen.py:75-86)
 *  BETWEEN_ROT3       keys [rot3 a, rot3 b]       consts [a_T_b q (4), sqrt_info_diag (3), epsilon]
 *      r = diag(s) * local_coordinates(a_T_b, a^-1 * b) (symforce/codegen/geo_factors_codegen.py:53-72)
 *  BARRON_VEC5        keys [vec5 x]               consts [y (5), mu, epsilon]
 *      r_i = Barron whitening of x_i - y_i with alpha = 2 - 1 / (1 - mu + eps), delta 1
 *      (symforce/opt/noise_models.py:318-428; the factor of test/symforce_gnc_codegen_test.py:24-31).
 *      mu is the graduated non-convexity parameter (sfg_set_factor_consts changes it).
 *  LINEAR_VEC5        keys [vec5 x]               consts [J (9 x 5 row-major), b (9)]
 *      r = J x + b     (test/symforce_levenberg_marquardt_test.cc:17-88)
 *  LINEAR_SCALAR2     keys [vec1 x, vec1 y]       consts [J (2 x 2 row-major), b (2)]
 *      r = J [x, y] + b   (test/symforce_linearizer_test.cc:16-43)
 * ------------------------------------------------------------------------------------------- */
enum {
  SFG_FACTOR_BEARING_POSE2 = 1,
  SFG_FACTOR_ODOMETRY_POSE2 = 2,
  SFG_FACTOR_SNAVELY_REPROJECTION = 3,
  SFG_FACTOR_BETWEEN_POSE3 = 4,
  SFG_FACTOR_PRIOR_POSE3 = 5,
  SFG_FACTOR_RANGE_POSE3 = 6,
  SFG_FACTOR_PRIOR_ROT3 = 7,
  SFG_FACTOR_BETWEEN_ROT3 = 8,
  SFG_FACTOR_BARRON_VEC5 = 9,
  SFG_FACTOR_LINEAR_VEC5 = 10,
  SFG_FACTOR_LINEAR_SCALAR2 = 11
};

typedef struct sfg_factor_batch_t {
  int32_t kind;          /* SFG_FACTOR_* */
  int32_t count;         /* number of factors in the batch (may be 0) */
  const int32_t* keys;   /* [count * num_keys(kind)] indices into the problem's key table */
  const double* consts;  /* [count * num_consts(kind)] */
} sfg_factor_batch_t;

/* A problem: the keys to optimize, in state-vector order (the reference's Linearizer key order,
 * symforce/opt/linearizer.cc:148-158), plus factor batches.  Residual rows are laid out batch by
 * batch, factor by factor.  If num_schur_keys > 0, the last num_schur_keys keys (all VEC3 and not
 * sharing a factor with each other) are eliminated by a Schur complement, as SparseSchurSolver
 * does for a block-diagonal C (symforce/opt/sparse_schur_solver.tcc:15-97). */
typedef struct sfg_problem_t {
  int32_t num_keys;
  const int32_t* key_types;          /* [num_keys] SFG_KEY_* */
  int32_t num_batches;
  const sfg_factor_batch_t* batches; /* [num_batches] */
  int32_t num_schur_keys;
} sfg_problem_t;

/* Plain-old-data mirror of optimizer_params_t (lcmtypes/symforce.lcm:134-200); defaults are
 * sfg_default_optimizer_params(), matching sym::DefaultOptimizerParams (symforce/opt/optimizer.cc:8-56).
 * verbose / check_derivatives / include_jacobians / debug_checks are accepted and ignored by the
 * device path (no per-iteration host logging; derivative checks live in the tests). */
typedef struct sfg_optimizer_params_t {
  int32_t verbose;
  int32_t debug_stats;
  int32_t check_derivatives;
  int32_t include_jacobians;
  int32_t debug_checks;
  double initial_lambda;
  double lambda_lower_bound;
  double lambda_upper_bound;
  int32_t lambda_update_type;
  double lambda_up_factor;
  double lambda_down_factor;
  double dynamic_lambda_update_beta;
  double dynamic_lambda_update_gamma;
  int32_t dynamic_lambda_update_p;
  int32_t use_diagonal_damping;
  int32_t use_unit_damping;
  int32_t keep_max_diagonal_damping;
  double diagonal_damping_min;
  int32_t iterations;
  double early_exit_min_reduction;
  double early_exit_min_absolute_error;
  int32_t enable_bold_updates;
} sfg_optimizer_params_t;

/* One record of optimization_iteration_t (lcmtypes/symforce.lcm:229-262) plus the device time
 * (ms since the start of the optimize call, read from the GPU global timer when the record was
 * written).  The update/values/residual debug vectors are not recorded. */
typedef struct sfg_iteration_t {
  int32_t iteration;
  int32_t update_accepted;
  double current_lambda;
  double new_error_linear;
  double new_error;
  double relative_reduction;
  double update_angle_change;
  double best_error;    /* error of the best state after this iteration */
  double elapsed_ms;    /* device time since the optimize call started */
} sfg_iteration_t;

/* optimization_stats_t (lcmtypes/symforce.lcm:302-336).  `iterations` is caller-owned with room
 * for `capacity` records (params.iterations + 1 suffices). */
typedef struct sfg_stats_t {
  sfg_iteration_t* iterations;
  int32_t capacity;
  int32_t num_iterations;
  int32_t best_index;
  int32_t status;
  int32_t failure_reason;
  int32_t kernel_launches;  /* device kernels the optimize call launched (graph nodes executed) */
  double device_ms;         /* CUDA-event time of the device work of the optimize call */
} sfg_stats_t;

/* Forms of the solver (besides the plain FP64 drop-in). */
enum { SFG_PRECISION_FP64 = 0, SFG_PRECISION_MIXED = 1 };
/* PCG_BLOCK_JACOBI / PCG_LEARNED: Schur complement over the points, then preconditioned conjugate
 * gradients on the reduced camera system with one 9 x 9 preconditioner block per camera (the keys
 * that share a factor with each other, e.g. pose + intrinsics).  BLOCK_JACOBI uses the inverse of
 * the reduced system's diagonal block; LEARNED corrects that block with a small network (see
 * "learned preconditioner" below).  The exact LDL^T of the reduced system is the fallback for every
 * solve whose FP64 relative residual |v - S y| / |v| is still above pcg_tol after pcg_max_iters
 * iterations.  Both require problem.num_schur_keys > 0. */
enum { SFG_LINEAR_SOLVER_SPARSE_LDLT = 0, SFG_LINEAR_SOLVER_SCHUR = 1,
       SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI = 2, SFG_LINEAR_SOLVER_PCG_LEARNED = 3 };
enum { SFG_ORDERING_NESTED_DISSECTION = 0, SFG_ORDERING_NATURAL = 1, SFG_ORDERING_MIN_DEGREE = 2 };

typedef struct sfg_form_params_t {
  int32_t precision;      /* SFG_PRECISION_* */
  int32_t linear_solver;  /* SFG_LINEAR_SOLVER_*; SCHUR requires problem.num_schur_keys > 0 */
  int32_t ordering;       /* SFG_ORDERING_* (block level) */
  int32_t device;         /* CUDA device ordinal */
  double epsilon;         /* the Optimizer's epsilon (symforce/opt/optimizer.h:90-94); default 10 * DBL_EPSILON */
  int32_t refine_steps;   /* MIXED: FP64 iterative-refinement steps per linear solve (default 1) */
  int32_t pcg_max_iters;  /* PCG forms: iteration cap of one reduced-system solve (default 500) */
  double pcg_tol;         /* PCG forms: FP64 relative residual target (default 1e-8) */
  int32_t pcg_coarse;     /* PCG forms: 1 adds to the camera-block preconditioner a coarse
                             correction on the 7 similarity-gauge directions of the camera poses
                             (POSE3 keys: world translation, rotation, scale), the near-null space
                             of a bundle-adjustment reduced system, while those directions stay
                             near-null under the damping; 0 (default): blocks only */
  int32_t pcg_band;       /* PCG forms: 0 (default): one preconditioner block per camera group
                             (block Jacobi, or the learned blocks); k in 1..6: the factorized sparse
                             approximate inverse M = G^T Lambda G, where block row i of G is the last
                             block row of chol(S_JJ)^-1 over J = {i} and the groups i-k .. i-1 coupled
                             to i in S (the Kaporin-optimal lower factor on that pattern, so that
                             G S G^T has unit diagonal blocks), and Lambda_i = I (BLOCK_JACOBI) or the
                             network's L L^T of group i (LEARNED); k = 0 is the block-diagonal case.
                             Not combined with pcg_coarse. */
} sfg_form_params_t;

typedef struct sfg_handle sfg_handle;

/* -------------------------------- library --------------------------------------------------- */
int32_t sfg_abi_version(void);
const char* sfg_last_error(void);
void sfg_default_optimizer_params(sfg_optimizer_params_t* out);
void sfg_default_form_params(sfg_form_params_t* out);
int32_t sfg_key_dims(int32_t key_type, int32_t* storage_dim, int32_t* tangent_dim);
int32_t sfg_factor_dims(int32_t kind, int32_t* num_keys, int32_t* num_consts, int32_t* residual_dim);

/* -------------------------------- sym::Optimizer --------------------------------------------
 * Replaces sym::Optimizer<double> construction (symforce/opt/optimizer.h:86-111) plus the first
 * Linearizer / LinearSolver analysis: uploads the structure, builds the block-sparse Hessian
 * layout, the Schur pair lists and the supernodal symbolic factorization.                      */
int32_t sfg_create(const sfg_problem_t* problem, const sfg_form_params_t* form, sfg_handle** out);
int32_t sfg_destroy(sfg_handle* h);
/* Values: the storage of every key of the problem, concatenated in key order. */
int32_t sfg_storage_dim(const sfg_handle* h, int64_t* storage_dim, int64_t* tangent_dim,
                        int64_t* residual_dim);
int32_t sfg_set_values(sfg_handle* h, const double* storage, int64_t n);
/* Optimizer::Optimize(values, num_iterations, populate_best_linearization, stats)
 * (symforce/opt/optimizer.tcc:79-89): runs the whole LM loop on the device; num_iterations < 0
 * means params->iterations.  Values stay on the device until sfg_get_values. */
int32_t sfg_optimize(sfg_handle* h, const sfg_optimizer_params_t* params, int32_t num_iterations,
                     sfg_stats_t* stats);
/* The loop of GncOptimizer::OptimizeContinue (symforce/opt/gnc_optimizer.h:113-121): ResetState on
 * the values the last call left (its best values), keeping lambda, nu and the iteration counter
 * (symforce/opt/levenberg_marquardt_solver.h:176-183); relax_damping != 0 applies
 * RelaxDampingToInitial first (lambda = min(lambda, initial_lambda), nu = dynamic beta, :170-174).
 * Runs at most num_iterations more iterations.  `stats` receives only the new records (there is no
 * iteration -1 record), num_iterations their count, and best_index the index among them of the
 * last new best, or -1 when none improved on the state the call started from.  Requires a prior
 * sfg_optimize on the handle. */
int32_t sfg_optimize_continue(sfg_handle* h, const sfg_optimizer_params_t* params,
                              int32_t num_iterations, int32_t relax_damping, sfg_stats_t* stats);
/* Replace the constants of one factor batch (layout as in sfg_problem_t, the caller's factor
 * order): the cost function changes, e.g. the convexity parameter mu of BARRON_VEC5 that a
 * graduated non-convexity schedule steps (the reference keeps it as a Values entry the factors
 * read, symforce/opt/gnc_optimizer.h:85-88). */
int32_t sfg_set_factor_consts(sfg_handle* h, int32_t batch, const double* consts, int64_t n);
/* GetBestValues (symforce/opt/levenberg_marquardt_solver.h:178-182). */
int32_t sfg_get_values(sfg_handle* h, double* storage, int64_t n);
/* Linearize the problem at the current values and return residual (M), rhs (N) and error; the
 * Hessian is returned in the reference's CSC lower layout (symforce/opt/linearizer.cc:148-356):
 * pass null arrays to query nnz. */
int32_t sfg_linearize(sfg_handle* h, double* residual, double* rhs, double* error);
int32_t sfg_hessian_lower(sfg_handle* h, int64_t* nnz, int32_t* col_ptr, int32_t* row_idx,
                          double* values);
/* OptimizationStats::cholesky_factor_sparsity (symforce/opt/optimization_stats.h:53-58, filled at
 * symforce/opt/levenberg_marquardt_solver.tcc:209-211): the unit lower factor of the handle's
 * exact factorization (the full damped Hessian, or the reduced camera system of the Schur forms)
 * as a compressed-column strict-lower matrix in the solver's ordering, with the values of the last
 * factorization; query and capacity convention as sfg_ldlt_lower. */
int32_t sfg_factor_lower(sfg_handle* h, int64_t* nnz, int32_t* col_ptr, int32_t* row_idx,
                         double* values);
/* The block ordering used by the linear solver, as new position of every state scalar. */
int32_t sfg_permutation(sfg_handle* h, int32_t* perm, int64_t n);
/* The fronts (supernodes) of the handle's exact factorization, in postorder: the pivot width and
 * the front size of each.  *count in: the capacity of width / size (0: query); out: the number of
 * fronts. */
int32_t sfg_fronts(sfg_handle* h, int32_t* count, int32_t* width, int32_t* size);
/* Time `reps` back-to-back launches of one stage of the iteration on the handle's stream with CUDA
 * events (after one warm-up launch) at the current values: SFG_STAGE_LINEARIZE (all factor
 * batches + staged reduction + cost), SFG_STAGE_SCHUR (point inverses, reduced system and rhs),
 * SFG_STAGE_FACTOR (numeric LDL^T), SFG_STAGE_SOLVE (triangular solves).  Requires a prior
 * sfg_optimize on the handle.  Also returns the stage's algorithmic bytes and multiply-adds. */
enum { SFG_STAGE_LINEARIZE = 0, SFG_STAGE_SCHUR = 1, SFG_STAGE_FACTOR = 2, SFG_STAGE_SOLVE = 3 };
int32_t sfg_time_stage(sfg_handle* h, int32_t stage, int32_t reps, double* ms_per_launch,
                       double* algorithmic_bytes, double* fmas);

/* -------------------------------- PCG forms -------------------------------------------------
 * Statistics of the reduced-system PCG solves of the last sfg_optimize call. */
typedef struct sfg_pcg_stats_t {
  int32_t solves;            /* reduced-system solves */
  int32_t fallbacks;         /* solves that missed pcg_tol and ran the exact LDL^T instead */
  int64_t iterations;        /* PCG iterations summed over the solves */
  int32_t max_iterations;    /* most iterations in one solve */
  int32_t last_iterations;
  double max_rel_residual;   /* largest final FP64 |v - S y| / |v| of a PCG solve */
  double last_rel_residual;
} sfg_pcg_stats_t;
int32_t sfg_get_pcg_stats(sfg_handle* h, sfg_pcg_stats_t* out);
/* The exact factorization as judge of a PCG step: at the values of the last accepted state and
 * the current lambda, solve the reduced system once with PCG and once with the exact LDL^T and
 * return |y_pcg - y_exact| / |y_exact|, the PCG iterations and its FP64 relative residual.
 * Requires a prior sfg_optimize on a PCG-form handle. */
int32_t sfg_pcg_step_error(sfg_handle* h, double* rel_step_error, int32_t* iterations,
                           double* rel_residual);

/* MIXED form: FP32 diagonal tiles of the factorization that had a near-singular pivot (one that kept
 * less than 1/4096 of its diagonal entry, or was not positive) and were factored again in FP64
 * from their input, counted over the handle's life (no counterpart in the reference). */
int32_t sfg_fp64_diag_tiles(sfg_handle* h, int64_t* count);

/* -------------------------------- learned preconditioner -------------------------------------
 * No counterpart in the reference.  One network per camera block: input = the camera's 9 x 9
 * reduced-system block scaled to unit diagonal (81 values, row-major), log(1 + rho_r) for its 9
 * rows (rho_r = sum over the row's entries outside the block of S_rc^2 / (S_rr S_cc)), the number
 * of neighbouring camera blocks / 16, and zero padding (96 inputs); two ReLU layers of 256; 45
 * outputs z, the row-major lower triangle of a 9 x 9 factor L with L_ii = softplus(z_ii + ln(e-1))
 * (zero outputs give L = I).  With D the block's diagonal and C C^T = D^-1/2 S_gg D^-1/2, the
 * preconditioner block is P_g = D^-1/2 C^-T L L^T C^-1 D^-1/2 (L = I: block Jacobi).
 * Weights are float32, packed as W1[96][256], b1[256], W2[256][256], b2[256], W3[256][45], b3[45]
 * (row = input).
 * A training sample is 114 floats: the 96 inputs, g_hat = C^-1 D^-1/2 v_g and
 * x_hat = C^T D^1/2 y_g for the block's part v_g of the reduced rhs and y_g of the exact solution;
 * its loss is |L L^T g_hat - x_hat|^2 / (|x_hat|^2 + 1e-30) (the error of P_g v_g against y_g
 * in the S_gg norm, relative) plus kaporin * (tr(L L^T) - log det(L L^T) - 9) / 9, averaged over
 * samples.  The second term is >= 0 and zero only at L = I: it is the block's share of Kaporin's
 * condition number (tr(K)/n) / det(K)^(1/n) of the preconditioned system K = P^1/2 S P^1/2, which
 * bounds the CG iteration count and which block Jacobi minimizes over all block-diagonal
 * preconditioners, so kaporin > 0 lets the network leave block Jacobi only where the first term
 * pays for it. */
#define SFG_PRECOND_BLOCK 9
#define SFG_PRECOND_FEATURES 96
#define SFG_PRECOND_HIDDEN 256
#define SFG_PRECOND_OUTPUTS 45
#define SFG_PRECOND_SAMPLE_FLOATS 114
#define SFG_PRECOND_NET_PARAMS (96 * 256 + 256 + 256 * 256 + 256 + 256 * 45 + 45)
int32_t sfg_set_preconditioner_weights(sfg_handle* h, const float* weights, int64_t n);
/* Record training samples of every camera block at every LM iteration of later sfg_optimize calls
 * (reduced system and its exact solution; any Schur-form handle), up to max_systems systems. */
int32_t sfg_collect_samples(sfg_handle* h, int32_t max_systems);
/* Copy the recorded samples out (count = blocks x systems recorded); cap in samples. */
int32_t sfg_get_samples(sfg_handle* h, float* samples, int64_t cap, int64_t* count);
typedef struct sfg_train_params_t {
  int32_t steps;        /* optimizer steps */
  int32_t batch;        /* samples per step (drawn without replacement, reshuffled per epoch) */
  float lr;             /* Adam learning rate (cosine decay to lr / 10) */
  float beta1, beta2, eps;
  uint64_t seed;        /* shuffling seed */
  int32_t device;
  float kaporin;        /* weight of the Kaporin term of the loss (0: none) */
} sfg_train_params_t;
/* Train the network on the GPU (Adam, hand-written forward / backward kernels).  weights holds the
 * initial weights and receives the trained ones; loss_curve (optional) receives the batch loss of
 * every step. */
int32_t sfg_precond_train(const float* samples, int64_t n, const sfg_train_params_t* params,
                          float* weights, float* loss_curve);
/* Mean loss over n samples and its gradient with respect to the weights (one forward + backward on
 * the GPU). */
int32_t sfg_precond_loss_grad(const float* samples, int64_t n, const float* weights, float kaporin,
                              double* loss, float* grad, int32_t device);
/* Network outputs z (45 per input row of 96 features). */
int32_t sfg_precond_infer(const float* features, int64_t n, const float* weights, float* out,
                          int32_t device);

/* -------------------------------- batched small problems -----------------------------------
 * Many independent problems of uneven size solved by one persistent kernel launch (captured in a
 * CUDA graph): each warp runs the whole LM loop of one problem at a time (the reference would run
 * one sym::Optimizer<double> per problem, symforce/opt/optimizer.h:72-94), taking problems
 * largest first from a device queue, in FP64.  A batch whose every problem is a Pose3 chain (every
 * key POSE3; unary PRIOR_POSE3 / RANGE_POSE3 factors and BETWEEN_POSE3 factors between consecutive
 * keys) has block-tridiagonal Hessians (6 x 6 blocks) factored by a block Cholesky recursion; any
 * other batch runs the dense path: any key types and factor kinds, at most 128 tangent dimensions a
 * problem (SFG_ERR_STRUCTURE above), every factor's keys distinct (SFG_ERR_STRUCTURE otherwise),
 * the dense Hessian factored by LDL^T; Schur keys are solved with the rest.  Values of all
 * problems are concatenated in problem order.  No reference counterpart for the batching itself. */
typedef struct sfg_batch sfg_batch;
typedef struct sfg_batch_result_t {
  int32_t num_iterations;   /* records, as optimization_stats_t.iterations.size() */
  int32_t best_index;
  int32_t status;
  int32_t failure_reason;
  double initial_error;
  double best_error;
} sfg_batch_result_t;
int32_t sfg_batch_create(const sfg_problem_t* problems, int32_t num_problems,
                         const sfg_form_params_t* form, sfg_batch** out);
int32_t sfg_batch_destroy(sfg_batch* b);
int32_t sfg_batch_storage_dim(const sfg_batch* b, int64_t* storage_dim);
int32_t sfg_batch_set_values(sfg_batch* b, const double* storage, int64_t n);
int32_t sfg_batch_get_values(sfg_batch* b, double* storage, int64_t n);
/* Optimize every problem (results: one entry per problem, may be null); device_ms: CUDA-event time
 * of the launch. */
int32_t sfg_batch_optimize(sfg_batch* b, const sfg_optimizer_params_t* params, int32_t num_iterations,
                           sfg_batch_result_t* results, double* device_ms);
/* The LM records of one problem from the last optimize call. */
int32_t sfg_batch_records(sfg_batch* b, int32_t problem, sfg_iteration_t* records, int32_t capacity,
                          int32_t* count);
/* Launch-shape autotuner: times one optimize per candidate (warps per CTA x CTAs per SM) on the
 * handle's own problems and keeps the fastest; returns the chosen warps per CTA and CTAs. */
int32_t sfg_batch_autotune(sfg_batch* b, const sfg_optimizer_params_t* params, int32_t* warps_per_cta,
                           int32_t* ctas);

/* -------------------------------- SparseCholeskySolver -------------------------------------
 * The LinearSolver concept on a user CSC lower matrix (symforce/opt/sparse_cholesky/
 * sparse_cholesky_solver.h:28-163): AnalyzeSparsityPattern -> sfg_ldlt_create, Factorize ->
 * sfg_ldlt_factorize, Solve/SolveInPlace -> sfg_ldlt_solve.  LDL^T with unit L, no pivoting.    */
typedef struct sfg_ldlt sfg_ldlt;
int32_t sfg_ldlt_create(int32_t n, const int32_t* col_ptr, const int32_t* row_idx,
                        int32_t ordering, int32_t device, sfg_ldlt** out);
int32_t sfg_ldlt_factorize(sfg_ldlt* s, const double* values);
int32_t sfg_ldlt_solve(sfg_ldlt* s, const double* b, double* x, int32_t nrhs);
int32_t sfg_ldlt_diagonal(sfg_ldlt* s, double* d);        /* D() in the solver's ordering */
int32_t sfg_ldlt_permutation(sfg_ldlt* s, int32_t* perm);  /* Permutation(): new index of old i */
/* L() (symforce/opt/sparse_cholesky/sparse_cholesky_solver.h:128-131; read by
 * symforce/opt/levenberg_marquardt_solver.tcc:209-211): the unit lower factor as a compressed-column
 * strict-lower n x n matrix in the solver's ordering, the supernodal pattern (explicit zeros
 * included).  Call with col_ptr, row_idx and values all null to query *nnz; otherwise *nnz is the
 * capacity on entry and the count on return; any of the three arrays may be null. */
int32_t sfg_ldlt_lower(sfg_ldlt* s, int64_t* nnz, int32_t* col_ptr, int32_t* row_idx, double* values);
int32_t sfg_ldlt_destroy(sfg_ldlt* s);

/* -------------------------------- SparseSchurSolver ----------------------------------------
 * symforce/opt/sparse_schur_solver.h:62-135: A (CSC lower) = [[B, E^T],[E, C]] with C block
 * diagonal and dense blocks; ComputeSymbolicSparsity(A, C_dim) -> sfg_schur_create,
 * Factorize -> sfg_schur_factorize, Solve -> sfg_schur_solve.                                  */
typedef struct sfg_schur sfg_schur;
int32_t sfg_schur_create(int32_t n, const int32_t* col_ptr, const int32_t* row_idx, int32_t c_dim,
                         int32_t device, sfg_schur** out);
int32_t sfg_schur_factorize(sfg_schur* s, const double* values);
int32_t sfg_schur_solve(sfg_schur* s, const double* b, double* x, int32_t nrhs);
int32_t sfg_schur_destroy(sfg_schur* s);

/* Self-test of the device wait caps (no counterpart in the reference): one CTA waits, with the
 * capped dependency wait of the persistent kernels, for a flag that nothing sets.  The cap ends
 * the wait without a fault; *device_status receives the device error word (1: a wait hit its cap)
 * and *ms (optional) the kernel's duration.  The device stays usable afterwards. */
int32_t sfg_selftest_wait_cap(int32_t device, int32_t* device_status, double* ms);

/* -------------------------------- dense solve without allocation ----------------------------
 * No counterpart in the reference.  Solves A x = b for a dense symmetric positive definite n x n
 * matrix (LDL^T, unit L, no pivoting; only the lower triangle of A is read) for callers that
 * cannot allocate device memory when they need the solve: code under an allocator that forbids
 * cudaMalloc / cudaFree (they allocate from and may synchronize the whole device), and plugins that
 * only receive device pointers from their host application.  A (column-major, leading dimension
 * lda), b and x are device pointers owned by the caller; `stream` is a cudaStream_t (null: the
 * default stream).  All working memory is a fixed set of file-scope device arrays (about 2.2 MB,
 * held on every GPU that loads the library until the process exits): n may be at most 512, larger
 * n is rejected with SFG_ERR_INVALID_ARGUMENT.  The call allocates nothing.  Its first call on a
 * device looks up the arrays' device addresses (cudaGetSymbolAddress), so make that first call
 * before any stream capture.  The call is synchronous: it copies the device status word to the
 * host and waits for `stream` (cudaStreamSynchronize) before it returns.  A zero or non-finite
 * pivot D (A singular, or not factorizable without pivoting) or a non-finite x returns
 * SFG_ERR_NUMERICAL.  Every call shares the same arrays, so calls that overlap on the GPU (other
 * threads, other streams) race; each call reinitializes everything it reads. */
int32_t sfg_dense_ldlt_solve_noalloc(int32_t n, const double* A, int64_t lda, const double* b,
                                     double* x, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SFGPU_H_ */
