// Device-side plain structs shared by the kernels and the host driver.  All pointers are device
// pointers; every array is laid out for coalesced access by consecutive threads (structure of
// arrays: entry-major, factor-minor).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sfg {

// LM state shared by every kernel of an optimization, in device memory.  The three state blocks
// (values + linearization) follow the reference's Init / New / Best / Free index juggling
// (symforce/opt/internal/levenberg_marquardt_state.h:33-170).
struct LmState {
  int init_idx, new_idx, best_idx, free_idx;
  int iteration;        // reference iteration_ (starts at -1)
  int num_records;      // records written
  int best_index;       // record index of the best iteration
  int status, failure_reason;
  int done;             // 1 when the loop must stop
  int have_last_update;
  int have_max_diagonal;
  int device_error;     // nonzero: a device loop hit its cap (see DeviceErrorCode)
  int max_iterations;
  double lambda, nu;
  double error[3];      // cached 0.5 |r|^2 per state block
  double linear_delta;  // 0.5 u.(rhs - d.u) of the current step
  double update_dot_last, update_norm2, last_norm2;
  unsigned long long t_start;  // globaltimer at the start of the optimize call
};

// Outcome of the reduced-system PCG solves (PCG forms).  The per-solve fields describe the last
// solve; need_fallback gates the exact factorization kernels that follow it.  The running totals
// are cleared at the start of every optimize call.
struct PcgState {
  int need_fallback;     // 1: the last solve missed its tolerance, the exact LDL^T runs
  int converged;
  int iterations;        // inner iterations of the last solve
  int outer;             // FP64 residual passes of the last solve
  double rel_residual;   // FP64 |v - S y| / |v| after the last solve
  long long total_iterations;
  int solves, fallbacks, max_iterations, pad;
  double max_rel_residual;
};

// Task kinds of the persistent factorization kernel.
// kTaskLookahead(k): the panel solve of tile (k+1, k), the update of diagonal tile (k+1, k+1) by
// that panel and the LDL^T of tile (k+1, k+1), in one CTA.
// kTaskChain: the whole critical chain of a front in one CTA: the LDL^T of tile (0, 0), then every
// look-ahead step k = 0 .. np - 2 in turn, the factor of tile (k, k) kept in shared memory.
// kTaskInverse(k): the inverse of tile (k, k)'s unit lower factor, for the triangular solves (FP64
// chains leave it out of the chain).
// kTaskUpdateTc: panel k's update of tiles (i0 .. i0 + cnt - 1, j) on the tensor cores (FP32
// fronts); z = i0 << 16 | j, w = k | cnt << 20.
enum TaskType {
  kTaskAssemble = 0,
  kTaskDiag = 1,
  kTaskTrsm = 2,
  kTaskUpdate = 3,
  kTaskLookahead = 4,
  kTaskChain = 5,
  kTaskInverse = 6,
  kTaskUpdateTc = 7
};

enum DeviceErrorCode {
  kDevOk = 0,
  kDevSpinTimeout = 1,   // a dependency wait in a persistent kernel exceeded its cap
  kDevBadTask = 2,
};

// LM parameters (optimizer_params_t subset used on the device).
struct LmParams {
  double initial_lambda, lambda_lower_bound, lambda_upper_bound;
  double lambda_up_factor, lambda_down_factor;
  double dynamic_beta, dynamic_gamma;
  double diagonal_damping_min, early_exit_min_reduction, early_exit_min_absolute_error;
  double epsilon;
  int lambda_update_type, dynamic_p;
  int use_diagonal_damping, use_unit_damping, keep_max_diagonal_damping;
  int enable_bold_updates;
  int iterations;
  // 1: continue an optimization (OptimizeContinue of symforce/opt/gnc_optimizer.h:113-121):
  // ResetState on the current values, keeping lambda, nu and the iteration counter, and write no
  // iteration -1 record; relax_damping additionally applies RelaxDampingToInitial first
  // (symforce/opt/levenberg_marquardt_solver.h:170-174)
  int continue_state, relax_damping;
};

// One factor batch as seen by the linearization kernel.
struct BatchDev {
  int count;
  int nent;                 // tdim*(tdim+1)/2 packed Hessian entries + tdim rhs entries
  const int32_t* keys;      // [nk][count]
  const double* consts;     // [nc][count]
  const int32_t* dest;      // [nent][count] sink index of each entry
  int64_t roff;             // residual row of the first factor
  int partial_base;         // first cost-partial slot of this batch
};

// Where linearization results go.  Sink index space: [0, nvals) Hessian block values,
// [nvals, nvals + N) rhs, [nvals + N, ...) shared staging for multi-source entries.
struct LinOut {
  const double* values;     // [3][S] storage of the three state blocks
  const int64_t* key_soff;  // storage offset of each key
  double* residual;         // [3][M]
  void* hess;               // [3][nvals] (T)
  void* rhs;                // [3][N] (T)
  void* stage;              // [nstage] (T)
  double* cost_partials;    // per-CTA partial sums of r^2
  int64_t S, M, N, nvals;
  const LmState* st;
  int which;                // 0: linearize Init, 1: linearize New
};

}  // namespace sfg
