// The Levenberg-Marquardt bookkeeping of LevenbergMarquardtSolver::Iterate
// (symforce/opt/levenberg_marquardt_solver.tcc:138-343) and its state blocks
// (symforce/opt/internal/levenberg_marquardt_state.h:33-270) as device functions on one LmState:
// the start of an optimize call, the initial record, and the accept / reject decision with the
// lambda update, best tracking, state-index juggling and early exits.  Both the single-problem
// graph (kernels_lm.cu) and the batched persistent kernel (kernels_batch.cu) call these, so the
// two share one definition of the algorithm.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "../../include/sfgpu.h"
#include "device.cuh"

namespace sfg {

__device__ __forceinline__ unsigned long long LmGlobalTimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Reset (symforce/opt/levenberg_marquardt_solver.h:163-175) + Step of the first Iterate.
__device__ __forceinline__ void LmBegin(const LmParams& p, LmState& st, int reset_indices) {
  if (p.continue_state) {
    // ResetState (symforce/opt/levenberg_marquardt_solver.h:176-183): lambda, nu and the iteration
    // counter carry over; the caller's values become New and every linearization is reset
    if (p.relax_damping) {
      st.lambda = fmin(st.lambda, p.initial_lambda);
      st.nu = p.dynamic_beta;
    }
    st.have_max_diagonal = 0;
    st.have_last_update = 0;
    st.num_records = 0;
    st.best_index = -1;
    st.status = 0;
    st.failure_reason = 0;
    st.done = 0;
    st.device_error = 0;
    st.t_start = LmGlobalTimer();
    const int t = st.init_idx;
    st.init_idx = st.new_idx;
    st.new_idx = t;
    st.iteration += 1;
    st.max_iterations = st.iteration + p.iterations;
    return;
  }
  if (reset_indices) {
    st.init_idx = 0;
    st.new_idx = 1;
    st.best_idx = 0;
    st.free_idx = 2;
  }
  st.lambda = p.initial_lambda;
  st.nu = p.dynamic_beta;
  st.have_max_diagonal = 0;
  st.have_last_update = 0;
  st.num_records = 0;
  st.best_index = 0;
  st.status = 0;
  st.failure_reason = 0;
  st.done = 0;
  st.device_error = 0;
  st.max_iterations = p.iterations;
  st.t_start = LmGlobalTimer();
  // Step(): swap New and Init; iteration_ = 0
  const int t = st.init_idx;
  st.init_idx = st.new_idx;
  st.new_idx = t;
  st.iteration = 0;
}

// First Iterate after relinearizing Init: SetBestToInit, the iteration -1 record, and the
// INITIAL_ERROR_NOT_FINITE check (symforce/opt/levenberg_marquardt_solver.tcc:151-186).
// Returns 1 if the loop runs.
__device__ __forceinline__ int LmFirstRecord(const LmParams& p, LmState& st, sfg_iteration_t* rec) {
  if (st.best_idx != st.init_idx) {
    if (st.best_idx != st.new_idx) st.free_idx = st.best_idx;
    st.best_idx = st.init_idx;
  }
  const double e = st.error[st.init_idx];
  if (p.continue_state) {
    // the iteration -1 record and the initial-error check belong to iteration 0 only
    // (symforce/opt/levenberg_marquardt_solver.tcc:157-186)
    if (st.iteration >= st.max_iterations) {
      st.done = 1;
      return 0;
    }
    return 1;
  }
  sfg_iteration_t r{};
  r.iteration = -1;
  r.new_error = e;
  r.current_lambda = st.lambda;
  r.best_error = e;
  r.elapsed_ms = double(LmGlobalTimer() - st.t_start) * 1e-6;
  if (rec) rec[0] = r;
  st.num_records = 1;
  int go = 1;
  if (!isfinite(e)) {
    st.status = SFG_STATUS_FAILED;
    st.failure_reason = SFG_FAILURE_INITIAL_ERROR_NOT_FINITE;
    st.done = 1;
    go = 0;
  } else if (st.max_iterations <= 0) {
    st.done = 1;
    go = 0;
  }
  return go;
}

// The decision half of Iterate.  sums = {u.(rhs - d.u), u.last, u.u, last.last}.  Writes the
// record (if `records`), sets *copy_last when the update must be kept for bold updates, and
// returns 1 when the loop stops.
__device__ __forceinline__ int LmDecide(const LmParams& p, LmState& st, sfg_iteration_t* records,
                                        const double* sums, int* copy_last) {
  const double eps = p.epsilon;
  const int init = st.init_idx, nw = st.new_idx;
  const double e_init = st.error[init];
  const double e_new = st.error[nw];
  const double relative_reduction = (e_init - e_new) / (e_init + eps);
  const double new_error_linear = e_init + 0.5 * sums[0];
  const double gain_ratio = (e_init - e_new) / (e_init - new_error_linear);
  sfg_iteration_t r{};
  r.iteration = st.iteration;
  r.current_lambda = st.lambda;
  r.new_error = e_new;
  r.new_error_linear = new_error_linear;
  r.relative_reduction = relative_reduction;
  int status = 0, reason = 0;
  if ((relative_reduction > -p.early_exit_min_reduction / 10 &&
       relative_reduction < p.early_exit_min_reduction) ||
      e_new < p.early_exit_min_absolute_error) {
    status = SFG_STATUS_SUCCESS;
  }
  bool accept = relative_reduction > 0;
  double angle = 0;
  if (p.enable_bold_updates && st.have_last_update && !accept) {
    angle = sums[1] / (sqrt(sums[3]) * sqrt(sums[2]));
    accept = ((1 - angle) * (1 - angle) * e_new) <= st.error[st.best_idx];
  }
  if (!accept && st.lambda >= p.lambda_upper_bound) {
    status = SFG_STATUS_FAILED;
    reason = SFG_FAILURE_LAMBDA_OUT_OF_BOUNDS;
  }
  double lambda = st.lambda;
  if (!accept) {
    if (p.lambda_update_type == SFG_LAMBDA_UPDATE_STATIC) {
      lambda *= p.lambda_up_factor;
    } else {
      lambda *= st.nu;
      st.nu *= 2;
    }
    st.init_idx = nw;  // SwapNewAndInit
    st.new_idx = init;
  } else {
    if (p.lambda_update_type == SFG_LAMBDA_UPDATE_STATIC) {
      lambda *= p.lambda_down_factor;
    } else {
      lambda *= fmax(1.0 / p.dynamic_gamma,
                     1.0 - (p.dynamic_beta - 1) * pow(2 * gain_ratio - 1, double(p.dynamic_p)));
      st.nu = 2;
    }
    st.have_last_update = 1;
    if (st.error[nw] <= st.error[st.best_idx]) {  // SetBestToNew
      if (st.best_idx != nw) {
        if (st.best_idx != init) st.free_idx = st.best_idx;
        st.best_idx = nw;
      }
      st.best_index = st.num_records;
    }
    if (st.best_idx == st.init_idx) {  // SetInitToNotBest
      st.init_idx = st.free_idx;
      st.free_idx = st.best_idx;
    }
  }
  lambda = fmin(fmax(lambda, p.lambda_lower_bound), p.lambda_upper_bound);
  st.lambda = lambda;
  if (p.use_diagonal_damping && p.keep_max_diagonal_damping) st.have_max_diagonal = 1;
  r.update_angle_change = angle;
  r.update_accepted = accept ? 1 : 0;
  r.best_error = st.error[st.best_idx];
  r.elapsed_ms = double(LmGlobalTimer() - st.t_start) * 1e-6;
  if (records) records[st.num_records] = r;
  st.num_records += 1;
  int done = 0;
  if (status != 0) {
    st.status = status;
    st.failure_reason = reason;
    done = 1;
  } else if (st.iteration + 1 >= st.max_iterations) {
    st.status = SFG_STATUS_HIT_ITERATION_LIMIT;
    st.failure_reason = 0;
    done = 1;
  }
  if (st.device_error) done = 1;
  st.done = done;
  if (!done) {  // Step() of the next Iterate
    const int t = st.init_idx;
    st.init_idx = st.new_idx;
    st.new_idx = t;
    st.iteration += 1;
  }
  *copy_last = (accept && p.enable_bold_updates) ? 1 : 0;
  return done;
}

// DampHessian (symforce/opt/levenberg_marquardt_solver.tcc:22-54) of one tangent scalar from its
// undamped diagonal entry; `max_diag` is the running maximum kept for keep_max_diagonal_damping.
__device__ __forceinline__ double LmDamping(const LmParams& p, const LmState& st, double undamped,
                                            double* max_diag) {
  const double lambda = st.lambda;
  double damp = 0.0;
  if (p.use_diagonal_damping) {
    if (p.keep_max_diagonal_damping) {
      const double m = !st.have_max_diagonal ? fmax(undamped, p.diagonal_damping_min)
                                             : fmax(*max_diag, undamped);
      *max_diag = m;
      damp = m * lambda;
    } else {
      damp = fmax(undamped, p.diagonal_damping_min) * lambda;
    }
  }
  if (p.use_unit_damping) damp += lambda;
  return damp;
}

}  // namespace sfg
