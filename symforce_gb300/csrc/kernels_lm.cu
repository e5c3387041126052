// Levenberg-Marquardt bookkeeping kernels: damping, retraction, the linearized error change, and
// the accept / reject decision.  Together with the linearization and linear-solve kernels they
// form one iteration of LevenbergMarquardtSolver::Iterate
// (symforce/opt/levenberg_marquardt_solver.tcc:138-343), executed entirely on the device; the
// loop runs as a CUDA graph whose while-condition this file's decide kernel sets.
#include "factor_math.cuh"
#include <algorithm>

#include "kernels.h"

namespace sfg {

namespace {

constexpr int kDeltaParts = 64;
constexpr int kDeltaThreads = 256;

__device__ __forceinline__ unsigned long long GlobalTimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// DampHessian (symforce/opt/levenberg_marquardt_solver.tcc:22-54): damping vector from the
// undamped diagonal of the Init block's Hessian.  The Hessian itself is left untouched: the
// damping is added where the damped matrix is assembled.
template <typename T>
__global__ void DampingKernel(DampDev d, const T* hess, int64_t nvals, const LmParams* p,
                              const LmState* st) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  const double lambda = st->lambda;
  const double undamped = double(hess[int64_t(st->init_idx) * nvals + d.diag_off[k]]);
  double damp = 0.0;
  if (p->use_diagonal_damping) {
    if (p->keep_max_diagonal_damping) {
      double m;
      if (!st->have_max_diagonal) {
        m = fmax(undamped, p->diagonal_damping_min);
      } else {
        m = fmax(d.max_diagonal[k], undamped);
      }
      d.max_diagonal[k] = m;
      damp = m * lambda;
    } else {
      damp = fmax(undamped, p->diagonal_damping_min) * lambda;
    }
  }
  if (p->use_unit_damping) damp += lambda;
  d.damping[k] = damp;
}

// Values::Retract (symforce/opt/values.cc:315-327) of the Init block into the New block.
__global__ void RetractKernel(RetractDev r, const LmParams* p, const LmState* st) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= r.nkeys) return;
  const double* a = r.values + int64_t(st->init_idx) * r.S + r.soff[k];
  double* o = r.values + int64_t(st->new_idx) * r.S + r.soff[k];
  const double* d = r.update + r.toff[k];
  switch (r.key_type[k]) {
    case SFG_KEY_POSE2: {  // gen/cpp/sym/ops/pose2/lie_group_ops.cc:58-82
      const double c = cos(d[0]), s = sin(d[0]);
      const double re = a[0], im = a[1];
      o[0] = re * c - im * s;
      o[1] = re * s + im * c;
      o[2] = a[2] + d[1];
      o[3] = a[3] + d[2];
      break;
    }
    case SFG_KEY_POSE3: {  // gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102
      const double eps = p->epsilon;
      const double n = sqrt(eps * eps + d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      const double c = cos(0.5 * n);
      const double s = sin(0.5 * n) / n;
      const double vx = s * d[0], vy = s * d[1], vz = s * d[2];
      const double a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
      o[0] = a3 * vx + a0 * c + a1 * vz - a2 * vy;
      o[1] = a3 * vy - a0 * vz + a1 * c + a2 * vx;
      o[2] = a3 * vz + a0 * vy - a1 * vx + a2 * c;
      o[3] = a3 * c - a0 * vx - a1 * vy - a2 * vz;
      o[4] = a[4] + d[3];
      o[5] = a[5] + d[4];
      o[6] = a[6] + d[5];
      break;
    }
    default: {
      const int n = r.key_type[k];  // VEC1..VEC3: the type value is the dimension
      for (int i = 0; i < n; ++i) o[i] = a[i] + d[i];
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kDeltaThreads) LinearDeltaKernel(const double* u, const T* rhs_all,
                                                                   const double* damping,
                                                                   const double* last, int64_t N,
                                                                   double* partials,
                                                                   const LmState* st, int bold) {
  __shared__ double red[4][kDeltaThreads / 32];
  const T* rhs = rhs_all + int64_t(st->init_idx) * N;
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N;
       i += int64_t(gridDim.x) * blockDim.x) {
    const double ui = u[i];
    s0 += ui * (double(rhs[i]) - damping[i] * ui);
    if (bold) {
      const double li = last[i];
      s1 += ui * li;
      s2 += ui * ui;
      s3 += li * li;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, d);
    s1 += __shfl_down_sync(0xffffffffu, s1, d);
    s2 += __shfl_down_sync(0xffffffffu, s2, d);
    s3 += __shfl_down_sync(0xffffffffu, s3, d);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = s0;
    red[1][w] = s1;
    red[2][w] = s2;
    red[3][w] = s3;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0;
    for (int q = 0; q < kDeltaThreads / 32; ++q) t += red[threadIdx.x][q];
    partials[threadIdx.x * kDeltaParts + blockIdx.x] = t;
  }
}

__global__ void CopyValuesKernel(const double* src, double* values, int64_t S, const LmState* st,
                                 int which) {
  const int state = which == 0 ? st->init_idx : (which == 1 ? st->new_idx : which - 2);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < S;
       i += int64_t(gridDim.x) * blockDim.x)
    values[int64_t(state) * S + i] = src[i];
}

// Reset (symforce/opt/levenberg_marquardt_solver.h:163-175) + Step of the first Iterate.
__global__ void BeginKernel(const LmParams* p, LmState* st, int reset_indices) {
  if (reset_indices) {
    st->init_idx = 0;
    st->new_idx = 1;
    st->best_idx = 0;
    st->free_idx = 2;
  }
  st->lambda = p->initial_lambda;
  st->nu = p->dynamic_beta;
  st->have_max_diagonal = 0;
  st->have_last_update = 0;
  st->num_records = 0;
  st->best_index = 0;
  st->status = 0;
  st->failure_reason = 0;
  st->done = 0;
  st->device_error = 0;
  st->max_iterations = p->iterations;
  st->t_start = GlobalTimer();
  // Step(): swap New and Init; iteration_ = 0
  const int t = st->init_idx;
  st->init_idx = st->new_idx;
  st->new_idx = t;
  st->iteration = 0;
}

// First Iterate after relinearizing Init: SetBestToInit, the iteration -1 record, and the
// INITIAL_ERROR_NOT_FINITE check (symforce/opt/levenberg_marquardt_solver.tcc:151-186).
__global__ void FirstRecordKernel(const LmParams* p, LmState* st, sfg_iteration_t* rec,
                                  cudaGraphConditionalHandle h, int use_cond) {
  if (st->best_idx != st->init_idx) {
    if (st->best_idx != st->new_idx) st->free_idx = st->best_idx;
    st->best_idx = st->init_idx;
  }
  const double e = st->error[st->init_idx];
  sfg_iteration_t r{};
  r.iteration = -1;
  r.new_error = e;
  r.current_lambda = st->lambda;
  r.best_error = e;
  r.elapsed_ms = double(GlobalTimer() - st->t_start) * 1e-6;
  rec[0] = r;
  st->num_records = 1;
  int go = 1;
  if (!isfinite(e)) {
    st->status = SFG_STATUS_FAILED;
    st->failure_reason = SFG_FAILURE_INITIAL_ERROR_NOT_FINITE;
    st->done = 1;
    go = 0;
  } else if (st->max_iterations <= 0) {
    st->done = 1;
    go = 0;
  }
  if (use_cond) cudaGraphSetConditional(h, go);
}

__global__ void DecideKernel(const LmParams* p, LmState* st, sfg_iteration_t* records,
                             const double* update, double* last_update, int64_t N,
                             const double* partials, int nparts, cudaGraphConditionalHandle h,
                             int use_cond) {
  __shared__ int s_copy;
  if (threadIdx.x == 0) {
    double sums[4] = {0, 0, 0, 0};
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < nparts; ++q) sums[c] += partials[c * nparts + q];
    const double eps = p->epsilon;
    const int init = st->init_idx, nw = st->new_idx;
    const double e_init = st->error[init];
    const double e_new = st->error[nw];
    const double relative_reduction = (e_init - e_new) / (e_init + eps);
    const double new_error_linear = e_init + 0.5 * sums[0];
    const double gain_ratio = (e_init - e_new) / (e_init - new_error_linear);
    sfg_iteration_t r{};
    r.iteration = st->iteration;
    r.current_lambda = st->lambda;
    r.new_error = e_new;
    r.new_error_linear = new_error_linear;
    r.relative_reduction = relative_reduction;
    int status = 0, reason = 0;
    if ((relative_reduction > -p->early_exit_min_reduction / 10 &&
         relative_reduction < p->early_exit_min_reduction) ||
        e_new < p->early_exit_min_absolute_error) {
      status = SFG_STATUS_SUCCESS;
    }
    bool accept = relative_reduction > 0;
    double angle = 0;
    if (p->enable_bold_updates && st->have_last_update && !accept) {
      angle = sums[1] / (sqrt(sums[3]) * sqrt(sums[2]));
      accept = ((1 - angle) * (1 - angle) * e_new) <= st->error[st->best_idx];
    }
    if (!accept && st->lambda >= p->lambda_upper_bound) {
      status = SFG_STATUS_FAILED;
      reason = SFG_FAILURE_LAMBDA_OUT_OF_BOUNDS;
    }
    double lambda = st->lambda;
    if (!accept) {
      if (p->lambda_update_type == SFG_LAMBDA_UPDATE_STATIC) {
        lambda *= p->lambda_up_factor;
      } else {
        lambda *= st->nu;
        st->nu *= 2;
      }
      st->init_idx = nw;  // SwapNewAndInit
      st->new_idx = init;
    } else {
      if (p->lambda_update_type == SFG_LAMBDA_UPDATE_STATIC) {
        lambda *= p->lambda_down_factor;
      } else {
        lambda *= fmax(1.0 / p->dynamic_gamma,
                       1.0 - (p->dynamic_beta - 1) * pow(2 * gain_ratio - 1, double(p->dynamic_p)));
        st->nu = 2;
      }
      st->have_last_update = 1;
      if (st->error[nw] <= st->error[st->best_idx]) {  // SetBestToNew
        if (st->best_idx != nw) {
          if (st->best_idx != init) st->free_idx = st->best_idx;
          st->best_idx = nw;
        }
        st->best_index = st->num_records;
      }
      if (st->best_idx == st->init_idx) {  // SetInitToNotBest
        st->init_idx = st->free_idx;
        st->free_idx = st->best_idx;
      }
    }
    lambda = fmin(fmax(lambda, p->lambda_lower_bound), p->lambda_upper_bound);
    st->lambda = lambda;
    if (p->use_diagonal_damping && p->keep_max_diagonal_damping) st->have_max_diagonal = 1;
    r.update_angle_change = angle;
    r.update_accepted = accept ? 1 : 0;
    r.best_error = st->error[st->best_idx];
    r.elapsed_ms = double(GlobalTimer() - st->t_start) * 1e-6;
    records[st->num_records] = r;
    st->num_records += 1;
    int done = 0;
    if (status != 0) {
      st->status = status;
      st->failure_reason = reason;
      done = 1;
    } else if (st->iteration + 1 >= st->max_iterations) {
      st->status = SFG_STATUS_HIT_ITERATION_LIMIT;
      st->failure_reason = 0;
      done = 1;
    }
    if (st->device_error) done = 1;
    st->done = done;
    if (!done) {  // Step() of the next Iterate
      const int t = st->init_idx;
      st->init_idx = st->new_idx;
      st->new_idx = t;
      st->iteration += 1;
    }
    if (use_cond) cudaGraphSetConditional(h, done ? 0 : 1);
    s_copy = (accept && p->enable_bold_updates) ? 1 : 0;
  }
  __syncthreads();
  if (s_copy)
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) last_update[i] = update[i];
}

// Optimize updates the caller's values with the best values (optimizer_utils.h:69): copy the Best
// block back into the input buffer so that the next optimize call starts from it.
__global__ void CopyBestKernel(const double* values, double* dst, int64_t S, const LmState* st) {
  const double* src = values + int64_t(st->best_idx) * S;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < S;
       i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = src[i];
}

}  // namespace

void LaunchCopyBest(const double* values, double* dst, int64_t S, const LmState* st,
                    cudaStream_t s) {
  const int threads = 256;
  int grid = int(std::min<int64_t>((S + threads - 1) / threads, 1024));
  CopyBestKernel<<<std::max(grid, 1), threads, 0, s>>>(values, dst, S, st);
}

int DeltaPartials() { return kDeltaParts; }

template <typename T>
void LaunchDamping(const DampDev& d, const void* hess, int64_t nvals, const LmParams* p,
                   LmState* st, cudaStream_t s) {
  const int threads = 256;
  DampingKernel<T><<<int((d.N + threads - 1) / threads), threads, 0, s>>>(
      d, static_cast<const T*>(hess), nvals, p, st);
}

void LaunchRetract(const RetractDev& r, const LmParams* p, LmState* st, cudaStream_t s) {
  const int threads = 128;
  RetractKernel<<<(r.nkeys + threads - 1) / threads, threads, 0, s>>>(r, p, st);
}

template <typename T>
void LaunchLinearDelta(const double* update, const void* rhs, const double* damping,
                       const double* last_update, int64_t N, double* partials, LmState* st,
                       int bold, cudaStream_t s) {
  LinearDeltaKernel<T><<<kDeltaParts, kDeltaThreads, 0, s>>>(
      update, static_cast<const T*>(rhs), damping, last_update, N, partials, st, bold);
}

void LaunchDecide(const LmParams* p, LmState* st, sfg_iteration_t* records, const double* update,
                  double* last_update, int64_t N, const double* delta_partials, int nparts,
                  cudaGraphConditionalHandle h, int use_cond, cudaStream_t s) {
  DecideKernel<<<1, 256, 0, s>>>(p, st, records, update, last_update, N, delta_partials, nparts,
                                 h, use_cond);
}

void LaunchBegin(const LmParams* p, LmState* st, int reset_indices, cudaStream_t s) {
  BeginKernel<<<1, 1, 0, s>>>(p, st, reset_indices);
}

void LaunchFirstRecord(const LmParams* p, LmState* st, sfg_iteration_t* records,
                       cudaGraphConditionalHandle h, int use_cond, cudaStream_t s) {
  FirstRecordKernel<<<1, 1, 0, s>>>(p, st, records, h, use_cond);
}

void LaunchCopyValues(const double* src, double* values, int64_t S, const LmState* st, int which,
                      cudaStream_t s) {
  const int threads = 256;
  int grid = int(std::min<int64_t>((S + threads - 1) / threads, 1024));
  if (grid < 1) grid = 1;
  CopyValuesKernel<<<grid, threads, 0, s>>>(src, values, S, st, which);
}

template void LaunchDamping<double>(const DampDev&, const void*, int64_t, const LmParams*, LmState*,
                                    cudaStream_t);
template void LaunchDamping<float>(const DampDev&, const void*, int64_t, const LmParams*, LmState*,
                                   cudaStream_t);
template void LaunchLinearDelta<double>(const double*, const void*, const double*, const double*,
                                        int64_t, double*, LmState*, int, cudaStream_t);
template void LaunchLinearDelta<float>(const double*, const void*, const double*, const double*,
                                       int64_t, double*, LmState*, int, cudaStream_t);

}  // namespace sfg
