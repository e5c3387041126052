// Levenberg-Marquardt bookkeeping kernels: damping, retraction, the linearized error change, and
// the accept / reject decision.  Together with the linearization and linear-solve kernels they
// form one iteration of LevenbergMarquardtSolver::Iterate
// (symforce/opt/levenberg_marquardt_solver.tcc:138-343), executed entirely on the device; the
// loop runs as a CUDA graph whose while-condition this file's decide kernel sets.
#include "factor_math.cuh"
#include <algorithm>

#include "kernels.h"
#include "lm_logic.cuh"

namespace sfg {

namespace {

constexpr int kDeltaParts = 64;
constexpr int kDeltaThreads = 256;

// DampHessian (symforce/opt/levenberg_marquardt_solver.tcc:22-54): damping vector from the
// undamped diagonal of the Init block's Hessian.  The Hessian itself is left untouched: the
// damping is added where the damped matrix is assembled.
template <typename T>
__global__ void DampingKernel(DampDev d, const T* hess, int64_t nvals, const LmParams* p,
                              const LmState* st) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  const double undamped = double(hess[int64_t(st->init_idx) * nvals + d.diag_off[k]]);
  const double damp = LmDamping(*p, *st, undamped, d.max_diagonal + k);
  d.damping[k] = damp;
}

// Values::Retract (symforce/opt/values.cc:315-327) of the Init block into the New block.
__global__ void RetractKernel(RetractDev r, const LmParams* p, const LmState* st) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= r.nkeys) return;
  const double* a = r.values + int64_t(st->init_idx) * r.S + r.soff[k];
  double* o = r.values + int64_t(st->new_idx) * r.S + r.soff[k];
  const double* d = r.update + r.toff[k];
  RetractKey(r.key_type[k], a, d, p->epsilon, o);
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
  LmBegin(*p, *st, reset_indices);
}

// First Iterate after relinearizing Init: SetBestToInit, the iteration -1 record, and the
// INITIAL_ERROR_NOT_FINITE check (symforce/opt/levenberg_marquardt_solver.tcc:151-186).
__global__ void FirstRecordKernel(const LmParams* p, LmState* st, sfg_iteration_t* rec,
                                  cudaGraphConditionalHandle h, int use_cond) {
  const int go = LmFirstRecord(*p, *st, rec);
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
    int copy = 0;
    const int done = LmDecide(*p, *st, records, sums, &copy);
    if (use_cond) cudaGraphSetConditional(h, done ? 0 : 1);
    s_copy = copy;
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
