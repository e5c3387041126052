// Factor linearization kernels (the device replacement of Linearizer::Relinearize,
// symforce/opt/linearizer.cc:54-120, and of the per-factor Factor::Linearize calls it makes).
//
// One thread evaluates one factor: it gathers its keys' storage, evaluates the residual in FP64
// and the tangent Jacobian in T, forms the packed lower Gauss-Newton block J^T J and J^T r, and
// writes each entry to its precomputed sink slot: directly into the block-sparse Hessian when the
// factor is the only contributor to that entry, otherwise into a staging slot that a second kernel
// sums in a fixed order (no atomics, bit-reproducible).  Keys, constants and sink indices are
// structure-of-arrays so that a warp's loads and stores of one entry are coalesced.
#include "factor_math.cuh"
#include "kernels.h"

namespace sfg {

namespace {

constexpr int kLinBlock = 128;

template <typename T>
__device__ __forceinline__ void SinkStore(int32_t idx, T v, T* hess, T* rhs, T* stage, int64_t nvals,
                                          int64_t N) {
  if (idx < nvals) {
    hess[idx] = v;
  } else if (idx < nvals + N) {
    rhs[idx - nvals] = v;
  } else {
    stage[idx - nvals - N] = v;
  }
}

template <int KIND, typename T>
__global__ void __launch_bounds__(kLinBlock) LinearizeKernel(LinOut o, BatchDev b) {
  using Tr = FactorTraits<KIND>;
  constexpr int TD = Tr::TD, RD = Tr::RD, NK = Tr::NK, NC = Tr::NC;
  __shared__ double red[kLinBlock / 32];
  const int state = o.which == 0 ? o.st->init_idx : (o.which == 1 ? o.st->new_idx : o.which - 2);
  const double* vals = o.values + int64_t(state) * o.S;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double err = 0.0;
  if (f < b.count) {
    double xs[NK][7];
    const double* xp[3];
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int key = __ldg(b.keys + int64_t(k) * b.count + f);
      const double* src = vals + __ldg(o.key_soff + key);
#pragma unroll
      for (int i = 0; i < Tr::KS(k); ++i) xs[k][i] = src[i];
      xp[k] = xs[k];
    }
    double c[NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) c[i] = __ldg(b.consts + int64_t(i) * b.count + f);
    double r[RD];
    T J[RD * TD];
    FactorEval<KIND, T>::Run(xp, c, r, J);
    double* res = o.residual + int64_t(state) * o.M + b.roff + int64_t(f) * RD;
#pragma unroll
    for (int i = 0; i < RD; ++i) {
      res[i] = r[i];
      err += r[i] * r[i];
    }
    T* hess = static_cast<T*>(o.hess) + int64_t(state) * o.nvals;
    T* rhs = static_cast<T*>(o.rhs) + int64_t(state) * o.N;
    T* stage = static_cast<T*>(o.stage);
    const int32_t* dest = b.dest + f;
    int e = 0;
#pragma unroll
    for (int a = 0; a < TD; ++a) {
#pragma unroll
      for (int q = 0; q <= a; ++q) {
        T h = T(0);
#pragma unroll
        for (int i = 0; i < RD; ++i) h += J[i * TD + a] * J[i * TD + q];
        SinkStore<T>(__ldg(dest + int64_t(e) * b.count), h, hess, rhs, stage, o.nvals, o.N);
        ++e;
      }
    }
#pragma unroll
    for (int a = 0; a < TD; ++a) {
      T g = T(0);
#pragma unroll
      for (int i = 0; i < RD; ++i) g += J[i * TD + a] * T(r[i]);
      SinkStore<T>(__ldg(dest + int64_t(e) * b.count), g, hess, rhs, stage, o.nvals, o.N);
      ++e;
    }
  }
  // deterministic block reduction of r^2: fixed shuffle tree, then warp 0
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) err += __shfl_down_sync(0xffffffffu, err, d);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = err;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kLinBlock / 32; ++w) s += red[w];
    o.cost_partials[b.partial_base + blockIdx.x] = s;
  }
}

// One warp per shared destination: lanes stride over its staged contributions (a camera block
// collects hundreds) and a fixed shuffle tree adds them, so the order is the same on every run.
template <typename T>
__global__ void ReduceStageKernel(ReduceDev r, LinOut o) {
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= r.ngroups) return;
  const int state = o.which == 0 ? o.st->init_idx : (o.which == 1 ? o.st->new_idx : o.which - 2);
  const T* stage = static_cast<const T*>(o.stage);
  T acc = T(0);
  const int64_t p1 = r.ptr[g + 1];
  for (int64_t q = r.ptr[g] + lane; q < p1; q += 32) acc += stage[q];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
  if (lane != 0) return;
  const int32_t d = r.dst[g];
  if (d < o.nvals) {
    static_cast<T*>(o.hess)[int64_t(state) * o.nvals + d] = acc;
  } else {
    static_cast<T*>(o.rhs)[int64_t(state) * o.N + (d - o.nvals)] = acc;
  }
}

__global__ void FinishCostKernel(const double* partials, int n, LmState* st, int which) {
  // one warp, fixed order
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 32) s += partials[i];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
  if (threadIdx.x == 0) {
    const int state = which == 0 ? st->init_idx : (which == 1 ? st->new_idx : which - 2);
    st->error[state] = 0.5 * s;
  }
}

}  // namespace

int LinearizeBlockSize() { return kLinBlock; }

template <typename T>
void LaunchLinearize(int kind, const LinOut& out, const BatchDev& b, cudaStream_t s) {
  if (b.count == 0) return;
  const int grid = (b.count + kLinBlock - 1) / kLinBlock;
  switch (kind) {
    case SFG_FACTOR_BEARING_POSE2:
      LinearizeKernel<SFG_FACTOR_BEARING_POSE2, T><<<grid, kLinBlock, 0, s>>>(out, b);
      break;
    case SFG_FACTOR_ODOMETRY_POSE2:
      LinearizeKernel<SFG_FACTOR_ODOMETRY_POSE2, T><<<grid, kLinBlock, 0, s>>>(out, b);
      break;
    case SFG_FACTOR_SNAVELY_REPROJECTION:
      LinearizeKernel<SFG_FACTOR_SNAVELY_REPROJECTION, T><<<grid, kLinBlock, 0, s>>>(out, b);
      break;
    case SFG_FACTOR_BETWEEN_POSE3:
      LinearizeKernel<SFG_FACTOR_BETWEEN_POSE3, T><<<grid, kLinBlock, 0, s>>>(out, b);
      break;
    case SFG_FACTOR_PRIOR_POSE3:
      LinearizeKernel<SFG_FACTOR_PRIOR_POSE3, T><<<grid, kLinBlock, 0, s>>>(out, b);
      break;
    case SFG_FACTOR_RANGE_POSE3:
      LinearizeKernel<SFG_FACTOR_RANGE_POSE3, T><<<grid, kLinBlock, 0, s>>>(out, b);
      break;
  }
}

template <typename T>
void LaunchReduceStage(const ReduceDev& r, const LinOut& out, cudaStream_t s) {
  if (r.ngroups == 0) return;
  const int warps = 8;
  ReduceStageKernel<T><<<(r.ngroups + warps - 1) / warps, 32 * warps, 0, s>>>(r, out);
}

void LaunchFinishCost(const double* partials, int npartials, LmState* st, int which,
                      cudaStream_t s) {
  FinishCostKernel<<<1, 32, 0, s>>>(partials, npartials, st, which);
}

template void LaunchLinearize<double>(int, const LinOut&, const BatchDev&, cudaStream_t);
template void LaunchLinearize<float>(int, const LinOut&, const BatchDev&, cudaStream_t);
template void LaunchReduceStage<double>(const ReduceDev&, const LinOut&, cudaStream_t);
template void LaunchReduceStage<float>(const ReduceDev&, const LinOut&, cudaStream_t);

}  // namespace sfg
