// Factor linearization kernels (the device replacement of Linearizer::Relinearize,
// symforce/opt/linearizer.cc:54-120, and of the per-factor Factor::Linearize calls it makes).
//
// One thread evaluates one factor: it gathers its keys' storage, evaluates the residual in FP64
// and the tangent Jacobian in T, forms the packed lower Gauss-Newton block J^T J and J^T r, and
// writes each entry to its precomputed sink slot: directly into the block-sparse Hessian when the
// factor is the only contributor to that entry, otherwise into a staging slot that a second kernel
// sums in a fixed order (no atomics, bit-reproducible).  Keys, constants and sink indices are
// structure-of-arrays so that a warp's loads and stores of one entry are coalesced.
//
// Factors are in the layout's device order: for a kind with merged key slots (a reprojection
// factor's camera) the factors of one camera are consecutive, and a warp whose 32 factors share
// the camera adds the camera entries of its lanes with a shuffle reduce-scatter (lane l ends with
// the warp's sum of entry l) and stores each sum once — the warp-shuffle reduction in place of
// 32 staged contributions.
#include "common.h"
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

// Lane l returns the sum over the warp's lanes of v[l]: five exchange levels, each lane keeping the
// half of its entries whose index bit matches its own lane bit and adding the partner's copy of
// that half (31 shuffles and adds per lane for 32 entries; a fixed order of additions).
template <typename T>
__device__ __forceinline__ T ReduceScatter32(T (&v)[32], int lane) {
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1) {
    const bool upper = (lane & w) != 0;
#pragma unroll
    for (int j = 0; j < w; ++j) {
      const T keep = upper ? v[j + w] : v[j];
      const T send = upper ? v[j] : v[j + w];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, w);
    }
  }
  return v[0];
}

template <typename Tr>
__host__ __device__ constexpr int MergedDims() {
  int d = 0;
  for (int k = 0; k < Tr::MK; ++k) d += Tr::KT(k);
  return d;
}

template <int KIND, typename T>
__global__ void __launch_bounds__(kLinBlock) LinearizeKernel(LinOut o, BatchDev b) {
  using Tr = FactorTraits<KIND>;
  constexpr int TD = Tr::TD, RD = Tr::RD, NK = Tr::NK, NC = Tr::NC;
  constexpr int NH = TD * (TD + 1) / 2;
  constexpr int MT = MergedDims<Tr>();      // tangent columns of the merged key slots
  constexpr int MH = MT * (MT + 1) / 2;     // their packed lower entries (a prefix of the packing)
  constexpr int NM = MH + MT;               // merged entries: packed prefix and rhs prefix
  __shared__ double red[kLinBlock / 32];
  const int state = o.which == 0 ? o.st->init_idx : (o.which == 1 ? o.st->new_idx : o.which - 2);
  const double* vals = o.values + int64_t(state) * o.S;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = f < b.count;
  int key[NK];
#pragma unroll
  for (int k = 0; k < NK; ++k) key[k] = valid ? __ldg(b.keys + int64_t(k) * b.count + f) : -1;
  bool merged = false;
  if constexpr (Tr::MK > 0) {
    // every lane takes part in every shuffle (no short-circuit around them)
    bool same = valid;
#pragma unroll
    for (int k = 0; k < Tr::MK; ++k) {
      const int first = __shfl_sync(0xffffffffu, key[k], 0);
      same = same && key[k] == first;
    }
    merged = __all_sync(0xffffffffu, same);
  }
  double err = 0.0;
  if (valid) {
    double xs[NK][7];
    const double* xp[3];
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const double* src = vals + __ldg(o.key_soff + key[k]);
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
    // entries this factor stores itself: all of them, or those outside the merged prefix
    int e = 0;
#pragma unroll
    for (int a = 0; a < TD; ++a) {
#pragma unroll
      for (int q = 0; q <= a; ++q) {
        if (a >= MT || !merged) {
          T h = T(0);
#pragma unroll
          for (int i = 0; i < RD; ++i) h += J[i * TD + a] * J[i * TD + q];
          SinkStore<T>(__ldg(dest + int64_t(e) * b.count), h, hess, rhs, stage, o.nvals, o.N);
        }
        ++e;
      }
    }
#pragma unroll
    for (int a = 0; a < TD; ++a) {
      if (a >= MT || !merged) {
        T g = T(0);
#pragma unroll
        for (int i = 0; i < RD; ++i) g += J[i * TD + a] * T(r[i]);
        SinkStore<T>(__ldg(dest + int64_t(e) * b.count), g, hess, rhs, stage, o.nvals, o.N);
      }
      ++e;
    }
    if constexpr (NM > 0) {
      if (merged) {
        // all 32 lanes are valid factors of one camera: 32 merged entries at a time
        const int32_t* dest0 = b.dest + (f - lane);
#pragma unroll
        for (int ch = 0; ch < (NM + 31) / 32; ++ch) {
          T v[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = T(0);
          int m = 0;
#pragma unroll
          for (int a = 0; a < MT; ++a) {
#pragma unroll
            for (int q = 0; q <= a; ++q) {
              if (m >= 32 * ch && m < 32 * ch + 32) {
                T h = T(0);
#pragma unroll
                for (int i = 0; i < RD; ++i) h += J[i * TD + a] * J[i * TD + q];
                v[m - 32 * ch] = h;
              }
              ++m;
            }
          }
#pragma unroll
          for (int a = 0; a < MT; ++a) {
            if (m >= 32 * ch && m < 32 * ch + 32) {
              T g = T(0);
#pragma unroll
              for (int i = 0; i < RD; ++i) g += J[i * TD + a] * T(r[i]);
              v[m - 32 * ch] = g;
            }
            ++m;
          }
          const T sum = ReduceScatter32<T>(v, lane);
          const int mm = 32 * ch + lane;
          if (mm < NM) {
            const int em = mm < MH ? mm : NH + (mm - MH);
            SinkStore<T>(__ldg(dest0 + int64_t(em) * b.count), sum, hess, rhs, stage, o.nvals, o.N);
          }
        }
      }
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

// One thread per shared destination adds its staged contributions in slot order (a point entry
// has one per observation; a camera entry one per warp of its observations, plus the partial
// warps at its ends), so the order is the same on every run.
template <typename T>
__global__ void ReduceStageKernel(ReduceDev r, LinOut o) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= r.ngroups) return;
  const int state = o.which == 0 ? o.st->init_idx : (o.which == 1 ? o.st->new_idx : o.which - 2);
  const T* stage = static_cast<const T*>(o.stage);
  const int64_t p0 = r.ptr[g], p1 = r.ptr[g + 1];
  T acc = stage[p0];
  for (int64_t q = p0 + 1; q < p1; ++q) acc += stage[q];
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

static_assert(FactorTraits<SFG_FACTOR_SNAVELY_REPROJECTION>::MK ==
                  MergedKeySlots(SFG_FACTOR_SNAVELY_REPROJECTION),
              "merged key slots of the kernel and of the host layout differ");
static_assert(kLinBlock % 32 == 0, "merged warps are aligned to the factor index");

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
#define SFG_GENERATED_CASE(KIND, NKEYS, NCONSTS, RDIM, K0, K1, K2, G) \
    case KIND:                                                         \
      LinearizeKernel<KIND, T><<<grid, kLinBlock, 0, s>>>(out, b);     \
      break;
      SFG_GENERATED_FACTORS(SFG_GENERATED_CASE)
#undef SFG_GENERATED_CASE
  }
}

template <typename T>
void LaunchReduceStage(const ReduceDev& r, const LinOut& out, cudaStream_t s) {
  if (r.ngroups == 0) return;
  const int threads = 128;
  ReduceStageKernel<T><<<(r.ngroups + threads - 1) / threads, threads, 0, s>>>(r, out);
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
