// Training kernels of the camera-block preconditioner network besides its GEMMs (which run on the
// tensor cores, kernels_tc.cu): column sums for bias gradients, the loss head (factor L from the
// outputs, P = L L^T applied to g_hat against x_hat, plus the Kaporin term) with its analytic
// gradient, batch gather and Adam.  Every reduction runs in a fixed order, so training is
// bit-reproducible.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace sfg {

namespace {

constexpr float kDiagShift = 0.54132485f;  // ln(e - 1)

__device__ __forceinline__ int Tri(int i, int j) { return i * (i + 1) / 2 + j; }

__global__ void ColSumKernel(int M, int N, const float* A, int64_t lda, float* out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += A[int64_t(m) * lda + n];
  out[n] = s;
}

__global__ void HeadKernel(int n, const float* z, const float* samples, int64_t lds, float scale,
                           float kaporin, float* dz, float* loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int kB = kPrecondBlock;
  const float* zi = z + int64_t(i) * kPrecondTri;
  const float* gh = samples + int64_t(i) * lds + kPrecondFeatures;
  const float* xh = gh + kB;
  float L[kPrecondTri], sig[kB];
#pragma unroll
  for (int r = 0; r < kB; ++r)
#pragma unroll
    for (int c = 0; c <= r; ++c) {
      const float zz = zi[Tri(r, c)];
      if (r == c) {
        const float x = zz + kDiagShift;
        L[Tri(r, r)] = x > 20.f ? x : log1pf(expf(x));
        sig[r] = 1.f / (1.f + expf(-x));
      } else {
        L[Tri(r, c)] = zz;
      }
    }
  // t = L^T g_hat, u = L t - x_hat
  float t[kB], u[kB], g[kB];
#pragma unroll
  for (int r = 0; r < kB; ++r) g[r] = gh[r];
#pragma unroll
  for (int c = 0; c < kB; ++c) {
    float s = 0.f;
#pragma unroll
    for (int r = c; r < kB; ++r) s += L[Tri(r, c)] * g[r];
    t[c] = s;
  }
  float xx = 0.f, uu = 0.f;
#pragma unroll
  for (int r = 0; r < kB; ++r) {
    float s = 0.f;
#pragma unroll
    for (int c = 0; c <= r; ++c) s += L[Tri(r, c)] * t[c];
    u[r] = s - xh[r];
    xx += xh[r] * xh[r];
    uu += u[r] * u[r];
  }
  const float inv = 1.f / (xx + 1e-30f);
  // Kaporin term kaporin * (tr(L L^T) - log det(L L^T) - 9) / 9
  float tr = 0.f, ld = 0.f;
#pragma unroll
  for (int r = 0; r < kB; ++r) {
#pragma unroll
    for (int c = 0; c <= r; ++c) tr += L[Tri(r, c)] * L[Tri(r, c)];
    ld += logf(L[Tri(r, r)]);
  }
  loss[i] = uu * inv + kaporin * (tr - 2.f * ld - float(kB)) * (1.f / kB);
  const float kf = 2.f * kaporin * (1.f / kB) * scale;
  // d loss / d L = (G + G^T) L with G = 2 u g^T / s, lower triangle, plus the Kaporin term's
  // 2 L - 2 diag(1 / L_rr), scaled
  const float f = 2.f * inv * scale;
  float* dzi = dz + int64_t(i) * kPrecondTri;
#pragma unroll
  for (int r = 0; r < kB; ++r)
#pragma unroll
    for (int c = 0; c <= r; ++c) {
      float s = 0.f;
#pragma unroll
      for (int k = c; k < kB; ++k) s += (u[r] * g[k] + g[r] * u[k]) * L[Tri(k, c)];
      s *= f;
      const float lrc = L[Tri(r, c)];
      s += kf * (r == c ? lrc - 1.f / lrc : lrc);
      dzi[Tri(r, c)] = r == c ? s * sig[r] : s;
    }
}

__global__ void SumKernel(int n, const float* loss, float scale, double* out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += double(loss[i]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = double(scale) * red[0];
}

__global__ void GatherKernel(int n, const float* samples, const int32_t* idx, float* rows) {
  const int64_t total = int64_t(n) * kSampleFloats;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / kSampleFloats, c = e - r * kSampleFloats;
    rows[e] = samples[int64_t(idx[r]) * kSampleFloats + c];
  }
}

__global__ void AdamKernel(int64_t n, float* w, const float* g, float* m, float* v, float lr,
                           float beta1, float beta2, float eps, float c1, float c2) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace

void LaunchColSum(int M, int N, const float* A, int64_t lda, float* out, cudaStream_t s) {
  const int threads = 128;
  ColSumKernel<<<(N + threads - 1) / threads, threads, 0, s>>>(M, N, A, lda, out);
}

void LaunchHead(int n, const float* z, const float* samples, int64_t lds, float scale, float kaporin,
                float* dz, float* loss, double* loss_sum, cudaStream_t s) {
  const int threads = 128;
  HeadKernel<<<(n + threads - 1) / threads, threads, 0, s>>>(n, z, samples, lds, scale, kaporin, dz,
                                                             loss);
  SumKernel<<<1, 256, 0, s>>>(n, loss, scale, loss_sum);
}

void LaunchGather(int n, const float* samples, const int32_t* idx, float* rows, cudaStream_t s) {
  const int threads = 256;
  const int64_t total = int64_t(n) * kSampleFloats;
  const int grid = int(std::min<int64_t>((total + threads - 1) / threads, 4096));
  GatherKernel<<<std::max(grid, 1), threads, 0, s>>>(n, samples, idx, rows);
}

void LaunchAdam(int64_t n, float* w, const float* g, float* m, float* v, float lr, float beta1,
                float beta2, float eps, float c1, float c2, cudaStream_t s) {
  const int threads = 256;
  const int grid = int(std::min<int64_t>((n + threads - 1) / threads, 1024));
  AdamKernel<<<grid, threads, 0, s>>>(n, w, g, m, v, lr, beta1, beta2, eps, c1, c2);
}

}  // namespace sfg
