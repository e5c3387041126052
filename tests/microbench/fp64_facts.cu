// GB300 FP64 facts behind the factorization's design (tests/test_gpu_microbench.py runs this):
//  1. dependent-chain latencies of FP64 primitives on one warp and on four (inline PTX, volatile);
//  2. FP64 issue: one warp's limit, and the SM's, with warps placed on chosen sub-partitions;
//  3. accuracy of rcp.approx.ftz.f64 and of the Newton-Raphson refinements against 1.0 / x;
//  4. whole-GPU FMA throughput, FP64 and FP32 (8 CTAs of 256 threads per SM, 8 chains a thread).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#define N 256
__global__ void Lat(double* out, long long* cyc, double a) {
  double x = a + 1e-3 * threadIdx.x;
  float f;
  long long t[16];
  int k = 0;
  t[k++] = clock64();
  for (int s = 0; s < N; ++s) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x) : "d"(1.0000001), "d"(1e-9));
  t[k++] = clock64();
  for (int s = 0; s < N; ++s) { asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(x)); asm volatile("cvt.f64.f32 %0, %1;" : "=d"(x) : "f"(f)); }
  t[k++] = clock64();
  for (int s = 0; s < N; ++s) { asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(x)); asm volatile("rcp.approx.ftz.f32 %0, %0;" : "+f"(f)); asm volatile("rcp.approx.ftz.f32 %0, %0;" : "+f"(f)); asm volatile("cvt.f64.f32 %0, %1;" : "=d"(x) : "f"(f)); }
  t[k++] = clock64();
  for (int s = 0; s < N; ++s) { asm volatile("rcp.approx.ftz.f64 %0, %0;" : "+d"(x)); asm volatile("rcp.approx.ftz.f64 %0, %0;" : "+d"(x)); }
  t[k++] = clock64();
  for (int s = 0; s < N; ++s) { asm volatile("div.rn.f64 %0, %1, %0;" : "+d"(x) : "d"(1.5)); }
  t[k++] = clock64();
  for (int s = 0; s < N; ++s) { asm volatile("mul.rn.f64 %0, %0, %1;" : "+d"(x) : "d"(1.0000001)); }
  t[k++] = clock64();
  // a pivot-reciprocal variant: fp32 seed + 2 Newton (4 fma) then feeds back
  for (int s = 0; s < N; ++s) {
    double y, e;
    asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(x));
    asm volatile("rcp.approx.ftz.f32 %0, %0;" : "+f"(f));
    asm volatile("cvt.f64.f32 %0, %1;" : "=d"(y) : "f"(f));
    asm volatile("fma.rn.f64 %0, %1, %2, %3;" : "=d"(e) : "d"(-x), "d"(y), "d"(1.0));
    asm volatile("fma.rn.f64 %0, %1, %2, %1;" : "=d"(y) : "d"(y), "d"(e));
    asm volatile("fma.rn.f64 %0, %1, %2, %3;" : "=d"(e) : "d"(-x), "d"(y), "d"(1.0));
    asm volatile("fma.rn.f64 %0, %1, %2, %1;" : "=d"(y) : "d"(y), "d"(e));
    x = 1.5 + 1e-12 * y;
  }
  t[k++] = clock64();
  // integer seed (exponent flip, ~4 bits) is not measured; shfl.sync f64 (two 32-bit halves)
  for (int s = 0; s < N; ++s) x = __shfl_sync(0xffffffffu, x, (threadIdx.x + 1) & 31);
  t[k++] = clock64();
  __shared__ double sh[128];
  for (int s = 0; s < N; ++s) { sh[threadIdx.x] = x; __syncthreads(); x = sh[(threadIdx.x + 3) & 127]; }
  t[k++] = clock64();
  if (threadIdx.x == 0) for (int i = 0; i + 1 < k; ++i) cyc[i] = t[i + 1] - t[i];
  out[threadIdx.x] = x;
}


__global__ void K(unsigned mask, int iters, double* out, long long* cyc) {
  const int w = threadIdx.x >> 5;
  double x = 1.0 + threadIdx.x * 1e-9, y = 0.999999, z = 1e-7;
  __syncthreads();
  long long t0 = clock64();
  if ((mask >> w) & 1) {
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x) : "d"(y), "d"(z));
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x) : "d"(y), "d"(z));
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x) : "d"(y), "d"(z));
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x) : "d"(y), "d"(z));
    }
  }
  long long t1 = clock64();
  __syncthreads();
  out[blockIdx.x * blockDim.x + threadIdx.x] = x;
  if ((threadIdx.x & 31) == 0) cyc[blockIdx.x * 16 + w] = ((mask >> w) & 1) ? (t1 - t0) : 0;
}
// independent chains per warp: ILP 4
__global__ void K4(unsigned mask, int iters, double* out, long long* cyc) {
  const int w = threadIdx.x >> 5;
  double a = 1.0 + threadIdx.x * 1e-9, b = a + 1e-3, c = a + 2e-3, d = a + 3e-3, y = 0.999999, z = 1e-7;
  __syncthreads();
  long long t0 = clock64();
  if ((mask >> w) & 1) {
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(a) : "d"(y), "d"(z));
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(b) : "d"(y), "d"(z));
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(c) : "d"(y), "d"(z));
      asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(d) : "d"(y), "d"(z));
    }
  }
  long long t1 = clock64();
  __syncthreads();
  out[blockIdx.x * blockDim.x + threadIdx.x] = a + b + c + d;
  if ((threadIdx.x & 31) == 0) cyc[blockIdx.x * 16 + w] = ((mask >> w) & 1) ? (t1 - t0) : 0;
}


__global__ void RcpErr(int n, uint64_t seed, double* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t s = seed + 0x9E3779B97F4A7C15ull * (i + 1);
  s ^= s >> 33; s *= 0xff51afd7ed558ccdull; s ^= s >> 33; s *= 0xc4ceb9fe1a85ec53ull; s ^= s >> 33;
  double m = 1.0 + double(s >> 11) * (1.0 / 9007199254740992.0);   // [1, 2)
  int ex = int((s >> 3) & 127) - 64;
  double x = ldexp(m, ex);
  double y; asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double q = 1.0 / x;
  double e0 = fabs(y - q) / q;
  double e = fma(-x, y, 1.0);
  double yc = fma(y, fma(e, e, e), y);          // cubic step
  double y1 = fma(y, e, y); double e1 = fma(-x, y1, 1.0); double y2 = fma(y1, e1, y1);  // two Newton steps
  out[4 * i + 0] = e0;
  out[4 * i + 1] = fabs(yc - q) / q;
  out[4 * i + 2] = fabs(y2 - q) / q;
  out[4 * i + 3] = (yc == q) ? 0.0 : 1.0;
}


template <typename T>
__global__ void Throughput(int iters, T* out) {
  T a[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) a[c] = T(1) + T(1e-3) * T(threadIdx.x + c);
  const T y = T(0.9999999), z = T(1e-7);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = fma(a[c], y, z);
  T s = T(0);
#pragma unroll
  for (int c = 0; c < 8; ++c) s += a[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <typename T>
double Tflops(int sms, int iters) {
  const int grid = sms * 8, threads = 256;
  T* out; cudaMalloc(&out, sizeof(T) * size_t(grid) * threads);
  Throughput<T><<<grid, threads>>>(iters, out);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  cudaEventRecord(e0);
  Throughput<T><<<grid, threads>>>(iters, out);
  cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms = 0; cudaEventElapsedTime(&ms, e0, e1);
  cudaFree(out);
  return 2.0 * 8 * double(iters) * grid * threads / (ms * 1e-3) / 1e12;
}
int main() {
  int ok = 1;
  {
    double* out; long long* cyc; cudaMalloc(&out, 1024 * 8); cudaMalloc(&cyc, 64 * 8);
    long long h[16];
    const char* names[] = {"fma.f64", "cvt f64->f32->f64 (pair)", "cvt + 2x rcp.f32 + cvt", "2x rcp.approx.f64",
                           "div.rn.f64", "mul.f64", "pivot recip (seed+4fma)+fma", "shfl f64", "smem st+bar+ld"};
    for (int threads : {32, 128})
      for (int rep = 0; rep < 2; ++rep) {
        Lat<<<1, threads>>>(out, cyc, 1.5);
        cudaMemcpy(h, cyc, 9 * 8, cudaMemcpyDeviceToHost);
        if (rep) for (int i = 0; i < 9; ++i) printf("latency %3d thr %-30s %7.1f cycles/step\n", threads, names[i], h[i] / double(N));
      }
    cudaFree(out); cudaFree(cyc);
  }
  {
    double* out; long long* cyc; long long h[16];
    cudaMalloc(&out, sizeof(double) * 512); cudaMalloc(&cyc, sizeof(long long) * 16);
    const int iters = 2000;
    struct { unsigned mask; const char* what; } cases[] = {
      {0x1, "1 warp"}, {0x3, "2 warps, 2 sub-partitions"}, {0x11, "2 warps, 1 sub-partition"},
      {0xF, "4 warps, 4 sub-partitions"}, {0x1111, "4 warps, 1 sub-partition"},
      {0xFF, "8 warps, 2 per sub-partition"}, {0xFFFF, "16 warps, 4 per sub-partition"}};
    for (int kind = 0; kind < 2; ++kind)
      for (auto& cs : cases) {
        if (kind == 0) K<<<1, 512>>>(cs.mask, iters, out, cyc); else K4<<<1, 512>>>(cs.mask, iters, out, cyc);
        cudaMemcpy(h, cyc, sizeof(h), cudaMemcpyDeviceToHost);
        long long mx = 0; for (int w = 0; w < 16; ++w) mx = h[w] > mx ? h[w] : mx;
        printf("issue %s %-32s %6.1f cycles per warp-instruction step\n", kind ? "ILP4 " : "chain", cs.what, double(mx) / (4.0 * iters));
      }
    cudaFree(out); cudaFree(cyc);
  }
  {
    const int n = 1 << 22;
    double* d; cudaMalloc(&d, sizeof(double) * 4 * n);
    double* h = new double[4 * size_t(n)];
    double mx[4] = {0, 0, 0, 0}; double neq = 0;
    for (int rep = 0; rep < 4; ++rep) {
      RcpErr<<<n / 256, 256>>>(n, 1234 + rep, d);
      cudaMemcpy(h, d, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost);
      for (int i = 0; i < n; ++i) { for (int k = 0; k < 3; ++k) mx[k] = fmax(mx[k], h[4 * i + k]); neq += h[4 * i + 3]; }
    }
    printf("rcp.approx.ftz.f64 max rel err %.3e (2^%.1f)\n", mx[0], log2(mx[0]));
    printf("cubic step max rel err %.3e, differs from 1/x in %.0f of %d\n", mx[1], neq, 4 * n);
    printf("two Newton steps max rel err %.3e\n", mx[2]);
    delete[] h; cudaFree(d);
  }
  {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    printf("throughput FP64 %.3f TFLOP/s\n", Tflops<double>(sms, 4000));
    printf("throughput FP32 %.3f TFLOP/s\n", Tflops<float>(sms, 40000));
  }
  cudaError_t e = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(e));
  return e == cudaSuccess && ok ? 0 : 1;
}
