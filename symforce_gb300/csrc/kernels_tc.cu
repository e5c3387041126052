// Tensor-core (tcgen05, TF32) GEMM of the preconditioner network, inference and training:
// out[M x N] = epilogue(A[M x K] B[K x N]) with strided operands (element (m, k) of A at
// A[m a_rs + k a_cs], element (k, n) of B at B[k b_rs + n b_cs]) and the epilogues none, + bias,
// ReLU(+ bias), or a ReLU mask (out = mask[m][n] > 0 ? v : 0).
//
//  - One CTA of 128 threads per 128-row x NP-column tile (NP = 128 for the hidden layers, 48 for the
//    45 outputs); the accumulator lives in tensor memory (TMEM, 128 lanes x NP FP32 columns,
//    allocated per CTA).
//  - K is consumed in chunks of 32: the threads stage the A and W chunks in shared memory in the
//    canonical K-major layout without swizzle (8-row x 16-byte core matrices; leading byte offset
//    = next core matrix along K, stride byte offset = next 8-row group), one elected thread issues
//    the MMAs (M = 128, N = NP, K = 8 each) and commits them to an mbarrier that the CTA waits on
//    before restaging.
//  - FP32 accuracy on the TF32 tensor pipe by the three-pass split x = hi + lo (hi: the top 11
//    significand bits, lo = x - hi): A W ~ A_hi W_hi + A_hi W_lo + A_lo W_hi, relative error ~2^-20.
//  - Epilogue: tcgen05.ld of 16 columns at a time (warp w reads TMEM lanes 32 w .. 32 w + 31, one row
//    per thread), bias, ReLU, store.
//  - Every mbarrier wait is capped; a cap hit sets the error word, and the CTA still waits (capped)
//    for its MMAs and frees its TMEM before returning.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"
#include "tc_common.cuh"

namespace sfg {

namespace {

constexpr int kTcThreads = 128;
using namespace tc;

struct TcArgs {
  const float* A;
  int64_t a_rs, a_cs;
  const float* B;
  int64_t b_rs, b_cs;
  int M, N, K;
  float* out;
  int64_t ldo;
  int epi;
  const float* bias;
  const float* mask;
  int64_t ldmask;
  int vec4;  // A rows are 16-byte aligned with unit column stride: 16-byte loads
  int* err;
};

template <int NP>
__global__ void __launch_bounds__(kTcThreads) TcGemmKernel(TcArgs g) {
  const float* A = g.A;
  const int M = g.M, K = g.K, N = g.N;
  static_assert(NP % 16 == 0 && NP >= 16 && NP <= 256, "N of a kind::tf32 MMA with M = 128");
  constexpr int kCols = NP <= 32 ? 32 : NP <= 64 ? 64 : NP <= 128 ? 128 : 256;  // TMEM columns
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  unsigned char* a_hi = tc_smem;
  unsigned char* a_lo = a_hi + kTcRows * kTcKc * 4;
  unsigned char* b_hi = a_lo + kTcRows * kTcKc * 4;
  unsigned char* b_lo = b_hi + NP * kTcKc * 4;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kTcRows;
  const int n0 = blockIdx.y * NP;  // this CTA's columns n0 .. n0 + NP of the output

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(&tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    MbarInit(&bar);
    s_fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t d_tmem = tmem_base;
  const uint32_t idesc = InstrDesc(NP);

  // Software pipeline over the K chunks: the global loads of chunk c + 1 go out (into registers)
  // while the MMAs of chunk c run; the registers are written to shared memory once those MMAs have
  // released it.
  constexpr int kAPer = kTcRows * (kTcKc / 4) / kTcThreads;  // 8 float4 per thread
  constexpr int kBPer = (NP + kTcThreads - 1) / kTcThreads;
  float4 av[kAPer];
  float bv[kBPer][kTcKc];
  auto load_chunk = [&](int k0) {
    // A: four consecutive k of one row per thread and step (eight threads cover a row's 32 k), so
    // a warp reads four full 128-byte rows per load
#pragma unroll
    for (int i = 0; i < kAPer; ++i) {
      const int idx = tid + i * kTcThreads;
      const int r = idx >> 3, k4 = (idx & 7) * 4, gr = row0 + r, gk = k0 + k4;
      if (g.vec4 && gr < M && gk + 3 < K) {
        av[i] = __ldg(reinterpret_cast<const float4*>(A + int64_t(gr) * g.a_rs + gk));
      } else {
        const float* ap = A + int64_t(gr) * g.a_rs + int64_t(gk) * g.a_cs;
        av[i].x = (gr < M && gk < K) ? __ldg(ap) : 0.f;
        av[i].y = (gr < M && gk + 1 < K) ? __ldg(ap + g.a_cs) : 0.f;
        av[i].z = (gr < M && gk + 2 < K) ? __ldg(ap + 2 * g.a_cs) : 0.f;
        av[i].w = (gr < M && gk + 3 < K) ? __ldg(ap + 3 * g.a_cs) : 0.f;
      }
    }
    // B^T: row n of the operand is column n0 + n of B (consecutive threads, consecutive n)
#pragma unroll
    for (int j = 0; j < kBPer; ++j) {
      const int n = tid + j * kTcThreads, gn = n0 + n;
#pragma unroll
      for (int k = 0; k < kTcKc; ++k) {
        const int gk = k0 + k;
        bv[j][k] = (n < NP && gn < N && gk < K) ? __ldg(g.B + int64_t(gk) * g.b_rs + int64_t(gn) * g.b_cs) : 0.f;
      }
    }
  };
  auto store_chunk = [&]() {
#pragma unroll
    for (int i = 0; i < kAPer; ++i) {
      const int idx = tid + i * kTcThreads;
      const int r = idx >> 3, k4 = (idx & 7) * 4;
      float4 hi4, lo4;
      hi4.x = TfHi(av[i].x);
      hi4.y = TfHi(av[i].y);
      hi4.z = TfHi(av[i].z);
      hi4.w = TfHi(av[i].w);
      lo4.x = av[i].x - hi4.x;
      lo4.y = av[i].y - hi4.y;
      lo4.z = av[i].z - hi4.z;
      lo4.w = av[i].w - hi4.w;
      const uint32_t o = ChunkOffset(r, k4);
      *reinterpret_cast<float4*>(a_hi + o) = hi4;
      *reinterpret_cast<float4*>(a_lo + o) = lo4;
    }
#pragma unroll
    for (int j = 0; j < kBPer; ++j) {
      const int n = tid + j * kTcThreads;
      if (n >= NP) continue;
#pragma unroll
      for (int k4 = 0; k4 < kTcKc; k4 += 4) {
        float4 hi4, lo4;
        hi4.x = TfHi(bv[j][k4]);
        hi4.y = TfHi(bv[j][k4 + 1]);
        hi4.z = TfHi(bv[j][k4 + 2]);
        hi4.w = TfHi(bv[j][k4 + 3]);
        lo4.x = bv[j][k4] - hi4.x;
        lo4.y = bv[j][k4 + 1] - hi4.y;
        lo4.z = bv[j][k4 + 2] - hi4.z;
        lo4.w = bv[j][k4 + 3] - hi4.w;
        const uint32_t o = ChunkOffset(n, k4);
        *reinterpret_cast<float4*>(b_hi + o) = hi4;
        *reinterpret_cast<float4*>(b_lo + o) = lo4;
      }
    }
  };

  uint32_t phase = 0;
  bool issued = false;
  if (K > 0) load_chunk(0);
  for (int k0 = 0; k0 < K; k0 += kTcKc) {
    if (issued) {
      // the MMAs of the previous chunk must have read shared memory before it is restaged
      if (!MbarWait(&bar, phase)) {
        if (lane == 0) atomicExch(g.err, kDevSpinTimeout);
        s_fail = 1;
      }
      phase ^= 1u;
      __syncthreads();
      if (s_fail) break;
    }
    store_chunk();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int j = 0; j < kTcKc / 8; ++j) {  // K = 8 per MMA: two core matrices along K
        const uint32_t off = uint32_t(j * 256);
        const uint32_t acc0 = (k0 > 0 || j > 0) ? 1u : 0u;
        MmaTf32(d_tmem, SmemDesc(SmemAddr(a_hi) + off), SmemDesc(SmemAddr(b_hi) + off), idesc, acc0);
        MmaTf32(d_tmem, SmemDesc(SmemAddr(a_hi) + off), SmemDesc(SmemAddr(b_lo) + off), idesc, 1u);
        MmaTf32(d_tmem, SmemDesc(SmemAddr(a_lo) + off), SmemDesc(SmemAddr(b_hi) + off), idesc, 1u);
      }
      MmaCommit(&bar);
    }
    issued = true;
    if (k0 + kTcKc < K) load_chunk(k0 + kTcKc);  // overlaps the MMAs just issued
  }
  // the last chunk's MMAs complete the accumulator
  if (issued && !s_fail) {
    if (!MbarWait(&bar, phase)) {
      if (lane == 0) atomicExch(g.err, kDevSpinTimeout);
      s_fail = 1;
    }
    phase ^= 1u;
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (issued && !s_fail) {
    // epilogue: row tid of the tile, 16 columns per TMEM load
    const int gr = row0 + tid;
#pragma unroll 1
    for (int c0 = 0; c0 < NP; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = d_tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (gr < M) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = n0 + c0 + i;
          if (c < N) {
            float y = __uint_as_float(v[i]);
            if (g.epi == kEpiBias || g.epi == kEpiBiasRelu) y += g.bias[c];
            if (g.epi == kEpiBiasRelu) y = fmaxf(y, 0.f);
            if (g.epi == kEpiMask && !(g.mask[int64_t(gr) * g.ldmask + c] > 0.f)) y = 0.f;
            g.out[int64_t(gr) * g.ldo + c] = y;
          }
        }
      }
    }
  } else if (issued) {
    // a wait gave up: give the MMAs a second (capped) chance to finish before the TMEM is freed
    (void)MbarWait(&bar, phase ^ 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(d_tmem), "r"(kCols) : "memory");
}

template <int NP>
size_t TcSmem() {
  return size_t(kTcRows) * kTcKc * 4 * 2 + size_t(NP) * kTcKc * 4 * 2;
}

template <int NP>
cudaError_t LaunchTc(TcArgs g, cudaStream_t s) {
  const size_t smem = TcSmem<NP>();
  const cudaError_t e = cudaFuncSetAttribute(TcGemmKernel<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return e;
  g.vec4 = (g.a_cs == 1 && g.a_rs % 4 == 0 && (reinterpret_cast<uintptr_t>(g.A) & 15) == 0) ? 1 : 0;
  const dim3 grid((g.M + kTcRows - 1) / kTcRows, (g.N + NP - 1) / NP);
  TcGemmKernel<NP><<<grid, kTcThreads, smem, s>>>(g);
  return cudaGetLastError();
}

}  // namespace

cudaError_t LaunchGemmTc(int M, int N, int K, const float* A, int64_t a_rs, int64_t a_cs, const float* B,
                         int64_t b_rs, int64_t b_cs, float* C, int64_t ldc, int epilogue, const float* bias,
                         const float* mask, int64_t ldmask, int* err, cudaStream_t s) {
  if (M == 0 || N == 0) return cudaSuccess;
  TcArgs g{A, a_rs, a_cs, B, b_rs, b_cs, M, N, K, C, ldc, epilogue, bias, mask, ldmask, 0, err};
  // 48 columns for the 45 outputs, otherwise tiles of 128 columns
  return N <= 48 ? LaunchTc<48>(g, s) : LaunchTc<128>(g, s);
}

cudaError_t LaunchMlpInferTc(const float* x, int64_t ldx, int64_t n, const float* weights, float* h1, float* h2,
                             float* z, int* err, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int F = kPrecondFeatures, H = kPrecondHidden, O = kPrecondTri;
  const float* W1 = weights;
  const float* b1 = W1 + F * H;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + H * O;
  const int m = int(n);
  cudaError_t e = LaunchGemmTc(m, H, F, x, ldx, 1, W1, H, 1, h1, H, kEpiBiasRelu, b1, nullptr, 0, err, s);
  if (e != cudaSuccess) return e;
  e = LaunchGemmTc(m, H, H, h1, H, 1, W2, H, 1, h2, H, kEpiBiasRelu, b2, nullptr, 0, err, s);
  if (e != cudaSuccess) return e;
  return LaunchGemmTc(m, O, H, h2, H, 1, W3, O, 1, z, O, kEpiBias, b3, nullptr, 0, err, s);
}

}  // namespace sfg
