// Linear solve of the damped Gauss-Newton system on the device.
//
//  - Schur complement over the trailing 3x3 point blocks (the SparseSchurSolver math,
//    symforce/opt/sparse_schur_solver.tcc:99-162): per point C^-1 (LL^T), W = C^-1 E, the
//    reduced system S = B - E^T W accumulated per S block in a fixed order, the reduced rhs, and
//    the point back-substitution.
//  - Multifrontal LDL^T (unit L, diagonal D, no pivoting: the factorization the reference computes
//    with its up-looking SparseCholeskySolver, symforce/opt/sparse_cholesky/
//    sparse_cholesky_solver.tcc:108-219) over a host-computed supernodal structure.  One
//    persistent kernel executes a topologically ordered list of tile tasks (front assembly,
//    diagonal-tile LDL^T, panel triangular solve, trailing update); dependencies are tile version
//    counters in global memory.  A CTA only waits on tasks that precede its own in the list, all
//    of which are held by running CTAs, so progress is guaranteed; every wait is capped and a cap
//    hit sets the error word and drains the kernel.
//  - The triangular solves, one task per front, forward in postorder and backward in reverse.
#include "factor_math.cuh"
#include <algorithm>

#include "kernels.h"
#include "tc_common.cuh"

namespace sfg {

namespace {

constexpr int kFactorThreads = 128;
// Tile entries each thread of a factorization CTA owns (entry e = threadIdx.x + n * kFactorThreads):
// a compile-time count, so that per-thread arrays over them stay in registers.
template <int TILE>
__host__ __device__ constexpr int TileEntriesPerThread() {
  static_assert(TILE * TILE % kFactorThreads == 0, "tiles split evenly over the CTA");
  return TILE * TILE / kFactorThreads;
}
constexpr unsigned kSpinLimit = 1u << 22;
constexpr int kFinal = 1 << 30;

__device__ __forceinline__ int LoadVolatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Thread 0 only.  Returns false if the wait gave up (error set by us or by another CTA).
__device__ bool WaitAtLeast(const int* addr, int v, int* err) {
  unsigned it = 0;
  while (LoadVolatile(addr) < v) {
    if (LoadVolatile(err) != 0) return false;
    if (++it > kSpinLimit) {
      atomicExch(err, kDevSpinTimeout);
      return false;
    }
    if (it > 64) __nanosleep(64);  // poll tightly first: most waits end within a few microseconds
  }
  __threadfence();
  return true;
}

__device__ __forceinline__ unsigned long long Clock64Global() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned SmId() {
  unsigned r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

template <typename T>
__device__ __forceinline__ T Ld(const T* p) { return __ldcg(p); }
template <typename T>
__device__ __forceinline__ void St(T* p, T v) { __stcg(p, v); }

// ---------------------------------------------------------------------------------------------
// Schur complement kernels
// ---------------------------------------------------------------------------------------------
// G = L^-1 E for one 3 x DK block E (row-major), li = L^-1 lower (00, 10, 11, 20, 21, 22) with
// C = L L^T: then E_k^T C^-1 E_l = G_k^T G_l, so the S terms read one array for both operands.
template <typename T, int DK>
__device__ __forceinline__ void PointG(const T* E, T* Gp, const T (&li)[6]) {
  T e[3 * DK];
#pragma unroll
  for (int i = 0; i < 3 * DK; ++i) e[i] = E[i];
#pragma unroll
  for (int c = 0; c < DK; ++c) {
    const T e0 = e[c], e1 = e[DK + c], e2 = e[2 * DK + c];
    Gp[c] = li[0] * e0;
    Gp[DK + c] = li[1] * e0 + li[2] * e1;
    Gp[2 * DK + c] = li[3] * e0 + li[4] * e1 + li[5] * e2;
  }
}
template <typename T>
__device__ __forceinline__ void PointGAny(const T* E, T* Gp, int dk, const T (&li)[6]) {
  for (int c = 0; c < dk; ++c) {
    const T e0 = E[c], e1 = E[dk + c], e2 = E[2 * dk + c];
    Gp[c] = li[0] * e0;
    Gp[dk + c] = li[1] * e0 + li[2] * e1;
    Gp[2 * dk + c] = li[3] * e0 + li[4] * e1 + li[5] * e2;
  }
}

// One thread per point: the Cholesky factor L of the damped 3 x 3 block, its inverse (kept) and
// t = C^-1 g.
template <typename T>
__global__ void SchurPointsKernel(SchurDev d, const T* hess_all, const T* rhs_all, int64_t nvals,
                                  int64_t N, const double* damping, T* cinv, T* tp,
                                  const LmState* st) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.npoints) return;
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const T* g = rhs_all + int64_t(st->init_idx) * N;
  const T* C = H + d.pt_diag[p];
  const int64_t toff = d.c_toff + 3 * int64_t(p);
  const T a00 = C[0] + T(damping[toff]);
  const T a10 = C[3];
  const T a11 = C[4] + T(damping[toff + 1]);
  const T a20 = C[6];
  const T a21 = C[7];
  const T a22 = C[8] + T(damping[toff + 2]);
  const T l00 = sqrt(a00);
  const T l10 = a10 / l00, l20 = a20 / l00;
  const T l11 = sqrt(a11 - l10 * l10);
  const T l21 = (a21 - l20 * l10) / l11;
  const T l22 = sqrt(a22 - l20 * l20 - l21 * l21);
  const T i00 = T(1) / l00, i11 = T(1) / l11, i22 = T(1) / l22;
  const T i10 = -l10 * i00 * i11;
  const T i21 = -l21 * i11 * i22;
  const T i20 = -(l20 * i00 + l21 * i10) * i22;
  const T c00 = i00 * i00 + i10 * i10 + i20 * i20;
  const T c10 = i11 * i10 + i21 * i20;
  const T c20 = i22 * i20;
  const T c11 = i11 * i11 + i21 * i21;
  const T c21 = i22 * i21;
  const T c22 = i22 * i22;
  T* ci = cinv + 9 * int64_t(p);  // L^-1 (C = L L^T), lower, row-major packed
  ci[0] = i00;
  ci[1] = i10; ci[2] = i11;
  ci[3] = i20; ci[4] = i21; ci[5] = i22;
  const T g0 = g[toff], g1 = g[toff + 1], g2 = g[toff + 2];
  T* t = tp + 3 * int64_t(p);
  t[0] = c00 * g0 + c10 * g1 + c20 * g2;
  t[1] = c10 * g0 + c11 * g1 + c21 * g2;
  t[2] = c20 * g0 + c21 * g1 + c22 * g2;
}

// One thread per E block: G = L^-1 E into the G buffer (at E's offset or point-major, as the layout
// chose), the block's loads all issued before its stores; the blocks are taken in the order of
// their G offsets (e_order), so that neighbouring threads write neighbouring addresses.
template <typename T>
__global__ void SchurWKernel(SchurDev d, const T* hess_all, int64_t nvals, const T* cinv, T* W,
                             const LmState* st) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= d.nE) return;
  const int64_t e = d.e_order ? d.e_order[q] : q;
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const T* ci = cinv + 9 * int64_t(d.pt_of_e[e]);
  const T li[6] = {ci[0], ci[1], ci[2], ci[3], ci[4], ci[5]};
  const int dk = d.pt_ekey_dim[e];
  const T* E = H + d.pt_eoff[e];
  T* Gp = W + d.pt_woff[e];
  if (dk == 6) PointG<T, 6>(E, Gp, li);
  else if (dk == 3) PointG<T, 3>(E, Gp, li);
  else PointGAny<T>(E, Gp, dk, li);
}

// S = B - sum_p G_pk^T G_pl over the S blocks' terms (points seen by both keys), G = L_p^-1 E (the
// G buffer; E_pk^T C_p^-1 E_pl = G_pk^T G_pl with C_p = L_p L_p^T), in two passes.
// Pass 1: one warp per chunk of at most chunk_terms terms of one block; each lane takes the
// chunk's terms in turn and accumulates the whole d_k x d_l product of its terms in registers (every
// G block is read once; a diagonal block only its lower triangle), then a butterfly
// reduce-scatter adds the lanes.  Pass 2: one warp per S block adds its chunks in order and writes
// B_kl (+ damping) - sum.  Chunks spread the heavy diagonal blocks (every observation of a camera)
// over many warps, which the FP64 pipe needs; the fixed orders make every run give the same bits.
// Key tangent dims are at most kMaxKeyDim.
constexpr int kMaxKeyDim = 6;
constexpr int kSchurWarps = 4;

// One exchange level of a butterfly reduce-scatter over the warp: the N values of v (entries
// [base, base + cnt) of the original order, the rest zero padding) are halved; lanes with bit O
// clear keep the lower ceil(N/2), the others the upper part, each adding its partner's copy of the
// half it keeps.  Five levels (O = 16 .. 1) leave every value summed over the 32 lanes in exactly
// one lane, for N/2 + N/4 + ... FP64 adds a lane instead of the 5 N of a shuffle tree per value.
template <typename T, int N, int O>
__device__ __forceinline__ void ReduceScatterLevel(T* v, int lane, int& base, int& cnt) {
  constexpr int H = (N + 1) / 2;
  const bool up = (lane & O) != 0;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const T lo = v[i];
    const T hi = H + i < N ? v[H + i] : T(0);
    const T send = up ? lo : hi;
    const T keep = up ? hi : lo;
    v[i] = keep + __shfl_xor_sync(0xffffffffu, send, O);
  }
  if (up) {
    base += H;
    cnt = cnt > H ? cnt - H : 0;
  } else {
    cnt = cnt < H ? cnt : H;
  }
  if constexpr (O > 1) ReduceScatterLevel<T, H, O / 2>(v, lane, base, cnt);
}
// Values a lane holds after the five levels for N inputs.
template <int N>
__host__ __device__ constexpr int ReduceScatterSlots() {
  int n = N;
  for (int l = 0; l < 5; ++l) n = (n + 1) / 2;
  return n;
}

// The products of one chunk for a block of DK x DL (compile-time sizes: only the block's entries are
// accumulated, which matters on the FP64 pipe), written as a 6 x 6 row-major partial.
template <typename T, int DK, int DL>
__device__ __forceinline__ void ChunkTerms(const SchurDev& d, const T* H, const T* W, int64_t t0,
                                           int64_t t1, int lane, T* out) {
  constexpr int N = DK * DL;
  T acc[N];
#pragma unroll
  for (int i = 0; i < N; ++i) acc[i] = T(0);
  for (int64_t t = t0 + lane; t < t1; t += 32) {
    const T* E = W + d.sb_eoff[t];
    const T* Wl = W + d.sb_woff[t];
    T e[3 * DK], w[3 * DL];
#pragma unroll
    for (int i = 0; i < 3 * DK; ++i) e[i] = E[i];
#pragma unroll
    for (int i = 0; i < 3 * DL; ++i) w[i] = Wl[i];
#pragma unroll
    for (int r = 0; r < DK; ++r)
#pragma unroll
      for (int c = 0; c < DL; ++c)
        acc[r * DL + c] += e[r] * w[c] + e[DK + r] * w[DL + c] + e[2 * DK + r] * w[2 * DL + c];
  }
  int base = 0, cnt = N;
  ReduceScatterLevel<T, N, 16>(acc, lane, base, cnt);
#pragma unroll
  for (int i = 0; i < ReduceScatterSlots<N>(); ++i)
    if (i < cnt) {
      const int ent = base + i, r = ent / DL, c = ent - r * DL;
      out[r * kMaxKeyDim + c] = acc[i];
    }
}

// A diagonal block (k = l, W_pk = C_p^-1 E_pk): its D (D + 1) / 2 lower entries, row-major packed;
// each is written to both triangles of the partial.
template <typename T, int D>
__device__ __forceinline__ void ChunkTermsSym(const SchurDev& d, const T* H, const T* W, int64_t t0,
                                              int64_t t1, int lane, T* out) {
  constexpr int N = D * (D + 1) / 2;
  T acc[N];
#pragma unroll
  for (int i = 0; i < N; ++i) acc[i] = T(0);
  for (int64_t t = t0 + lane; t < t1; t += 32) {
    const T* E = W + d.sb_eoff[t];
    const T* Wl = W + d.sb_woff[t];
    T e[3 * D], w[3 * D];
#pragma unroll
    for (int i = 0; i < 3 * D; ++i) e[i] = E[i];
#pragma unroll
    for (int i = 0; i < 3 * D; ++i) w[i] = Wl[i];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c <= r; ++c)
        acc[r * (r + 1) / 2 + c] += e[r] * w[c] + e[D + r] * w[D + c] + e[2 * D + r] * w[2 * D + c];
  }
  int base = 0, cnt = N;
  ReduceScatterLevel<T, N, 16>(acc, lane, base, cnt);
#pragma unroll
  for (int i = 0; i < ReduceScatterSlots<N>(); ++i)
    if (i < cnt) {
      const int ent = base + i;
      int r = 0;
      while ((r + 1) * (r + 2) / 2 <= ent) ++r;
      const int c = ent - r * (r + 1) / 2;
      out[r * kMaxKeyDim + c] = acc[i];
      out[c * kMaxKeyDim + r] = acc[i];
    }
}

// Any other key sizes (up to kMaxKeyDim): runtime bounds inside the 6 x 6 accumulator.
template <typename T>
__device__ __forceinline__ void ChunkTermsAny(const SchurDev& d, const T* H, const T* W, int dk, int dl,
                                              int64_t t0, int64_t t1, int lane, T* out) {
  constexpr int D = kMaxKeyDim;
  constexpr int N = D * D;
  T acc[N];
#pragma unroll
  for (int i = 0; i < N; ++i) acc[i] = T(0);
  for (int64_t t = t0 + lane; t < t1; t += 32) {
    const T* E = W + d.sb_eoff[t];
    const T* Wl = W + d.sb_woff[t];
    T e[3 * D], w[3 * D];
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
      for (int i = 0; i < D; ++i) {
        e[q * D + i] = i < dk ? E[q * dk + i] : T(0);
        w[q * D + i] = i < dl ? Wl[q * dl + i] : T(0);
      }
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = 0; c < D; ++c)
        acc[r * D + c] += e[r] * w[c] + e[D + r] * w[D + c] + e[2 * D + r] * w[2 * D + c];
  }
  int base = 0, cnt = N;
  ReduceScatterLevel<T, N, 16>(acc, lane, base, cnt);
#pragma unroll
  for (int i = 0; i < ReduceScatterSlots<N>(); ++i)
    if (i < cnt) out[base + i] = acc[i];
}

template <typename T>
__global__ void __launch_bounds__(32 * kSchurWarps)
    SchurChunkKernel(SchurDev d, const T* hess_all, int64_t nvals, const T* W, const LmState* st) {
  const int ch = blockIdx.x * kSchurWarps + (threadIdx.x >> 5);
  if (ch >= d.nchunks) return;
  const int lane = threadIdx.x & 31;
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const int sb = d.ch_block[ch];
  const int dk = d.sb_dk[sb], dl = d.sb_dl[sb];
  const int64_t t0 = d.ch_begin[ch];
  const int64_t t1 = min(t0 + d.chunk_terms, d.sb_ptr[sb + 1]);
  T* out = static_cast<T*>(d.partials) + int64_t(ch) * (kMaxKeyDim * kMaxKeyDim);
  // one case per chunk (warp-uniform): the key sizes of bundle adjustment and 2D / 3D poses
  const bool diag = d.sb_diag_toff[sb] >= 0;
  switch (dk * 8 + dl + (diag ? 64 : 0)) {
    case 64 + 6 * 8 + 6: ChunkTermsSym<T, 6>(d, H, W, t0, t1, lane, out); break;
    case 64 + 3 * 8 + 3: ChunkTermsSym<T, 3>(d, H, W, t0, t1, lane, out); break;
    case 64 + 2 * 8 + 2: ChunkTermsSym<T, 2>(d, H, W, t0, t1, lane, out); break;
    case 64 + 1 * 8 + 1: ChunkTermsSym<T, 1>(d, H, W, t0, t1, lane, out); break;
    case 6 * 8 + 6: ChunkTerms<T, 6, 6>(d, H, W, t0, t1, lane, out); break;
    case 3 * 8 + 6: ChunkTerms<T, 3, 6>(d, H, W, t0, t1, lane, out); break;
    case 6 * 8 + 3: ChunkTerms<T, 6, 3>(d, H, W, t0, t1, lane, out); break;
    case 3 * 8 + 3: ChunkTerms<T, 3, 3>(d, H, W, t0, t1, lane, out); break;
    default: ChunkTermsAny<T>(d, H, W, dk, dl, t0, t1, lane, out);
  }
}

template <typename T>
__global__ void SchurFinishKernel(SchurDev d, const T* hess_all, int64_t nvals, const double* damping,
                                  T* S, const LmState* st) {
  const int sb = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (sb >= d.nsblocks) return;
  const int lane = threadIdx.x & 31;
  const int dk = d.sb_dk[sb], dl = d.sb_dl[sb];
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const int64_t hoff = d.sb_hoff[sb];
  const int diag_toff = d.sb_diag_toff[sb];
  const T* part = static_cast<const T*>(d.partials);
  for (int ent = lane; ent < dk * dl; ent += 32) {
    const int r = ent / dl, c = ent - r * dl;
    T acc = T(0);
    for (int64_t ch = d.sb_chunk_ptr[sb]; ch < d.sb_chunk_ptr[sb + 1]; ++ch)
      acc += part[ch * (kMaxKeyDim * kMaxKeyDim) + r * kMaxKeyDim + c];
    T v = hoff >= 0 ? H[hoff + ent] : T(0);
    if (diag_toff >= 0 && r == c) v += T(damping[diag_toff + r]);
    S[d.sb_soff[sb] + ent] = v - acc;
  }
}

// One warp per reduced-system scalar: v_i = g_i - sum_p (E_p^T t_p)_i, fixed shuffle tree.
template <typename T>
__global__ void SchurRhsKernel(SchurDev d, const T* hess_all, int64_t nvals, const T* rhs_all,
                               int64_t N, const T* tp, T* v, const LmState* st) {
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= d.nB) return;
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const T* g = rhs_all + int64_t(st->init_idx) * N;
  // two entries per lane in flight (their index loads, then their operand loads), added in order
  auto term = [&](int64_t q, T (&et)[6]) {
    const int dk = d.r_dk[q];
    const T* E = H + d.r_eoff[q] + d.r_ecol[q];
    const T* t = tp + 3 * int64_t(d.r_pt[q]);
    et[0] = E[0];
    et[1] = E[dk];
    et[2] = E[2 * dk];
    et[3] = t[0];
    et[4] = t[1];
    et[5] = t[2];
  };
  T acc = T(0);
  const int64_t q1 = d.r_ptr[i + 1];
  int64_t q = d.r_ptr[i] + lane;
  for (; q + 32 < q1; q += 64) {
    T a[6], b[6];
    term(q, a);
    term(q + 32, b);
    acc += a[0] * a[3] + a[1] * a[4] + a[2] * a[5];
    acc += b[0] * b[3] + b[1] * b[4] + b[2] * b[5];
  }
  if (q < q1) {
    T a[6];
    term(q, a);
    acc += a[0] * a[3] + a[1] * a[4] + a[2] * a[5];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) v[i] = g[i] - acc;
}

// The same per reduced-system key: one warp per key k (d_k scalars), lanes over the points that see
// it (the list of its first scalar), each point's E_pk block read once, whole and contiguous (a
// key's blocks lie consecutively in the Hessian values); the lanes' d_k sums are added by the
// butterfly reduce-scatter.  v_k = g_k - sum_p E_pk^T t_p.
template <typename T, int DK>
__device__ __forceinline__ void RhsKeyTerms(const SchurDev& d, const T* H, const T* tp, int64_t q0,
                                            int64_t q1, int lane, T* sum, int* base, int* cnt) {
  constexpr int N = DK;
  T acc[N];
#pragma unroll
  for (int c = 0; c < N; ++c) acc[c] = T(0);
  for (int64_t q = q0 + lane; q < q1; q += 32) {
    const T* E = H + d.r_eoff[q];
    const T* t = tp + 3 * int64_t(d.r_pt[q]);
    T e[3 * N];
#pragma unroll
    for (int i = 0; i < 3 * N; ++i) e[i] = E[i];
    const T t0 = t[0], t1 = t[1], t2 = t[2];
#pragma unroll
    for (int c = 0; c < N; ++c) acc[c] += e[c] * t0 + e[N + c] * t1 + e[2 * N + c] * t2;
  }
  int b = 0, n = N;
  ReduceScatterLevel<T, N, 16>(acc, lane, b, n);
#pragma unroll
  for (int i = 0; i < ReduceScatterSlots<N>(); ++i) sum[i] = acc[i];
  *base = b;
  *cnt = n;
}

constexpr int kRhsKeyWarpsMin = 1024;  // keys below which the rhs runs a warp per scalar

template <typename T>
__global__ void SchurRhsKeyKernel(SchurDev d, const T* hess_all, int64_t nvals, const T* rhs_all,
                                  int64_t N, const T* tp, T* v, const LmState* st) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= d.nBk) return;
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const T* g = rhs_all + int64_t(st->init_idx) * N;
  const int i0 = d.bkey_toff[k], dk = d.bkey_toff[k + 1] - i0;
  const int64_t q0 = d.r_ptr[i0], q1 = d.r_ptr[i0 + 1];
  T sum[2];
  int base = 0, cnt = 0;
  if (dk == 6) RhsKeyTerms<T, 6>(d, H, tp, q0, q1, lane, sum, &base, &cnt);
  else if (dk == 3) RhsKeyTerms<T, 3>(d, H, tp, q0, q1, lane, sum, &base, &cnt);
  else {
    // other key sizes: one lane per component, in point order
    if (lane < dk) {
      T acc = T(0);
      for (int64_t q = q0; q < q1; ++q) {
        const T* E = H + d.r_eoff[q];
        const T* t = tp + 3 * int64_t(d.r_pt[q]);
        acc += E[lane] * t[0] + E[dk + lane] * t[1] + E[2 * dk + lane] * t[2];
      }
      v[i0 + lane] = g[i0 + lane] - acc;
    }
    return;
  }
  for (int i = 0; i < cnt; ++i) v[i0 + base + i] = g[i0 + base + i] - sum[i];
}

// s = W y for one 3 x DK block (all loads issued first; the sums in column order).
template <typename T, int DK>
__device__ __forceinline__ void BlockTimes(const T* Wp, const double* yk, T (&s)[3]) {
  T w[3 * DK], yv[DK];
#pragma unroll
  for (int i = 0; i < 3 * DK; ++i) w[i] = Wp[i];
#pragma unroll
  for (int c = 0; c < DK; ++c) yv[c] = T(yk[c]);
  s[0] = s[1] = s[2] = T(0);
#pragma unroll
  for (int c = 0; c < DK; ++c) {
    s[0] += w[c] * yv[c];
    s[1] += w[DK + c] * yv[c];
    s[2] += w[2 * DK + c] * yv[c];
  }
}
template <typename T>
__device__ __forceinline__ void BlockTimesAny(const T* Wp, const double* yk, int dk, T (&s)[3]) {
  s[0] = s[1] = s[2] = T(0);
  for (int c = 0; c < dk; ++c) {
    const T yc = T(yk[c]);
    s[0] += Wp[c] * yc;
    s[1] += Wp[dk + c] * yc;
    s[2] += Wp[2 * dk + c] * yc;
  }
}

// Point back-substitution z_p = t_p - C_p^-1 sum_k E_pk y_k = t_p - L_p^-T sum_k G_pk y_k, and
// update = -[y; z].
template <typename T>
__global__ void SchurBackSubKernel(SchurDev d, const double* y, const T* W, const T* tp, const T* cinv,
                                   double* update) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < d.npoints) {
    const int p = t;
    T z0 = T(0), z1 = T(0), z2 = T(0);  // sum_k G_pk y_k
    for (int64_t e = d.pt_eptr[p]; e < d.pt_eptr[p + 1]; ++e) {
      const int dk = d.pt_ekey_dim[e];
      const T* Wp = W + d.pt_woff[e];
      const double* yk = y + d.pt_ekey_toff[e];
      T s[3];
      if (dk == 6) BlockTimes<T, 6>(Wp, yk, s);
      else if (dk == 3) BlockTimes<T, 3>(Wp, yk, s);
      else BlockTimesAny<T>(Wp, yk, dk, s);
      z0 += s[0];
      z1 += s[1];
      z2 += s[2];
    }
    const T* li = cinv + 9 * int64_t(p);  // L^-1 lower (00, 10, 11, 20, 21, 22)
    const T w0 = li[0] * z0 + li[1] * z1 + li[3] * z2;
    const T w1 = li[2] * z1 + li[4] * z2;
    const T w2 = li[5] * z2;
    double* u = update + d.c_toff + 3 * int64_t(p);
    u[0] = -double(tp[3 * int64_t(p)] - w0);
    u[1] = -double(tp[3 * int64_t(p) + 1] - w1);
    u[2] = -double(tp[3 * int64_t(p) + 2] - w2);
  } else if (t < d.npoints + d.nB) {
    const int i = t - d.npoints;
    update[i] = -double(y[i]);
  }
}

// ---------------------------------------------------------------------------------------------
// Multifrontal LDL^T: persistent tile-task kernel
// ---------------------------------------------------------------------------------------------
struct Geom {
  int w, m, np, nt, base;
  int64_t foff;
};

__device__ __forceinline__ Geom FrontGeom(const FactorDev& f, int s) {
  Geom g;
  g.w = f.sn_w[s];
  g.m = f.sn_m[s];
  g.np = f.npiv[s];
  g.nt = f.ntiles[s];
  g.base = f.tile_base[s];
  g.foff = f.sn_foff[s];
  return g;
}
__device__ __forceinline__ int TileStart(const Geom& g, int t, int tile) {
  return t < g.np ? t * tile : g.w + (t - g.np) * tile;
}
__device__ __forceinline__ int TileSize(const Geom& g, int t, int tile) {
  return t < g.np ? min(tile, g.w - t * tile) : min(tile, g.m - TileStart(g, t, tile));
}
__device__ __forceinline__ int StateIdx(const Geom& g, int i, int j) { return g.base + i * (i + 1) / 2 + j; }

// Shared tiles are stored transposed (column index major, row index minor) so that the lanes of a
// warp, which walk consecutive rows, read consecutive words.
template <typename T, int TILE>
struct alignas(16) TileSmem {
  T a[TILE * TILE];  // a and b are contiguous: together they hold a double tile (FP64 redo of a tile)
  T b[TILE * TILE];
  T c[TILE * TILE];
  T w[TILE * TILE];  // L D of the look-ahead's panel tile
  T e[sizeof(T) == 8 ? TILE * TILE : 1];  // FP64 look-ahead: the diagonal tile
  T d[TILE];
};

// Reciprocal for the pivot chain.  FP64 division is a long dependent instruction sequence on this
// GPU (~560 cycles measured; every dependent FP64 operation costs ~64), so doubles take the
// hardware's approximate FP64 reciprocal (rcp.approx.ftz.f64, ~18 cycles) and two Newton-Raphson
// steps y <- y + y (1 - x y), whose error squares at each step.  Inputs whose reciprocal leaves the
// normal range (the approximation flushes subnormals) take the IEEE division.
template <typename T>
__device__ __forceinline__ T PivotReciprocal(T x) { return T(1) / x; }
template <>
__device__ __forceinline__ double PivotReciprocal<double>(double x) {
  const int ex = __double2hiint(x) & 0x7FF00000;  // biased exponent field
  if (ex < 0x00200000 || ex >= 0x7FD00000) return 1.0 / x;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// Per-phase clock stamps of a traced task (SFG_TRACE_FACTOR): `ready` is the task's trace record
// + 1; phase i goes to record slot 4 + i.
__device__ __forceinline__ void Stamp(unsigned long long* ready, int i) {
  if (ready && threadIdx.x == 0) ready[3 + i] = Clock64Global();
}

// Broadcast of thread 0's wait result.
__device__ __forceinline__ bool CtaWait(bool ok_thread0, int* s_flag,
                                        unsigned long long* ready = nullptr) {
  if (threadIdx.x == 0) *s_flag = ok_thread0 ? 1 : 0;
  if (threadIdx.x == 0 && ready) *ready = Clock64Global();
  __syncthreads();
  const bool ok = *s_flag != 0;
  __syncthreads();
  return ok;
}

// Publish a tile version: the CTA barrier orders every thread's writes before thread 0's fence,
// and the fence (cumulative) before the flag store that other CTAs acquire.
__device__ __forceinline__ void Signal(int* addr, int v) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicExch(addr, v);
  }
}
// The same for a completion count that several CTAs add to.
__device__ __forceinline__ void SignalAdd(int* addr) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(addr, 1);
  }
}

// Load a b_r x b_c tile at (r0, c0) of a column-major front into smem, transposed: dst[c*TILE + r].
template <typename T, int TILE>
__device__ __forceinline__ void LoadTileT(const T* Fs, int m, int r0, int c0, int br, int bc, T* dst) {
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    if (r < br && c < bc) dst[c * TILE + r] = Ld(Fs + (r0 + r) + int64_t(c0 + c) * m);
  }
}

// The same tile into registers (entry e = threadIdx.x + n * kFactorThreads; zero outside), so that
// its loads can be in flight across a barrier, and from there into shared memory.
template <typename T, int TILE>
__device__ __forceinline__ void LoadTileRegs(const T* Fs, int m, int r0, int c0, int br, int bc,
                                             T (&v)[TileEntriesPerThread<TILE>()]) {
#pragma unroll
  for (int n = 0; n < TileEntriesPerThread<TILE>(); ++n) {
    const int e = threadIdx.x + n * kFactorThreads, r = e % TILE, c = e / TILE;
    v[n] = (r < br && c < bc) ? Ld(Fs + (r0 + r) + int64_t(c0 + c) * m) : T(0);
  }
}
template <typename T, int TILE>
__device__ __forceinline__ void StoreTileRegs(const T (&v)[TileEntriesPerThread<TILE>()], T* dst) {
#pragma unroll
  for (int n = 0; n < TileEntriesPerThread<TILE>(); ++n) {
    const int e = threadIdx.x + n * kFactorThreads;
    dst[(e / TILE) * TILE + e % TILE] = v[n];
  }
}

// Assemble one tile column of a front from host-flattened lists: zero it, write the original
// entries (+ damping on the diagonal), then add the children's update entries round by round
// (within a round every destination is distinct).
template <typename T, int TILE>
__device__ void TaskAssemble(const FactorDev& f, int s, int tj, const T* A, const double* damping,
                             T* F, int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  bool ok = true;
  if (threadIdx.x == 0) {
    for (int q = f.child_ptr[s]; q < f.child_ptr[s + 1] && ok; ++q) {
      const int c = f.child_list[q];
      const Geom gc = FrontGeom(f, c);
      for (int i = gc.np; i < gc.nt && ok; ++i)
        for (int j = gc.np; j <= i && ok; ++j)
          ok = WaitAtLeast(f.tile_state + StateIdx(gc, i, j), 1 + gc.np, f.error);
    }
  }
  if (!CtaWait(ok, s_flag, ready)) return;
  T* Fs = F + g.foff;
  const int m = g.m;
  const int c0 = TileStart(g, tj, TILE), c1 = c0 + TileSize(g, tj, TILE);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int c = c0 + warp; c < c1; c += nwarp)
    for (int r = c + lane; r < m; r += 32) St(Fs + r + int64_t(c) * m, T(0));
  __syncthreads();
  const int slot = f.col_base[s] + tj;
  for (int64_t e = f.a_ptr[slot] + threadIdx.x; e < f.a_ptr[slot + 1]; e += blockDim.x) {
    T v = A[f.a_src[e]];
    const int dmp = f.a_damp[e];
    if (dmp >= 0 && damping) v += T(damping[dmp]);
    St(Fs + f.a_dst[e], v);
  }
  for (int64_t rb = f.e_rptr[slot]; rb < f.e_rptr[slot + 1]; ++rb) {
    __syncthreads();
    for (int64_t e = f.e_round[rb] + threadIdx.x; e < f.e_round[rb + 1]; e += blockDim.x) {
      T* dst = Fs + f.e_dst[e];
      St(dst, Ld(dst) + Ld(F + f.e_src[e]));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) __threadfence();
  __syncthreads();
  for (int i = tj + threadIdx.x; i < g.nt; i += blockDim.x) atomicExch(f.tile_state + StateIdx(g, i, tj), 1);
}

// ---- FP64 tiles (16 x 16).  On this GPU a warp issues an FP64 instruction about once per 64
// cycles on its own SM sub-partition (a one-warp elimination of a tile measured 20 us against 12.6
// us for the same work spread over four warps), so FP64 tile work is spread over all four warps of
// the CTA (one per sub-partition) with as few FP64 instructions per warp and step as possible.

// x 2^s, exact while the result stays a normal number (otherwise the library's scalbn).
__device__ __forceinline__ double Pow2Scale(double x, int s) {
  const int hi = __double2hiint(x), ex = (hi >> 20) & 0x7FF, ne = ex + s;
  if (ex != 0 && ex != 0x7FF && ne > 0 && ne < 0x7FF)
    return __hiloint2double(hi + s * (1 << 20), __double2loint(x));
  return scalbn(x, s);
}
// Unbiased binary exponent of a pivot; 0 (no scaling) for zero, subnormal, infinite or NaN pivots.
__device__ __forceinline__ int PivotExponent(double p) {
  const int ex = (__double2hiint(p) >> 20) & 0x7FF;
  return (ex == 0 || ex == 0x7FF) ? 0 : ex - 1023;
}

// Fraction-free LDL^T of the b x b leading part of a TILE x TILE FP64 tile held transposed in
// shared memory (a[c * TILE + r] = A(r, c), lower part used).  Pivot k replaces every trailing
// lower entry by B(r, c) <- 2^-e_k (P_k B(r, c) - B(r, k) B(c, k)), P_k = B(k, k), e_k its binary
// exponent: the Schur complement of the right-looking elimination times S_{k+1} = m_0 ... m_k (m_i
// the mantissa of P_i, |m_i| in [1, 2)), so that no division sits on the pivot chain, only one
// FP64 multiply and one multiply-add per entry.  The entries right of column 0 are held in
// registers, one per thread for 16 x 16 tiles (120 entries), four for 32 x 32 (496); one CTA
// barrier per pivot.  At the end d_k = P_k / S_k and L(r, k) = B(r, k) / P_k, one reciprocal per
// column, formed in parallel.  Measured on one GB300 SM, a 16 x 16 tile takes 7,000 cycles against
// 14,200 for the elimination with a reciprocal per pivot and two barriers, at the same accuracy
// against a long double factorization.  On return column j below the diagonal holds L(:, j), the
// diagonal D, and dinv[0, b) = D^-1 (if dinv is not null); s_rp is TILE doubles of scratch.
template <int TILE>
__device__ void DiagLdltF64(double* a, int b, double* dinv, double* s_rp) {
  static_assert(TILE <= 32, "one lane per pivot in the final scan");
  constexpr int kEntries = TILE * (TILE - 1) / 2;
  constexpr int kPer = (kEntries + kFactorThreads - 1) / kFactorThreads;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  // entry e = t + q * kFactorThreads -> (r, c), 1 <= c <= r < TILE, column-major
  int r[kPer], c[kPer];
  double v[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = t + q * kFactorThreads;
    int cc = 1, start = 0;
    while (cc < TILE - 1 && e >= start + (TILE - cc)) {
      start += TILE - cc;
      ++cc;
    }
    c[q] = (e < kEntries) ? cc : TILE;
    r[q] = (e < kEntries) ? cc + (e - start) : 0;
    if (r[q] >= b) c[q] = TILE;
    v[q] = c[q] < TILE ? a[c[q] * TILE + r[q]] : 0.0;
  }
  for (int k = 0; k + 1 < b; ++k) {
    const double p = a[k * (TILE + 1)];
    const int ek = PivotExponent(p);
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      if (c[q] < TILE && c[q] > k) {
        const double m = a[k * TILE + r[q]] * a[k * TILE + c[q]];
        v[q] = Pow2Scale(fma(p, v[q], -m), -ek);
        a[c[q] * TILE + r[q]] = v[q];
      }
    }
    __syncthreads();
  }
  double dk = 0.0, sk = 1.0;
  if (warp == 0) {
    // S_k = m_0 ... m_{k-1}: exclusive product scan over the pivots' mantissas
    const double p = lane < b ? a[lane * (TILE + 1)] : 1.0;
    double x = lane < b ? Pow2Scale(p, -PivotExponent(p)) : 1.0;
#pragma unroll
    for (int off = 1; off < TILE; off <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x *= y;
    }
    sk = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) sk = 1.0;
    dk = p * PivotReciprocal<double>(sk);
  } else if (warp == 1 && lane < TILE) {
    s_rp[lane] = lane < b ? PivotReciprocal<double>(a[lane * (TILE + 1)]) : 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kPer; ++q)
    if (c[q] < TILE && r[q] > c[q]) a[c[q] * TILE + r[q]] = v[q] * s_rp[c[q]];
  for (int rr = 1 + t; rr < b; rr += kFactorThreads) a[rr] *= s_rp[0];  // column 0
  if (warp == 0 && lane < b) {
    a[lane * (TILE + 1)] = dk;
    if (dinv) dinv[lane] = sk * s_rp[lane];
  }
  __syncthreads();
}

// Inverse of the unit lower factor held in `a` (strict lower part of the b x b leading block, as
// the diagonal LDL^T leaves it) into li (transposed like the tiles; identity outside the block), by
// forward substitution on all columns at once: the strict lower entries (r > c) in registers, one
// per thread for 16 x 16 tiles, four for 32 x 32; one multiply-add per entry and step, one CTA
// barrier per step.
template <typename T, int TILE>
__device__ void UnitLowerInverse(const T* a, int b, T* li) {
  constexpr int kEntries = TILE * (TILE - 1) / 2;
  constexpr int kPer = (kEntries + kFactorThreads - 1) / kFactorThreads;
  const int t = threadIdx.x;
  for (int e = t; e < TILE * TILE; e += blockDim.x) li[e] = (e % (TILE + 1) == 0) ? T(1) : T(0);
  // entry e = t + q * kFactorThreads -> (r, c), r > c, column-major
  int r[kPer], c[kPer];
  T v[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = t + q * kFactorThreads;
    int cc = 0, start = 0;
    while (cc < TILE - 2 && e >= start + (TILE - 1 - cc)) {
      start += TILE - 1 - cc;
      ++cc;
    }
    c[q] = (e < kEntries) ? cc : TILE;
    r[q] = (e < kEntries) ? cc + 1 + (e - start) : 0;
    if (r[q] >= b) c[q] = TILE;
    v[q] = T(0);
  }
  __syncthreads();
  for (int q = 0; q + 1 < b; ++q) {
    // Li(r, c) -= L(r, q) Li(q, c) for r > q >= c; row q of Li is final after step q - 1
#pragma unroll
    for (int n = 0; n < kPer; ++n) {
      if (c[n] < TILE && r[n] > q && c[n] <= q) {
        const T lrq = a[q * TILE + r[n]];
        v[n] = (c[n] == q) ? -lrq : v[n] - lrq * li[c[n] * TILE + q];
        li[c[n] * TILE + r[n]] = v[n];
      }
    }
    __syncthreads();
  }
}

// Panel solve X = F L^-T D^-1 of a 16 x 16 FP64 tile by forward substitution (no inverse on the
// critical path): Y L^T = F row by row, then X = Y D^-1.  f: F transposed in shared memory, l: the
// diagonal tile's unit lower factor (transposed, strict lower part), dinv: D^-1 (bk entries).
// Thread t takes row r = t / 8 and columns g = t % 8 and g + 8 in registers; the eight threads of a
// row are lanes of one warp, and step q takes y_q from its owner by a shuffle.  Writes X into x_out
// and Y = X D into y_out (transposed, zero outside bi x bk).
__device__ void PanelSolveSubstF64(const double* f, const double* l, const double* dinv, int bi, int bk,
                                   double* x_out, double* y_out) {
  constexpr unsigned kAll = 0xffffffffu;
  const int t = threadIdx.x;
  const int r = t >> 3, g = t & 7;
  const int lane = t & 31, base = lane & ~7;
  double y0 = (r < bi && g < bk) ? f[g * 16 + r] : 0.0;
  double y1 = (r < bi && g + 8 < bk) ? f[(g + 8) * 16 + r] : 0.0;
#pragma unroll
  for (int q = 0; q < 15; ++q) {
    const double yq = __shfl_sync(kAll, q < 8 ? y0 : y1, base + (q & 7));
    if (q < bk) {
      if (g > q && g < bk) y0 = fma(-yq, l[q * 16 + g], y0);
      if (g + 8 > q && g + 8 < bk) y1 = fma(-yq, l[q * 16 + g + 8], y1);
    }
  }
  const bool in0 = r < bi && g < bk, in1 = r < bi && g + 8 < bk;
  y_out[g * 16 + r] = in0 ? y0 : 0.0;
  y_out[(g + 8) * 16 + r] = in1 ? y1 : 0.0;
  x_out[g * 16 + r] = in0 ? y0 * dinv[g] : 0.0;
  x_out[(g + 8) * 16 + r] = in1 ? y1 * dinv[g + 8] : 0.0;
}

// A pivot of an FP32 diagonal tile that kept less than this fraction of its diagonal entry (more
// than 12 of FP32's 24 bits cancelled), or is not positive, sends the tile to the FP64 redo.
constexpr float kNearSingularPivot = 1.0f / 4096.0f;

// LDL^T of a 32 x 32 FP32 diagonal tile held transposed in shared memory (b x b of it), CTA-wide:
// the 496 entries right of column 0 are held four per thread in registers; pivot k takes the
// hardware's approximate reciprocal of P_k (every thread forms it), and each trailing entry takes
// one multiply and one multiply-add, B(r, c) -= (B(r, k) / P_k) B(c, k), with the columns scaled
// to L once at the end; one CTA barrier per pivot.  Measured on one GB300 SM: 9,800 cycles per
// tile against 17,900 for one warp with the rows in registers, at the same accuracy.  Sets
// *redo_flag when a pivot kept less than kNearSingularPivot of its input diagonal entry (orig) or
// is not positive.
template <int TILE>
__device__ void DiagLdltF32(float* a, const float* orig, int b, int* redo_flag) {
  constexpr int kEntries = TILE * (TILE - 1) / 2;
  constexpr int kPer = (kEntries + kFactorThreads - 1) / kFactorThreads;
  const int t = threadIdx.x;
  int r[kPer], c[kPer];
  float v[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = t + q * kFactorThreads;
    int cc = 1, start = 0;
    while (cc < TILE - 1 && e >= start + (TILE - cc)) {
      start += TILE - cc;
      ++cc;
    }
    c[q] = (e < kEntries) ? cc : TILE;
    r[q] = (e < kEntries) ? cc + (e - start) : 0;
    if (r[q] >= b) c[q] = TILE;
    v[q] = c[q] < TILE ? a[c[q] * TILE + r[q]] : 0.f;
  }
  bool redo = false;
  for (int k = 0; k + 1 < b; ++k) {
    const float p = a[k * (TILE + 1)];
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(p));
    if (t == 0) redo = redo || !(p > kNearSingularPivot * fabsf(orig[k * (TILE + 1)]));
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      if (c[q] < TILE && c[q] > k) {
        const float lr = a[k * TILE + r[q]] * inv;
        v[q] = fmaf(-lr, a[k * TILE + c[q]], v[q]);
        a[c[q] * TILE + r[q]] = v[q];
      }
    }
    __syncthreads();
  }
  if (t == 0 && b > 0)
    redo = redo || !(a[(b - 1) * (TILE + 1)] > kNearSingularPivot * fabsf(orig[(b - 1) * (TILE + 1)]));
#pragma unroll
  for (int q = 0; q < kPer; ++q)
    if (c[q] < TILE && r[q] > c[q]) a[c[q] * TILE + r[q]] = v[q] / a[c[q] * (TILE + 1)];
  for (int rr = 1 + t; rr < b; rr += kFactorThreads) a[rr] = a[rr] / a[0];  // column 0
  if (t == 0 && redo) *redo_flag = 1;
  __syncthreads();
}

// LDL^T of diagonal tile k, held transposed in shared memory `a` (b x b of it), plus the explicit
// inverse of its unit lower factor (for the triangular solves, and for the FP32 panel solves, which
// are small products with it); writes L, D and the inverse and publishes the tile.  FP64 tiles take
// the fraction-free CTA-wide elimination, FP32 tiles the CTA-wide one with approximate pivot
// reciprocals.  An FP32
// tile with a near-singular pivot is factored again in FP64 from its saved input and rounded back
// (counted in f.fp64_tiles).
template <typename T, int TILE>
__device__ void DiagCore(const FactorDev& f, const Geom& g, int s, int k, T* F, T* Linv, T* a,
                         TileSmem<T, TILE>& sm, unsigned long long* tr = nullptr) {
  static_assert(TILE <= 32, "one lane per tile row");
  const int b = TileSize(g, k, TILE), r0 = TileStart(g, k, TILE);
  T* Fs = F + g.foff;
  T* li = sm.b;
  if constexpr (sizeof(T) == 8) {
    static_assert(sizeof(T) != 8 || TILE == 16, "the FP64 tile kernels are written for 16 x 16 tiles");
    __shared__ double s_rp[16];
    DiagLdltF64<16>(a, b, sm.d, s_rp);
    Stamp(tr, 3);
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
      const int r = e % TILE, c = e / TILE;
      if (r < b && c < b && r >= c) St(Fs + (r0 + r) + int64_t(r0 + c) * g.m, a[c * TILE + r]);
    }
    Signal(f.tile_state + StateIdx(g, k, k), kFinal);
    // the inverse of L is for the triangular solves only (the FP64 panel solves substitute), so
    // it is formed after the tile is published, off the front's critical chain
    UnitLowerInverse<double, 16>(a, b, li);
    T* Lk = Linv + f.linv_base[s] + int64_t(k) * TILE * TILE;
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) St(Lk + e, li[e]);
    return;
  } else {
    // the tile's input, kept for an FP64 redo
    T* orig = sm.c;
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) orig[e] = a[e];
    __shared__ int s_redo;
    if (threadIdx.x == 0) s_redo = 0;
    __syncthreads();
    DiagLdltF32<TILE>(a, orig, b, &s_redo);
    Stamp(tr, 3);
    if (s_redo) {
      // FP64 redo from the saved input: the double tile occupies a and b
      double* dt = reinterpret_cast<double*>(sm.a);
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) dt[e] = double(orig[e]);
      __syncthreads();
      __shared__ double s_rp[TILE];
      DiagLdltF64<TILE>(dt, b, nullptr, s_rp);
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) orig[e] = T(dt[e]);
      __syncthreads();
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) a[e] = orig[e];
      if (threadIdx.x == 0 && f.fp64_tiles) atomicAdd(f.fp64_tiles, 1);
      __syncthreads();
    }
    UnitLowerInverse<T, TILE>(a, b, li);
  }
  T* Lk = Linv + f.linv_base[s] + int64_t(k) * TILE * TILE;
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    St(Lk + e, li[e]);  // stored transposed like the shared tiles
    if (r < b && c < b && r >= c) St(Fs + (r0 + r) + int64_t(r0 + c) * g.m, a[c * TILE + r]);
  }
  Signal(f.tile_state + StateIdx(g, k, k), kFinal);
}

template <typename T, int TILE>
__device__ void TaskDiag(const FactorDev& f, int s, int k, T* F, T* Linv, TileSmem<T, TILE>& sm,
                         int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  bool ok = true;
  if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, k, k), 1 + k, f.error);
  if (!CtaWait(ok, s_flag, ready)) return;
  const int b = TileSize(g, k, TILE), r0 = TileStart(g, k, TILE);
  LoadTileT<T, TILE>(F + g.foff, g.m, r0, r0, b, b, sm.a);
  __syncthreads();
  Stamp(ready, 0);
  DiagCore<T, TILE>(f, g, s, k, F, Linv, sm.a, sm, ready);
}

// sum_{q < n} x[q * TILE + r] y[q * TILE + c] over two tiles held transposed in shared memory, with
// two accumulation chains (a dependent FP64 multiply-add costs 64 cycles on this GPU) added at
// the end in a fixed order.
template <typename T, int TILE>
__device__ __forceinline__ T PanelDot(const T* x, const T* y, int r, int c, int n) {
  T s0 = T(0), s1 = T(0);
  int q = 0;
  for (; q + 2 <= n; q += 2) {
    s0 = fma(x[q * TILE + r], y[q * TILE + c], s0);
    s1 = fma(x[(q + 1) * TILE + r], y[(q + 1) * TILE + c], s1);
  }
  if (q < n) s0 = fma(x[q * TILE + r], y[q * TILE + c], s0);
  return s0 + s1;
}

// Panel solve L_ik = F_ik L_kk^-T D_k^-1 as a product with the stored inverse.
template <typename T, int TILE>
__device__ void TaskTrsm(const FactorDev& f, int s, int i, int k, T* F, const T* Linv,
                         TileSmem<T, TILE>& sm, int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  bool ok = true;
  if (threadIdx.x == 0) {
    ok = WaitAtLeast(f.tile_state + StateIdx(g, k, k), kFinal, f.error) &&
         WaitAtLeast(f.tile_state + StateIdx(g, i, k), 1 + k, f.error);
  }
  if (!CtaWait(ok, s_flag, ready)) return;
  const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
  const int bi = TileSize(g, i, TILE), ri = TileStart(g, i, TILE);
  T* Fs = F + g.foff;
  LoadTileT<T, TILE>(Fs, g.m, ri, ck, bi, bk, sm.a);  // F_ik
  if constexpr (sizeof(T) == 8) {
    LoadTileT<T, TILE>(Fs, g.m, ck, ck, bk, bk, sm.b);  // L_kk (strict lower) and D_k
    __syncthreads();
    for (int c = threadIdx.x; c < bk; c += blockDim.x) sm.d[c] = PivotReciprocal<T>(sm.b[c * TILE + c]);
    __syncthreads();
    PanelSolveSubstF64(sm.a, sm.b, sm.d, bi, bk, sm.c, sm.w);
    __syncthreads();
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
      const int r = e % TILE, c = e / TILE;
      if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, sm.c[c * TILE + r]);
    }
    Signal(f.tile_state + StateIdx(g, i, k), kFinal);
    return;
  }
  const T* Lk = Linv + f.linv_base[s] + int64_t(k) * TILE * TILE;
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) sm.b[e] = Ld(Lk + e);
  for (int c = threadIdx.x; c < bk; c += blockDim.x)
    sm.d[c] = PivotReciprocal<T>(Ld(Fs + int64_t(ck + c) * (g.m + 1)));
  __syncthreads();
  // W(r, c) = sum_{q <= c} F(r, q) Li(c, q);  Li(c, q) = b[q * TILE + c]; two accumulation chains
  constexpr int kPer = TileEntriesPerThread<TILE>();
  T out[kPer];
#pragma unroll
  for (int n = 0; n < kPer; ++n) {
    const int e = threadIdx.x + n * kFactorThreads, r = e % TILE, c = e / TILE;
    out[n] = PanelDot<T, TILE>(sm.a, sm.b, r, c, min(c + 1, bk)) * sm.d[c < bk ? c : 0];
  }
#pragma unroll
  for (int n = 0; n < kPer; ++n) {
    const int e = threadIdx.x + n * kFactorThreads, r = e % TILE, c = e / TILE;
    if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, out[n]);
  }
  Signal(f.tile_state + StateIdx(g, i, k), kFinal);
}

// Lower part of a b x b diagonal tile held transposed in shared memory, back to its front.
template <typename T, int TILE>
__device__ __forceinline__ void StoreDiagLower(T* Fs, int m, int r0, int b, const T* a) {
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    if (r < b && c < b && r >= c) St(Fs + (r0 + r) + int64_t(r0 + c) * m, a[c * TILE + r]);
  }
}

// Per-phase time of a traced chain task, summed over its steps into record slots 4 .. 7 (thread 0;
// `ready` is the task's trace record + 1): 0 waits, 1 tile loads, 2 panel solve and diagonal
// update, 3 diagonal factorization.
struct ChainClock {
  unsigned long long* ready;
  unsigned long long last = 0;
  __device__ explicit ChainClock(unsigned long long* r) : ready(r) {
    if (ready && threadIdx.x == 0) last = Clock64Global();
  }
  __device__ void Lap(int phase) {
    if (ready && threadIdx.x == 0) {
      const unsigned long long now = Clock64Global();
      ready[3 + phase] += now - last;
      last = now;
    }
  }
};

// The critical chain of a front in one CTA (kTaskChain): the LDL^T of tile (0, 0), then for every
// panel k < np - 1 the panel solve of tile i = k + 1, the update of diagonal tile (i, i) by it,
// F_ii -= L_ik D_k L_ik^T (after every earlier panel's update of that tile, which other CTAs
// apply), and the LDL^T of (i, i).  The factor of the pivot tile stays in shared memory from one
// step to the next, so a step waits for and loads only the two tiles the other CTAs' updates
// produce.  (Applying panel k - 1's update of tile (i, k) in the chain as well, instead of waiting
// for it, measured slower at 50 cameras: the wait moves to the panel solve that update needs.)
// FP64: the chain keeps L_kk and D_k^-1 (the panel solve substitutes against L_kk) and leaves the
// explicit inverses of the diagonal factors to kTaskInverse.  FP32: the chain keeps L_kk^-1 and
// D_k^-1 (the panel solve is a product with the inverse, which DiagCore forms and stores).
template <typename T, int TILE>
__device__ void TaskChain(const FactorDev& f, int s, T* F, T* Linv, TileSmem<T, TILE>& sm,
                          int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  T* Fs = F + g.foff;
  bool ok = true;
  if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, 0, 0), 1, f.error);
  if (!CtaWait(ok, s_flag, ready)) return;
  if (ready && threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) ready[3 + q] = 0;
  ChainClock clk(ready);
  const int b0 = TileSize(g, 0, TILE);
  if constexpr (sizeof(T) == 8) {
    static_assert(sizeof(T) != 8 || TILE == 16, "the FP64 tile kernels are written for 16 x 16 tiles");
    __shared__ double s_rp[16];
    double* lk = sm.b;  // factor of the pivot tile (k, k)
    double* di = sm.e;  // the next diagonal tile
    LoadTileT<T, TILE>(Fs, g.m, 0, 0, b0, b0, lk);
    __syncthreads();
    clk.Lap(1);
    DiagLdltF64<16>(lk, b0, sm.d, s_rp);
    StoreDiagLower<T, TILE>(Fs, g.m, 0, b0, lk);
    Signal(f.tile_state + StateIdx(g, 0, 0), kFinal);
    clk.Lap(3);
    for (int k = 0; k + 1 < g.np; ++k) {
      const int i = k + 1;
      const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
      const int bi = TileSize(g, i, TILE), ri = TileStart(g, i, TILE);
      // F_ii is normally ready long before the panel tile (k+1, k), which waits on the update by
      // panel k - 1: its loads are issued into registers and land while that wait runs
      if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, i, i), 1 + k, f.error);
      if (!CtaWait(ok, s_flag)) return;
      T fii[TileEntriesPerThread<TILE>()];
      LoadTileRegs<T, TILE>(Fs, g.m, ri, ri, bi, bi, fii);
      if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, i, k), 1 + k, f.error);
      if (!CtaWait(ok, s_flag)) return;
      clk.Lap(0);
      LoadTileT<T, TILE>(Fs, g.m, ri, ck, bi, bk, sm.a);  // F_ik
      StoreTileRegs<T, TILE>(fii, di);
      __syncthreads();
      clk.Lap(1);
      PanelSolveSubstF64(sm.a, lk, sm.d, bi, bk, sm.c, sm.w);
      __syncthreads();
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
        const int r = e % TILE, c = e / TILE;
        if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, sm.c[c * TILE + r]);
      }
      Signal(f.tile_state + StateIdx(g, i, k), kFinal);
      // F_ii -= Y X^T (Y = X D), lower part
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
        const int r = e % TILE, c = e / TILE;
        if (r >= bi || c > r) continue;
        di[c * TILE + r] -= PanelDot<T, TILE>(sm.w, sm.c, r, c, bk);
      }
      __syncthreads();
      clk.Lap(2);
      DiagLdltF64<16>(di, bi, sm.d, s_rp);
      StoreDiagLower<T, TILE>(Fs, g.m, ri, bi, di);
      Signal(f.tile_state + StateIdx(g, i, i), kFinal);
      clk.Lap(3);
      double* tmp = lk;
      lk = di;
      di = tmp;
    }
  } else {
    LoadTileT<T, TILE>(Fs, g.m, 0, 0, b0, b0, sm.a);
    __syncthreads();
    clk.Lap(1);
    DiagCore<T, TILE>(f, g, s, 0, F, Linv, sm.a, sm);  // leaves L_00^-1 in sm.b
    for (int c = threadIdx.x; c < b0; c += blockDim.x) sm.d[c] = PivotReciprocal<T>(sm.a[c * TILE + c]);
    clk.Lap(3);
    for (int k = 0; k + 1 < g.np; ++k) {
      const int i = k + 1;
      const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
      const int bi = TileSize(g, i, TILE), ri = TileStart(g, i, TILE);
      // F_ii's loads are issued into registers while the wait for the panel tile runs (as FP64)
      if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, i, i), 1 + k, f.error);
      if (!CtaWait(ok, s_flag)) return;
      T fii[TileEntriesPerThread<TILE>()];
      LoadTileRegs<T, TILE>(Fs, g.m, ri, ri, bi, bi, fii);
      if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, i, k), 1 + k, f.error);
      if (!CtaWait(ok, s_flag)) return;
      clk.Lap(0);
      LoadTileT<T, TILE>(Fs, g.m, ri, ck, bi, bk, sm.a);  // F_ik
      __syncthreads();
      clk.Lap(1);
      // L_ik (r, c) = sum_{q <= c} F(r, q) Li(c, q) / D_c, into c[] (transposed) and the front, and
      // L_ik D into w[]
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
        const int r = e % TILE, c = e / TILE;
        const T acc = PanelDot<T, TILE>(sm.a, sm.b, r, c, min(c + 1, bk));
        const T l = (r < bi && c < bk) ? acc * sm.d[c < bk ? c : 0] : T(0);
        sm.c[c * TILE + r] = l;
        sm.w[c * TILE + r] = (r < bi && c < bk) ? acc : T(0);  // F Li^T = L D
        if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, l);
      }
      Signal(f.tile_state + StateIdx(g, i, k), kFinal);
      StoreTileRegs<T, TILE>(fii, sm.a);  // F_ii
      __syncthreads();
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
        const int r = e % TILE, c = e / TILE;
        if (r >= bi || c > r) continue;
        sm.a[c * TILE + r] -= PanelDot<T, TILE>(sm.w, sm.c, r, c, bk);
      }
      __syncthreads();
      clk.Lap(2);
      DiagCore<T, TILE>(f, g, s, i, F, Linv, sm.a, sm);
      for (int c = threadIdx.x; c < bi; c += blockDim.x) sm.d[c] = PivotReciprocal<T>(sm.a[c * TILE + c]);
      clk.Lap(3);
    }
  }
}

// The explicit inverse of diagonal tile k's unit lower factor (kTaskInverse; FP64 chains), for the
// triangular solves.
template <typename T, int TILE>
__device__ void TaskInverse(const FactorDev& f, int s, int k, const T* F, T* Linv, TileSmem<T, TILE>& sm,
                            int* s_flag, unsigned long long* ready) {
  if constexpr (sizeof(T) == 8) {
    const Geom g = FrontGeom(f, s);
    bool ok = true;
    if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, k, k), kFinal, f.error);
    if (!CtaWait(ok, s_flag, ready)) return;
    const int b = TileSize(g, k, TILE), c0 = TileStart(g, k, TILE);
    LoadTileT<T, TILE>(F + g.foff, g.m, c0, c0, b, b, sm.a);
    __syncthreads();
    UnitLowerInverse<double, 16>(sm.a, b, sm.b);
    T* Lk = Linv + f.linv_base[s] + int64_t(k) * TILE * TILE;
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) St(Lk + e, sm.b[e]);
  } else {
    if (threadIdx.x == 0) atomicExch(f.error, kDevBadTask);
  }
}

template <typename T, int TILE>
__device__ void TaskUpdate(const FactorDev& f, int s, int i, int j, int k, T* F,
                           TileSmem<T, TILE>& sm, int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  bool ok = true;
  // The panel tile (j, k) is the one that usually comes last (on a front's critical path it is
  // the chain's panel solve): the target and L_ik are waited for, loaded and scaled by D first.
  if (threadIdx.x == 0) {
    ok = WaitAtLeast(f.tile_state + StateIdx(g, i, k), kFinal, f.error) &&
         WaitAtLeast(f.tile_state + StateIdx(g, i, j), 1 + k, f.error);
  }
  if (!CtaWait(ok, s_flag, ready)) return;
  const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
  const int bi = TileSize(g, i, TILE), ri = TileStart(g, i, TILE);
  const int bj = TileSize(g, j, TILE), rj = TileStart(g, j, TILE);
  T* Fs = F + g.foff;
  constexpr int kPer = TileEntriesPerThread<TILE>();
  T cdst[kPer];
#pragma unroll
  for (int n = 0; n < kPer; ++n) {
    const int e = threadIdx.x + n * kFactorThreads, r = e % TILE, c = e / TILE;
    cdst[n] = (r < bi && c < bj) ? Ld(Fs + (ri + r) + int64_t(rj + c) * g.m) : T(0);
  }
  LoadTileT<T, TILE>(Fs, g.m, ri, ck, bi, bk, sm.a);  // L_ik ((k, k) is final before it)
  for (int c = threadIdx.x; c < bk; c += blockDim.x) sm.d[c] = Ld(Fs + int64_t(ck + c) * (g.m + 1));
  __syncthreads();
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int c = e / TILE;
    if (c < bk) sm.a[e] *= sm.d[c];  // L_ik D
  }
  if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, j, k), kFinal, f.error);
  if (!CtaWait(ok, s_flag)) return;
  LoadTileT<T, TILE>(Fs, g.m, rj, ck, bj, bk, sm.b);  // L_jk
  __syncthreads();
#pragma unroll
  for (int n = 0; n < kPer; ++n) {
    const int e = threadIdx.x + n * kFactorThreads, r = e % TILE, c = e / TILE;
    if (r >= bi || c >= bj || (i == j && r < c)) continue;
    St(Fs + (ri + r) + int64_t(rj + c) * g.m, cdst[n] - PanelDot<T, TILE>(sm.a, sm.b, r, c, bk));
  }
  Signal(f.tile_state + StateIdx(g, i, j), 2 + k);
}

// ---- Tensor-core trailing updates (FP32 fronts).  A column of up to four row tiles i0 ..
// i0 + cnt - 1 takes panel k's update as one product: C -= (L_ik D_k) L_jk^T, M = 128 rows (the
// four tiles), N = 32 (tile column j), K = the panel's width, on the tcgen05 tensor cores in
// kind::tf32 with the three-pass split x = hi + lo (A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32-level
// accuracy), the accumulator in the CTA's 32 TMEM columns.  The operands are staged by the threads
// in the canonical K-major layout (no swizzle) in the CTA's shared tile storage; thread 0 issues the
// twelve MMAs and commits them to an mbarrier; warp w reads TMEM lanes 32 w .. 32 w + 31 (tile
// i0 + w) and subtracts them from the front.  The target and L_ik are waited for and staged before
// the usually later panel tile L_jk.
constexpr int kTcUpdRows = tc::kTcRows;                         // 4 tiles of 32
constexpr size_t kTcUpdBytes = size_t(kTcUpdRows) * 32 * 4 * 2  // A hi / lo
                               + size_t(32) * 32 * 4 * 2;       // B hi / lo
constexpr int kTcUpdCols = 32;                                  // TMEM columns per CTA

template <typename T, int TILE>
__device__ void TaskUpdateTc(const FactorDev& f, int s, int i0, int cnt, int j, int k, T* F, unsigned char* smem,
                             uint32_t tmem, uint64_t* bar, uint32_t& phase, int* s_flag,
                             unsigned long long* ready) {
  static_assert(TILE == 32 && sizeof(T) == 4, "tensor-core updates are for FP32 tiles of 32");
  using namespace tc;
  const Geom g = FrontGeom(f, s);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  bool ok = true;
  if (tid == 0)
    for (int q = 0; q < cnt && ok; ++q)
      ok = WaitAtLeast(f.tile_state + StateIdx(g, i0 + q, k), kFinal, f.error) &&
           WaitAtLeast(f.tile_state + StateIdx(g, i0 + q, j), 1 + k, f.error);
  if (!CtaWait(ok, s_flag, ready)) return;
  const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
  const int bj = TileSize(g, j, TILE), rj = TileStart(g, j, TILE);
  T* Fs = F + g.foff;
  unsigned char* a_hi = smem;
  unsigned char* a_lo = a_hi + kTcUpdRows * 32 * 4;
  unsigned char* b_hi = a_lo + kTcUpdRows * 32 * 4;
  unsigned char* b_lo = b_hi + 32 * 32 * 4;
  // A row tid: row tid % 32 of tile i0 + warp, times D_k (lane q of the warp holds d_q)
  {
    const int it = i0 + warp;
    const bool in_tile = warp < cnt && lane < TileSize(g, it < g.nt ? it : 0, TILE);
    const float dq = lane < bk ? Ld(Fs + int64_t(ck + lane) * (g.m + 1)) : 0.f;
    const T* arow = Fs + (in_tile ? TileStart(g, it, TILE) + lane : 0) + int64_t(ck) * g.m;
#pragma unroll
    for (int q4 = 0; q4 < 32; q4 += 4) {
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float d = __shfl_sync(0xffffffffu, dq, q4 + u);
        v[u] = (in_tile && q4 + u < bk) ? Ld(arow + int64_t(q4 + u) * g.m) * d : 0.f;
      }
      float4 hi4, lo4;
      hi4.x = TfHi(v[0]);
      hi4.y = TfHi(v[1]);
      hi4.z = TfHi(v[2]);
      hi4.w = TfHi(v[3]);
      lo4.x = v[0] - hi4.x;
      lo4.y = v[1] - hi4.y;
      lo4.z = v[2] - hi4.z;
      lo4.w = v[3] - hi4.w;
      const uint32_t o = ChunkOffset(tid, q4);
      *reinterpret_cast<float4*>(a_hi + o) = hi4;
      *reinterpret_cast<float4*>(a_lo + o) = lo4;
    }
  }
  if (tid == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, j, k), kFinal, f.error);
  if (!CtaWait(ok, s_flag)) return;
  // B row n = row n of L_jk (the product's column n), K along the row; thread: row tid / 4, 8 k
  {
    const int n = tid >> 2, qb = (tid & 3) * 8;
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      v[u] = (n < bj && qb + u < bk) ? Ld(Fs + (rj + n) + int64_t(ck + qb + u) * g.m) : 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float4 hi4, lo4;
      hi4.x = TfHi(v[4 * h]);
      hi4.y = TfHi(v[4 * h + 1]);
      hi4.z = TfHi(v[4 * h + 2]);
      hi4.w = TfHi(v[4 * h + 3]);
      lo4.x = v[4 * h] - hi4.x;
      lo4.y = v[4 * h + 1] - hi4.y;
      lo4.z = v[4 * h + 2] - hi4.z;
      lo4.w = v[4 * h + 3] - hi4.w;
      const uint32_t o = ChunkOffset(n, qb + 4 * h);
      *reinterpret_cast<float4*>(b_hi + o) = hi4;
      *reinterpret_cast<float4*>(b_lo + o) = lo4;
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (tid == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t idesc = InstrDesc(32);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {  // K = 8 per MMA: two core matrices along K
      const uint32_t off = uint32_t(kk * 256);
      MmaTf32(tmem, SmemDesc(SmemAddr(a_hi) + off), SmemDesc(SmemAddr(b_hi) + off), idesc, kk > 0 ? 1u : 0u);
      MmaTf32(tmem, SmemDesc(SmemAddr(a_hi) + off), SmemDesc(SmemAddr(b_lo) + off), idesc, 1u);
      MmaTf32(tmem, SmemDesc(SmemAddr(a_lo) + off), SmemDesc(SmemAddr(b_hi) + off), idesc, 1u);
    }
    MmaCommit(bar);
  }
  const bool done = __all_sync(0xffffffffu, MbarWait(bar, phase));  // warp-uniform for tcgen05.ld
  if (!done) {
    if (lane == 0) atomicExch(f.error, kDevSpinTimeout);
    (void)MbarWait(bar, phase);  // a second (capped) chance before the storage is reused
  }
  phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (done && warp < cnt) {
    const int it = i0 + warp, ri = TileStart(g, it, TILE), bi = TileSize(g, it, TILE);
#pragma unroll
    for (int c0 = 0; c0 < 32; c0 += 16) {
      uint32_t v[16];
      TmemLoad16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int c = c0 + u;
        if (lane < bi && c < bj && (it != j || lane >= c)) {
          T* dst = Fs + (ri + lane) + int64_t(rj + c) * g.m;
          St(dst, Ld(dst) - __uint_as_float(v[u]));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    for (int q = 0; q < cnt; ++q) atomicExch(f.tile_state + StateIdx(g, i0 + q, j), 2 + k);
  }
}

template <typename T, int TILE, int MINB>
__global__ void __launch_bounds__(kFactorThreads, MINB) FactorKernel(FactorDev f, const T* A,
                                                               const double* damping, T* F,
                                                               T* Linv) {
  // the tile storage; FP32 kernels also stage tensor-core update operands in it (one task at a time)
  constexpr bool kTc = sizeof(T) == 4;
  constexpr size_t kSmemBytes = (kTc && kTcUpdBytes > sizeof(TileSmem<T, TILE>)) ? kTcUpdBytes : sizeof(TileSmem<T, TILE>);
  __shared__ __align__(1024) unsigned char smem_raw[kSmemBytes];
  TileSmem<T, TILE>& sm = *reinterpret_cast<TileSmem<T, TILE>*>(smem_raw);
  __shared__ int s_task, s_next, s_ok, s_flag;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  if (f.gate && *f.gate == 0) return;
  A += int64_t(f.st->init_idx) * f.a_stride;
  uint32_t phase = 0;
  if constexpr (kTc) {
    if ((threadIdx.x >> 5) == 0) tc::TmemAlloc(&s_tmem, kTcUpdCols);
    if (threadIdx.x == 0) tc::MbarInit(&s_bar);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  // A chain task runs on an SM of its own where it can (its FP64 work otherwise queues behind the
  // co-resident CTAs' updates on the SM's shared FP64 pipe): its CTA flags the SM, and the SM's
  // other CTAs leave the kernel after their claimed tasks.  At most f.iso_limit SMs are flagged,
  // so the other tasks keep CTAs to run on.
  const unsigned smid = SmId();
  int* sm_flag = (f.sm_flags && smid < unsigned(kSmFlagSlots)) ? f.sm_flags + smid : nullptr;
  __shared__ int s_chain_cta;
  if (threadIdx.x == 0) {
    s_chain_cta = 0;
    s_next = atomicAdd(f.counters, 1);
  }
  for (;;) {
    if (threadIdx.x == 0) {
      s_ok = LoadVolatile(f.error) == 0;
      s_task = s_ok ? s_next : f.ntasks;
      // fetch the following task now so that the atomic's latency overlaps this task; not under a
      // chain task, which waits on tasks after it in the list: one of them, claimed here and held
      // until the chain ends, would never run
      s_next = -1;
      if (s_task < f.ntasks) {
        if (f.tasks[s_task].x == kTaskChain) {
          s_chain_cta = 1;
          if (sm_flag && LoadVolatile(sm_flag) == 0 && atomicAdd(f.sm_flags + kSmFlagSlots, 1) < f.iso_limit)
            atomicExch(sm_flag, 1);
        } else if (s_chain_cta || !sm_flag || LoadVolatile(sm_flag) == 0) {
          s_next = atomicAdd(f.counters, 1);
        }
      }
    }
    __syncthreads();
    const int t = s_task;
    if (t >= f.ntasks) break;
    const int4 task = f.tasks[t];
    const int i = task.z >> 16, j = task.z & 0xffff, k = task.w & 0xfffff;
    unsigned long long* ready = f.trace ? f.trace + 8 * int64_t(t) + 1 : nullptr;
    if (f.trace && threadIdx.x == 0) {
      f.trace[8 * int64_t(t)] = Clock64Global();
      f.trace[8 * int64_t(t) + 3] = SmId();
    }
    switch (task.x) {
      case kTaskAssemble: TaskAssemble<T, TILE>(f, task.y, j, A, damping, F, &s_flag, ready); break;
      case kTaskDiag: TaskDiag<T, TILE>(f, task.y, k, F, Linv, sm, &s_flag, ready); break;
      case kTaskTrsm: TaskTrsm<T, TILE>(f, task.y, i, k, F, Linv, sm, &s_flag, ready); break;
      case kTaskUpdate: TaskUpdate<T, TILE>(f, task.y, i, j, k, F, sm, &s_flag, ready); break;
      case kTaskChain: TaskChain<T, TILE>(f, task.y, F, Linv, sm, &s_flag, ready); break;
      case kTaskInverse: TaskInverse<T, TILE>(f, task.y, k, F, Linv, sm, &s_flag, ready); break;
      case kTaskUpdateTc:
        if constexpr (kTc) {
          TaskUpdateTc<T, TILE>(f, task.y, i, task.w >> 20, j, task.w & 0xfffff, F, smem_raw, s_tmem, &s_bar,
                                phase, &s_flag, ready);
          break;
        }
        [[fallthrough]];
      default:
        if (threadIdx.x == 0) atomicExch(f.error, kDevBadTask);
    }
    __syncthreads();
    if (f.trace && threadIdx.x == 0) f.trace[8 * int64_t(t) + 2] = Clock64Global();
    if (threadIdx.x == 0 && s_next < 0) {
      // after a chain, or on an SM given to a chain (this CTA then leaves)
      s_next = (s_chain_cta || !sm_flag || LoadVolatile(sm_flag) == 0) ? atomicAdd(f.counters, 1) : f.ntasks;
    }
  }
  if constexpr (kTc) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::TmemFree(s_tmem, kTcUpdCols);
  }
}

// ---------------------------------------------------------------------------------------------
// Triangular solves: task t < ns is the forward solve of front t (postorder), task ns + q the
// backward solve of front ns - 1 - q (reverse postorder).  Dynamic shared memory: max_m scalars.
// Within a front the row tiles (the factorization's pivot tiles, then the update rows in tiles of
// the same height) belong to the CTA's warps in turn (tile i to warp i mod warps).  A pivot tile is
// solved by its warp with the inverse of its unit lower factor that the factorization kept (a
// product: independent rows instead of a chain of TILE dependent multiply-adds) as soon as the
// contributions of every earlier tile are in, and published through a counter in shared memory;
// each warp applies each published tile to its own row tiles, the tile after it first.  No CTA
// barrier sits between tiles, so the solve of the next tile overlaps the bulk of the updates: on a
// 450-wide FP64 front the bulk is ~100k multiply-adds, about 30 us of one SM's FP64 pipe.
// ---------------------------------------------------------------------------------------------
constexpr int kSolveThreads = 256;
// Dynamic shared memory of a solve CTA: the largest front's scalars, plus one warp's width of
// slack (every read is bounded by the front; the slack only keeps a short last tile's lanes inside
// the allocation), then one tile of received values per warp (solves shared by several CTAs).
template <typename T>
size_t SolveSmemBytes(int max_m) {
  return (size_t(max_m) + 32 + size_t(kSolveThreads / 32) * 32) * sizeof(T);
}

// sum_{c = c0}^{c1 - 1} a[c * stride] x[c] with four independent accumulation chains, added in a
// fixed order.
template <typename T>
__device__ __forceinline__ T RowDot(const T* a, int64_t stride, const T* x, int c0, int c1) {
  T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
  int c = c0;
  for (; c + 4 <= c1; c += 4) {
    s0 += Ld(a + int64_t(c) * stride) * x[c];
    s1 += Ld(a + int64_t(c + 1) * stride) * x[c + 1];
    s2 += Ld(a + int64_t(c + 2) * stride) * x[c + 2];
    s3 += Ld(a + int64_t(c + 3) * stride) * x[c + 3];
  }
  for (; c < c1; ++c) s0 += Ld(a + int64_t(c) * stride) * x[c];
  return (s0 + s1) + (s2 + s3);
}

// Spin (capped) until the CTA's count of published tiles reaches n.  On the cap the error word is
// set and the caller goes on (with a wrong result, which the error word reports), so that every
// warp still reaches the CTA's barriers.
__device__ __forceinline__ void WaitPublished(const volatile int* s_done, int n, int* err) {
  unsigned it = 0;
  while (*s_done < n) {
    if (++it > kSpinLimit) {
      atomicExch(err, kDevSpinTimeout);
      break;
    }
  }
  __threadfence_block();
}
// Publish: every lane's shared-memory writes before the counter (warp-wide call).
__device__ __forceinline__ void Publish(volatile int* s_done, int n) {
  __threadfence_block();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) *s_done = n;
}

// One warp's share of a TILE x TILE block: lane = (row, part), each part takes TILE / kSplit
// columns (two parts of 8 for FP64 tiles, one of 32 for FP32).  Loaded into registers ahead of
// use, so that the loads of the next block are in flight while the warp waits or computes.
template <typename T, int TILE>
struct WarpBlock {
  static constexpr int kSplit = 32 / TILE, kCols = TILE / kSplit;
  T v[kCols];
  int n;  // columns of the block: x is read below n only (a short last tile may end the front)
  // a(r, c) = base[r * rs + c * cs] for r < br, c < bc (zero elsewhere)
  __device__ __forceinline__ void Load(const T* base, int64_t rs, int64_t cs, int br, int bc) {
    const int lane = threadIdx.x & 31, row = lane % TILE, part = lane / TILE;
    n = bc;
#pragma unroll
    for (int q = 0; q < kCols; ++q) {
      const int c = part * kCols + q;
      v[q] = (row < br && c < bc) ? __ldg(base + row * rs + c * cs) : T(0);
    }
  }
  // sum_{c < n} a(row, c) x[c] over the whole row (the parts' sums added by a shuffle), two chains
  __device__ __forceinline__ T Dot(const T* x) const {
    const int part = (threadIdx.x & 31) / TILE;
    T s0 = T(0), s1 = T(0);
#pragma unroll
    for (int q = 0; q < kCols; q += 2) {
      const int c = part * kCols + q;
      if (c < n) s0 += v[q] * x[c];
      if (q + 1 < kCols && c + 1 < n) s1 += v[q + 1] * x[c + 1];
    }
    T acc = s0 + s1;
    if (kSplit == 2) acc += __shfl_xor_sync(0xffffffffu, acc, 16);
    return acc;
  }
};

// Forward solve L y = x of a front's pivot columns (y over the pivot rows; the update rows get
// x - L_21 y), in place in xs.  Every warp of the CTA calls it; s_done is 0 and the CTA barrier
// behind the caller's writes of xs.  A warp loads the blocks of its next tile (and, for the tile
// it solves next, that tile's inverse) before it waits for the tile they multiply.
template <typename T, int TILE>
__device__ void ForwardFront(const Geom& g, const T* Fs, const T* Li, T* xs, volatile int* s_done, int* err) {
  const int m = g.m, np = g.np, nt = g.nt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int row = lane % TILE, part = lane / TILE;
  WarpBlock<T, TILE> inv, cur, nxt;
  // y_i = L_ii^-1 x_i (the inverse, with (r, c) at c * TILE + r, in inv)
  auto solve = [&](int i) {
    const int ri = i * TILE, bi = min(TILE, g.w - ri);
    const T y = inv.Dot(xs + ri);
    __syncwarp();
    if (part == 0 && row < bi) xs[ri + row] = y;
    Publish(s_done, i + 1);
  };
  auto load_inv = [&](int i) {
    const int bi = min(TILE, g.w - i * TILE);
    inv.Load(Li + int64_t(i) * TILE * TILE, 1, TILE, bi, bi);
  };
  if (warp == 0) {
    load_inv(0);
    solve(0);
  }
  for (int j = 0; j < np; ++j) {
    const int cj = j * TILE, bj = min(TILE, g.w - cj);
    // this warp's row tiles after j, in order (tile j + 1 first when it is this warp's)
    int i = j + 1 + ((warp - (j + 1)) % nw + nw) % nw;
    if (i < nt) cur.Load(Fs + TileStart(g, i, TILE) + int64_t(cj) * m, 1, m, TileSize(g, i, TILE), bj);
    if (i == j + 1 && i < np) load_inv(i);
    WaitPublished(s_done, j + 1, err);
    for (; i < nt; i += nw) {
      const int ri = TileStart(g, i, TILE), bi = TileSize(g, i, TILE);
      if (i + nw < nt) nxt.Load(Fs + TileStart(g, i + nw, TILE) + int64_t(cj) * m, 1, m, TileSize(g, i + nw, TILE), bj);
      const T u = cur.Dot(xs + cj);
      if (part == 0 && row < bi) xs[ri + row] -= u;
      if (i == j + 1 && i < np) {
        __syncwarp();
        solve(i);
      }
      cur = nxt;
    }
  }
  __syncthreads();
}

// Backward solve L^T x = z over a front's pivot columns, in place in xs[0, w) (z there on entry:
// D^-1 y minus the update rows' contributions).  Mirror of ForwardFront: tiles from the last
// down, tile j to warp j mod warps; the blocks are L_ij^T, lane row = column of L_ij.
template <typename T, int TILE>
__device__ void BackwardFront(const Geom& g, const T* Fs, const T* Li, T* xs, volatile int* s_done, int* err) {
  const int m = g.m, np = g.np;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int row = lane % TILE, part = lane / TILE;
  WarpBlock<T, TILE> inv, cur, nxt;
  // x_j = L_jj^-T z_j: x(c) = sum_r Li(r, c) z(r), Li(r, c) at c * TILE + r
  auto solve = [&](int j) {
    const int cj = j * TILE, bj = min(TILE, g.w - cj);
    const T x = inv.Dot(xs + cj);
    __syncwarp();
    if (part == 0 && row < bj) xs[cj + row] = x;
    Publish(s_done, np - j);
  };
  auto load_inv = [&](int j) {
    const int bj = min(TILE, g.w - j * TILE);
    inv.Load(Li + int64_t(j) * TILE * TILE, TILE, 1, bj, bj);
  };
  if (warp == (np - 1) % nw) {
    load_inv(np - 1);
    solve(np - 1);
  }
  for (int i = np - 1; i >= 1; --i) {
    const int ri = i * TILE, bi = min(TILE, g.w - ri);
    // this warp's tiles before i, from i - 1 down (tile i - 1 first when it is this warp's)
    int j = i - 1;
    j -= ((j - warp) % nw + nw) % nw;
    // block (c, r) = L_ij(r, c) = Fs[(ri + r) + (cj + c) m]
    if (j >= 0) cur.Load(Fs + ri + int64_t(j * TILE) * m, m, 1, min(TILE, g.w - j * TILE), bi);
    if (j == i - 1) load_inv(j);
    WaitPublished(s_done, np - i, err);
    for (; j >= 0; j -= nw) {
      const int cj = j * TILE, bj = min(TILE, g.w - cj);
      const int jn = j - nw;
      if (jn >= 0) nxt.Load(Fs + ri + int64_t(jn * TILE) * m, m, 1, min(TILE, g.w - jn * TILE), bi);
      const T u = cur.Dot(xs + ri);
      if (part == 0 && row < bj) xs[cj + row] -= u;
      if (j == i - 1) {
        __syncwarp();
        solve(j);
      }
      cur = nxt;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------------------------
// Solves of wide fronts by several CTAs.  One CTA's FP64 pipe caps a front's solve (a 450-wide
// front's ~100k multiply-adds per direction take ~37 us of one SM), so a front with more tiles than
// a CTA has warps is split: pivot-block CTAs own kSolveBlockTiles consecutive pivot tiles each (one
// per warp: the chain steps inside a block pass through shared memory), update CTAs own the
// update-row tiles (forward only; tile np + u + ku l to CTA u).  Values a CTA needs from another
// CTA go through global memory without flags: the exchange buffers (ysave for the forward y, xb
// for the backward x, front-local order) hold an unset pattern — a signalling NaN, which no
// arithmetic produces — until the owner stores the value, and a reader polls each value until it
// is set.  The buffers are reset to the pattern before every solve launch.  Every CTA waits only on
// CTAs with lower task numbers (forward: earlier blocks; backward: later blocks, numbered first),
// so the persistent task order cannot deadlock.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ bool IsUnset(double v) {
  return __double_as_longlong(v) == static_cast<long long>(0x7FF4DEAD0BADF00DULL);
}
__device__ __forceinline__ bool IsUnset(float v) { return __float_as_uint(v) == 0x7FA5DEADu; }
__device__ __forceinline__ double LdRelaxed(const double* p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ float LdRelaxed(const float* p) {
  float v;
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void StRelaxed(double* p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" : : "l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void StRelaxed(float* p, float v) {
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" : : "l"(p), "f"(v) : "memory");
}

// First attempt at the bn values of a published tile (lane l reads value l mod TILE).
template <typename T, int TILE>
__device__ __forceinline__ T PeekTile(const T* p, int bn) {
  const int l = (threadIdx.x & 31) % TILE;
  return l < bn ? LdRelaxed(p + l) : T(0);
}
// Spin (capped, and given up when the error word is set) until all bn values of the tile are set,
// starting from the PeekTile value v, then copy them to the warp's scratch (zero past bn).
template <typename T, int TILE>
__device__ __forceinline__ void ReceiveTile(const T* p, int bn, T v, T* scratch, int* err) {
  const int lane = threadIdx.x & 31, l = lane % TILE;
  const bool need = l < bn;
  unsigned it = 0;
  while (!__all_sync(0xffffffffu, !need || !IsUnset(v))) {
    if (++it > kSpinLimit || ((it & 255u) == 0 && LoadVolatile(err) != 0)) {
      if (lane == 0 && it > kSpinLimit) atomicExch(err, kDevSpinTimeout);
      break;
    }
    if (need && IsUnset(v)) v = LdRelaxed(p + l);
  }
  if (lane < TILE) scratch[lane] = need ? v : T(0);
  __syncwarp();
}

// Forward solve of front g by CTA `cta` of kp pivot-block CTAs and ku update CTAs (xs holds the
// CTA's own rows: b plus the children's contributions; yx = the front's forward exchange values).
// Warp q of pivot CTA c takes pivot tile c kSolveBlockTiles + q: it applies every earlier column
// (received from global memory for earlier blocks, from shared memory inside its block), solves
// the tile and stores y to shared memory and to yx.  Update CTA warps take update tiles and apply
// every pivot column.
template <typename T, int TILE>
__device__ void ForwardMulti(const Geom& g, const T* Fs, const T* Li, T* xs, T* yx, T* scratch,
                             volatile int* s_done, int cta, int kp, int ku, int* err) {
  const int m = g.m, np = g.np, nt = g.nt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row = lane % TILE, part = lane / TILE;
  if (warp >= kSolveBlockTiles) return;
  WarpBlock<T, TILE> inv, cur, nxt;
  if (cta < kp) {
    const int b0 = cta * kSolveBlockTiles, i = b0 + warp;
    if (i >= np) return;
    const int ri = i * TILE, bi = min(TILE, g.w - ri);
    inv.Load(Li + int64_t(i) * TILE * TILE, 1, TILE, bi, bi);
    if (i > 0) cur.Load(Fs + ri, 1, m, bi, min(TILE, g.w));
    T pv = b0 > 0 ? PeekTile<T, TILE>(yx, min(TILE, g.w)) : T(0);
    for (int j = 0; j < i; ++j) {
      const int cj = j * TILE, bj = min(TILE, g.w - cj);
      const T* x;
      if (j < b0) {
        ReceiveTile<T, TILE>(yx + cj, bj, pv, scratch, err);
        x = scratch;
        if (j + 1 < b0) pv = PeekTile<T, TILE>(yx + cj + TILE, min(TILE, g.w - cj - TILE));
      } else {
        WaitPublished(s_done, j - b0 + 1, err);
        x = xs + cj;
      }
      if (j + 1 < i) nxt.Load(Fs + ri + int64_t(cj + TILE) * m, 1, m, bi, min(TILE, g.w - cj - TILE));
      const T u = cur.Dot(x);
      if (part == 0 && row < bi) xs[ri + row] -= u;
      cur = nxt;
      __syncwarp();
    }
    const T y = inv.Dot(xs + ri);
    __syncwarp();
    if (part == 0 && row < bi) {
      xs[ri + row] = y;
      StRelaxed(yx + ri + row, y);
    }
    Publish(s_done, warp + 1);
    return;
  }
  // update CTA: tiles np + u + ku (warp + kSolveBlockTiles r), r = 0, 1, ...
  const int u = cta - kp, step = ku * kSolveBlockTiles;
  const int i0 = np + u + ku * warp;
  if (i0 >= nt) return;
  T pv = PeekTile<T, TILE>(yx, min(TILE, g.w));
  for (int j = 0; j < np; ++j) {
    const int cj = j * TILE, bj = min(TILE, g.w - cj);
    cur.Load(Fs + TileStart(g, i0, TILE) + int64_t(cj) * m, 1, m, TileSize(g, i0, TILE), bj);
    ReceiveTile<T, TILE>(yx + cj, bj, pv, scratch, err);
    if (j + 1 < np) pv = PeekTile<T, TILE>(yx + cj + TILE, min(TILE, g.w - cj - TILE));
    for (int i = i0; i < nt; i += step) {
      const int ri = TileStart(g, i, TILE), bi = TileSize(g, i, TILE);
      if (i + step < nt) nxt.Load(Fs + TileStart(g, i + step, TILE) + int64_t(cj) * m, 1, m, TileSize(g, i + step, TILE), bj);
      const T v = cur.Dot(scratch);
      if (part == 0 && row < bi) xs[ri + row] -= v;
      cur = nxt;
    }
    __syncwarp();
  }
}

// Backward solve of front g's pivot columns by pivot-block CTA `blk` (xs holds its rows' z: D^-1 y
// minus the update rows' contributions; xe = the front's backward exchange values).  Warp q takes
// tile blk kSolveBlockTiles + q and applies L_ij^T x_i of every later tile i (received from global
// memory for later blocks, from shared memory inside its block), then solves it.
template <typename T, int TILE>
__device__ void BackwardMulti(const Geom& g, const T* Fs, const T* Li, T* xs, T* xe, T* scratch,
                              volatile int* s_done, int blk, int* err) {
  const int m = g.m, np = g.np;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row = lane % TILE, part = lane / TILE;
  if (warp >= kSolveBlockTiles) return;
  const int b0 = blk * kSolveBlockTiles, j = b0 + warp;
  const int top = min(b0 + kSolveBlockTiles, np) - 1;  // the block's last tile, published first
  if (j > top) return;
  const int cj = j * TILE, bj = min(TILE, g.w - cj);
  WarpBlock<T, TILE> inv, cur, nxt;
  inv.Load(Li + int64_t(j) * TILE * TILE, TILE, 1, bj, bj);
  if (j < np - 1) cur.Load(Fs + (np - 1) * TILE + int64_t(cj) * m, m, 1, bj, min(TILE, g.w - (np - 1) * TILE));
  T pv = top < np - 1 ? PeekTile<T, TILE>(xe + (np - 1) * TILE, min(TILE, g.w - (np - 1) * TILE)) : T(0);
  for (int i = np - 1; i > j; --i) {
    const int ri = i * TILE, bi = min(TILE, g.w - ri);
    const T* x;
    if (i > top) {
      ReceiveTile<T, TILE>(xe + ri, bi, pv, scratch, err);
      x = scratch;
      if (i - 1 > top) pv = PeekTile<T, TILE>(xe + ri - TILE, TILE);
    } else {
      WaitPublished(s_done, top - i + 1, err);
      x = xs + ri;
    }
    if (i - 1 > j) nxt.Load(Fs + ri - TILE + int64_t(cj) * m, m, 1, bj, TILE);
    const T u = cur.Dot(x);
    if (part == 0 && row < bj) xs[cj + row] -= u;
    cur = nxt;
    __syncwarp();
  }
  const T x = inv.Dot(xs + cj);
  __syncwarp();
  if (part == 0 && row < bj) {
    xs[cj + row] = x;
    StRelaxed(xe + cj + row, x);
  }
  Publish(s_done, top - j + 1);
}

// Rows of a front a solve CTA owns: all of them for a one-CTA solve, else its block's pivot rows
// (pivot CTA) or its update tiles' rows (update CTA).
__device__ __forceinline__ bool OwnsRow(const Geom& g, int tile, int q, int cta, int kp, int ku) {
  if (kp == 0) return true;
  if (cta < kp) return q < g.w && q / (tile * kSolveBlockTiles) == cta;
  return q >= g.w && ((q - g.w) / tile) % ku == cta - kp;
}

template <typename T>
__global__ void __launch_bounds__(kSolveThreads) SolveKernel(FactorDev f, const T* F, const T* Linv,
                                                              const T* b, T* ycon, T* ysave, T* xperm,
                                                              T* x, T* xb) {
  constexpr int kTile = sizeof(T) == 8 ? kFactorTileF64 : kFactorTileF32;
  static_assert(kTile <= 32 && kSolveThreads >= 32, "warp 0 holds a tile's rows");
  extern __shared__ unsigned char smem_raw[];
  T* xs = reinterpret_cast<T*>(smem_raw);
  T* scratch = xs + (f.max_m + 32) + (threadIdx.x >> 5) * 32;
  __shared__ int s_task, s_ok, s_flag, s_done;
  int* fwd_done = f.front_flags;
  int* bwd_done = f.front_flags + f.ns;
  if (f.gate && *f.gate == 0) return;
  b += int64_t(f.st->init_idx) * f.b_stride;
  const bool split = f.solve_front != nullptr;
  const int nfwd = split ? f.solve_nf : f.ns;
  const int ntasks = split ? f.solve_nf + f.solve_nb : 2 * f.ns;
  // CTAs that signal a front's forward / backward completion
  auto fwd_ctas = [&](int s) { return split && f.solve_kp[s] > 0 ? f.solve_kp[s] + f.solve_ku[s] : 1; };
  auto bwd_ctas = [&](int s) { return split && f.solve_kp[s] > 0 ? f.solve_kp[s] : 1; };
  for (;;) {
    if (threadIdx.x == 0) {
      s_ok = LoadVolatile(f.error) == 0;
      s_task = s_ok ? atomicAdd(f.counters + 1, 1) : ntasks;
    }
    __syncthreads();
    const int t = s_task;
    if (t >= ntasks) return;
    const bool forward = t < nfwd;
    const int s = split ? f.solve_front[t] : (forward ? t : f.ns - 1 - (t - f.ns));
    const int sub = split ? f.solve_sub[t] : 0;
    const int kp = split ? f.solve_kp[s] : 0, ku = split ? f.solve_ku[s] : 0;
    const Geom g = FrontGeom(f, s);
    if (forward) {
      bool ok = true;
      if (threadIdx.x == 0)
        for (int q = f.child_ptr[s]; q < f.child_ptr[s + 1] && ok; ++q)
          ok = WaitAtLeast(fwd_done + f.child_list[q], fwd_ctas(f.child_list[q]), f.error);
      if (CtaWait(ok, &s_flag)) {
        const int32_t* idx = f.idx + f.idx_off[s];
        const T* Fs = F + g.foff;
        for (int q = threadIdx.x; q < g.m; q += blockDim.x)
          if (OwnsRow(g, kTile, q, sub, kp, ku)) xs[q] = q < g.w ? b[f.scalar_old[idx[q]]] : T(0);
        if (threadIdx.x == 0) s_done = 0;
        __syncthreads();
        for (int q = f.child_ptr[s]; q < f.child_ptr[s + 1]; ++q) {
          const int c = f.child_list[q];
          const int hc = f.sn_m[c] - f.sn_w[c];
          const int32_t* rel = f.rel + f.rel_off[c];
          for (int r = threadIdx.x; r < hc; r += blockDim.x)
            if (OwnsRow(g, kTile, rel[r], sub, kp, ku)) xs[rel[r]] += Ld(ycon + f.rel_off[c] + r);
          __syncthreads();
        }
        if (kp == 0) {
          ForwardFront<T, kTile>(g, Fs, Linv + f.linv_base[s], xs, &s_done, f.error);
          for (int q = threadIdx.x; q < g.w; q += blockDim.x) St(ysave + f.idx_off[s] + q, xs[q]);
        } else if constexpr (sizeof(T) == 8) {
          // pivot CTAs store their y in ysave as they solve
          ForwardMulti<T, kTile>(g, Fs, Linv + f.linv_base[s], xs, ysave + f.idx_off[s], scratch,
                                 &s_done, sub, kp, ku, f.error);
          __syncthreads();
        }
        for (int r = threadIdx.x; r < g.m - g.w; r += blockDim.x)
          if (OwnsRow(g, kTile, g.w + r, sub, kp, ku)) St(ycon + f.rel_off[s] + r, xs[g.w + r]);
        SignalAdd(fwd_done + s);
      }
    } else {
      const int blk = kp - 1 - sub;  // backward tasks take a front's blocks from the last one down
      bool ok = true;
      if (threadIdx.x == 0) {
        const int p = f.parent[s];
        ok = p >= 0 ? WaitAtLeast(bwd_done + p, bwd_ctas(p), f.error)
                    : WaitAtLeast(fwd_done + s, fwd_ctas(s), f.error);
      }
      if (CtaWait(ok, &s_flag)) {
        const int32_t* idx = f.idx + f.idx_off[s];
        const T* Fs = F + g.foff;
        const int h = g.m - g.w;
        T* xa = xs + g.w;
        for (int r = threadIdx.x; r < h; r += blockDim.x) xa[r] = Ld(xperm + idx[g.w + r]);
        __syncthreads();
        for (int q = threadIdx.x; q < g.w; q += blockDim.x)
          if (OwnsRow(g, kTile, q, blk, kp, ku)) {
            const T z = Ld(ysave + f.idx_off[s] + q) / Ld(Fs + int64_t(q) * (g.m + 1));
            xs[q] = z - RowDot(Fs + int64_t(q) * g.m + g.w, int64_t(1), xa, 0, h);
          }
        if (threadIdx.x == 0) s_done = 0;
        __syncthreads();
        if (kp == 0) {
          BackwardFront<T, kTile>(g, Fs, Linv + f.linv_base[s], xs, &s_done, f.error);
        } else if constexpr (sizeof(T) == 8) {
          BackwardMulti<T, kTile>(g, Fs, Linv + f.linv_base[s], xs, xb + f.idx_off[s], scratch,
                                  &s_done, blk, f.error);
          __syncthreads();
        }
        for (int q = threadIdx.x; q < g.w; q += blockDim.x)
          if (OwnsRow(g, kTile, q, blk, kp, ku)) {
            St(xperm + idx[q], xs[q]);
            x[f.scalar_old[idx[q]]] = xs[q];
          }
        SignalAdd(bwd_done + s);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// FP64 iterative refinement of a low-precision factorization: r = b - (A + diag(damping)) y with
// A the matrix that was factored (block-sparse lower, used symmetrically) in its stored precision
// and every product and sum in FP64.  One warp per scalar row; lanes take row segments in turn
// and a fixed shuffle tree adds them.
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void RefineResidualKernel(SpmvDev m, const T* A_all, const double* damping, const T* b_all,
                                     const double* y, double* r, T* r_lo, const LmState* st,
                                     const int* gate) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= m.n || (gate && *gate == 0)) return;
  const T* A = A_all + int64_t(st->init_idx) * m.a_stride;
  const T* b = b_all + int64_t(st->init_idx) * m.b_stride;
  double acc = 0.0;
  for (int64_t q = m.row_ptr[row] + lane; q < m.row_ptr[row + 1]; q += 32) {
    const T* a = A + m.seg_base[q];
    const int stride = m.seg_stride[q], n = m.seg_len[q];
    const double* x = y + m.seg_x[q];
    for (int c = 0; c < n; ++c) acc += double(a[int64_t(c) * stride]) * x[c];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    if (damping) acc += damping[row] * y[row];
    const double res = double(b[row]) - acc;
    r[row] = res;
    r_lo[row] = T(res);
  }
}

template <typename T>
__global__ void WidenKernel(const T* x, double* y, int64_t n, const int* gate) {
  if (gate && *gate == 0) return;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] = double(x[i]);
}

template <typename T>
__global__ void AccumulateKernel(const T* dx, double* y, int64_t n, const int* gate) {
  if (gate && *gate == 0) return;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] += double(dx[i]);
}

__global__ void ResetFactorStateKernel(int* tile_state, int nstates, int* front_flags, int nflags,
                                       int* counters, const int* gate, unsigned* unset,
                                       int64_t unset_words, int elem) {
  if (gate && *gate == 0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nstates; i += gridDim.x * blockDim.x)
    tile_state[i] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nflags; i += gridDim.x * blockDim.x)
    front_flags[i] = 0;
  // the unset pattern of IsUnset: 0x7FF4DEAD0BADF00D (double, low word first), 0x7FA5DEAD (float)
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < unset_words;
       i += int64_t(gridDim.x) * blockDim.x)
    unset[i] = elem == 8 ? ((i & 1) ? 0x7FF4DEADu : 0x0BADF00Du) : 0x7FA5DEADu;
  if (blockIdx.x == 0 && threadIdx.x < 2) counters[threadIdx.x] = 0;
}

template <typename T>
__global__ void NegateKernel(const T* x, double* u, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    u[i] = -double(x[i]);
}

}  // namespace

void LaunchResetFactorState(int* tile_state, int nstates, int* front_flags, int nflags,
                            int* counters, cudaStream_t s, const int* gate, void* unset,
                            int64_t n_unset, int elem) {
  const int threads = 256;
  const int64_t words = unset ? n_unset * elem / 4 : 0;
  int64_t work = std::max<int64_t>(std::max(nstates, nflags), words);
  const int grid = int(std::min<int64_t>(std::max<int64_t>((work + threads - 1) / threads, 1), 1024));
  ResetFactorStateKernel<<<grid, threads, 0, s>>>(tile_state, nstates, front_flags, nflags, counters,
                                                  gate, static_cast<unsigned*>(unset), words, elem);
}

template <typename T>
void LaunchNegate(const void* x, double* u, int64_t n, cudaStream_t s) {
  const int threads = 256;
  int grid = int(std::min<int64_t>((n + threads - 1) / threads, 1024));
  NegateKernel<T><<<std::max(grid, 1), threads, 0, s>>>(static_cast<const T*>(x), u, n);
}
template void LaunchNegate<double>(const void*, double*, int64_t, cudaStream_t);
template void LaunchNegate<float>(const void*, double*, int64_t, cudaStream_t);

template <typename T>
void LaunchRefineResidual(const SpmvDev& m, const void* A, const double* damping, const void* b,
                          const double* y, double* r, void* r_lo, const LmState* st, cudaStream_t s,
                          const int* gate) {
  const int warps = 8;
  RefineResidualKernel<T><<<(m.n + warps - 1) / warps, 32 * warps, 0, s>>>(
      m, static_cast<const T*>(A), damping, static_cast<const T*>(b), y, r, static_cast<T*>(r_lo), st,
      gate);
}
template <typename T>
void LaunchWiden(const void* x, double* y, int64_t n, cudaStream_t s, const int* gate) {
  const int threads = 256;
  const int grid = int(std::min<int64_t>(std::max<int64_t>((n + threads - 1) / threads, 1), 1024));
  WidenKernel<T><<<grid, threads, 0, s>>>(static_cast<const T*>(x), y, n, gate);
}
template <typename T>
void LaunchAccumulate(const void* dx, double* y, int64_t n, cudaStream_t s, const int* gate) {
  const int threads = 256;
  const int grid = int(std::min<int64_t>(std::max<int64_t>((n + threads - 1) / threads, 1), 1024));
  AccumulateKernel<T><<<grid, threads, 0, s>>>(static_cast<const T*>(dx), y, n, gate);
}
template void LaunchRefineResidual<double>(const SpmvDev&, const void*, const double*, const void*,
                                           const double*, double*, void*, const LmState*, cudaStream_t,
                                           const int*);
template void LaunchRefineResidual<float>(const SpmvDev&, const void*, const double*, const void*,
                                          const double*, double*, void*, const LmState*, cudaStream_t,
                                          const int*);
template void LaunchWiden<double>(const void*, double*, int64_t, cudaStream_t, const int*);
template void LaunchWiden<float>(const void*, double*, int64_t, cudaStream_t, const int*);
template void LaunchAccumulate<double>(const void*, double*, int64_t, cudaStream_t, const int*);
template void LaunchAccumulate<float>(const void*, double*, int64_t, cudaStream_t, const int*);

int FactorThreads() { return kFactorThreads; }

namespace {
// Self-test of the capped dependency wait: thread 0 waits for a flag that nothing sets, with the
// same wait the persistent kernels use; the cap ends the wait and sets the error word.
__global__ void WaitCapSelfTestKernel(const int* flag, int* err) {
  if (threadIdx.x == 0 && blockIdx.x == 0) (void)WaitAtLeast(flag, 1, err);
}
}  // namespace

cudaError_t LaunchWaitCapSelfTest(const int* flag, int* err, cudaStream_t s) {
  WaitCapSelfTestKernel<<<1, 32, 0, s>>>(flag, err);
  return cudaGetLastError();
}

int SolveWarps() { return kSolveThreads / 32; }

template <typename T>
void ConfigureSolve(int max_m) {
  const size_t smem = SolveSmemBytes<T>(max_m);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(SolveKernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
}
template void ConfigureSolve<double>(int);
template void ConfigureSolve<float>(int);

template <typename T>
void LaunchSchurPoints(const SchurDev& d, const void* hess, const void* rhs, int64_t nvals,
                       int64_t N, const double* damping, void* cinv, void* W, void* tp,
                       const LmState* st, cudaStream_t s) {
  if (d.npoints == 0) return;
  const int threads = 128;
  SchurPointsKernel<T><<<(d.npoints + threads - 1) / threads, threads, 0, s>>>(
      d, static_cast<const T*>(hess), static_cast<const T*>(rhs), nvals, N, damping,
      static_cast<T*>(cinv), static_cast<T*>(tp), st);
  if (d.nE > 0)
    SchurWKernel<T><<<int((d.nE + threads - 1) / threads), threads, 0, s>>>(
        d, static_cast<const T*>(hess), nvals, static_cast<const T*>(cinv), static_cast<T*>(W), st);
}

template <typename T>
void LaunchSchurBuildS(const SchurDev& d, const void* hess, int64_t nvals, const double* damping,
                       const void* W, void* S, const LmState* st, cudaStream_t s) {
  if (d.nsblocks == 0) return;
  if (d.nchunks > 0)
    SchurChunkKernel<T><<<(d.nchunks + kSchurWarps - 1) / kSchurWarps, 32 * kSchurWarps, 0, s>>>(
        d, static_cast<const T*>(hess), nvals, static_cast<const T*>(W), st);
  constexpr int kWarps = 8;
  SchurFinishKernel<T><<<(d.nsblocks + kWarps - 1) / kWarps, 32 * kWarps, 0, s>>>(
      d, static_cast<const T*>(hess), nvals, damping, static_cast<T*>(S), st);
}

template <typename T>
void LaunchSchurRhs(const SchurDev& d, const void* hess, int64_t nvals, const void* rhs, int64_t N,
                    const void* tp, void* v, const LmState* st, cudaStream_t s) {
  if (d.nB == 0) return;
  const int warps = 4;
  // a warp per key reads every E block once but has d_k times fewer warps than a warp per scalar:
  // it is taken when the keys alone fill the GPU (1,000 cameras: 2,000 keys; 50 cameras: 100)
  // SFG_SCHUR_RHS_PER_SCALAR=0 / 1 overrides
  static const int force = [] {
    const char* e = std::getenv("SFG_SCHUR_RHS_PER_SCALAR");
    return e ? std::atoi(e) : -1;
  }();
  const bool per_scalar = force >= 0 ? force != 0 : d.nBk < kRhsKeyWarpsMin;
  if (per_scalar)
    SchurRhsKernel<T><<<(d.nB + warps - 1) / warps, 32 * warps, 0, s>>>(
        d, static_cast<const T*>(hess), nvals, static_cast<const T*>(rhs), N,
        static_cast<const T*>(tp), static_cast<T*>(v), st);
  else
    SchurRhsKeyKernel<T><<<(d.nBk + warps - 1) / warps, 32 * warps, 0, s>>>(
        d, static_cast<const T*>(hess), nvals, static_cast<const T*>(rhs), N,
        static_cast<const T*>(tp), static_cast<T*>(v), st);
}

template <typename T>
void LaunchSchurBackSub(const SchurDev& d, const void* y, const void* W, const void* tp, const void* cinv,
                        double* update, cudaStream_t s) {
  const int n = d.npoints + d.nB;
  const int threads = 128;
  SchurBackSubKernel<T><<<(n + threads - 1) / threads, threads, 0, s>>>(
      d, static_cast<const double*>(y), static_cast<const T*>(W), static_cast<const T*>(tp),
      static_cast<const T*>(cinv), update);
}

template <typename T>
void LaunchFactor(const FactorDev& f, const void* A, const double* damping, void* F, void* Linv,
                  int grid, cudaStream_t s) {
  constexpr int kTile = sizeof(T) == 8 ? kFactorTileF64 : kFactorTileF32;
  // FP64 plans of many fronts take the build for more resident CTAs (fewer registers a thread):
  // more trailing updates in flight; a single front's chain runs faster with more registers
  if constexpr (sizeof(T) == 8) {
    if (f.wide) {
      static const cudaError_t carveout = cudaFuncSetAttribute(
          FactorKernel<T, kTile, kFactorCtasPerSmWide>, cudaFuncAttributePreferredSharedMemoryCarveout,
          int(cudaSharedmemCarveoutMaxShared));
      (void)carveout;
      FactorKernel<T, kTile, kFactorCtasPerSmWide><<<grid, kFactorThreads, 0, s>>>(
          f, static_cast<const T*>(A), damping, static_cast<T*>(F), static_cast<T*>(Linv));
      return;
    }
  }
  static const cudaError_t carveout = cudaFuncSetAttribute(
      FactorKernel<T, kTile, kFactorCtasPerSm>, cudaFuncAttributePreferredSharedMemoryCarveout,
      int(cudaSharedmemCarveoutMaxShared));
  (void)carveout;
  FactorKernel<T, kTile, kFactorCtasPerSm><<<grid, kFactorThreads, 0, s>>>(
      f, static_cast<const T*>(A), damping, static_cast<T*>(F), static_cast<T*>(Linv));
}

template <typename T>
void LaunchSolve(const FactorDev& f, const void* F, const void* Linv, const void* b, void* ycon,
                 void* ysave, void* xperm, void* x, void* xb, int grid, cudaStream_t s) {
  const size_t smem = SolveSmemBytes<T>(f.max_m);
  SolveKernel<T><<<grid, kSolveThreads, smem, s>>>(
      f, static_cast<const T*>(F), static_cast<const T*>(Linv), static_cast<const T*>(b),
      static_cast<T*>(ycon), static_cast<T*>(ysave), static_cast<T*>(xperm), static_cast<T*>(x),
      static_cast<T*>(xb));
}

template void LaunchSchurPoints<double>(const SchurDev&, const void*, const void*, int64_t, int64_t,
                                        const double*, void*, void*, void*, const LmState*, cudaStream_t);
template void LaunchSchurPoints<float>(const SchurDev&, const void*, const void*, int64_t, int64_t,
                                       const double*, void*, void*, void*, const LmState*, cudaStream_t);
template void LaunchSchurBuildS<double>(const SchurDev&, const void*, int64_t, const double*,
                                        const void*, void*, const LmState*, cudaStream_t);
template void LaunchSchurBuildS<float>(const SchurDev&, const void*, int64_t, const double*,
                                       const void*, void*, const LmState*, cudaStream_t);
template void LaunchSchurRhs<double>(const SchurDev&, const void*, int64_t, const void*, int64_t,
                                     const void*, void*, const LmState*, cudaStream_t);
template void LaunchSchurRhs<float>(const SchurDev&, const void*, int64_t, const void*, int64_t,
                                    const void*, void*, const LmState*, cudaStream_t);
template void LaunchSchurBackSub<double>(const SchurDev&, const void*, const void*, const void*,
                                         const void*, double*, cudaStream_t);
template void LaunchSchurBackSub<float>(const SchurDev&, const void*, const void*, const void*,
                                        const void*, double*, cudaStream_t);
template void LaunchFactor<double>(const FactorDev&, const void*, const double*, void*, void*, int,
                                   cudaStream_t);
template void LaunchFactor<float>(const FactorDev&, const void*, const double*, void*, void*, int,
                                  cudaStream_t);
template void LaunchSolve<double>(const FactorDev&, const void*, const void*, const void*, void*, void*, void*,
                                  void*, void*, int, cudaStream_t);
template void LaunchSolve<float>(const FactorDev&, const void*, const void*, const void*, void*, void*, void*,
                                 void*, void*, int, cudaStream_t);

}  // namespace sfg
