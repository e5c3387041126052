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

namespace sfg {

namespace {

constexpr int kFactorThreads = 128;
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
// W = C^-1 E for one 3 x DK block E (row-major); cm = C^-1 entries (00, 10, 20, 11, 21, 22).
template <typename T, int DK>
__device__ __forceinline__ void PointW(const T* E, T* Wp, const T (&cm)[6]) {
  T e[3 * DK];
#pragma unroll
  for (int i = 0; i < 3 * DK; ++i) e[i] = E[i];
#pragma unroll
  for (int c = 0; c < DK; ++c) {
    const T e0 = e[c], e1 = e[DK + c], e2 = e[2 * DK + c];
    Wp[c] = cm[0] * e0 + cm[1] * e1 + cm[2] * e2;
    Wp[DK + c] = cm[1] * e0 + cm[3] * e1 + cm[4] * e2;
    Wp[2 * DK + c] = cm[2] * e0 + cm[4] * e1 + cm[5] * e2;
  }
}
template <typename T>
__device__ __forceinline__ void PointWAny(const T* E, T* Wp, int dk, const T (&cm)[6]) {
  for (int c = 0; c < dk; ++c) {
    const T e0 = E[c], e1 = E[dk + c], e2 = E[2 * dk + c];
    Wp[c] = cm[0] * e0 + cm[1] * e1 + cm[2] * e2;
    Wp[dk + c] = cm[1] * e0 + cm[3] * e1 + cm[4] * e2;
    Wp[2 * dk + c] = cm[2] * e0 + cm[4] * e1 + cm[5] * e2;
  }
}

// One thread per point: C^-1 of the damped 3 x 3 block (by its Cholesky factor) and t = C^-1 g.
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
  T* ci = cinv + 9 * int64_t(p);
  ci[0] = c00; ci[1] = c10; ci[2] = c20;
  ci[3] = c10; ci[4] = c11; ci[5] = c21;
  ci[6] = c20; ci[7] = c21; ci[8] = c22;
  const T g0 = g[toff], g1 = g[toff + 1], g2 = g[toff + 2];
  T* t = tp + 3 * int64_t(p);
  t[0] = c00 * g0 + c10 * g1 + c20 * g2;
  t[1] = c10 * g0 + c11 * g1 + c21 * g2;
  t[2] = c20 * g0 + c21 * g1 + c22 * g2;
}

// One thread per E block (the blocks of a point are consecutive, so neighbouring threads share its
// C^-1): W = C^-1 E, the block's loads all issued before its stores.
template <typename T>
__global__ void SchurWKernel(SchurDev d, const T* hess_all, int64_t nvals, const T* cinv, T* W,
                             const LmState* st) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= d.nE) return;
  const T* H = hess_all + int64_t(st->init_idx) * nvals;
  const T* ci = cinv + 9 * int64_t(d.pt_of_e[e]);
  const T cm[6] = {ci[0], ci[1], ci[2], ci[4], ci[5], ci[8]};
  const int dk = d.pt_ekey_dim[e];
  const T* E = H + d.pt_eoff[e];
  T* Wp = W + d.pt_woff[e];
  if (dk == 6) PointW<T, 6>(E, Wp, cm);
  else if (dk == 3) PointW<T, 3>(E, Wp, cm);
  else PointWAny<T>(E, Wp, dk, cm);
}

// S = B - sum_p E_pk^T W_pl over the S blocks' terms (points seen by both keys), in two passes.
// Pass 1: one warp per chunk of at most chunk_terms terms of one block; each lane takes the
// chunk's terms in turn and accumulates the whole d_k x d_l product of its terms in registers (every
// E and W block is read once), then a fixed shuffle tree adds the lanes.  Pass 2: one warp per S
// block adds its chunks in order and writes B_kl (+ damping) - sum.  Chunks spread the heavy
// diagonal blocks (every observation of a camera) over many warps, which the FP64 pipe needs; the
// fixed orders make every run give the same bits.  Key tangent dims are at most kMaxKeyDim.
constexpr int kMaxKeyDim = 6;
constexpr int kSchurWarps = 4;

// The products of one chunk for a block of DK x DL (compile-time sizes: only the block's entries are
// accumulated, which matters on the FP64 pipe), written as a 6 x 6 row-major partial.
template <typename T, int DK, int DL>
__device__ __forceinline__ void ChunkTerms(const SchurDev& d, const T* H, const T* W, int64_t t0,
                                           int64_t t1, int lane, T* out) {
  T acc[DK * DL];
#pragma unroll
  for (int i = 0; i < DK * DL; ++i) acc[i] = T(0);
  for (int64_t t = t0 + lane; t < t1; t += 32) {
    const T* E = H + d.sb_eoff[t];
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
#pragma unroll
  for (int i = 0; i < DK * DL; ++i) {
    T v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    acc[i] = v;
  }
  if (lane == 0)
#pragma unroll
    for (int r = 0; r < DK; ++r)
#pragma unroll
      for (int c = 0; c < DL; ++c) out[r * kMaxKeyDim + c] = acc[r * DL + c];
}

// Any other key sizes (up to kMaxKeyDim): runtime bounds inside the 6 x 6 accumulator.
template <typename T>
__device__ __forceinline__ void ChunkTermsAny(const SchurDev& d, const T* H, const T* W, int dk, int dl,
                                              int64_t t0, int64_t t1, int lane, T* out) {
  constexpr int D = kMaxKeyDim;
  T acc[D * D];
#pragma unroll
  for (int i = 0; i < D * D; ++i) acc[i] = T(0);
  for (int64_t t = t0 + lane; t < t1; t += 32) {
    const T* E = H + d.sb_eoff[t];
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
#pragma unroll
  for (int i = 0; i < D * D; ++i) {
    T v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    acc[i] = v;
  }
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < D * D; ++i) out[i] = acc[i];
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
  switch (dk * 8 + dl) {
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

// Point back-substitution z_p = t_p - sum_k W_pk y_k, and update = -[y; z].
template <typename T>
__global__ void SchurBackSubKernel(SchurDev d, const double* y, const T* W, const T* tp,
                                   double* update) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < d.npoints) {
    const int p = t;
    T z0 = tp[3 * int64_t(p)], z1 = tp[3 * int64_t(p) + 1], z2 = tp[3 * int64_t(p) + 2];
    for (int64_t e = d.pt_eptr[p]; e < d.pt_eptr[p + 1]; ++e) {
      const int dk = d.pt_ekey_dim[e];
      const T* Wp = W + d.pt_woff[e];
      const double* yk = y + d.pt_ekey_toff[e];
      T s[3];
      if (dk == 6) BlockTimes<T, 6>(Wp, yk, s);
      else if (dk == 3) BlockTimes<T, 3>(Wp, yk, s);
      else BlockTimesAny<T>(Wp, yk, dk, s);
      z0 -= s[0];
      z1 -= s[1];
      z2 -= s[2];
    }
    double* u = update + d.c_toff + 3 * int64_t(p);
    u[0] = -double(z0);
    u[1] = -double(z1);
    u[2] = -double(z2);
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

// Load a b_r x b_c tile at (r0, c0) of a column-major front into smem, transposed: dst[c*TILE + r].
template <typename T, int TILE>
__device__ __forceinline__ void LoadTileT(const T* Fs, int m, int r0, int c0, int br, int bc, T* dst) {
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    if (r < br && c < bc) dst[c * TILE + r] = Ld(Fs + (r0 + r) + int64_t(c0 + c) * m);
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

// LDL^T of diagonal tile k, held transposed in shared memory `a` (b x b of it), plus the explicit
// inverse of its unit lower factor (kept for the panel solves, which then become small matrix
// products); writes L, D and the inverse and publishes the tile.  This task is on the critical path
// of every front, and the two precisions take the form that measured fastest for them on one
// GB300 SM (TILE 16 FP64: CTA-wide steps 12.6 us, one warp 18-32 us; TILE 32 FP32: one warp with
// the rows in registers and a rolled pivot loop 12 us, CTA-wide steps 37 us).
// CTA-wide right-looking LDL^T steps of a tile held transposed in shared memory (b x b of it), one
// barrier per pivot: every thread forms the pivot's reciprocal itself (same bits everywhere), and
// column j is scaled during step j + 1, which does not read it.
template <typename D, int TILE>
__device__ __forceinline__ void LdltStepsCta(D* a, int b) {
  D inv_prev = D(0);
  for (int j = 0; j < b; ++j) {
    const D inv = PivotReciprocal<D>(a[j * TILE + j]);
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
      const int r = e % TILE, c = e / TILE;
      if (c > j && r >= c && r < b) a[c * TILE + r] -= a[j * TILE + r] * (a[j * TILE + c] * inv);
      if (j > 0 && c == j - 1 && r > c && r < b) a[c * TILE + r] *= inv_prev;
    }
    inv_prev = inv;
    __syncthreads();
  }
}

// ---- FP64 tiles (16 x 16).  On this GPU a warp issues an FP64 instruction about once per 64
// cycles on its own SM sub-partition (a one-warp elimination of a tile measured 20 us against 12.6
// us for the same work spread over four warps), so FP64 tile work is spread over all four warps of
// the CTA (one per sub-partition) with as few FP64 instructions per warp and step as possible.

// Lower entries of a 16 x 16 tile in column-major order: entry e -> (r, c), r >= c.
__device__ __forceinline__ void LowerEntry16(int e, int* r, int* c) {
  int cc = 0, start = 0;
  while (cc < 15 && e >= start + (16 - cc)) {
    start += 16 - cc;
    ++cc;
  }
  *c = cc;
  *r = cc + (e - start);
}

// Right-looking LDL^T of the b x b leading part of a 16 x 16 FP64 tile held transposed in shared
// memory (a[c * 16 + r] = A(r, c), lower part used): on return column j below the diagonal holds
// L(:, j) and the diagonal D.  Warp 0 forms each pivot's reciprocal; warps 1-3 own the 136 lower
// entries (at most two per thread) in registers, form the products A(r, j) A(c, j) while warp 0
// works on the reciprocal, then apply one multiply-add per entry once it is published.  Two CTA
// barriers per pivot.
__device__ void DiagLdltF64(double* a, int b, double* s_inv) {
  const int t = threadIdx.x;
  int r0 = 0, c0 = 16, r1 = 0, c1 = 16;  // c = 16: no entry
  double v0 = 0.0, v1 = 0.0;
  if (t >= 32) {
    const int e = t - 32;
    LowerEntry16(e, &r0, &c0);
    if (r0 >= b) c0 = 16;
    if (e + 96 < 136) {
      LowerEntry16(e + 96, &r1, &c1);
      if (r1 >= b) c1 = 16;
    }
    if (c0 < 16) v0 = a[c0 * 16 + r0];
    if (c1 < 16) v1 = a[c1 * 16 + r1];
  }
  for (int j = 0; j < b; ++j) {
    double p0 = 0.0, p1 = 0.0;
    if (t < 32) {
      const double inv = PivotReciprocal<double>(a[j * 16 + j]);
      if (t == 0) *s_inv = inv;
    } else {
      if (c0 < 16 && c0 > j) p0 = a[j * 16 + r0] * a[j * 16 + c0];
      if (c1 < 16 && c1 > j) p1 = a[j * 16 + r1] * a[j * 16 + c1];
    }
    __syncthreads();
    if (t >= 32) {
      const double inv = *s_inv;
      if (c0 < 16) {
        if (c0 > j) {
          v0 = fma(-p0, inv, v0);
          a[c0 * 16 + r0] = v0;
        } else if (c0 == j && r0 > j) {
          v0 *= inv;  // L(r, j)
          a[c0 * 16 + r0] = v0;
        }
      }
      if (c1 < 16) {
        if (c1 > j) {
          v1 = fma(-p1, inv, v1);
          a[c1 * 16 + r1] = v1;
        } else if (c1 == j && r1 > j) {
          v1 *= inv;
          a[c1 * 16 + r1] = v1;
        }
      }
    }
    __syncthreads();
  }
}

// Inverse of the unit lower factor held in `a` (strict lower part of the b x b leading block, as
// DiagLdltF64 leaves it) into li (transposed like the tiles; identity outside the block), by forward
// substitution on all columns at once: one entry (r > c) per thread, one multiply-add per step.
__device__ void UnitLowerInverseF64(const double* a, int b, double* li) {
  const int t = threadIdx.x;
  for (int e = t; e < 256; e += blockDim.x) li[e] = (e % 17 == 0) ? 1.0 : 0.0;
  // strict lower entries (120): e -> (r, c) with r > c, column-major
  int r = 0, c = 16;
  if (t < 120) {
    int cc = 0, start = 0;
    while (cc < 14 && t >= start + (15 - cc)) {
      start += 15 - cc;
      ++cc;
    }
    c = cc;
    r = cc + 1 + (t - start);
    if (r >= b) c = 16;
  }
  __syncthreads();
  double v = 0.0;
  for (int q = 0; q + 1 < b; ++q) {
    // Li(r, c) -= L(r, q) Li(q, c) for r > q >= c; row q of Li is final after step q - 1
    if (c < 16 && r > q && c <= q) {
      v = (c == q) ? -a[q * 16 + r] : fma(-a[q * 16 + r], li[c * 16 + q], v);
      li[c * 16 + r] = v;
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

// LDL^T of diagonal tile k, held transposed in shared memory `a` (b x b of it), plus the explicit
// inverse of its unit lower factor (kept for the panel solves, which then become small matrix
// products); writes L, D and the inverse and publishes the tile.  This task is on the critical path
// of every front, and the two precisions take the form that measured fastest for them on one
// GB300 SM (TILE 16 FP64: CTA-wide steps 12.6 us, one warp 18-32 us; TILE 32 FP32: one warp with
// the rows in registers and a rolled pivot loop 12 us, CTA-wide steps 37 us).  An FP32 tile with a
// near-singular pivot is factored again in FP64 from its saved input and rounded back (counted in
// f.fp64_tiles).
template <typename T, int TILE>
__device__ void DiagCore(const FactorDev& f, const Geom& g, int s, int k, T* F, T* Linv, T* a,
                         TileSmem<T, TILE>& sm, unsigned long long* tr = nullptr) {
  static_assert(TILE <= 32, "one lane per tile row");
  const int b = TileSize(g, k, TILE), r0 = TileStart(g, k, TILE);
  T* Fs = F + g.foff;
  T* li = sm.b;
  if constexpr (sizeof(T) == 8) {
    static_assert(sizeof(T) != 8 || TILE == 16, "the FP64 tile kernels are written for 16 x 16 tiles");
    __shared__ double s_inv;
    DiagLdltF64(a, b, &s_inv);
    Stamp(tr, 3);
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
      const int r = e % TILE, c = e / TILE;
      if (r < b && c < b && r >= c) St(Fs + (r0 + r) + int64_t(r0 + c) * g.m, a[c * TILE + r]);
    }
    Signal(f.tile_state + StateIdx(g, k, k), kFinal);
    // the inverse of L is for the triangular solves only (the FP64 panel solves substitute), so
    // it is formed after the tile is published, off the front's critical chain
    UnitLowerInverseF64(a, b, li);
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
    constexpr unsigned kAll = 0xffffffffu;
    // one warp, lane r holds row r in registers; the pivot loop is unrolled so that every register
    // index is static (FP32 issues at full rate from one warp, unlike FP64), and the multipliers
    // reach the other rows by shuffles
    if (threadIdx.x < 32) {
      const int r = threadIdx.x;
      T row[TILE];
#pragma unroll
      for (int c = 0; c < TILE; ++c) row[c] = (r < b && c <= r) ? a[c * TILE + (r < TILE ? r : 0)] : T(0);
      bool redo = false;
#pragma unroll
      for (int j = 0; j < TILE; ++j) {
        if (j < b) {
          const T dj = __shfl_sync(kAll, row[j], j);
          redo = redo || !(dj > kNearSingularPivot * fabsf(float(orig[j * TILE + j])));
          const T inv = PivotReciprocal<T>(dj);
          const T lrj = row[j] * inv;
#pragma unroll
          for (int c = j + 1; c < TILE; ++c) {
            const T lcj = __shfl_sync(kAll, lrj, c);
            if (r >= c) row[c] -= row[j] * lcj;
          }
          if (r < b && r >= j) a[j * TILE + r] = r > j ? lrj : row[j];  // L(r, j), or d_j on the diagonal
        }
      }
      if (r == 0 && redo) s_redo = 1;
    }
    __syncthreads();
    Stamp(tr, 3);
    if (s_redo) {
      // FP64 redo from the saved input: the double tile occupies a and b
      double* dt = reinterpret_cast<double*>(sm.a);
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) dt[e] = double(orig[e]);
      __syncthreads();
      LdltStepsCta<double, TILE>(dt, b);
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) orig[e] = T(dt[e]);
      __syncthreads();
      for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) a[e] = orig[e];
      if (threadIdx.x == 0 && f.fp64_tiles) atomicAdd(f.fp64_tiles, 1);
      __syncthreads();
    }
    if (threadIdx.x < 32) {
      const int r = threadIdx.x;
      T lrow[TILE];
#pragma unroll
      for (int c = 0; c < TILE; ++c) lrow[c] = T(c == r ? 1 : 0);
      for (int q = 0; q + 1 < b; ++q) {
        const T lrq = (r > q && r < b) ? a[q * TILE + r] : T(0);
#pragma unroll
        for (int c = 0; c < TILE; ++c) {
          const T liqc = __shfl_sync(kAll, lrow[c], q);
          if (c <= q) lrow[c] -= lrq * liqc;
        }
      }
      if (r < TILE)
#pragma unroll
        for (int c = 0; c < TILE; ++c) li[c * TILE + r] = lrow[c];
    }
    __syncthreads();
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
  T out[TILE * TILE >= kFactorThreads ? TILE * TILE / kFactorThreads : 1];
  int n = 0;
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x, ++n) {
    const int r = e % TILE, c = e / TILE;
    out[n] = PanelDot<T, TILE>(sm.a, sm.b, r, c, min(c + 1, bk)) * sm.d[c < bk ? c : 0];
  }
  n = 0;
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x, ++n) {
    const int r = e % TILE, c = e / TILE;
    if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, out[n]);
  }
  Signal(f.tile_state + StateIdx(g, i, k), kFinal);
}

// The critical chain of panel k in one CTA: panel solve of tile i = k + 1 (as TaskTrsm, kept in
// shared memory), the update of diagonal tile (i, i) by it, F_ii -= L_ik D_k L_ik^T (after every
// earlier panel's update of that tile), and the LDL^T of (i, i).  This saves two hand-offs between
// CTAs (and two tile reloads) per panel on the longest dependency path of a front.
// FP64 look-ahead: the three tiles it reads are waited for and loaded in one round (the diagonal
// tile (i, i) is normally ready long before), the panel solve substitutes against L_kk, and the
// diagonal tile is factored by the CTA-wide kernel.
template <typename T, int TILE>
__device__ void LookaheadF64(const FactorDev& f, int s, int i, int k, T* F, T* Linv, TileSmem<T, TILE>& sm,
                             int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  bool ok = true;
  if (threadIdx.x == 0) {
    ok = WaitAtLeast(f.tile_state + StateIdx(g, k, k), kFinal, f.error) &&
         WaitAtLeast(f.tile_state + StateIdx(g, i, k), 1 + k, f.error) &&
         WaitAtLeast(f.tile_state + StateIdx(g, i, i), 1 + k, f.error);
  }
  if (!CtaWait(ok, s_flag, ready)) return;
  const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
  const int bi = TileSize(g, i, TILE), ri = TileStart(g, i, TILE);
  T* Fs = F + g.foff;
  LoadTileT<T, TILE>(Fs, g.m, ri, ck, bi, bk, sm.a);  // F_ik
  LoadTileT<T, TILE>(Fs, g.m, ck, ck, bk, bk, sm.b);  // L_kk and D_k
  LoadTileT<T, TILE>(Fs, g.m, ri, ri, bi, bi, sm.e);  // F_ii
  __syncthreads();
  for (int c = threadIdx.x; c < bk; c += blockDim.x) sm.d[c] = PivotReciprocal<T>(sm.b[c * TILE + c]);
  __syncthreads();
  Stamp(ready, 0);
  PanelSolveSubstF64(sm.a, sm.b, sm.d, bi, bk, sm.c, sm.w);
  __syncthreads();
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, sm.c[c * TILE + r]);
  }
  Signal(f.tile_state + StateIdx(g, i, k), kFinal);
  Stamp(ready, 1);
  // F_ii -= Y X^T (Y = X D), lower part
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    if (r >= bi || c > r) continue;
    sm.e[c * TILE + r] -= PanelDot<T, TILE>(sm.w, sm.c, r, c, bk);
  }
  __syncthreads();
  Stamp(ready, 2);
  DiagCore<T, TILE>(f, g, s, i, F, Linv, sm.e, sm, ready);
}

template <typename T, int TILE>
__device__ void TaskLookahead(const FactorDev& f, int s, int i, int k, T* F, T* Linv,
                              TileSmem<T, TILE>& sm, int* s_flag, unsigned long long* ready) {
  if constexpr (sizeof(T) == 8) {
    LookaheadF64<T, TILE>(f, s, i, k, F, Linv, sm, s_flag, ready);
    return;
  }
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
  const T* Lk = Linv + f.linv_base[s] + int64_t(k) * TILE * TILE;
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) sm.b[e] = Ld(Lk + e);
  for (int c = threadIdx.x; c < bk; c += blockDim.x)
    sm.d[c] = PivotReciprocal<T>(Ld(Fs + int64_t(ck + c) * (g.m + 1)));
  __syncthreads();
  Stamp(ready, 0);
  // L_ik (r, c) = sum_{q <= c} F(r, q) Li(c, q) / D_c, into c[] (transposed) and the front, and
  // L_ik D into w[]
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    const T acc = PanelDot<T, TILE>(sm.a, sm.b, r, c, min(c + 1, bk));
    const T inv = sm.d[c < bk ? c : 0];
    const T l = (r < bi && c < bk) ? acc * inv : T(0);
    sm.c[c * TILE + r] = l;
    sm.w[c * TILE + r] = (r < bi && c < bk) ? acc : T(0);  // F Li^T = L D
    if (r < bi && c < bk) St(Fs + (ri + r) + int64_t(ck + c) * g.m, l);
  }
  Signal(f.tile_state + StateIdx(g, i, k), kFinal);
  Stamp(ready, 1);
  // F_ii after every earlier panel's update, minus L_ik D_k L_ik^T (lower part), in a[]
  ok = true;
  if (threadIdx.x == 0) ok = WaitAtLeast(f.tile_state + StateIdx(g, i, i), 1 + k, f.error);
  if (!CtaWait(ok, s_flag)) return;
  LoadTileT<T, TILE>(Fs, g.m, ri, ri, bi, bi, sm.a);
  __syncthreads();
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int r = e % TILE, c = e / TILE;
    if (r >= bi || c > r) continue;
    sm.a[c * TILE + r] -= PanelDot<T, TILE>(sm.w, sm.c, r, c, bk);
  }
  __syncthreads();
  Stamp(ready, 2);
  DiagCore<T, TILE>(f, g, s, i, F, Linv, sm.a, sm, ready);
}

template <typename T, int TILE>
__device__ void TaskUpdate(const FactorDev& f, int s, int i, int j, int k, T* F,
                           TileSmem<T, TILE>& sm, int* s_flag, unsigned long long* ready) {
  const Geom g = FrontGeom(f, s);
  bool ok = true;
  if (threadIdx.x == 0) {
    ok = WaitAtLeast(f.tile_state + StateIdx(g, i, k), kFinal, f.error) &&
         WaitAtLeast(f.tile_state + StateIdx(g, j, k), kFinal, f.error) &&
         WaitAtLeast(f.tile_state + StateIdx(g, i, j), 1 + k, f.error);
  }
  if (!CtaWait(ok, s_flag, ready)) return;
  const int bk = TileSize(g, k, TILE), ck = TileStart(g, k, TILE);
  const int bi = TileSize(g, i, TILE), ri = TileStart(g, i, TILE);
  const int bj = TileSize(g, j, TILE), rj = TileStart(g, j, TILE);
  T* Fs = F + g.foff;
  constexpr int kPer = TILE * TILE >= kFactorThreads ? TILE * TILE / kFactorThreads : 1;
  T cdst[kPer];
  {
    int n = 0;
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x, ++n) {
      const int r = e % TILE, c = e / TILE;
      cdst[n] = (r < bi && c < bj) ? Ld(Fs + (ri + r) + int64_t(rj + c) * g.m) : T(0);
    }
  }
  LoadTileT<T, TILE>(Fs, g.m, ri, ck, bi, bk, sm.a);  // L_ik
  LoadTileT<T, TILE>(Fs, g.m, rj, ck, bj, bk, sm.b);  // L_jk
  for (int c = threadIdx.x; c < bk; c += blockDim.x) sm.d[c] = Ld(Fs + int64_t(ck + c) * (g.m + 1));
  __syncthreads();
  for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
    const int c = e / TILE;
    if (c < bk) sm.b[e] *= sm.d[c];  // L_jk D
  }
  __syncthreads();
  {
    int n = 0;
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x, ++n) {
      const int r = e % TILE, c = e / TILE;
      if (r >= bi || c >= bj || (i == j && r < c)) continue;
      St(Fs + (ri + r) + int64_t(rj + c) * g.m, cdst[n] - PanelDot<T, TILE>(sm.a, sm.b, r, c, bk));
    }
  }
  Signal(f.tile_state + StateIdx(g, i, j), 2 + k);
}

template <typename T, int TILE>
__global__ void __launch_bounds__(kFactorThreads, kFactorCtasPerSm) FactorKernel(FactorDev f, const T* A,
                                                               const double* damping, T* F,
                                                               T* Linv) {
  __shared__ TileSmem<T, TILE> sm;
  __shared__ int s_task, s_next, s_ok, s_flag;
  if (f.gate && *f.gate == 0) return;
  A += int64_t(f.st->init_idx) * f.a_stride;
  if (threadIdx.x == 0) s_next = atomicAdd(f.counters, 1);
  for (;;) {
    if (threadIdx.x == 0) {
      s_ok = LoadVolatile(f.error) == 0;
      s_task = s_ok ? s_next : f.ntasks;
      // fetch the following task now so that the atomic's latency overlaps this task
      if (s_task < f.ntasks) s_next = atomicAdd(f.counters, 1);
    }
    __syncthreads();
    const int t = s_task;
    if (t >= f.ntasks) return;
    const int4 task = f.tasks[t];
    const int i = task.z >> 16, j = task.z & 0xffff, k = task.w;
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
      case kTaskLookahead: TaskLookahead<T, TILE>(f, task.y, i, k, F, Linv, sm, &s_flag, ready); break;
      default:
        if (threadIdx.x == 0) atomicExch(f.error, kDevBadTask);
    }
    __syncthreads();
    if (f.trace && threadIdx.x == 0) f.trace[8 * int64_t(t) + 2] = Clock64Global();
  }
}

// ---------------------------------------------------------------------------------------------
// Triangular solves: task t < ns is the forward solve of front t (postorder), task ns + q the
// backward solve of front ns - 1 - q (reverse postorder).  Dynamic shared memory: max_m scalars.
// The pivot columns go in the factorization's pivot tiles.  A tile's triangle is solved with the
// inverse of its unit lower factor that the factorization kept (a product whose rows are
// independent: four-chain dot products instead of a chain of TILE dependent multiply-adds), by
// warp 0, which also updated the tile's rows in the step before (so a warp barrier orders them);
// then every thread updates its rows with the tile (independent loads).  One CTA barrier per tile.
// Warp 0 loads the next tile's inverse row while the current tile's update runs.
// ---------------------------------------------------------------------------------------------
// Threads of a solve task: the rows below a tile are updated one row per thread, each row a few
// dependent multiply-add chains after one round of L2 loads, so more threads shorten the step of a
// wide front (256: a 450-wide front needs at most two rows per thread).
constexpr int kSolveThreads = 256;

// sum_{c = c0}^{c1 - 1} a[c * stride] x[c] with four independent accumulation chains (a dependent
// FP64 multiply-add costs 64 cycles on this GPU), added in a fixed order.
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

// sum_{c < n} v[c] x[c] over a register row, four chains, fixed order (x is read below n only)
template <typename T, int TILE>
__device__ __forceinline__ T RegDot(const T (&v)[TILE], const T* x, int n) {
  T s[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
  for (int c = 0; c < TILE; ++c)
    if (c < n) s[c & 3] += v[c] * x[c];
  return (s[0] + s[1]) + (s[2] + s[3]);
}

// Row `lane` of the inverse of pivot tile k (forward: row of L^-1, entries c <= lane) or column
// `lane` (backward: row of L^-T, entries c >= lane); zeros outside the tile's b rows.  The inverse
// is stored with (r, c) at c * TILE + r.
template <typename T, int TILE, bool kTransposed>
__device__ __forceinline__ void LoadInvRow(const T* Li, int k, int b, int lane, T (&v)[TILE]) {
  const T* L = Li + int64_t(k) * TILE * TILE;
#pragma unroll
  for (int c = 0; c < TILE; ++c) {
    const bool in = lane < b && c < b && (kTransposed ? c >= lane : c <= lane);
    v[c] = in ? Ld(kTransposed ? L + lane * TILE + c : L + c * TILE + lane) : T(0);
  }
}

// Pivot tiles go in steps of SUP = 32 / TILE tiles (two FP64 tiles of 16, one FP32 tile of 32), one
// per TILE lanes of warp 0, so that a step spans 32 columns.  Within a step, the lanes of a later
// tile first subtract the earlier tile's contribution (its rows of L, loaded ahead like the inverse
// rows), then apply their tile's inverse.
template <typename T, int TILE>
__device__ void ForwardFront(const Geom& g, const T* Fs, const T* Li, T* xs) {
  constexpr int SUP = 32 / TILE;
  static_assert(SUP * TILE == 32 && SUP <= 2, "a step is warp 0: one or two pivot tiles");
  const int m = g.m, t = threadIdx.x;
  const int grp = (t & 31) / TILE, lr = (t & 31) % TILE;
  T inv[TILE], lft[TILE];
  // inverse row of tile k0 + grp; for the second tile, its row lr against the first tile's columns
  auto prefetch = [&](int k0) {
    const int k = k0 + grp, pk = k * TILE;
    const int b = k < g.np ? min(TILE, g.w - pk) : 0;
    LoadInvRow<T, TILE, false>(Li, k < g.np ? k : 0, b, lr, inv);
#pragma unroll
    for (int c = 0; c < TILE; ++c)
      lft[c] = (grp > 0 && lr < b) ? Ld(Fs + (pk + lr) + int64_t(k0 * TILE + c) * m) : T(0);
  };
  if (t < 32) prefetch(0);
  for (int k0 = 0; k0 < g.np; k0 += SUP) {
    const int p0 = k0 * TILE, p2 = min(p0 + SUP * TILE, g.w);
    if (t < 32) {
      // the step's rows were last updated by warp 0 (or before the caller's CTA barrier)
      __syncwarp();
#pragma unroll
      for (int j = 0; j < SUP; ++j) {
        const int pj = p0 + j * TILE, bj = min(TILE, p2 - pj);  // bj <= 0: no such tile
        T y = T(0);
        if (j > 0) {
          if (grp == j && lr < bj) xs[pj + lr] -= RegDot<T, TILE>(lft, xs + p0, TILE);
          __syncwarp();
        }
        if (grp == j && lr < bj) y = RegDot<T, TILE>(inv, xs + pj, bj);
        __syncwarp();
        if (grp == j && lr < bj) xs[pj + lr] = y;
        __syncwarp();
      }
      if (k0 + SUP < g.np) prefetch(k0 + SUP);
    }
    __syncthreads();
    // thread i updates rows p2 + i, p2 + i + blockDim, ...: the next step's rows fall to warp 0
    for (int r = p2 + t; r < m; r += blockDim.x) xs[r] -= RowDot(Fs + r, int64_t(m), xs, p0, p2);
  }
  __syncthreads();
}

template <typename T, int TILE>
__device__ void BackwardFront(const Geom& g, const T* Fs, const T* Li, T* xs) {
  constexpr int SUP = 32 / TILE;
  const int m = g.m, t = threadIdx.x;
  const int grp = (t & 31) / TILE, lr = (t & 31) % TILE;
  T inv[TILE], lft[TILE];
  // row lr of the inverse transposed of tile k0 + grp; for the first tile of a two-tile step, its
  // column lr of L against the second tile's rows (the entries of L^T row lr)
  auto prefetch = [&](int k0) {
    const int k = k0 + grp, pk = k * TILE;
    const int b = k < g.np ? min(TILE, g.w - pk) : 0;
    LoadInvRow<T, TILE, true>(Li, k < g.np ? k : 0, b, lr, inv);
    const int k1 = k0 + 1, b1 = k1 < g.np ? min(TILE, g.w - k1 * TILE) : 0;
#pragma unroll
    for (int c = 0; c < TILE; ++c)
      lft[c] = (SUP > 1 && grp == 0 && lr < b && c < b1) ? Ld(Fs + (k1 * TILE + c) + int64_t(pk + lr) * m)
                                                          : T(0);
  };
  const int last = g.np > 0 ? ((g.np - 1) / SUP) * SUP : 0;
  if (t < 32 && g.np > 0) prefetch(last);
  for (int k0 = last; k0 >= 0 && g.np > 0; k0 -= SUP) {
    const int p0 = k0 * TILE, p2 = min(p0 + SUP * TILE, g.w);
    if (t < 32) {
      __syncwarp();
#pragma unroll
      for (int jj = SUP - 1; jj >= 0; --jj) {
        const int pj = p0 + jj * TILE, bj = min(TILE, p2 - pj);
        if (bj > 0) {
          T y = T(0);
          if (jj < SUP - 1) {
            const int pn = pj + TILE;  // the later tile of the step, solved just before
            if (grp == jj && lr < bj) xs[pj + lr] -= RegDot<T, TILE>(lft, xs + pn, p2 - pn);
            __syncwarp();
          }
          if (grp == jj && lr < bj) y = RegDot<T, TILE>(inv, xs + pj, bj);
          __syncwarp();
          if (grp == jj && lr < bj) xs[pj + lr] = y;
          __syncwarp();
        }
      }
      if (k0 - SUP >= 0) prefetch(k0 - SUP);
    }
    __syncthreads();
    // thread i updates rows p0 - 1 - i, ...: the previous step's rows fall to warp 0
    for (int i = t; i < p0; i += blockDim.x) {
      const int r = p0 - 1 - i;
      xs[r] -= RowDot(Fs + int64_t(r) * m, int64_t(1), xs, p0, p2);
    }
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kSolveThreads) SolveKernel(FactorDev f, const T* F, const T* Linv,
                                                              const T* b, T* ycon, T* ysave, T* xperm,
                                                              T* x) {
  constexpr int kTile = sizeof(T) == 8 ? kFactorTileF64 : kFactorTileF32;
  static_assert(kTile <= 32 && kSolveThreads >= 32, "warp 0 holds a tile's rows");
  extern __shared__ unsigned char smem_raw[];
  T* xs = reinterpret_cast<T*>(smem_raw);
  __shared__ int s_task, s_ok, s_flag;
  int* fwd_done = f.front_flags;
  int* bwd_done = f.front_flags + f.ns;
  if (f.gate && *f.gate == 0) return;
  b += int64_t(f.st->init_idx) * f.b_stride;
  for (;;) {
    if (threadIdx.x == 0) {
      s_ok = LoadVolatile(f.error) == 0;
      s_task = s_ok ? atomicAdd(f.counters + 1, 1) : 2 * f.ns;
    }
    __syncthreads();
    const int t = s_task;
    if (t >= 2 * f.ns) return;
    if (t < f.ns) {
      const int s = t;
      const Geom g = FrontGeom(f, s);
      bool ok = true;
      if (threadIdx.x == 0)
        for (int q = f.child_ptr[s]; q < f.child_ptr[s + 1] && ok; ++q)
          ok = WaitAtLeast(fwd_done + f.child_list[q], 1, f.error);
      if (CtaWait(ok, &s_flag)) {
        const int32_t* idx = f.idx + f.idx_off[s];
        const T* Fs = F + g.foff;
        for (int q = threadIdx.x; q < g.m; q += blockDim.x)
          xs[q] = q < g.w ? b[f.scalar_old[idx[q]]] : T(0);
        __syncthreads();
        for (int q = f.child_ptr[s]; q < f.child_ptr[s + 1]; ++q) {
          const int c = f.child_list[q];
          const int hc = f.sn_m[c] - f.sn_w[c];
          const int32_t* rel = f.rel + f.rel_off[c];
          for (int r = threadIdx.x; r < hc; r += blockDim.x) xs[rel[r]] += Ld(ycon + f.rel_off[c] + r);
          __syncthreads();
        }
        ForwardFront<T, kTile>(g, Fs, Linv + f.linv_base[s], xs);
        for (int q = threadIdx.x; q < g.w; q += blockDim.x) St(ysave + f.idx_off[s] + q, xs[q]);
        for (int r = threadIdx.x; r < g.m - g.w; r += blockDim.x) St(ycon + f.rel_off[s] + r, xs[g.w + r]);
        Signal(fwd_done + s, 1);
      }
    } else {
      const int s = f.ns - 1 - (t - f.ns);
      const Geom g = FrontGeom(f, s);
      bool ok = true;
      if (threadIdx.x == 0) {
        const int p = f.parent[s];
        ok = p >= 0 ? WaitAtLeast(bwd_done + p, 1, f.error) : WaitAtLeast(fwd_done + s, 1, f.error);
      }
      if (CtaWait(ok, &s_flag)) {
        const int32_t* idx = f.idx + f.idx_off[s];
        const T* Fs = F + g.foff;
        const int h = g.m - g.w;
        T* xa = xs + g.w;
        for (int r = threadIdx.x; r < h; r += blockDim.x) xa[r] = Ld(xperm + idx[g.w + r]);
        __syncthreads();
        for (int q = threadIdx.x; q < g.w; q += blockDim.x) {
          const T z = Ld(ysave + f.idx_off[s] + q) / Ld(Fs + int64_t(q) * (g.m + 1));
          xs[q] = z - RowDot(Fs + int64_t(q) * g.m + g.w, int64_t(1), xa, 0, h);
        }
        __syncthreads();
        BackwardFront<T, kTile>(g, Fs, Linv + f.linv_base[s], xs);
        for (int q = threadIdx.x; q < g.w; q += blockDim.x) {
          St(xperm + idx[q], xs[q]);
          x[f.scalar_old[idx[q]]] = xs[q];
        }
        Signal(bwd_done + s, 1);
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
                                       int* counters, const int* gate) {
  if (gate && *gate == 0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nstates; i += gridDim.x * blockDim.x)
    tile_state[i] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nflags; i += gridDim.x * blockDim.x)
    front_flags[i] = 0;
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
                            int* counters, cudaStream_t s, const int* gate) {
  const int threads = 256;
  int grid = (std::max(nstates, nflags) + threads - 1) / threads;
  grid = std::min(std::max(grid, 1), 1024);
  ResetFactorStateKernel<<<grid, threads, 0, s>>>(tile_state, nstates, front_flags, nflags, counters,
                                                  gate);
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

template <typename T>
void ConfigureSolve(int max_m) {
  const size_t smem = size_t(max_m) * sizeof(T);
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
  SchurRhsKernel<T><<<(d.nB + warps - 1) / warps, 32 * warps, 0, s>>>(
      d, static_cast<const T*>(hess), nvals, static_cast<const T*>(rhs), N,
      static_cast<const T*>(tp), static_cast<T*>(v), st);
}

template <typename T>
void LaunchSchurBackSub(const SchurDev& d, const void* y, const void* W, const void* tp,
                        double* update, cudaStream_t s) {
  const int n = d.npoints + d.nB;
  const int threads = 128;
  SchurBackSubKernel<T><<<(n + threads - 1) / threads, threads, 0, s>>>(
      d, static_cast<const double*>(y), static_cast<const T*>(W), static_cast<const T*>(tp), update);
}

template <typename T>
void LaunchFactor(const FactorDev& f, const void* A, const double* damping, void* F, void* Linv,
                  int grid, cudaStream_t s) {
  constexpr int kTile = sizeof(T) == 8 ? kFactorTileF64 : kFactorTileF32;
  FactorKernel<T, kTile><<<grid, kFactorThreads, 0, s>>>(f, static_cast<const T*>(A), damping,
                                                         static_cast<T*>(F), static_cast<T*>(Linv));
}

template <typename T>
void LaunchSolve(const FactorDev& f, const void* F, const void* Linv, const void* b, void* ycon,
                 void* ysave, void* xperm, void* x, int grid, cudaStream_t s) {
  // dynamic shared memory: the largest front's scalars
  const size_t smem = size_t(f.max_m) * sizeof(T);
  SolveKernel<T><<<grid, kSolveThreads, smem, s>>>(
      f, static_cast<const T*>(F), static_cast<const T*>(Linv), static_cast<const T*>(b),
      static_cast<T*>(ycon), static_cast<T*>(ysave), static_cast<T*>(xperm), static_cast<T*>(x));
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
                                         double*, cudaStream_t);
template void LaunchSchurBackSub<float>(const SchurDev&, const void*, const void*, const void*,
                                        double*, cudaStream_t);
template void LaunchFactor<double>(const FactorDev&, const void*, const double*, void*, void*, int,
                                   cudaStream_t);
template void LaunchFactor<float>(const FactorDev&, const void*, const double*, void*, void*, int,
                                  cudaStream_t);
template void LaunchSolve<double>(const FactorDev&, const void*, const void*, const void*, void*, void*,
                                  void*, void*, int, cudaStream_t);
template void LaunchSolve<float>(const FactorDev&, const void*, const void*, const void*, void*, void*,
                                 void*, void*, int, cudaStream_t);

}  // namespace sfg
