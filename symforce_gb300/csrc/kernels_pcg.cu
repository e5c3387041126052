// Preconditioned conjugate gradients on the reduced camera system (the PCG forms).
//
//  - Camera-block features: each camera's 9 x 9 block of S scaled to unit diagonal, the rows'
//    coupling to other blocks, the block degree; and the block's scaled Cholesky factor.
//  - Preconditioner blocks P_g = D^-1/2 C^-T L L^T C^-1 D^-1/2 with L from the network (or I:
//    block Jacobi).
//  - One persistent kernel per reduced-system solve: FP64 residual passes r = v - S y around
//    inner PCG solves in the matrix precision, until |r| <= tol |v| or the iteration cap.  Three
//    lanes-groups of nine lanes per warp own the nine rows of one camera block each, so applying
//    P_g is a warp-shuffle product and every thread keeps its row of P_g in registers.  Dot
//    products are reduced in FP64 in a fixed order (warp tree, CTA order, then the same fixed
//    order over CTAs in every CTA), so every CTA takes the same branch and runs are reproducible.
//    Multi-CTA solves use a grid barrier (cooperative launch: all CTAs resident) on one arrival
//    counter that only grows within a launch (zeroed before it), so a CTA waits for the counter to
//    reach its barrier's count and nobody has to release the others; the waits are capped and a
//    cap hit sets the device error word.
//  (The network's inference pass runs on the tensor cores: kernels_tc.cu.)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <string>

#include "common.h"
#include "kernels.h"

namespace sfg {

namespace {

constexpr int kB = kPrecondBlock;
constexpr unsigned kSpinLimit = 1u << 22;
constexpr float kDiagShift = 0.54132485f;  // ln(e - 1): softplus(kDiagShift) = 1
constexpr int kPcgMultiThreads = 256;
// gauge coarse correction: kept while tr(Z^T S Z) / tr(Z^T S_blocks Z) is at most this (a CPU study
// of 30- and 100-camera problems: at 4e-4 the correction saved 25-45 % of the iterations, at 3e-2
// 7-18 %, at 0.8 it cost 30 %)
constexpr double kCoarseMaxRatio = 0.05;
constexpr size_t kPcgStagedMax = 200 * 1024;  // shared memory of a staged one-CTA solve

__device__ __forceinline__ float Softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }

__device__ __forceinline__ int Tri(int i, int j) { return i * (i + 1) / 2 + j; }

// ---------------------------------------------------------------------------------------------
// Features
// ---------------------------------------------------------------------------------------------
// One warp per reduced-system row: rho = sum over entries outside the row's block of
// S_rc^2 / (S_rr S_cc).
template <typename T>
__global__ void PrecondRowKernel(PrecondDev pd, SpmvDev m, const T* S, float* rho) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= m.n) return;
  const int grow = pd.scalar_group[row];
  const float drow = float(S[pd.sdiag_off[row]]);
  float acc = 0.f;
  for (int64_t q = m.row_ptr[row] + lane; q < m.row_ptr[row + 1]; q += 32) {
    const T* a = S + m.seg_base[q];
    const int stride = m.seg_stride[q], n = m.seg_len[q], x0 = m.seg_x[q];
    for (int c = 0; c < n; ++c) {
      const int col = x0 + c;
      if (pd.scalar_group[col] == grow) continue;
      const float v = float(a[int64_t(c) * stride]);
      const float dc = float(S[pd.sdiag_off[col]]);
      acc += v * v / fmaxf(drow * dc, 1e-30f);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) rho[row] = acc;
}

// One thread per camera block: inputs of the network and the block's scaled Cholesky factor.
template <typename T>
__global__ void PrecondFeatureKernel(PrecondDev pd, const T* S, const float* rho, float* feats,
                                     float* fac) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= pd.ng) return;
  const int32_t* gi = pd.gidx + size_t(g) * kB;
  const int64_t* go = pd.goff + size_t(g) * kB * kB;
  float dis[kB];
#pragma unroll
  for (int a = 0; a < kB; ++a) {
    const int64_t o = go[a * kB + a];
    const float d = o >= 0 ? float(S[o]) : 1.f;
    dis[a] = d > 0.f ? rsqrtf(d) : 1.f;
  }
  float A[kB * kB];
#pragma unroll
  for (int a = 0; a < kB; ++a)
#pragma unroll
    for (int b = 0; b < kB; ++b) {
      const int64_t o = go[a * kB + b];
      float v;
      if (o >= 0) v = float(S[o]) * dis[a] * dis[b];
      else v = (o == -1 && a == b) ? 1.f : 0.f;
      A[a * kB + b] = v;
    }
  float* fo = feats + size_t(g) * kPrecondFeatures;
#pragma unroll
  for (int i = 0; i < kB * kB; ++i) fo[i] = A[i];
#pragma unroll
  for (int a = 0; a < kB; ++a) fo[kB * kB + a] = gi[a] >= 0 ? log1pf(rho[gi[a]]) : 0.f;
  fo[kB * kB + kB] = pd.degree[g] * (1.f / 16.f);
#pragma unroll
  for (int i = kB * kB + kB + 1; i < kPrecondFeatures; ++i) fo[i] = 0.f;
  // C C^T = A (lower, packed); identity if A is not numerically positive definite
  float C[kPrecondTri];
  bool ok = true;
#pragma unroll
  for (int i = 0; i < kB; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      float s = A[i * kB + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= C[Tri(i, k)] * C[Tri(j, k)];
      if (i == j) {
        if (!(s > 1e-12f)) {
          ok = false;
          s = 1.f;
        }
        C[Tri(i, i)] = sqrtf(s);
      } else {
        C[Tri(i, j)] = s / C[Tri(j, j)];
      }
    }
  float* fc = fac + size_t(g) * kPrecondFac;
#pragma unroll
  for (int i = 0; i < kB; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) fc[Tri(i, j)] = ok ? C[Tri(i, j)] : (i == j ? 1.f : 0.f);
#pragma unroll
  for (int a = 0; a < kB; ++a) fc[kPrecondTri + a] = dis[a];
}

// P_g = Q Q^T, Q = D^-1/2 C^-T L.
template <typename T>
__global__ void PrecondAssembleKernel(int ng, const float* fac, const float* z, T* P) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  const float* fc = fac + size_t(g) * kPrecondFac;
  float C[kPrecondTri], L[kPrecondTri];
#pragma unroll
  for (int i = 0; i < kPrecondTri; ++i) C[i] = fc[i];
  if (z) {
    const float* zg = z + size_t(g) * kPrecondTri;
#pragma unroll
    for (int i = 0; i < kB; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j) L[Tri(i, j)] = i == j ? Softplus(zg[Tri(i, i)] + kDiagShift) : zg[Tri(i, j)];
  } else {
#pragma unroll
    for (int i = 0; i < kB; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j) L[Tri(i, j)] = i == j ? 1.f : 0.f;
  }
  // M = C^-T L: back substitution with the upper triangle C^T, column by column
  float Q[kB * kB];
#pragma unroll
  for (int j = 0; j < kB; ++j)
#pragma unroll
    for (int i = kB - 1; i >= 0; --i) {
      float s = i >= j ? L[Tri(i, j)] : 0.f;
#pragma unroll
      for (int k = i + 1; k < kB; ++k) s -= C[Tri(k, i)] * Q[k * kB + j];
      Q[i * kB + j] = s / C[Tri(i, i)];
    }
#pragma unroll
  for (int i = 0; i < kB; ++i) {
    const float d = fc[kPrecondTri + i];
#pragma unroll
    for (int j = 0; j < kB; ++j) Q[i * kB + j] *= d;
  }
  T* Pg = P + size_t(g) * kB * kB;
#pragma unroll
  for (int a = 0; a < kB; ++a)
#pragma unroll
    for (int b = 0; b <= a; ++b) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < kB; ++k) s += Q[a * kB + k] * Q[b * kB + k];
      Pg[a * kB + b] = T(s);
      Pg[b * kB + a] = T(s);
    }
}

// ---------------------------------------------------------------------------------------------
// Band preconditioner: factorized sparse approximate inverse M = G^T Lambda G
// ---------------------------------------------------------------------------------------------
// Block row l of G is the last block row of R^-1, R R^T = D^-1/2 S_JJ D^-1/2 over the groups J_l
// (ascending, l last), times D^-1/2: then G S G^T has identity diagonal blocks, and with J_l = {l}
// it is C^-1 D^-1/2 of the block-diagonal preconditioner, so that Lambda = L L^T keeps the
// meaning it has there.  One warp per group row, the scaled S_JJ (n = 9 |J_l|) in shared memory
// with an odd row stride; a block Cholesky by 9 x 9 blocks (the diagonal block by rows, the panel
// by forward substitution in registers, the trailing update with lanes over independent entries),
// then X R = [0 I] by block columns from the right.  A pivot that is not numerically positive
// retries with J_l = {l}; if that fails too the row is D^-1/2 (Jacobi).
__host__ __device__ constexpr int BandLd(int band) { return 9 * (band + 1) + ((band + 1) % 2 == 0 ? 1 : 0); }
__host__ __device__ constexpr int BandWarpElems(int band) {
  return 9 * (band + 1) * BandLd(band) + 9 * (band + 1) + kB * 9 * (band + 1);
}

template <typename T>
__global__ void BandFactorKernel(BandDev bd, const T* Sb) {
  extern __shared__ __align__(16) unsigned char band_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int l = blockIdx.x * (blockDim.x >> 5) + warp;
  if (l >= bd.ng) return;  // warp-uniform
  const int LD = BandLd(bd.band), XLD = 9 * (bd.band + 1);
  T* A = reinterpret_cast<T*>(band_smem) + size_t(warp) * BandWarpElems(bd.band);
  T* dis = A + XLD * LD;  // D^-1/2 of the rows; negative: an identity row (padding)
  T* X = dis + XLD;       // [9][XLD] last block row of R^-1
  const int K1 = bd.band + 1;
  const int nj = bd.nj[l];
  const int32_t* jg = bd.jgrp + size_t(l) * K1;
  const int32_t* jb = bd.jblk + size_t(l) * K1 * K1;
  T* Gl = static_cast<T*>(bd.G) + size_t(l) * K1 * kB * kB;
  const T tiny = T(sizeof(T) == 8 ? 1e-12 : 1e-6);
  auto pair_of = [](int p, int& s1, int& s2) {
    s1 = 0;
    while ((s1 + 1) * (s1 + 2) / 2 <= p) ++s1;
    s2 = p - s1 * (s1 + 1) / 2;
  };
  int s0 = -1;  // first group of J_l that the factor used (-1: none)
  for (int attempt = 0; attempt < 2 && s0 < 0; ++attempt) {
    const int first = attempt == 0 ? 0 : nj - 1;
    const int m = nj - first, n = m * kB, npairs = m * (m + 1) / 2;
    // lane p: the stored block of lower pair p (at most 28 pairs); every row's padding flag
    int pblk = -1;
    if (lane < npairs) {
      int s1, s2;
      pair_of(lane, s1, s2);
      pblk = jb[(first + s1) * K1 + first + s2];
    }
    bool padr[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int r = lane + 32 * q;
      padr[q] = r < n ? bd.gidx[size_t(jg[first + r / kB]) * kB + r % kB] < 0 : true;
    }
    // the raw blocks, four pairs (twelve loads a lane) in flight at a time
    for (int p0 = 0; p0 < npairs; p0 += 4) {
      T v[4][3];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int p = p0 + u;
        const int blk = __shfl_sync(0xffffffffu, pblk, p);
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const int e = lane + 32 * t;
          v[u][t] = (p < npairs && blk >= 0 && e < kB * kB) ? Sb[size_t(blk) * (kB * kB) + e] : T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int p = p0 + u;
        if (p >= npairs) break;
        int s1, s2;
        pair_of(p, s1, s2);
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const int e = lane + 32 * t;
          if (e < kB * kB) A[(kB * s1 + e / kB) * LD + kB * s2 + e % kB] = v[u][t];
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int r = lane + 32 * q;
      if (r < n) {
        const T d = A[r * LD + r];
        dis[r] = (!padr[q] && d > T(0)) ? T(1) / sqrt(d) : T(-1);
      }
    }
    __syncwarp();
    // D^-1/2 S_JJ D^-1/2 (lower), identity rows for padding
    for (int r = 0; r < n; ++r)
      for (int c = lane; c <= r; c += 32) {
        T v = A[r * LD + c];
        if (dis[r] < T(0) || dis[c] < T(0)) v = r == c ? T(1) : T(0);
        else v *= dis[r] * dis[c];
        A[r * LD + c] = v;
      }
    __syncwarp();
    // block Cholesky
    bool ok = true;
    for (int sb = 0; sb < m && ok; ++sb) {
      T* Ass = A + kB * sb * LD + kB * sb;
      for (int j = 0; j < kB; ++j) {  // the diagonal block, lanes over its rows
        T v = T(0);
        if (lane < kB && lane >= j) {
          v = Ass[lane * LD + j];
          for (int k = 0; k < j; ++k) v -= Ass[lane * LD + k] * Ass[j * LD + k];
        }
        const T piv = __shfl_sync(0xffffffffu, v, j);
        if (!(piv > tiny)) {  // the same value in every lane: a warp-uniform exit
          ok = false;
          break;
        }
        const T ljj = sqrt(piv);
        if (lane == j) Ass[j * LD + j] = ljj;
        else if (lane < kB && lane > j) Ass[lane * LD + j] = v / ljj;
        __syncwarp();
      }
      if (!ok) break;
      // the panel below: L_ts = A_ts L_ss^-T, a row per lane in registers
      for (int i = kB * (sb + 1) + lane; i < n; i += 32) {
        T x[kB];
#pragma unroll
        for (int c = 0; c < kB; ++c) x[c] = A[i * LD + kB * sb + c];
#pragma unroll
        for (int c = 0; c < kB; ++c) {
#pragma unroll
          for (int k = 0; k < c; ++k) x[c] -= x[k] * Ass[c * LD + k];
          x[c] /= Ass[c * LD + c];
        }
#pragma unroll
        for (int c = 0; c < kB; ++c) A[i * LD + kB * sb + c] = x[c];
      }
      __syncwarp();
      // the trailing lower blocks (t, u), sb < u <= t < m: A_tu -= L_ts L_us^T
      const int q = m - 1 - sb;
      const int tp = q * (q + 1) / 2;
      for (int pr = 0; pr < tp; ++pr) {
        int tt, uu;
        pair_of(pr, tt, uu);
        const int t = sb + 1 + tt, u = sb + 1 + uu;
        for (int e = lane; e < kB * kB; e += 32) {
          const int r = e / kB, c = e % kB;
          if (t == u && c > r) continue;
          const T* lt = A + (kB * t + r) * LD + kB * sb;
          const T* lu = A + (kB * u + c) * LD + kB * sb;
          T acc = A[(kB * t + r) * LD + kB * u + c];
#pragma unroll
          for (int k = 0; k < kB; ++k) acc -= lt[k] * lu[k];
          A[(kB * t + r) * LD + kB * u + c] = acc;
        }
      }
      __syncwarp();
    }
    if (!ok) {
      __syncwarp();
      continue;
    }
    // X R = [0 I] by block columns from the right: X_s R_ss = delta(s, m - 1) I - sum_{t > s} X_t R_ts
    for (int sb = m - 1; sb >= 0; --sb) {
      for (int e = lane; e < kB * kB; e += 32) {
        const int r = e / kB, c = e % kB;
        T b = (sb == m - 1 && r == c) ? T(1) : T(0);
        for (int t = sb + 1; t < m; ++t) {
          const T* xr = X + r * XLD + kB * t;
#pragma unroll
          for (int k = 0; k < kB; ++k) b -= xr[k] * A[(kB * t + k) * LD + kB * sb + c];
        }
        X[r * XLD + kB * sb + c] = b;
      }
      __syncwarp();
      if (lane < kB) {  // row `lane` of X_s: x R_ss = b, from the last column down
        const T* Ass = A + kB * sb * LD + kB * sb;
        T x[kB];
#pragma unroll
        for (int c = 0; c < kB; ++c) x[c] = X[lane * XLD + kB * sb + c];
#pragma unroll
        for (int c = kB - 1; c >= 0; --c) {
#pragma unroll
          for (int k = c + 1; k < kB; ++k) x[c] -= x[k] * Ass[k * LD + c];
          x[c] /= Ass[c * LD + c];
        }
#pragma unroll
        for (int c = 0; c < kB; ++c) X[lane * XLD + kB * sb + c] = x[c];
      }
      __syncwarp();
    }
    s0 = first;
  }
  // block (l, l - band + slot) of G: X's columns of that group times D^-1/2
  for (int e = lane; e < K1 * kB * kB; e += 32) {
    const int slot = e / (kB * kB), rc = e - slot * (kB * kB), r = rc / kB, c = rc % kB;
    const int grp = l - bd.band + slot;
    T v = T(0);
    if (s0 >= 0) {
      for (int sg = s0; sg < nj; ++sg)
        if (jg[sg] == grp) {
          const int col = (sg - s0) * kB + c;
          v = X[r * XLD + col] * (dis[col] < T(0) ? T(1) : dis[col]);
        }
    } else if (grp == l && r == c) {  // Jacobi row
      const int blk = jb[(nj - 1) * K1 + nj - 1];
      const T d = blk >= 0 ? Sb[size_t(blk) * (kB * kB) + r * kB + r] : T(0);
      v = d > T(0) ? T(1) / sqrt(d) : T(1);
    }
    Gl[e] = v;
  }
}

// M_{a, a - d} = sum over l = a .. min(a - d + band, ng - 1) of G_{l,a}^T Lambda_l G_{l,a-d}; one
// warp per (a, d), four warps per CTA.  All the terms' blocks (and network outputs) are loaded into
// shared memory at once, then added in l order.
constexpr int kBandAsmWarps = 4;
template <typename T>
__global__ void BandAssembleKernel(BandDev bd, const float* z, T* Mb) {
  constexpr int kT = kPcgMaxBand + 1;
  __shared__ T sg[kBandAsmWarps][kT][2][kB * kB];
  __shared__ float sz[kBandAsmWarps][kT][kPrecondTri];
  __shared__ T stt[kBandAsmWarps][2][kB * kB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int K1 = bd.band + 1;
  const int idx = blockIdx.x * kBandAsmWarps + warp;
  if (idx >= bd.ng * K1) return;  // warp-uniform
  const int a = idx / K1, b = a - idx % K1;
  const int nterm = b >= 0 ? min(b + bd.band, bd.ng - 1) - a + 1 : 0;
  for (int e = lane; e < nterm * 2 * kB * kB; e += 32) {
    const int t = e / (2 * kB * kB), w = (e / (kB * kB)) & 1, x = e % (kB * kB);
    const int l = a + t;
    const int slot = (w ? b : a) - l + bd.band;
    sg[warp][t][w][x] = static_cast<const T*>(bd.G)[(size_t(l) * K1 + slot) * (kB * kB) + x];
  }
  if (z)
    for (int e = lane; e < nterm * kPrecondTri; e += 32)
      sz[warp][e / kPrecondTri][e % kPrecondTri] = z[size_t(a + e / kPrecondTri) * kPrecondTri + e % kPrecondTri];
  __syncwarp();
  T acc[3] = {T(0), T(0), T(0)};
  T* Lm = stt[warp][0];
  T* tt = stt[warp][1];
  for (int t = 0; t < nterm; ++t) {
    const T* ga = sg[warp][t][0];
    T* gb = sg[warp][t][1];
    if (z) {  // gb <- L (L^T gb)
      const float* zl = sz[warp][t];
      for (int e = lane; e < kB * kB; e += 32) {
        const int i = e / kB, j = e % kB;
        Lm[e] = j > i ? T(0) : i == j ? T(Softplus(zl[Tri(i, i)] + kDiagShift)) : T(zl[Tri(i, j)]);
      }
      __syncwarp();
      for (int e = lane; e < kB * kB; e += 32) {
        const int x = e / kB, c = e % kB;
        T s = T(0);
        for (int y = x; y < kB; ++y) s += Lm[y * kB + x] * gb[y * kB + c];
        tt[e] = s;
      }
      __syncwarp();
      for (int e = lane; e < kB * kB; e += 32) {
        const int x = e / kB, c = e % kB;
        T s = T(0);
        for (int y = 0; y <= x; ++y) s += Lm[x * kB + y] * tt[y * kB + c];
        gb[e] = s;
      }
      __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int e = lane + 32 * k;
      if (e < kB * kB) {
        const int r = e / kB, c = e % kB;
        T s = T(0);
#pragma unroll
        for (int x = 0; x < kB; ++x) s += ga[x * kB + r] * gb[x * kB + c];
        acc[k] += s;
      }
    }
    __syncwarp();
  }
  T* out = Mb + size_t(idx) * (kB * kB);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int e = lane + 32 * k;
    if (e < kB * kB) out[e] = acc[k];
  }
}

// Training samples of the current system: inputs, g_hat = C^-1 D^-1/2 v_g, x_hat = C^T D^1/2 y_g.
template <typename T>
__global__ void CollectSamplesKernel(PrecondDev pd, const float* feats, const float* fac,
                                     const T* v, const double* y, float* samples, int max_systems,
                                     const LmState* st) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int slot = st->num_records - 1;
  if (g >= pd.ng || slot < 0 || slot >= max_systems) return;
  const int32_t* gi = pd.gidx + size_t(g) * kB;
  const float* fc = fac + size_t(g) * kPrecondFac;
  float* out = samples + (size_t(slot) * pd.ng + g) * kSampleFloats;
  const float* fi = feats + size_t(g) * kPrecondFeatures;
  for (int i = 0; i < kPrecondFeatures; ++i) out[i] = fi[i];
  float gh[kB];
#pragma unroll
  for (int i = 0; i < kB; ++i) {
    float s = gi[i] >= 0 ? float(v[gi[i]]) * fc[kPrecondTri + i] : 0.f;
#pragma unroll
    for (int k = 0; k < i; ++k) s -= fc[Tri(i, k)] * gh[k];
    gh[i] = s / fc[Tri(i, i)];
  }
  float yd[kB];
#pragma unroll
  for (int i = 0; i < kB; ++i) yd[i] = gi[i] >= 0 ? float(y[gi[i]]) / fc[kPrecondTri + i] : 0.f;
#pragma unroll
  for (int i = 0; i < kB; ++i) {
    float s = 0.f;
#pragma unroll
    for (int k = i; k < kB; ++k) s += fc[Tri(k, i)] * yd[k];
    out[kPrecondFeatures + i] = gh[i];
    out[kPrecondFeatures + kB + i] = s;
  }
}

// ---------------------------------------------------------------------------------------------
// PCG
// ---------------------------------------------------------------------------------------------
// Barrier number `epoch` (1, 2, ... within the launch; kept by thread 0 of each CTA): arrive on
// the counter, then wait until all nblocks CTAs have arrived epoch times.
// Thread 0 only: arrive and wait.  The arrival is a release (the CTA's writes, ordered before it by
// a CTA barrier, become visible with it) and the polls acquire, so no separate fences sit on the
// path.
__device__ void GridArriveWait(unsigned* bar, unsigned nblocks, unsigned& epoch, int* err) {
  const unsigned target = ++epoch * nblocks;
  asm volatile("red.release.gpu.global.add.u32 [%0], 1;" : : "l"(bar) : "memory");
  unsigned it = 0, count;
  for (;;) {
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(count) : "l"(bar) : "memory");
    if (count >= target) break;
    if (++it > kSpinLimit) {
      atomicExch(err, kDevSpinTimeout);
      break;
    }
    if ((it & 63) == 0 && *reinterpret_cast<volatile int*>(err) != 0) break;
  }
}
__device__ void GridBarrier(unsigned* bar, unsigned nblocks, unsigned& epoch, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) GridArriveWait(bar, nblocks, epoch, err);
  __syncthreads();
}

// 1 / x for the CG scalars: the hardware's approximate FP64 reciprocal and two Newton-Raphson
// steps (on this GPU one FP64 division costs ~560 cycles, one dependent FP64 operation ~64);
// inputs outside the range where the approximation is normal take the IEEE division.
__device__ __forceinline__ double FastRecip(double x) {
  const int ex = __double2hiint(x) & 0x7FF00000;
  if (ex < 0x00200000 || ex >= 0x7FD00000) return 1.0 / x;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

template <typename T>
__device__ __forceinline__ T ApplyBlock(const T (&prow)[kB], T r, int gbase) {
  T acc = T(0);
#pragma unroll
  for (int b = 0; b < kB; ++b) acc += prow[b] * __shfl_sync(0xffffffffu, r, gbase + b);
  return acc;
}

// Vectors that other threads wrote in this launch: shared memory (staged) or L2 (grid-wide).
template <bool kStaged, typename V>
__device__ __forceinline__ V LdX(const V* p) {
  if constexpr (kStaged) return *p;
  else return __ldcg(p);
}
template <bool kStaged, typename V>
__device__ __forceinline__ void StX(V* p, V v) {
  if constexpr (kStaged) *p = v;
  else __stcg(p, v);
}

// Row a of group row g of S times x (group-major): the stored lower blocks of the row, and the
// transposed stored blocks (h, g) for the neighbours h > g (addressing chosen without branching).
template <typename Acc, bool kStaged, typename T, typename V>
__device__ __forceinline__ Acc GroupRow(const T* Sb, const int2* gent, int e0, int e1, int stride,
                                        int a, const V* x) {
  // entries e0, e0 + stride, ... of the row; blocks are taken U at a time with all their loads
  // issued before the multiply-adds, so U round trips to L2 overlap; U shrinks with the operand
  // width to stay within the 64 registers of a 1024-thread CTA
  constexpr int U = sizeof(T) + sizeof(V) == 8 ? 4 : sizeof(T) + sizeof(V) == 12 ? 2 : 1;
  Acc acc = Acc(0);
  int e = e0;
  for (; e + (U - 1) * stride < e1; e += U * stride) {
    T sv[U][kB];
    V xv[U][kB];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int2 en = gent[e + u * stride];
      const int tr = en.y & 1;
      const T* row = Sb + size_t(en.x) * (kB * kB) + (tr ? a : a * kB);
      const int step = tr ? kB : 1;
      const V* xh = x + size_t(en.y >> 1) * kB;
#pragma unroll
      for (int b = 0; b < kB; ++b) {
        sv[u][b] = row[b * step];
        xv[u][b] = LdX<kStaged>(xh + b);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int b = 0; b < kB; ++b) acc += Acc(sv[u][b]) * Acc(xv[u][b]);
  }
  for (; e < e1; e += stride) {
    const int2 en = gent[e];
    const int tr = en.y & 1;
    const T* row = Sb + size_t(en.x) * (kB * kB) + (tr ? a : a * kB);
    const int step = tr ? kB : 1;
    const V* xh = x + size_t(en.y >> 1) * kB;
#pragma unroll
    for (int b = 0; b < kB; ++b) acc += Acc(row[b * step]) * Acc(LdX<kStaged>(xh + b));
  }
  return acc;
}

// Row a of group row g of the diagonal block S_gg times x (the entry of the row's list whose
// neighbour is g itself); entries e0, e0 + stride, ... as GroupRow.
template <bool kStaged, typename T, typename V>
__device__ __forceinline__ T DiagBlockRow(const T* Sb, const int2* gent, int e0, int e1, int stride, int a,
                                          const V* x, int g) {
  T acc = T(0);
  for (int e = e0; e < e1; e += stride) {
    const int2 en = gent[e];
    if ((en.y >> 1) != g) continue;
    const int tr = en.y & 1;
    const T* row = Sb + size_t(en.x) * (kB * kB) + (tr ? a : a * kB);
    const int step = tr ? kB : 1;
    const V* xh = x + size_t(g) * kB;
#pragma unroll
    for (int b = 0; b < kB; ++b) acc += row[b * step] * T(LdX<kStaged>(xh + b));
  }
  return acc;
}

// Sum of a row's partial products over the SPLIT lanes that share the row (lanes a, a + 9, a + 18),
// added in the same order in every one of them, so all hold the same bits.
template <int SPLIT, typename V>
__device__ __forceinline__ V CombineSplit(V x, int a) {
  if constexpr (SPLIT == 1) {
    return x;
  } else {
    const V t0 = __shfl_sync(0xffffffffu, x, a);
    const V t1 = __shfl_sync(0xffffffffu, x, a + kB);
    const V t2 = __shfl_sync(0xffffffffu, x, a + 2 * kB);
    return (t0 + t1) + t2;
  }
}

template <typename T> struct PairOf;
template <> struct PairOf<float> { using type = float2; };
template <> struct PairOf<double> { using type = double2; };

// Row a of group row g of the band preconditioner M times x_h = r_h - alpha q_h (kQ) or r_h, over
// the neighbours h = g + j, j = -band + phase, -band + phase + stride, ... <= band; (r, q) of
// every row interleaved in rq.  M_{g,h} is the stored block (g, g - h) for h <= g and the
// transposed block (h, h - g) above.  Lane a of the row's nine lanes (gbase + a) loads entry a of
// x_h and the nine lanes exchange them by shuffles; three blocks at a time, every load issued
// before the multiply-adds.  Called by all lanes of the warp with the same trip count (lanes with
// ok_row false add nothing).
template <bool kQ, int SPLIT, typename T>
__device__ __forceinline__ T BandRow(const T* Mb, int band, int ng, int g, int a, int gbase, int phase,
                                     bool ok_row, const typename PairOf<T>::type* rq, T alpha) {
  constexpr int U = sizeof(T) == 8 ? 2 : 3;
  const int K1 = band + 1;
  const int per_phase = (2 * band + SPLIT) / SPLIT;  // blocks of phase 0, the most of any phase
  const int trips = (per_phase + U - 1) / U;
  T acc = T(0);
  for (int t = 0; t < trips; ++t) {
    T mv[U][kB], xe[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = -band + phase + (t * U + u) * SPLIT;
      const int h = g + j;
      const bool ok = ok_row && j <= band && h >= 0 && h < ng;
      const int hc = ok ? h : 0;
      const T* blk = j <= 0 ? Mb + (size_t(ok ? g : 0) * K1 + (ok ? -j : 0)) * (kB * kB) + a * kB
                            : Mb + (size_t(hc) * K1 + (ok ? j : 0)) * (kB * kB) + a;
      const int step = j <= 0 ? 1 : kB;
#pragma unroll
      for (int b = 0; b < kB; ++b) mv[u][b] = ok ? blk[b * step] : T(0);
      const auto v = __ldcg(rq + size_t(hc) * kB + a);
      xe[u] = ok ? (kQ ? v.x - alpha * v.y : v.x) : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int b = 0; b < kB; ++b) acc += mv[u][b] * __shfl_sync(0xffffffffu, xe[u], gbase + b);
  }
  return acc;
}

struct PcgShared {
  double2 red[32];
  double vnorm, target2, rel;
  double rz, alpha, beta;
  int iters, stop, broke, converged;
  unsigned epoch;  // grid barriers passed (thread 0 only)
  double E[kGaugeDim * kGaugeDim];  // coarse correction: (Z^T S Z)^-1
  double cg[kGaugeDim];             // coarse correction of the current residual: E Z^T r
  double sums[32];                  // results of GridReduceN
  double trs, trd;                  // tr(Z^T S Z), tr(Z^T S_blocks Z)
  double zsz[kGaugeDim * (kGaugeDim + 1) / 2];  // Z^T S Z, packed lower
};

// Sum (a, b) over the grid: a warp tree in Acc, the CTA's warps in order (warp 0, Acc), and the CTAs
// in order (every CTA's warp 0, in FP64, so every CTA gets the same bits).  Thread 0 of every CTA
// then runs epi(sum_a, sum_b) (in Acc for one CTA, FP64 across CTAs), which writes the scalars the
// threads need into shared memory; they are visible to all threads on return.
template <typename Acc, typename Epi>
__device__ __forceinline__ void GridReduce(Acc a, Acc b, const PcgDev& d, int& seq, PcgShared& sm,
                                           Epi epi) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int grid = gridDim.x;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  Acc* red = reinterpret_cast<Acc*>(sm.red);
  __syncthreads();  // every thread has read the previous scalars
  if (lane == 0) {
    red[2 * warp] = a;
    red[2 * warp + 1] = b;
  }
  __syncthreads();
  double2* part = reinterpret_cast<double2*>(d.partials) + size_t(seq & 1) * grid;
  if (warp == 0) {
    Acc ta = lane < nwarp ? red[2 * lane] : Acc(0);
    Acc tb = lane < nwarp ? red[2 * lane + 1] : Acc(0);
    // as many levels as the CTA has warps need (nwarp <= 2^levels)
    for (int o = 1; o < nwarp; o <<= 1) {
      const Acc ua = __shfl_xor_sync(0xffffffffu, ta, o);
      const Acc ub = __shfl_xor_sync(0xffffffffu, tb, o);
      ta += ua;  // a butterfly: every lane ends with the same bits
      tb += ub;
    }
    if (lane == 0) {
      if (grid == 1) epi(ta, tb);
      else __stcg(part + blockIdx.x, make_double2(double(ta), double(tb)));
    }
  }
  if (grid > 1 && warp == 0) {
    // thread 0 stored the partial after the CTA barrier that ordered every thread's writes before
    // it; only warp 0 needs the others' partials
    if (lane == 0) GridArriveWait(d.bar, grid, sm.epoch, d.err);
    __syncwarp();
    {
      // four partials per lane in flight at once, added in CTA order
      double ta = 0.0, tb = 0.0;
      for (int q0 = lane; q0 < grid; q0 += 128) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          v[u] = q0 + 32 * u < grid ? __ldcg(part + q0 + 32 * u) : make_double2(0.0, 0.0);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          ta += v[u].x;
          tb += v[u].y;
        }
      }
      for (int o = 1; o < min(grid, 32); o <<= 1) {
        const double ua = __shfl_xor_sync(0xffffffffu, ta, o);
        const double ub = __shfl_xor_sync(0xffffffffu, tb, o);
        ta += ua;
        tb += ub;
      }
      if (lane == 0) epi(Acc(ta), Acc(tb));
    }
  }
  __syncthreads();
  ++seq;
}

// Sum of N values (N <= kPcgReduceMax) over the grid in FP64, in the fixed orders of GridReduce
// (warp trees, the CTA's warps in order, the CTAs in order); thread 0 of every CTA then runs
// epi(sums), whose shared-memory writes are visible to all threads on return.  red: shared scratch
// of 32 x N doubles.
template <int N, typename Epi>
__device__ __forceinline__ void GridReduceN(double (&v)[N], const PcgDev& d, int& seq, PcgShared& sm,
                                            double* red, Epi epi) {
  static_assert(N <= kPcgReduceMax && N <= 32, "partials hold kPcgReduceMax values per CTA");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int grid = gridDim.x;
#pragma unroll
  for (int n = 0; n < N; ++n)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[n] += __shfl_down_sync(0xffffffffu, v[n], o);
  __syncthreads();  // every thread has read the previous scalars
  if (lane == 0)
#pragma unroll
    for (int n = 0; n < N; ++n) red[warp * N + n] = v[n];
  __syncthreads();
  double* part = d.partials + size_t(seq & 1) * grid * kPcgReduceMax;
  double* sums = sm.sums;
  if (warp == 0) {
    // lane n < N sums value n over the CTA's warps in order
    if (lane < N) {
      double t = 0.0;
      for (int w = 0; w < nwarp; ++w) t += red[w * N + lane];
      if (grid == 1) sums[lane] = t;
      else __stcg(part + size_t(blockIdx.x) * kPcgReduceMax + lane, t);
    }
    __syncwarp();
    if (grid == 1 && lane == 0) epi(sums);
  }
  if (grid > 1 && warp == 0) {
    if (lane == 0) GridArriveWait(d.bar, grid, sm.epoch, d.err);
    __syncwarp();
    {
      // lane l takes the CTAs l, l + 32, ... (all N values each, the loads in flight together),
      // then a warp tree per value: a fixed order, the same bits in every CTA
      double t[N];
#pragma unroll
      for (int n = 0; n < N; ++n) t[n] = 0.0;
      for (int q = lane; q < grid; q += 32)
#pragma unroll
        for (int n = 0; n < N; ++n) t[n] += __ldcg(part + size_t(q) * kPcgReduceMax + n);
      for (int o = 1; o < min(grid, 32); o <<= 1)
#pragma unroll
        for (int n = 0; n < N; ++n) t[n] += __shfl_xor_sync(0xffffffffu, t[n], o);
      if (lane == 0)
#pragma unroll
        for (int n = 0; n < N; ++n) sums[n] = t[n];
      __syncwarp();
      if (lane == 0) epi(sums);
    }
  }
  __syncthreads();
  ++seq;
}

// The gauge coarse correction's 7 x 7 matrix E = (Z^T S Z)^-1 from the packed lower triangle of
// Z^T S Z (28 values), by an LDL^T and the solve of the seven unit vectors; false when Z^T S Z is
// not positive definite (then no coarse correction: E = 0).  Thread 0 of each CTA, same bits in all.
__device__ bool GaugeInverse(const double* g, double* E) {
  constexpr int K = kGaugeDim;
  double a[K][K], d[K];
  for (int i = 0; i < K; ++i)
    for (int j = 0; j <= i; ++j) a[i][j] = a[j][i] = g[i * (i + 1) / 2 + j];
  // A = L D L^T (unit L below the diagonal)
  for (int k = 0; k < K; ++k) {
    double dk = a[k][k];
    for (int q = 0; q < k; ++q) dk -= a[k][q] * a[k][q] * d[q];
    if (!(dk > 1e-300 * (fabs(a[k][k]) + 1e-300)) || !(dk < 1e300)) return false;
    d[k] = dk;
    for (int i = k + 1; i < K; ++i) {
      double v = a[i][k];
      for (int q = 0; q < k; ++q) v -= a[i][q] * a[k][q] * d[q];
      a[i][k] = v / dk;
    }
  }
  for (int c = 0; c < K; ++c) {
    double x[K];
    for (int i = 0; i < K; ++i) {
      double v = i == c ? 1.0 : 0.0;
      for (int q = 0; q < i; ++q) v -= a[i][q] * x[q];
      x[i] = v;
    }
    for (int i = 0; i < K; ++i) x[i] /= d[i];
    for (int i = K - 1; i >= 0; --i)
      for (int q = i + 1; q < K; ++q) x[i] -= a[q][i] * x[q];
    for (int i = 0; i < K; ++i) E[i * K + c] = x[i];
  }
  return true;
}

// One stamp of the optional iteration trace (CTA 0, thread 0).
__device__ __forceinline__ void PcgStamp(const PcgDev& d, int it, int phase) {
  if (d.trace && blockIdx.x == 0 && threadIdx.x == 0 && it < d.trace_cap) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    d.trace[1 + 4 * size_t(it) + phase] = t;
  }
}

// Vector arithmetic in the matrix precision T (FP32 in the mixed form); inner products, CG scalars,
// the residual passes and the stopping decisions in FP64.
// SPLIT 1: three camera blocks per warp (lanes 9 q + a, row a of block q).  SPLIT 3: one camera
// block per warp and three lanes per row (lanes 9 q + a for q = 0..2), each taking every third
// entry of the row's product with S, so a row waits on a third of the L2 round trips; the vectors
// are kept in all three lanes (same bits) and only lane a reduces and stores.
// kCoarse: the preconditioner adds a coarse correction on the camera poses' similarity gauge,
// M^-1 r = P r + Z E Z^T r with E = (Z^T S Z)^-1 (an additive two-level preconditioner; Z from
// LaunchGaugeBasis).  S Z is formed once per launch and kept by row, so that the product of a search
// direction stays one pass over S: S z = S (P r) + (S Z) c, c = E Z^T r, and Z^T r rides in the
// grid reduction that already follows the update of r.
template <typename T, bool kStaged, int SPLIT, bool kCoarse, bool kBand>
__global__ void __launch_bounds__(1024) PcgKernel(PcgDev d) {
  static_assert(SPLIT == 1 || SPLIT == 3, "one or three lanes per row");
  static_assert(!(kCoarse && kBand), "the coarse correction goes with the block-diagonal preconditioner");
  extern __shared__ __align__(16) unsigned char pcg_smem[];
  __shared__ PcgShared sm;
  __shared__ double redn[kCoarse ? 32 * (2 + kGaugeDim) : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = lane / kB;  // 0..2; 3: idle lanes 27..31
  const int a = lane - slot * kB;
  const int ng = d.pd.ng;
  const int sub = SPLIT == 1 ? slot : 0;    // camera block of the lane within the warp
  const int split = SPLIT == 1 ? 0 : slot;  // entry phase of the lane within its row
  const int g = (blockIdx.x * (blockDim.x >> 5) + warp) * (3 / SPLIT) + sub;
  const bool in_group = slot < 3 && g < ng;
  const int s = in_group ? d.pd.gidx[size_t(g) * kB + a] : -1;
  const bool row_ok = s >= 0;
  const bool own = row_ok && split == 0;  // reduces and stores the row
  const bool store = in_group && split == 0;
  const int gbase = slot < 3 ? slot * kB : 0;
  const size_t gi = size_t(in_group ? g : 0) * kB + a;
  const int e0 = in_group ? d.gptr[g] + split : 0, e1 = in_group ? d.gptr[g + 1] : 0;
  const T* Sb;
  const int2* gent;
  T* zv;
  double* ygv;
  if constexpr (kStaged) {
    const int nent = d.gptr[ng];
    double* sy = reinterpret_cast<double*>(pcg_smem);
    int2* se = reinterpret_cast<int2*>(sy + size_t(ng) * kB);
    T* sS = reinterpret_cast<T*>(se + nent);
    T* sz = sS + size_t(d.nbl) * kB * kB;
    const T* gS = static_cast<const T*>(d.Sb);
    for (size_t i = threadIdx.x; i < size_t(d.nbl) * kB * kB; i += blockDim.x) sS[i] = gS[i];
    for (int i = threadIdx.x; i < nent; i += blockDim.x) se[i] = d.gent[i];
    for (int i = threadIdx.x; i < ng * kB; i += blockDim.x) {
      sz[i] = T(0);
      sy[i] = 0.0;
    }
    Sb = sS;
    gent = se;
    zv = sz;
    ygv = sy;
  } else {
    Sb = static_cast<const T*>(d.Sb);
    gent = d.gent;
    zv = static_cast<T*>(d.z);
    ygv = d.yg;
  }
  if (threadIdx.x == 0) {
    sm.epoch = 0;
    sm.iters = 0;
    sm.converged = 0;
    sm.broke = 0;
    sm.rel = 0.0;
  }
  const T* v = static_cast<const T*>(d.v);
  const T* P = static_cast<const T*>(d.P);
  T prow[kB];
#pragma unroll
  for (int b = 0; b < kB; ++b) prow[b] = (!kBand && row_ok) ? P[(size_t(g) * kB + a) * kB + b] : T(0);
  using T2 = typename PairOf<T>::type;
  const T* Mb = static_cast<const T*>(d.Mb);
  T2* rq = static_cast<T2*>(d.RQ);
  // the preconditioned residual of this row: the block product in registers, or a row of the
  // band preconditioner over the (r, q) that every row stored before the last grid reduction
  auto precond = [&](T r, T alpha, bool with_q) -> T {
    if constexpr (kBand) {
      const T zb = with_q ? BandRow<true, SPLIT>(Mb, d.band, ng, g, a, gbase, split, in_group, rq, alpha)
                          : BandRow<false, SPLIT>(Mb, d.band, ng, g, a, gbase, split, in_group, rq, alpha);
      return CombineSplit<SPLIT>(zb, a);
    } else {
      return ApplyBlock(prow, r, gbase);
    }
  };
  int seq = 0;
  const double vs = row_ok ? double(v[s]) : 0.0;
  GridReduce<double>(own ? vs * vs : 0.0, 0.0, d, seq, sm, [&](double x, double) {
    sm.vnorm = sqrt(x);
    sm.converged = sm.vnorm > 0.0 ? 0 : 1;  // zero rhs: y = 0
  });
  const double vnorm = sm.vnorm;
  const size_t nrows = size_t(ng) * kB;
  const T* zg = static_cast<const T*>(d.zg);
  T* szg = static_cast<T*>(d.szg);
  if constexpr (kCoarse) {
    // S Z by row (kept for the products), then Z^T S Z over the grid and its inverse
    // Column j of Z^T S Z (rows i = 0 .. 6; the lower part is kept) per grid reduction, with
    // z_j^T S_blocks z_j (the camera blocks alone).  The correction is kept only while the gauge
    // directions are near-null next to what the blocks see, tr(Z^T S Z) <= kCoarseMaxRatio
    // tr(Z^T S_blocks Z): with large damping they are not, and the correction costs iterations.
    if (threadIdx.x == 0) {
      sm.trs = 0.0;
      sm.trd = 0.0;
    }
    for (int j = 0; j < kGaugeDim; ++j) {
      const T sz = CombineSplit<SPLIT>(
          in_group ? GroupRow<T, kStaged>(Sb, gent, e0, e1, SPLIT, a, zg + j * nrows) : T(0), a);
      const T dz = CombineSplit<SPLIT>(
          in_group ? DiagBlockRow<kStaged>(Sb, gent, e0, e1, SPLIT, a, zg + j * nrows, g) : T(0), a);
      if (store) szg[j * nrows + gi] = sz;
      const double zj = row_ok ? double(zg[j * nrows + gi]) : 0.0;
      double zs[kGaugeDim + 1];
#pragma unroll
      for (int i = 0; i < kGaugeDim; ++i) zs[i] = own ? double(row_ok ? zg[i * nrows + gi] : T(0)) * double(sz) : 0.0;
      zs[kGaugeDim] = own ? zj * double(dz) : 0.0;
      GridReduceN<kGaugeDim + 1>(zs, d, seq, sm, redn, [&](double* gs) {
        for (int i = j; i < kGaugeDim; ++i) sm.zsz[i * (i + 1) / 2 + j] = gs[i];
        sm.trs += gs[j];
        sm.trd += gs[kGaugeDim];
        if (j == kGaugeDim - 1 &&
            (!(sm.trs <= kCoarseMaxRatio * sm.trd) || !GaugeInverse(sm.zsz, sm.E)))
          for (int q = 0; q < kGaugeDim * kGaugeDim; ++q) sm.E[q] = 0.0;
      });
    }
  }
  // the coarse correction c = E Z^T r from the reduced Z^T r (thread 0 of each CTA)
  auto coarse_of = [&](const double* ztr) {
    for (int i = 0; i < kGaugeDim; ++i) {
      double c = 0.0;
      for (int j = 0; j < kGaugeDim; ++j) c += sm.E[i * kGaugeDim + j] * ztr[j];
      sm.cg[i] = c;
    }
  };
  auto z_plus_coarse = [&](T zb) {  // P r + Z c of this row
    T z = zb;
#pragma unroll
    for (int i = 0; i < kGaugeDim; ++i) z += (row_ok ? zg[i * nrows + gi] : T(0)) * T(sm.cg[i]);
    return z;
  };
  double y64 = 0.0;
  int outer = 0, traced = 0;
  while (!sm.converged) {
    double r64 = vs;
    if (outer > 0) {
      const double sy = CombineSplit<SPLIT>(
          in_group ? GroupRow<double, kStaged>(Sb, gent, e0, e1, SPLIT, a, ygv) : 0.0, a);
      if (in_group) r64 = vs - sy;
    }
    if constexpr (kBand) {
      if (store) __stcg(rq + gi, T2{T(r64), T(0)});
    }
    GridReduce<double>(own ? r64 * r64 : 0.0, 0.0, d, seq, sm, [&](double x, double) {
      sm.rel = sqrt(x) / vnorm;
      sm.converged = sm.rel <= d.tol ? 1 : 0;
      sm.stop = (sm.converged || outer >= d.max_outer || sm.iters >= d.max_iters || sm.broke ||
                 !(sm.rel == sm.rel)) ? 1 : 0;
      const double target = fmax(0.5 * d.tol * vnorm, d.inner_floor * sqrt(x));
      sm.target2 = target * target;  // the inner solves stop once |r|^2 <= target^2
    });
    if (sm.stop) break;
    ++outer;
    // inner PCG on S dx = r (x0 = 0): vectors and the products with S and P in the matrix
    // precision T, inner products and the CG scalars in FP64 (FP32 sums of a few thousand terms
    // lose the digits the recurrences need on these ill-conditioned systems).  The product uses
    // w = S z and q = w + beta q so that one grid reduction separates the product from the update.
    T r = T(r64);
    T zz = precond(r, T(0), false);
    if (store) StX<kStaged>(zv + gi, zz);
    T zf = zz;  // the preconditioned residual (with the coarse correction)
    if constexpr (kCoarse) {
      double rv[1 + kGaugeDim];
      rv[0] = own ? double(r) * double(zz) : 0.0;
#pragma unroll
      for (int i = 0; i < kGaugeDim; ++i) rv[1 + i] = own ? double(r) * double(zg[i * nrows + gi]) : 0.0;
      GridReduceN<1 + kGaugeDim>(rv, d, seq, sm, redn, [&](double* g) {
        coarse_of(g + 1);
        double rz = g[0];
        for (int i = 0; i < kGaugeDim; ++i) rz += sm.cg[i] * g[1 + i];
        sm.rz = rz;
      });
      zf = z_plus_coarse(zz);
    } else {
      GridReduce<double>(own ? double(r) * double(zz) : 0.0, 0.0, d, seq, sm,
                         [&](double x, double) { sm.rz = x; });
    }
    T p = T(0), qv = T(0), dx = T(0), beta = T(0);
    for (;;) {
      T w = CombineSplit<SPLIT>(in_group ? GroupRow<T, kStaged>(Sb, gent, e0, e1, SPLIT, a, zv) : T(0), a);
      PcgStamp(d, traced, 0);
      if constexpr (kCoarse) {
#pragma unroll
        for (int i = 0; i < kGaugeDim; ++i) w += (row_ok ? szg[i * nrows + gi] : T(0)) * T(sm.cg[i]);
      }
      p = zf + beta * p;
      qv = w + beta * qv;
      if constexpr (kBand) {
        if (store) __stcg(rq + gi, T2{r, qv});
      }
      GridReduce<double>(own ? double(p) * double(qv) : 0.0, 0.0, d, seq, sm, [&](double pq, double) {
        const double rz = sm.rz;
        if (!(pq > 0.0) || !(pq < 1e300) || !(fabs(rz) < 1e300)) sm.broke = 1;
        else sm.alpha = rz * FastRecip(pq);
      });
      PcgStamp(d, traced, 1);
      if (sm.broke) break;
      const T alpha = T(sm.alpha);
      dx += alpha * p;
      r -= alpha * qv;
      zz = precond(r, alpha, true);
      if (store) StX<kStaged>(zv + gi, zz);
      PcgStamp(d, traced, 2);
      if constexpr (kCoarse) {
        double rv[2 + kGaugeDim];
        rv[0] = own ? double(r) * double(zz) : 0.0;
        rv[1] = own ? double(r) * double(r) : 0.0;
#pragma unroll
        for (int i = 0; i < kGaugeDim; ++i) rv[2 + i] = own ? double(r) * double(zg[i * nrows + gi]) : 0.0;
        GridReduceN<2 + kGaugeDim>(rv, d, seq, sm, redn, [&](double* g) {
          coarse_of(g + 2);
          double rz = g[0];
          for (int i = 0; i < kGaugeDim; ++i) rz += sm.cg[i] * g[2 + i];
          sm.iters += 1;
          sm.stop = (g[1] <= sm.target2 || sm.iters >= d.max_iters) ? 1 : 0;
          sm.beta = rz * FastRecip(sm.rz);
          sm.rz = rz;
        });
        zf = z_plus_coarse(zz);
      } else {
        GridReduce<double>(own ? double(r) * double(zz) : 0.0, own ? double(r) * double(r) : 0.0, d, seq, sm,
                           [&](double rz, double rr) {
          sm.iters += 1;
          sm.stop = (rr <= sm.target2 || sm.iters >= d.max_iters) ? 1 : 0;
          sm.beta = rz * FastRecip(sm.rz);
          sm.rz = rz;
        });
        zf = zz;
      }
      PcgStamp(d, traced++, 3);
      if (sm.stop) break;
      beta = T(sm.beta);
    }
    y64 += double(dx);
    if (store) StX<kStaged>(ygv + gi, y64);
    if (gridDim.x > 1) GridBarrier(d.bar, gridDim.x, sm.epoch, d.err);
    else __syncthreads();
  }
  if (own) __stcg(d.y + s, y64);
  if (d.trace && blockIdx.x == 0 && threadIdx.x == 0) d.trace[0] = (unsigned long long)traced;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    PcgState* ps = d.ps;
    const int conv = sm.converged;
    ps->converged = conv;
    ps->need_fallback = conv ? 0 : 1;
    ps->iterations = sm.iters;
    ps->outer = outer;
    ps->rel_residual = sm.rel;
    ps->total_iterations += sm.iters;
    ps->solves += 1;
    ps->fallbacks += conv ? 0 : 1;
    ps->max_iterations = max(ps->max_iterations, sm.iters);
    ps->max_rel_residual = fmax(ps->max_rel_residual, sm.rel);
  }
}

// Z (T [7][ng * 9], column-major by group row) of the similarity gauge at the current camera
// poses (POSE3 storage qx qy qz qw tx ty tz, tangent [rotation, translation], the pose mapping world
// to camera coordinates): moving the world by a translation e_a moves a pose's translation by
// -R e_a; rotating it by e_a moves a pose's rotation by -e_a; scaling it moves the translation by t
// (the null vectors of an undamped bundle-adjustment Hessian, restricted to the cameras).
template <typename T>
__global__ void GaugeBasisKernel(PcgDev d, const double* values, int64_t S, const LmState* st) {
  const int64_t rows = int64_t(d.pd.ng) * kB;
  const int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  double z[kGaugeDim] = {0, 0, 0, 0, 0, 0, 0};
  const int64_t so = d.gauge_soff[row];
  if (so >= 0) {
    const double* x = values + int64_t(st->init_idx) * S + so;
    const double qx = x[0], qy = x[1], qz = x[2], qw = x[3];
    const int c = d.gauge_comp[row];
    if (c < 3) {
      z[3 + c] = -1.0;
    } else {
      const int i = c - 3;  // row i of R
      const double R[3][3] = {{1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qw * qz), 2 * (qx * qz + qw * qy)},
                              {2 * (qx * qy + qw * qz), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qw * qx)},
                              {2 * (qx * qz - qw * qy), 2 * (qy * qz + qw * qx), 1 - 2 * (qx * qx + qy * qy)}};
      for (int a = 0; a < 3; ++a) z[a] = -R[i][a];
      z[6] = x[4 + i];
    }
  }
  T* zg = static_cast<T*>(d.zg);
  for (int j = 0; j < kGaugeDim; ++j) zg[j * rows + row] = T(z[j]);
}

template <typename T>
__global__ void GroupBlocksKernel(const int64_t* off, int64_t n, const T* S, T* Sb) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t o = off[i];
    Sb[i] = o >= 0 ? S[o] : T(0);
  }
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------------
template <typename T>
void LaunchPrecondFeatures(const PrecondDev& pd, const SpmvDev& m, const void* S, float* rho,
                           float* feats, float* fac, cudaStream_t s) {
  if (pd.ng == 0) return;
  const int warps = 8;
  PrecondRowKernel<T><<<(m.n + warps - 1) / warps, 32 * warps, 0, s>>>(pd, m, static_cast<const T*>(S), rho);
  const int threads = 64;
  PrecondFeatureKernel<T><<<(pd.ng + threads - 1) / threads, threads, 0, s>>>(
      pd, static_cast<const T*>(S), rho, feats, fac);
}

template <typename T>
void LaunchPrecondAssemble(int ng, const float* fac, const float* z, void* P, cudaStream_t s) {
  if (ng == 0) return;
  const int threads = 64;
  PrecondAssembleKernel<T><<<(ng + threads - 1) / threads, threads, 0, s>>>(ng, fac, z, static_cast<T*>(P));
}

template <typename T>
void LaunchCollectSamples(const PrecondDev& pd, const float* feats, const float* fac, const void* v,
                          const double* y, float* samples, int max_systems, PcgState* ps,
                          const LmState* st, cudaStream_t s) {
  (void)ps;
  if (pd.ng == 0) return;
  const int threads = 64;
  CollectSamplesKernel<T><<<(pd.ng + threads - 1) / threads, threads, 0, s>>>(
      pd, feats, fac, static_cast<const T*>(v), y, samples, max_systems, st);
}

template <typename T, int SPLIT>
int PcgMaxResidentCtas(int threads, int num_sms) {
  // the coarse and band variants use more registers and shared memory: the smallest count
  int per_sm = 0, per_sm_c = 0, per_sm_b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, PcgKernel<T, false, SPLIT, false, false>, threads, 0) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_c, PcgKernel<T, false, SPLIT, true, false>, threads, 0) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_b, PcgKernel<T, false, SPLIT, false, true>, threads, 0) !=
          cudaSuccess)
    return 0;
  return std::min(std::min(per_sm, per_sm_c), per_sm_b) * num_sms;
}

template <typename T>
void PcgShape(int ng, int num_sms, int* grid, int* threads, int* split) {
  *split = 1;
  const int warps = std::max(1, (ng + 2) / 3);
  if (warps <= 32) {  // one CTA, three camera blocks per warp (staged in shared memory if it fits)
    *grid = 1;
    *threads = 32 * warps;
    return;
  }
  // CTA size of multi-CTA solves; SFG_PCG_CTA_THREADS (a multiple of 32, at most 1024) overrides
  int t = kPcgMultiThreads;
  if (const char* e = std::getenv("SFG_PCG_CTA_THREADS")) {
    const int v = std::atoi(e);
    if (v >= 32 && v <= 1024 && v % 32 == 0) t = v;
  }
  *threads = t;
  // three lanes per row when one warp per camera block still fits on the device at once
  const int grid3 = (ng + t / 32 - 1) / (t / 32);
  if (grid3 <= PcgMaxResidentCtas<T, 3>(t, num_sms)) {
    *split = 3;
    *grid = grid3;
    return;
  }
  const int per_cta = 3 * (t / 32);
  *grid = (ng + per_cta - 1) / per_cta;
  const int cap = PcgMaxResidentCtas<T, 1>(t, num_sms);
  if (*grid > cap)
    throw Error(SFG_ERR_STRUCTURE, "the reduced system has " + std::to_string(ng) +
                                       " camera blocks, more than one PCG launch can hold (" +
                                       std::to_string(cap) + " CTAs)");
}
template void PcgShape<double>(int, int, int*, int*, int*);
template void PcgShape<float>(int, int, int*, int*, int*);

template <typename T>
size_t PcgStagedSmem(int ng, int nbl, int nent) {
  const size_t bytes = size_t(ng) * kB * 8 + size_t(nent) * 8 + size_t(nbl) * kB * kB * sizeof(T) +
                       size_t(ng) * kB * sizeof(T);
  return bytes > kPcgStagedMax ? 0 : bytes;
}
template size_t PcgStagedSmem<double>(int, int, int);
template size_t PcgStagedSmem<float>(int, int, int);

template <typename T>
void ConfigurePcg() {
  cudaFuncSetAttribute(PcgKernel<T, true, 1, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(kPcgStagedMax));
  cudaFuncSetAttribute(PcgKernel<T, true, 1, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(kPcgStagedMax));
  cudaFuncSetAttribute(PcgKernel<T, true, 1, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(kPcgStagedMax));
}
template void ConfigurePcg<double>();
template void ConfigurePcg<float>();

template <typename T>
void LaunchGroupBlocks(const int64_t* off, int64_t n, const void* S, void* Sb, cudaStream_t s) {
  const int threads = 256;
  const int grid = int(std::min<int64_t>((n + threads - 1) / threads, 4096));
  GroupBlocksKernel<T><<<std::max(grid, 1), threads, 0, s>>>(off, n, static_cast<const T*>(S),
                                                            static_cast<T*>(Sb));
}
template void LaunchGroupBlocks<double>(const int64_t*, int64_t, const void*, void*, cudaStream_t);
template void LaunchGroupBlocks<float>(const int64_t*, int64_t, const void*, void*, cudaStream_t);

template <typename T, bool kCoarse, bool kBand>
cudaError_t LaunchPcgVariant(const PcgDev& d, int grid, int threads, cudaStream_t s) {
  if (grid == 1) {
    if (d.staged) {
      PcgKernel<T, true, 1, kCoarse, kBand><<<1, threads, size_t(d.staged), s>>>(d);
    } else {
      PcgKernel<T, false, 1, kCoarse, kBand><<<1, threads, 0, s>>>(d);
    }
    return cudaGetLastError();
  }
  const cudaError_t e = cudaMemsetAsync(d.bar, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (d.split == 3) return cudaLaunchKernelEx(&cfg, PcgKernel<T, false, 3, kCoarse, kBand>, d);
  return cudaLaunchKernelEx(&cfg, PcgKernel<T, false, 1, kCoarse, kBand>, d);
}

template <typename T>
cudaError_t LaunchPcg(const PcgDev& d, int grid, int threads, cudaStream_t s) {
  if (d.band > 0) return LaunchPcgVariant<T, false, true>(d, grid, threads, s);
  return d.coarse ? LaunchPcgVariant<T, true, false>(d, grid, threads, s)
                  : LaunchPcgVariant<T, false, false>(d, grid, threads, s);
}

template <typename T>
void LaunchBandFactor(const BandDev& b, const void* Sb, cudaStream_t s) {
  if (b.ng == 0) return;
  // warps per CTA: as many as 48 KB of shared memory holds (at most 8)
  const size_t per_warp = size_t(BandWarpElems(b.band)) * sizeof(T);
  const int w = int(std::max<size_t>(1, std::min<size_t>(8, (48 * 1024) / per_warp)));
  BandFactorKernel<T><<<(b.ng + w - 1) / w, 32 * w, w * per_warp, s>>>(b, static_cast<const T*>(Sb));
}

template <typename T>
void LaunchBandAssemble(const BandDev& b, const float* z, void* Mb, cudaStream_t s) {
  const int n = b.ng * (b.band + 1);
  if (n == 0) return;
  BandAssembleKernel<T><<<(n + kBandAsmWarps - 1) / kBandAsmWarps, 32 * kBandAsmWarps, 0, s>>>(
      b, z, static_cast<T*>(Mb));
}
template void LaunchBandFactor<double>(const BandDev&, const void*, cudaStream_t);
template void LaunchBandFactor<float>(const BandDev&, const void*, cudaStream_t);
template void LaunchBandAssemble<double>(const BandDev&, const float*, void*, cudaStream_t);
template void LaunchBandAssemble<float>(const BandDev&, const float*, void*, cudaStream_t);

template <typename T>
void LaunchGaugeBasis(const PcgDev& d, const double* values, int64_t S, const LmState* st, cudaStream_t s) {
  const int64_t rows = int64_t(d.pd.ng) * kB;
  if (rows == 0) return;
  const int threads = 256;
  GaugeBasisKernel<T><<<int((rows + threads - 1) / threads), threads, 0, s>>>(d, values, S, st);
}
template void LaunchGaugeBasis<double>(const PcgDev&, const double*, int64_t, const LmState*, cudaStream_t);
template void LaunchGaugeBasis<float>(const PcgDev&, const double*, int64_t, const LmState*, cudaStream_t);
template cudaError_t LaunchPcg<double>(const PcgDev&, int, int, cudaStream_t);
template cudaError_t LaunchPcg<float>(const PcgDev&, int, int, cudaStream_t);

void LaunchPcgBegin(PcgState* ps, cudaStream_t s) { cudaMemsetAsync(ps, 0, sizeof(PcgState), s); }

template void LaunchPrecondFeatures<double>(const PrecondDev&, const SpmvDev&, const void*, float*,
                                            float*, float*, cudaStream_t);
template void LaunchPrecondFeatures<float>(const PrecondDev&, const SpmvDev&, const void*, float*,
                                           float*, float*, cudaStream_t);
template void LaunchPrecondAssemble<double>(int, const float*, const float*, void*, cudaStream_t);
template void LaunchPrecondAssemble<float>(int, const float*, const float*, void*, cudaStream_t);
template void LaunchCollectSamples<double>(const PrecondDev&, const float*, const float*, const void*,
                                           const double*, float*, int, PcgState*, const LmState*,
                                           cudaStream_t);
template void LaunchCollectSamples<float>(const PrecondDev&, const float*, const float*, const void*,
                                          const double*, float*, int, PcgState*, const LmState*,
                                          cudaStream_t);
}  // namespace sfg
