// Thousands of independent small problems in one persistent launch.
//
// Each warp takes a problem from a device queue (largest first) and runs its entire
// Levenberg-Marquardt loop (symforce/opt/levenberg_marquardt_solver.tcc:138-343, through the same
// lm_logic.cuh bookkeeping as the single-problem graph) before taking the next one, so uneven
// problem sizes balance across the GPU without any host round trip.  Supported problems are Pose3
// chains: unary prior / range factors and between factors on consecutive poses, so the Hessian is
// block tridiagonal (6 x 6 blocks) in key order.  Per iteration the warp
//   - linearizes: lane k accumulates pose k's unary factors and the between factor (k, k+1), whose
//     pose-(k+1) part is handed over through the workspace (fixed order, no atomics);
//   - factors H + D block by block, C_k C_k^T = A_kk + D_k - B_k B_k^T with B_k = A_k,k-1 C_k-1^-T,
//     keeping C_k^-1 so that both triangular solves are small matrix-vector products;
//   - retracts, relinearizes the new state and decides.
// Everything is FP64; reciprocal square roots start from an FP32 seed refined by two Newton steps
// (y <- y (3 - x y^2) / 2), which reach FP64 accuracy without the FP64 divide / square-root
// sequences, whose latency dominates these short dependent chains on GB300.
#include "factor_math.cuh"
#include <algorithm>

#include "kernels.h"
#include "lm_logic.cuh"

namespace sfg {

namespace {

constexpr int kScratch = 6 * 36 + 3 * 6;  // per-warp shared scratch (doubles)

struct Ws {
  double *vals, *Hd, *Ho, *g, *carry, *bwa, *damp, *maxd, *upd, *last, *Ci, *B, *y;
};

__device__ __forceinline__ Ws SlotWs(const BatchLmDev& d, int slot) {
  const size_t n = size_t(d.nmax);
  double* w = d.ws + size_t(slot) * kBatchWsPerPose * n;
  Ws s;
  s.vals = w;  w += 3 * 7 * n;
  s.Hd = w;    w += 3 * 36 * n;
  s.Ho = w;    w += 3 * 36 * n;
  s.g = w;     w += 3 * 6 * n;
  s.carry = w; w += 27 * n;
  s.bwa = w;   w += 27 * n;
  s.damp = w;  w += 6 * n;
  s.maxd = w;  w += 6 * n;
  s.upd = w;   w += 6 * n;
  s.last = w;  w += 6 * n;
  s.Ci = w;    w += 36 * n;
  s.B = w;     w += 36 * n;
  s.y = w;     w += 6 * n;
  return s;
}

__device__ __forceinline__ int Tri(int i, int j) { return i * (i + 1) / 2 + j; }

// Butterfly sum: every lane gets the same bits (IEEE addition is commutative).
__device__ __forceinline__ double WarpSum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Linearize state block s: H (full diagonal blocks, sub-diagonal blocks), rhs, and 0.5 |r|^2.
// Two passes keep few values live per lane: the between factors (lane per pose k, factor (k, k+1))
// write their three blocks and two rhs parts to the workspace; the unary factors (lane per pose)
// accumulate in registers and add the between parts of their pose.
__device__ double Linearize(const BatchLmDev& d, const Ws& w, int64_t pose0, int n, int s, int lane) {
  const size_t N = size_t(d.nmax);
  const double* V = w.vals + size_t(s) * 7 * N;
  double* Hd = w.Hd + size_t(s) * 36 * N;
  double* Ho = w.Ho + size_t(s) * 36 * N;
  double* g = w.g + size_t(s) * 6 * N;
  double err = 0.0;
  for (int k = lane; k + 1 < n; k += 32) {
    const int64_t gp = pose0 + k;
    double* own = w.bwa + size_t(k) * 27;       // pose k's part: H lower (21) + rhs (6)
    double* cr = w.carry + size_t(k + 1) * 27;  // pose k+1's part
    double* ho = Ho + size_t(k + 1) * 36;       // block (k+1, k)
    for (int i = 0; i < 27; ++i) own[i] = cr[i] = 0.0;
    for (int i = 0; i < 36; ++i) ho[i] = 0.0;
    for (int64_t f = d.bw_ptr[gp]; f < d.bw_ptr[gp + 1]; ++f) {
      const int rev = d.bw_rev[f];
      const double* x[2] = {V + 7 * (rev ? k + 1 : k), V + 7 * (rev ? k : k + 1)};
      double r[6], J[72];
      FactorEval<SFG_FACTOR_BETWEEN_POSE3, double>::Run(x, d.consts + d.bw_coff[f], r, J);
      const int ca = rev ? 6 : 0, cb = rev ? 0 : 6;
      for (int i = 0; i < 6; ++i) {
        err += r[i] * r[i];
        for (int a = 0; a < 6; ++a) {
          const double ja = J[i * 12 + ca + a], jb = J[i * 12 + cb + a];
          own[21 + a] += ja * r[i];
          cr[21 + a] += jb * r[i];
          for (int b = 0; b <= a; ++b) {
            own[Tri(a, b)] += ja * J[i * 12 + ca + b];
            cr[Tri(a, b)] += jb * J[i * 12 + cb + b];
          }
          for (int b = 0; b < 6; ++b) ho[a * 6 + b] += jb * J[i * 12 + ca + b];
        }
      }
    }
  }
  __syncwarp();
  for (int k = lane; k < n; k += 32) {
    const int64_t gp = pose0 + k;
    double h[21], gk[6];
#pragma unroll
    for (int i = 0; i < 21; ++i) h[i] = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) gk[i] = 0.0;
    for (int64_t f = d.un_ptr[gp]; f < d.un_ptr[gp + 1]; ++f) {
      const double* c = d.consts + d.un_coff[f];
      const double* x[1] = {V + 7 * k};
      if (d.un_kind[f] == SFG_FACTOR_RANGE_POSE3) {
        double r[1], J[6];
        FactorEval<SFG_FACTOR_RANGE_POSE3, double>::Run(x, c, r, J);
        err += r[0] * r[0];
        // the range Jacobian has no rotation part: only the translation block changes
#pragma unroll
        for (int a = 3; a < 6; ++a) {
          gk[a] += J[a] * r[0];
#pragma unroll
          for (int b = 3; b <= a; ++b) h[Tri(a, b)] += J[a] * J[b];
        }
      } else {
        double r[6], J[36];
        FactorEval<SFG_FACTOR_PRIOR_POSE3, double>::Run(x, c, r, J);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          err += r[i] * r[i];
#pragma unroll
          for (int a = 0; a < 6; ++a) {
            gk[a] += J[i * 6 + a] * r[i];
#pragma unroll
            for (int b = 0; b <= a; ++b) h[Tri(a, b)] += J[i * 6 + a] * J[i * 6 + b];
          }
        }
      }
    }
    if (k + 1 < n) {
      const double* own = w.bwa + size_t(k) * 27;
#pragma unroll
      for (int i = 0; i < 21; ++i) h[i] += own[i];
#pragma unroll
      for (int a = 0; a < 6; ++a) gk[a] += own[21 + a];
    }
    if (k > 0) {
      const double* cr = w.carry + size_t(k) * 27;
#pragma unroll
      for (int i = 0; i < 21; ++i) h[i] += cr[i];
#pragma unroll
      for (int a = 0; a < 6; ++a) gk[a] += cr[21 + a];
    }
    double* hd = Hd + size_t(k) * 36;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
#pragma unroll
      for (int b = 0; b <= a; ++b) hd[a * 6 + b] = hd[b * 6 + a] = h[Tri(a, b)];
      g[size_t(k) * 6 + a] = gk[a];
    }
  }
  __syncwarp();
  return 0.5 * WarpSum(err);
}

// (H + D) x = g by block Cholesky; writes upd = -x.
__device__ void FactorSolve(const BatchLmDev& d, const Ws& w, int n, int s, int lane, double* sm) {
  const size_t N = size_t(d.nmax);
  const double* Hd = w.Hd + size_t(s) * 36 * N;
  const double* Ho = w.Ho + size_t(s) * 36 * N;
  const double* g = w.g + size_t(s) * 6 * N;
  double* sA = sm;
  double* sC = sm + 36;
  double* sCi = sm + 72;       // C_k^-1 (lower)
  double* sCiPrev = sm + 108;  // C_k-1^-1
  double* sB = sm + 144;
  double* sInv = sm + 180;     // 1 / C_jj
  double* sv = sm + 186;       // 6-vectors
  double* sv2 = sm + 192;
  for (int k = 0; k < n; ++k) {
    // B = A_k,k-1 C_k-1^-T
    if (k > 0) {
      const double* O = Ho + size_t(k) * 36;
      for (int e = lane; e < 36; e += 32) {
        const int i = e / 6, j = e - 6 * (e / 6);
        double acc = 0.0;
        for (int p = 0; p <= j; ++p) acc += O[i * 6 + p] * sCiPrev[j * 6 + p];
        sB[e] = acc;
        w.B[size_t(k) * 36 + e] = acc;
      }
    }
    __syncwarp();
    if (lane < 21) {
      int i = 0;
      while (Tri(i + 1, 0) <= lane) ++i;
      const int j = lane - Tri(i, 0);
      double a = Hd[size_t(k) * 36 + i * 6 + j] + (i == j ? w.damp[size_t(k) * 6 + i] : 0.0);
      if (k > 0)
        for (int p = 0; p < 6; ++p) a -= sB[i * 6 + p] * sB[j * 6 + p];
      sA[i * 6 + j] = a;
    }
    __syncwarp();
    for (int j = 0; j < 6; ++j) {
      if (lane == j) {
        double t = sA[j * 6 + j];
        for (int p = 0; p < j; ++p) t -= sC[j * 6 + p] * sC[j * 6 + p];
        const double r = RsqrtD(t);
        sC[j * 6 + j] = t * r;
        sInv[j] = r;
      }
      __syncwarp();
      if (lane > j && lane < 6) {
        double t = sA[lane * 6 + j];
        for (int p = 0; p < j; ++p) t -= sC[lane * 6 + p] * sC[j * 6 + p];
        sC[lane * 6 + j] = t * sInv[j];
      }
      __syncwarp();
    }
    // C^-1: lane c computes column c
    if (lane < 6) {
      const int c = lane;
      for (int i = 0; i < 6; ++i) {
        double v;
        if (i < c) v = 0.0;
        else if (i == c) v = sInv[c];
        else {
          double t = 0.0;
          for (int p = c; p < i; ++p) t += sC[i * 6 + p] * sCi[p * 6 + c];
          v = -t * sInv[i];
        }
        sCi[i * 6 + c] = v;
      }
    }
    __syncwarp();
    for (int e = lane; e < 36; e += 32) {
      w.Ci[size_t(k) * 36 + e] = sCi[e];
      sCiPrev[e] = sCi[e];
    }
    __syncwarp();
  }
  // forward: y_k = C_k^-1 (g_k - B_k y_k-1)
  for (int k = 0; k < n; ++k) {
    if (lane < 6) {
      double t = g[size_t(k) * 6 + lane];
      if (k > 0)
        for (int j = 0; j < 6; ++j) t -= w.B[size_t(k) * 36 + lane * 6 + j] * sv[j];
      sv2[lane] = t;
    }
    __syncwarp();
    if (lane < 6) {
      double t = 0.0;
      for (int j = 0; j <= lane; ++j) t += w.Ci[size_t(k) * 36 + lane * 6 + j] * sv2[j];
      w.y[size_t(k) * 6 + lane] = t;
    }
    __syncwarp();
    if (lane < 6) sv[lane] = w.y[size_t(k) * 6 + lane];
    __syncwarp();
  }
  // backward: x_k = C_k^-T (y_k - B_k+1^T x_k+1)
  for (int k = n - 1; k >= 0; --k) {
    if (lane < 6) {
      double t = w.y[size_t(k) * 6 + lane];
      if (k + 1 < n)
        for (int i = 0; i < 6; ++i) t -= w.B[size_t(k + 1) * 36 + i * 6 + lane] * sv[i];
      sv2[lane] = t;
    }
    __syncwarp();
    if (lane < 6) {
      double t = 0.0;
      for (int i = lane; i < 6; ++i) t += w.Ci[size_t(k) * 36 + i * 6 + lane] * sv2[i];
      sv[lane] = t;  // read by the lanes only after the next __syncwarp
      w.upd[size_t(k) * 6 + lane] = -t;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// Dense path: problems of any key and factor kinds (tangent dimension up to kBatchDenseMaxN), one
// warp per problem as above, with the Hessian dense in the slot's workspace (L2-resident).
//   - linearize: factors in rounds of 32, one lane each (residual and Jacobian into the slot's
//     scratch), then the warp adds the round's J^T J / J^T r entries factor by factor in factor
//     order (lanes over a factor's entries, which fall on distinct Hessian entries because a
//     factor's keys are distinct): the same bits on every run, no atomics;
//   - factor: right-looking LDL^T of H + D (the lanes over the trailing lower entries of a pivot),
//     then column-oriented unit-lower solves and D^-1;
//   - retract every key by its type, relinearize, decide (lm_logic.cuh, as the chain path).
// ---------------------------------------------------------------------------------------------
struct DnWs {
  double *vals, *H, *F, *g, *damp, *maxd, *upd, *last, *y, *Js;
};
constexpr int kDnJs = kBatchDenseRd * (kBatchDenseTd + 1) + 1;  // r, J, then rd and td
constexpr int kDnBatch = 8;  // trailing-update entries a lane keeps in flight

__device__ __forceinline__ DnWs DenseWs(const BatchLmDev& d, int slot) {
  const size_t n = size_t(d.nmax_t), sm = size_t(d.smax);
  double* w = d.ws + size_t(slot) * size_t(d.ws_stride);
  DnWs s;
  s.vals = w;  w += 3 * sm;
  s.H = w;     w += 3 * n * n;
  s.F = w;     w += n * n;
  s.g = w;     w += 3 * n;
  s.damp = w;  w += n;
  s.maxd = w;  w += n;
  s.upd = w;   w += n;
  s.last = w;  w += n;
  s.y = w;     w += 2 * n;
  s.Js = w;
  return s;
}

template <int KIND>
__device__ __forceinline__ void EvalKind(const double* const* x, const double* c, double* r, double* J,
                                         int* rd, int* td) {
  static_assert(FactorTraits<KIND>::RD <= kBatchDenseRd && FactorTraits<KIND>::TD <= kBatchDenseTd &&
                    FactorTraits<KIND>::NK <= kBatchDenseKeys,
                "dense batch scratch holds the factor");
  FactorEval<KIND, double>::Run(x, c, r, J);
  *rd = FactorTraits<KIND>::RD;
  *td = FactorTraits<KIND>::TD;
}

// Residual r and row-major Jacobian J (rd x td) of a factor of any kind.
__device__ void EvalAny(int kind, const double* const* x, const double* c, double* r, double* J, int* rd,
                        int* td) {
  *rd = 0;
  *td = 0;
  switch (kind) {
    case SFG_FACTOR_BEARING_POSE2: EvalKind<SFG_FACTOR_BEARING_POSE2>(x, c, r, J, rd, td); break;
    case SFG_FACTOR_ODOMETRY_POSE2: EvalKind<SFG_FACTOR_ODOMETRY_POSE2>(x, c, r, J, rd, td); break;
    case SFG_FACTOR_SNAVELY_REPROJECTION: EvalKind<SFG_FACTOR_SNAVELY_REPROJECTION>(x, c, r, J, rd, td); break;
    case SFG_FACTOR_BETWEEN_POSE3: EvalKind<SFG_FACTOR_BETWEEN_POSE3>(x, c, r, J, rd, td); break;
    case SFG_FACTOR_PRIOR_POSE3: EvalKind<SFG_FACTOR_PRIOR_POSE3>(x, c, r, J, rd, td); break;
    case SFG_FACTOR_RANGE_POSE3: EvalKind<SFG_FACTOR_RANGE_POSE3>(x, c, r, J, rd, td); break;
#define SFG_DENSE_CASE(KIND, NKEYS, NCONSTS, RDIM, K0, K1, K2, G) \
    case KIND: EvalKind<KIND>(x, c, r, J, rd, td); break;
      SFG_GENERATED_FACTORS(SFG_DENSE_CASE)
#undef SFG_DENSE_CASE
  }
}

__device__ __forceinline__ int KeyTangentDim(int type) {
  switch (type) {
    case SFG_KEY_POSE2: return 3;
    case SFG_KEY_POSE3: return 6;
    case SFG_KEY_ROT3: return 3;
    default: return type <= SFG_KEY_VEC3 ? type : type - SFG_KEY_VEC4 + 4;
  }
}

// Row of entry e of a packed lower triangle (row-major: row i holds entries i (i + 1) / 2 ...).
__device__ __forceinline__ int TriRow(int e) {
  int i = int((sqrtf(8.0f * float(e) + 1.0f) - 1.0f) * 0.5f);
  if ((i + 1) * (i + 2) / 2 <= e) ++i;
  if (i * (i + 1) / 2 > e) --i;
  return i;
}

// Linearize state block s of problem prob: H (lower part of an n x n row-major block), g = J^T r,
// and 0.5 |r|^2 (returned to every lane).
__device__ double DnLinearize(const BatchLmDev& d, const DnWs& w, int prob, int s, int lane) {
  const int n = d.dn_n[prob];
  const size_t nm = size_t(d.nmax_t);
  const double* V = w.vals + size_t(s) * size_t(d.smax);
  double* H = w.H + size_t(s) * nm * nm;
  double* g = w.g + size_t(s) * nm;
  for (int i = lane; i < n * n; i += 32) H[i] = 0.0;
  for (int i = lane; i < n; i += 32) g[i] = 0.0;
  __syncwarp();
  double err = 0.0;
  const int64_t f0 = d.f_ptr[prob], f1 = d.f_ptr[prob + 1];
  for (int64_t fb = f0; fb < f1; fb += 32) {
    const int cnt = int(f1 - fb < 32 ? f1 - fb : 32);
    if (lane < cnt) {
      const int64_t f = fb + lane;
      const int32_t* fk = d.f_key + f * kBatchDenseKeys;
      const double* x[kBatchDenseKeys];
#pragma unroll
      for (int q = 0; q < kBatchDenseKeys; ++q) x[q] = fk[q] >= 0 ? V + d.key_soff[fk[q]] : V;
      double* js = w.Js + size_t(lane) * kDnJs;
      int rd = 0, td = 0;
      EvalAny(d.f_kind[f], x, d.consts + d.f_coff[f], js, js + kBatchDenseRd, &rd, &td);
      for (int i = 0; i < rd; ++i) err += js[i] * js[i];
      js[kDnJs - 1] = double(rd * 256 + td);
    }
    __syncwarp();
    for (int q = 0; q < cnt; ++q) {
      const int32_t* fk = d.f_key + (fb + q) * kBatchDenseKeys;
      const double* js = w.Js + size_t(q) * kDnJs;
      const int code = int(js[kDnJs - 1]), rd = code >> 8, td = code & 255;
      const double* r = js;
      const double* J = js + kBatchDenseRd;
      // the factor's tangent columns on the problem's tangent vector
      int cols[kBatchDenseTd];
      int nc = 0;
#pragma unroll
      for (int k = 0; k < kBatchDenseKeys; ++k) {
        if (fk[k] < 0) continue;
        const int t = KeyTangentDim(d.key_type[fk[k]]), o = d.key_toff[fk[k]];
        for (int j = 0; j < t && nc < kBatchDenseTd; ++j) cols[nc++] = o + j;
      }
      if (nc != td) continue;  // (the host admits only factors whose key types give td columns)
      const int ntri = td * (td + 1) / 2;
      // the lane's entries of this factor (at most kDnFactorEntries): products first, then the
      // read-modify-writes with their loads in flight together
      constexpr int kDnFactorEntries = (kBatchDenseTd * (kBatchDenseTd + 1) / 2 + kBatchDenseTd + 31) / 32;
      double val[kDnFactorEntries], old[kDnFactorEntries];
      double* dst[kDnFactorEntries];
#pragma unroll
      for (int u = 0; u < kDnFactorEntries; ++u) {
        const int e = lane + 32 * u;
        dst[u] = nullptr;
        val[u] = 0.0;
        if (e < ntri) {
          const int a = TriRow(e), b = e - a * (a + 1) / 2;
          double v = 0.0;
          for (int i = 0; i < rd; ++i) v += J[i * td + a] * J[i * td + b];
          const int ga = cols[a], gb = cols[b];
          dst[u] = H + size_t(max(ga, gb)) * n + min(ga, gb);
          val[u] = v;
        } else if (e < ntri + td) {
          const int a = e - ntri;
          double v = 0.0;
          for (int i = 0; i < rd; ++i) v += J[i * td + a] * r[i];
          dst[u] = g + cols[a];
          val[u] = v;
        }
      }
#pragma unroll
      for (int u = 0; u < kDnFactorEntries; ++u) old[u] = dst[u] ? *dst[u] : 0.0;
#pragma unroll
      for (int u = 0; u < kDnFactorEntries; ++u)
        if (dst[u]) *dst[u] = old[u] + val[u];
      __syncwarp();
    }
  }
  return 0.5 * WarpSum(err);
}

// (H + D) x = g by LDL^T (no pivoting, as the reference's sparse LDL^T); writes upd = -x.
__device__ void DnFactorSolve(const BatchLmDev& d, const DnWs& w, int prob, int s, int lane) {
  const int n = d.dn_n[prob];
  const size_t nm = size_t(d.nmax_t);
  const double* H = w.H + size_t(s) * nm * nm;
  const double* g = w.g + size_t(s) * nm;
  double* F = w.F;
  double* y = w.y;
  double* l = w.y + nm;  // the scaled pivot column
  for (int i = lane; i < n * n; i += 32) {
    const int r = i / n, c = i - (i / n) * n;
    F[i] = c <= r ? H[i] + (r == c ? w.damp[r] : 0.0) : 0.0;
  }
  __syncwarp();
  for (int k = 0; k < n; ++k) {
    const double inv = 1.0 / F[size_t(k) * n + k];
    for (int j = k + 1 + lane; j < n; j += 32) l[j] = F[size_t(j) * n + k] * inv;
    __syncwarp();
    // trailing update, kDnBatch entries a lane in flight: their loads issue before any store
    const int m = n - k - 1, cnt = m * (m + 1) / 2;
    for (int e0 = lane; e0 < cnt; e0 += 32 * kDnBatch) {
      double fv[kDnBatch], av[kDnBatch], bv[kDnBatch];
      size_t at[kDnBatch];
#pragma unroll
      for (int u = 0; u < kDnBatch; ++u) {
        const int e = e0 + 32 * u;
        at[u] = 0;
        fv[u] = av[u] = bv[u] = 0.0;
        if (e < cnt) {
          const int ii = TriRow(e), jj = e - ii * (ii + 1) / 2;
          const int i = k + 1 + ii, j = k + 1 + jj;
          at[u] = size_t(i) * n + j;
          fv[u] = F[at[u]];
          av[u] = F[size_t(i) * n + k];
          bv[u] = l[j];
        }
      }
#pragma unroll
      for (int u = 0; u < kDnBatch; ++u)
        if (e0 + 32 * u < cnt) F[at[u]] = fv[u] - av[u] * bv[u];
    }
    __syncwarp();
    for (int j = k + 1 + lane; j < n; j += 32) F[size_t(j) * n + k] = l[j];
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) y[i] = g[i];
  __syncwarp();
  for (int j = 0; j < n; ++j) {  // L y = g, unit L
    const double yj = y[j];
    for (int i = j + 1 + lane; i < n; i += 32) y[i] -= F[size_t(i) * n + j] * yj;
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) y[i] /= F[size_t(i) * n + i];
  __syncwarp();
  for (int i = n - 1; i > 0; --i) {  // L^T x = D^-1 y
    const double xi = y[i];
    for (int j = lane; j < i; j += 32) y[j] -= F[size_t(i) * n + j] * xi;
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) w.upd[i] = -y[i];
  __syncwarp();
}

// One problem of the dense path, start to finish (the warp's LM loop).
__device__ void DenseProblem(const BatchLmDev& d, const LmParams& p, const DnWs& w, LmState& st, int prob,
                             int lane) {
  const int n = d.dn_n[prob], S = d.dn_s[prob], nk = d.dn_nk[prob], k0 = d.dn_k0[prob];
  const int64_t s0 = d.dn_s0[prob];
  const size_t sm = size_t(d.smax), nm = size_t(d.nmax_t);
  sfg_iteration_t* rec = d.records ? d.records + size_t(prob) * d.rec_cap : nullptr;
  if (lane == 0) {
    st = LmState{};
    LmBegin(p, st, 1);
  }
  __syncwarp();
  for (int i = lane; i < S; i += 32) w.vals[size_t(st.init_idx) * sm + i] = d.values_in[s0 + i];
  __syncwarp();
  {
    const int init = st.init_idx;
    const double e = DnLinearize(d, w, prob, init, lane);
    if (lane == 0) st.error[init] = e;
  }
  __syncwarp();
  int go = 0;
  if (lane == 0) go = LmFirstRecord(p, st, rec);
  go = __shfl_sync(0xffffffffu, go, 0);
  while (go) {
    const int init = st.init_idx, nw = st.new_idx;
    const double* H = w.H + size_t(init) * nm * nm;
    for (int i = lane; i < n; i += 32) w.damp[i] = LmDamping(p, st, H[size_t(i) * n + i], w.maxd + i);
    __syncwarp();
    DnFactorSolve(d, w, prob, init, lane);
    for (int k = lane; k < nk; k += 32) {
      const int kg = k0 + k;
      RetractKey(d.key_type[kg], w.vals + size_t(init) * sm + d.key_soff[kg], w.upd + d.key_toff[kg],
                 p.epsilon, w.vals + size_t(nw) * sm + d.key_soff[kg]);
    }
    __syncwarp();
    const double e_new = DnLinearize(d, w, prob, nw, lane);
    const double* g = w.g + size_t(init) * nm;
    double s0s = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int i = lane; i < n; i += 32) {
      const double u = w.upd[i];
      s0s += u * (g[i] - w.damp[i] * u);
      if (p.enable_bold_updates) {
        const double l = w.last[i];
        s1 += u * l;
        s2 += u * u;
        s3 += l * l;
      }
    }
    double sums[4] = {WarpSum(s0s), WarpSum(s1), WarpSum(s2), WarpSum(s3)};
    int done = 0, copy = 0;
    if (lane == 0) {
      st.error[nw] = e_new;
      done = LmDecide(p, st, rec, sums, &copy);
    }
    done = __shfl_sync(0xffffffffu, done, 0);
    copy = __shfl_sync(0xffffffffu, copy, 0);
    if (copy)
      for (int i = lane; i < n; i += 32) w.last[i] = w.upd[i];
    __syncwarp();
    go = !done;
  }
  for (int i = lane; i < S; i += 32) d.values_out[s0 + i] = w.vals[size_t(st.best_idx) * sm + i];
  if (lane == 0) d.st[prob] = st;
  __syncwarp();
}

template <int kWarps, int kMinBlocks, bool kDense>
__global__ void __launch_bounds__(32 * kWarps, kMinBlocks) BatchLmKernel(BatchLmDev d, const LmParams* pp) {
  __shared__ LmState sst[kWarps];
  __shared__ double sscr[kWarps][kScratch];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = blockIdx.x * (blockDim.x >> 5) + warp;
  const LmParams p = *pp;
  const Ws w = SlotWs(d, slot);
  LmState& st = sst[warp];
  double* sm = sscr[warp];
  const size_t NM = size_t(d.nmax);
  for (;;) {
    int job = 0;
    if (lane == 0) job = atomicAdd(d.counter, 1);
    job = __shfl_sync(0xffffffffu, job, 0);
    if (job >= d.nprob) break;
    const int prob = d.order[job];
    if constexpr (kDense) {
      DenseProblem(d, p, DenseWs(d, slot), st, prob, lane);
      continue;
    }
    const int n = d.n[prob];
    const int64_t pose0 = d.pose0[prob];
    sfg_iteration_t* rec = d.records ? d.records + size_t(prob) * d.rec_cap : nullptr;
    if (lane == 0) {
      st = LmState{};
      LmBegin(p, st, 1);
    }
    __syncwarp();
    {
      const int init = st.init_idx;
      for (int i = lane; i < 7 * n; i += 32) w.vals[size_t(init) * 7 * NM + i] = d.values_in[pose0 * 7 + i];
    }
    __syncwarp();
    {
      const int init = st.init_idx;
      const double e = Linearize(d, w, pose0, n, init, lane);
      if (lane == 0) st.error[init] = e;
    }
    __syncwarp();
    int go = 0;
    if (lane == 0) go = LmFirstRecord(p, st, rec);
    go = __shfl_sync(0xffffffffu, go, 0);
    while (go) {
      const int init = st.init_idx, nw = st.new_idx;
      const double* Hd = w.Hd + size_t(init) * 36 * NM;
      for (int i = lane; i < 6 * n; i += 32) {
        const int k = i / 6, a = i - 6 * (i / 6);
        w.damp[i] = LmDamping(p, st, Hd[size_t(k) * 36 + a * 7], w.maxd + i);
      }
      __syncwarp();
      FactorSolve(d, w, n, init, lane, sm);
      for (int k = lane; k < n; k += 32)
        RetractPose3(w.vals + size_t(init) * 7 * NM + 7 * k, w.upd + 6 * k, p.epsilon,
                     w.vals + size_t(nw) * 7 * NM + 7 * k);
      __syncwarp();
      const double e_new = Linearize(d, w, pose0, n, nw, lane);
      // u.(rhs - d.u) with rhs of the Init block, and the bold-update products
      const double* g = w.g + size_t(init) * 6 * NM;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      for (int i = lane; i < 6 * n; i += 32) {
        const double u = w.upd[i];
        s0 += u * (g[i] - w.damp[i] * u);
        if (p.enable_bold_updates) {
          const double l = w.last[i];
          s1 += u * l;
          s2 += u * u;
          s3 += l * l;
        }
      }
      double sums[4] = {WarpSum(s0), WarpSum(s1), WarpSum(s2), WarpSum(s3)};
      int done = 0, copy = 0;
      if (lane == 0) {
        st.error[nw] = e_new;
        done = LmDecide(p, st, rec, sums, &copy);
      }
      done = __shfl_sync(0xffffffffu, done, 0);
      copy = __shfl_sync(0xffffffffu, copy, 0);
      if (copy)
        for (int i = lane; i < 6 * n; i += 32) w.last[i] = w.upd[i];
      __syncwarp();
      go = !done;
    }
    {
      const int best = st.best_idx;
      for (int i = lane; i < 7 * n; i += 32) d.values_out[pose0 * 7 + i] = w.vals[size_t(best) * 7 * NM + i];
    }
    if (lane == 0) d.st[prob] = st;
    __syncwarp();
  }
}

}  // namespace

// Launch shapes the autotuner chooses from: warps per CTA and the register budget implied by the
// minimum resident CTAs per SM (fewer registers: more warps in flight to hide FP64 latency); each
// for the chain and the dense path.
template <int W, int B>
struct Shape {
  static int MaxCtasPerSm(bool dense) {
    int per_sm = 0;
    const cudaError_t e =
        dense ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, BatchLmKernel<W, B, true>, 32 * W, 0)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, BatchLmKernel<W, B, false>, 32 * W, 0);
    return e == cudaSuccess ? per_sm : 0;
  }
  static void Launch(const BatchLmDev& d, const LmParams* p, int ctas, cudaStream_t s) {
    if (d.dense) BatchLmKernel<W, B, true><<<ctas, 32 * W, 0, s>>>(d, p);
    else BatchLmKernel<W, B, false><<<ctas, 32 * W, 0, s>>>(d, p);
  }
};

int BatchShapes() { return 5; }

int BatchShapeWarps(int shape) {
  constexpr int w[5] = {8, 4, 2, 4, 2};
  return shape >= 0 && shape < 5 ? w[shape] : 0;
}

int BatchMaxCtasPerSm(int shape, bool dense) {
  switch (shape) {
    case 0: return Shape<8, 1>::MaxCtasPerSm(dense);
    case 1: return Shape<4, 4>::MaxCtasPerSm(dense);
    case 2: return Shape<2, 8>::MaxCtasPerSm(dense);
    case 3: return Shape<4, 6>::MaxCtasPerSm(dense);
    case 4: return Shape<2, 16>::MaxCtasPerSm(dense);
  }
  return 0;
}

void LaunchBatchLm(const BatchLmDev& d, const LmParams* p, int ctas, int shape, cudaStream_t s) {
  cudaMemsetAsync(d.counter, 0, sizeof(int), s);
  switch (shape) {
    case 0: Shape<8, 1>::Launch(d, p, ctas, s); break;
    case 1: Shape<4, 4>::Launch(d, p, ctas, s); break;
    case 2: Shape<2, 8>::Launch(d, p, ctas, s); break;
    case 3: Shape<4, 6>::Launch(d, p, ctas, s); break;
    case 4: Shape<2, 16>::Launch(d, p, ctas, s); break;
  }
}

}  // namespace sfg
