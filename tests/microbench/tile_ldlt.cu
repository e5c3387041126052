// Diagonal-tile LDL^T variants of the factorization, timed on one GB300 SM and at four CTAs per SM,
// and checked against a long double / double factorization (tests/test_gpu_microbench.py runs
// this).  FP64 16 x 16: a reciprocal per pivot with two barriers (the earlier design) against the
// fraction-free elimination the library uses; FP32 32 x 32: one warp with the rows in registers
// (the earlier design) against the CTA-wide elimination the library uses.
#include <cstdio>
#include <cstdint>
#include <cmath>
#include <vector>
#include <random>
__device__ __forceinline__ double PivotReciprocal(double x) {
  const int ex = __double2hiint(x) & 0x7FF00000;
  if (ex < 0x00200000 || ex >= 0x7FD00000) return 1.0 / x;
  double y; asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0); y = fma(y, e, y); e = fma(-x, y, 1.0); return fma(y, e, y);
}
__device__ __forceinline__ void LowerEntry16(int e, int* r, int* c) {
  int cc = 0, start = 0;
  while (cc < 15 && e >= start + (16 - cc)) { start += 16 - cc; ++cc; }
  *c = cc; *r = cc + (e - start);
}
__device__ void DiagLdltF64(double* a, int b, double* s_inv) {
  const int t = threadIdx.x;
  int r0 = 0, c0 = 16, r1 = 0, c1 = 16;
  double v0 = 0.0, v1 = 0.0;
  if (t >= 32) {
    const int e = t - 32;
    LowerEntry16(e, &r0, &c0);
    if (r0 >= b) c0 = 16;
    if (e + 96 < 136) { LowerEntry16(e + 96, &r1, &c1); if (r1 >= b) c1 = 16; }
    if (c0 < 16) v0 = a[c0 * 16 + r0];
    if (c1 < 16) v1 = a[c1 * 16 + r1];
  }
  for (int j = 0; j < b; ++j) {
    double p0 = 0.0, p1 = 0.0;
    if (t < 32) {
      const double inv = PivotReciprocal(a[j * 16 + j]);
      if (t == 0) *s_inv = inv;
    } else {
      if (c0 < 16 && c0 > j) p0 = a[j * 16 + r0] * a[j * 16 + c0];
      if (c1 < 16 && c1 > j) p1 = a[j * 16 + r1] * a[j * 16 + c1];
    }
    __syncthreads();
    if (t >= 32) {
      const double inv = *s_inv;
      if (c0 < 16) {
        if (c0 > j) { v0 = fma(-p0, inv, v0); a[c0 * 16 + r0] = v0; }
        else if (c0 == j && r0 > j) { v0 *= inv; a[c0 * 16 + r0] = v0; }
      }
      if (c1 < 16) {
        if (c1 > j) { v1 = fma(-p1, inv, v1); a[c1 * 16 + r1] = v1; }
        else if (c1 == j && r1 > j) { v1 *= inv; a[c1 * 16 + r1] = v1; }
      }
    }
    __syncthreads();
  }
}
// x * 2^s, exact while the result stays normal
__device__ __forceinline__ double Pow2Scale(double x, int s) {
  const int hi = __double2hiint(x), ex = (hi >> 20) & 0x7FF, ne = ex + s;
  if (ex != 0 && ex != 0x7FF && ne > 0 && ne < 0x7FF)
    return __hiloint2double(hi + s * (1 << 20), __double2loint(x));
  return scalbn(x, s);
}
__device__ __forceinline__ int PivotExponent(double p) {
  const int ex = (__double2hiint(p) >> 20) & 0x7FF;
  return (ex == 0 || ex == 0x7FF) ? 0 : ex - 1023;
}
template <bool kNamed>
__device__ void DiagLdltFF(double* a, int b, double* s_rp) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  // entry (r, c), 1 <= c <= r <= 15, column-major, one per thread t < 120
  int r = 0, c = 16;
  if (t < 120) {
    int cc = 1, start = 0;
    while (cc < 15 && t >= start + (16 - cc)) { start += 16 - cc; ++cc; }
    c = cc; r = cc + (t - start);
    if (r >= b) c = 16;
  }
  double v = (c < 16) ? a[c * 16 + r] : 0.0;
  for (int k = 0; k + 1 < b; ++k) {
    const double p = a[k * 17];
    const int ek = PivotExponent(p);
    if (c < 16 && c > k) {
      const double m = a[k * 16 + r] * a[k * 16 + c];
      v = Pow2Scale(fma(p, v, -m), -ek);
      a[c * 16 + r] = v;
    }
    if (kNamed) {
      // warps whose entries all lie in columns <= k neither write now nor read later
      if (k < 3) __syncthreads();
      else if (k < 4) { if (warp >= 1) asm volatile("bar.sync 1, 96;" ::: "memory"); }
      else if (k < 8) { if (warp >= 2) asm volatile("bar.sync 2, 64;" ::: "memory"); }
      else { if (warp == 3) __syncwarp(); }
    } else {
      __syncthreads();
    }
  }
  __syncthreads();
  // P_k = a[k * 17]; S_k = prod_{i < k} mant(P_i); d_k = P_k / S_k; L(r, c) = B(r, c) / P_c
  double dk = 0.0;
  if (warp == 0) {
    const double p = lane < b ? a[lane * 17] : 1.0;
    double x = lane < b ? Pow2Scale(p, -PivotExponent(p)) : 1.0;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x *= y;
    }
    double s = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) s = 1.0;
    dk = p * PivotReciprocal(s);
  } else if (warp == 1 && lane < 16) {
    s_rp[lane] = lane < b ? PivotReciprocal(a[lane * 17]) : 0.0;
  }
  __syncthreads();
  if (c < 16 && r > c) a[c * 16 + r] = v * s_rp[c];
  if (t >= 112 && t < 127) {  // column 0, rows 1..15
    const int rr = t - 111;
    if (rr < b) a[rr] = a[rr] * s_rp[0];
  }
  if (warp == 0 && lane < b) a[lane * 17] = dk;
  __syncthreads();
}

// Fraction-free elimination two pivots per CTA barrier: for the pair (k, k + 1) with P = B(k, k),
// Q = B(k + 1, k + 1), X = B(k + 1, k), D = P Q - X^2, every trailing entry (c >= k + 2) becomes
// 2^-e(D) [D B(r, c) - B(r, k) u_c - B(r, k + 1) w_c], u_c = Q B(c, k) - X B(c, k + 1),
// w_c = P B(c, k + 1) - X B(c, k): the Schur complement of the 2 x 2 block times D (the block's
// determinant), so the stored matrix stays the true Schur complement times a product of pivot
// mantissas.  At the end d_k = P_k / S_k, L(r, k) = B(r, k) / P_k for the first column of a pair
// (and single pivots), and d_k+1 = D / (P S_k), L(r, k + 1) = (P B(r, k + 1) - X B(r, k)) / D for
// the second.
__device__ void DiagLdltFF2(double* a, int b, double* s_rp, double* s_aux) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int r = 0, c = 16;
  if (t < 120) {
    int cc = 1, start = 0;
    while (cc < 15 && t >= start + (16 - cc)) { start += 16 - cc; ++cc; }
    c = cc; r = cc + (t - start);
    if (r >= b) c = 16;
  }
  double v = (c < 16) ? a[c * 16 + r] : 0.0;
  int k = 0;
  for (; k + 2 < b; k += 2) {
    const double P = a[k * 17], Q = a[(k + 1) * 17], X = a[k * 16 + k + 1];
    const double D = fma(P, Q, -(X * X));
    const int eD = PivotExponent(D);
    if (c < 16 && c >= k + 2) {
      const double ar = a[k * 16 + r], br = a[(k + 1) * 16 + r];
      const double ac = a[k * 16 + c], bc = a[(k + 1) * 16 + c];
      const double uc = fma(Q, ac, -(X * bc)), wc = fma(P, bc, -(X * ac));
      double in = D * v;
      in = fma(-ar, uc, in);
      in = fma(-br, wc, in);
      v = Pow2Scale(in, -eD);
      a[c * 16 + r] = v;
    }
    __syncthreads();
  }
  if (k + 1 < b) {  // one single pivot left before the last column
    const double p = a[k * 17];
    const int ek = PivotExponent(p);
    if (c < 16 && c > k) {
      const double m = a[k * 16 + r] * a[k * 16 + c];
      v = Pow2Scale(fma(p, v, -m), -ek);
      a[c * 16 + r] = v;
    }
    __syncthreads();
  }
  const int npair = (b >= 3) ? (b - 1) / 2 : 0;  // pairs (0,1) .. (2 npair - 2, 2 npair - 1)
  double dk = 0.0;
  if (warp == 0) {
    // event factor of column j: a pair's first column mant(D), its second 1, a single mant(P)
    const bool first = lane < 2 * npair && (lane & 1) == 0, second = lane < 2 * npair && (lane & 1);
    double P = lane < b ? a[lane * 17] : 1.0, Dp = 1.0;
    if (first) {
      const double Q = a[(lane + 1) * 17], X = a[lane * 16 + lane + 1];
      Dp = fma(P, Q, -(X * X));
    }
    const double Dsec = __shfl_up_sync(0xffffffffu, Dp, 1);  // a pair's D, at its second column
    const double Psec = __shfl_up_sync(0xffffffffu, P, 1);
    double f = lane < b ? (first ? Pow2Scale(Dp, -PivotExponent(Dp)) : second ? 1.0 : Pow2Scale(P, -PivotExponent(P))) : 1.0;
    double x = f;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x *= y;
    }
    double S = __shfl_up_sync(0xffffffffu, x, 1);  // exclusive product
    if (lane == 0) S = 1.0;
    const double Sprev = __shfl_up_sync(0xffffffffu, S, 1);  // the pair's scale, at its second column
    if (second) dk = Dsec * PivotReciprocal(Psec * Sprev);
    else dk = P * PivotReciprocal(S);
    if (lane < 16) {
      s_rp[lane] = lane < b ? (second ? PivotReciprocal(Dsec) : PivotReciprocal(P)) : 0.0;
      s_aux[lane] = second ? 1.0 : 0.0;
    }
  }
  __syncthreads();
  // every L value is formed before any is stored (a pair's second column reads its first)
  double lv = 0.0, l0 = 0.0;
  if (c < 16 && r > c) {
    if (s_aux[c] != 0.0) {  // second column of a pair: (P b_r - X a_r) / D
      const double P = a[(c - 1) * 17], X = a[(c - 1) * 16 + c], ar = a[(c - 1) * 16 + r];
      lv = fma(P, v, -(X * ar)) * s_rp[c];
    } else {
      lv = v * s_rp[c];
    }
  }
  const int rr = t - 111;  // threads 112..126: column 0, rows 1..15
  if (t >= 112 && t < 127 && rr < b) l0 = a[rr] * s_rp[0];
  __syncthreads();
  if (c < 16 && r > c) a[c * 16 + r] = lv;
  if (t >= 112 && t < 127 && rr < b) a[rr] = l0;
  if (warp == 0 && lane < b) a[lane * 17] = dk;
  __syncthreads();
}

template <int V>
__global__ void __launch_bounds__(128) BenchF64(const double* tiles, int ntiles, int b, int reps, double* out,
                                             long long* cycles) {
  __shared__ double a[256], keep[256], s[16], aux[16];
  const int tile = blockIdx.x % ntiles;
  for (int e = threadIdx.x; e < 256; e += 128) keep[e] = tiles[int64_t(tile) * 256 + e];
  __syncthreads();
  long long total = 0;
  for (int it = 0; it < reps; ++it) {
    for (int e = threadIdx.x; e < 256; e += 128) a[e] = keep[e];
    __syncthreads();
    const long long t0 = clock64();
    if (V == 0) DiagLdltF64(a, b, s);
    else if (V == 1) DiagLdltFF<false>(a, b, s);
    else if (V == 2) DiagLdltFF<true>(a, b, s);
    else DiagLdltFF2(a, b, s, aux);
    __syncthreads();
    total += clock64() - t0;
  }
  if (blockIdx.x < ntiles)
    for (int e = threadIdx.x; e < 256; e += 128) out[int64_t(blockIdx.x) * 256 + e] = a[e];
  if (threadIdx.x == 0) cycles[blockIdx.x] = total / reps;
}

// reference LDL^T in long double; a is column-major 16 x 16 (a[c * 16 + r]), b x b used
static void RefLdlt(const double* a, int b, long double* L, long double* D) {
  long double w[256];
  for (int i = 0; i < 256; ++i) w[i] = a[i];
  for (int k = 0; k < b; ++k) {
    D[k] = w[k * 16 + k];
    for (int r = k + 1; r < b; ++r) L[k * 16 + r] = w[k * 16 + r] / D[k];
    for (int c = k + 1; c < b; ++c)
      for (int r = c; r < b; ++r) w[c * 16 + r] -= L[k * 16 + r] * D[k] * L[k * 16 + c];
  }
}

int RunF64() {
  const int ntiles = 608;
  std::mt19937_64 rng(7);
  std::normal_distribution<double> N(0.0, 1.0);
  std::vector<double> tiles(size_t(ntiles) * 256);
  for (int t = 0; t < ntiles; ++t) {
    double* A = &tiles[size_t(t) * 256];
    const int kind = t % 4;  // 0: SPD well conditioned, 1: SPD wide scale, 2: indefinite, 3: SPD near singular
    double M[256];
    for (int i = 0; i < 256; ++i) M[i] = N(rng);
    for (int r = 0; r < 16; ++r)
      for (int c = 0; c < 16; ++c) {
        double s = 0;
        for (int q = 0; q < 16; ++q) s += M[q * 16 + r] * M[q * 16 + c];
        A[c * 16 + r] = s / 16 + (r == c ? (kind == 3 ? 1e-9 : 1.0) : 0.0);
      }
    if (kind == 1) {
      double sc[16];
      for (int i = 0; i < 16; ++i) sc[i] = std::pow(10.0, 12.0 * (i % 5) / 4.0 - 3.0);
      for (int r = 0; r < 16; ++r) for (int c = 0; c < 16; ++c) A[c * 16 + r] *= sc[r] * sc[c];
    }
    if (kind == 2) for (int i = 0; i < 16; ++i) A[i * 17] = N(rng);
  }
  double* d_t; double* d_o; long long* d_c;
  cudaMalloc(&d_t, sizeof(double) * tiles.size());
  cudaMalloc(&d_o, sizeof(double) * tiles.size());
  cudaMalloc(&d_c, sizeof(long long) * 608);
  cudaMemcpy(d_t, tiles.data(), sizeof(double) * tiles.size(), cudaMemcpyHostToDevice);
  std::vector<double> out(tiles.size());
  std::vector<long long> cyc(608);
  const char* names[4] = {"reciprocal, 2 barriers", "fraction-free, 1 barrier", "fraction-free, named barriers",
                          "fraction-free, 2 pivots a barrier"};
  for (int b : {16, 11}) {
    for (int V = 0; V < 4; ++V) {
      for (int grid : {1, 608}) {
        if (V == 0) BenchF64<0><<<grid, 128>>>(d_t, ntiles, b, 200, d_o, d_c);
        if (V == 1) BenchF64<1><<<grid, 128>>>(d_t, ntiles, b, 200, d_o, d_c);
        if (V == 2) BenchF64<2><<<grid, 128>>>(d_t, ntiles, b, 200, d_o, d_c);
        if (V == 3) BenchF64<3><<<grid, 128>>>(d_t, ntiles, b, 200, d_o, d_c);
        cudaDeviceSynchronize();
        cudaMemcpy(cyc.data(), d_c, sizeof(long long) * grid, cudaMemcpyDeviceToHost);
        double mean = 0; for (int g = 0; g < grid; ++g) mean += cyc[g]; mean /= grid;
        printf("b=%2d %-32s grid %3d: %7.0f cycles per tile\n", b, names[V], grid, mean);
      }
      cudaMemcpy(out.data(), d_o, sizeof(double) * out.size(), cudaMemcpyDeviceToHost);
      double worst[4] = {0, 0, 0, 0};
      for (int t = 0; t < ntiles; ++t) {
        long double L[256] = {0}, D[16];
        RefLdlt(&tiles[size_t(t) * 256], b, L, D);
        const double* o = &out[size_t(t) * 256];
        double e = 0;
        for (int k = 0; k < b; ++k) {
          e = std::fmax(e, double(fabsl((o[k * 17] - D[k]) / D[k])));
          for (int r = k + 1; r < b; ++r) {
            long double sc = fabsl(L[k * 16 + r]) + 1e-300L;
            long double colmax = 0; for (int q = k + 1; q < b; ++q) colmax = std::fmax(double(colmax), double(fabsl(L[k * 16 + q])));
            e = std::fmax(e, double(fabsl(o[k * 16 + r] - L[k * 16 + r]) / (colmax + 1e-300L)));
            (void)sc;
          }
        }
        worst[t % 4] = std::fmax(worst[t % 4], e);
      }
      printf("     max rel err vs long double: spd %.2e  spd-scaled %.2e  indefinite %.2e  near-singular %.2e\n",
             worst[0], worst[1], worst[2], worst[3]);
    }
  }
  return 0;
}

constexpr float kNearSingularPivot = 1.0f / 4096.0f;
template <typename T, int TILE>
__device__ __noinline__ void DiagElimWarp(T* a, const T* orig, int b, int* redo_flag) {
  constexpr unsigned kAll = 0xffffffffu;
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
      const T inv = T(1) / dj;
      const T lrj = row[j] * inv;
#pragma unroll
      for (int c = j + 1; c < TILE; ++c) {
        const T lcj = __shfl_sync(kAll, lrj, c);
        if (r >= c) row[c] -= row[j] * lcj;
      }
      if (r < b && r >= j) a[j * TILE + r] = r > j ? lrj : row[j];
    }
  }
  if (r == 0 && redo) *redo_flag = 1;
}
// entry q of thread t: e = t + 128 q over (r, c), 1 <= c <= r <= 31, column-major
__device__ __forceinline__ void LowerEntry32(int e, int* r, int* c) {
  int cc = 1, start = 0;
  while (cc < 31 && e >= start + (32 - cc)) { start += 32 - cc; ++cc; }
  *c = cc; *r = cc + (e - start);
}
template <bool kFastRcp>
__device__ void DiagLdltCta32(float* a, const float* orig, int b, int* redo_flag) {
  const int t = threadIdx.x;
  int r[4], c[4];
  float v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int e = t + 128 * q;
    if (e < 496) { LowerEntry32(e, &r[q], &c[q]); if (r[q] >= b) c[q] = 32; } else { r[q] = 0; c[q] = 32; }
    v[q] = c[q] < 32 ? a[c[q] * 32 + r[q]] : 0.f;
  }
  bool redo = false;
  for (int k = 0; k + 1 < b; ++k) {
    const float p = a[k * 33];
    float inv;
    if (kFastRcp) asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(p)); else inv = 1.0f / p;
    if (t == 0) redo = redo || !(p > kNearSingularPivot * fabsf(orig[k * 33]));
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (c[q] < 32 && c[q] > k) {
        const float lr = a[k * 32 + r[q]] * inv;
        v[q] = fmaf(-lr, a[k * 32 + c[q]], v[q]);
        a[c[q] * 32 + r[q]] = v[q];
      }
    }
    __syncthreads();
  }
  // scale the columns: L(r, c) = B(r, c) / d_c (d_c = a[c * 33]); column 0 separately
  if (t == 0) redo = redo || !(a[(b - 1) * 33] > kNearSingularPivot * fabsf(orig[(b - 1) * 33]));
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (c[q] < 32 && r[q] > c[q]) a[c[q] * 32 + r[q]] = v[q] / a[c[q] * 33];
  if (t >= 1 && t < b) a[t] = a[t] / a[0];
  if (t == 0 && redo) *redo_flag = 1;
  __syncthreads();
}

template <int V>
__global__ void __launch_bounds__(128) BenchF32(const float* tiles, int ntiles, int b, int reps, float* out,
                                             long long* cycles) {
  __shared__ float a[1024], keep[1024];
  __shared__ int redo;
  const int tile = blockIdx.x % ntiles;
  for (int e = threadIdx.x; e < 1024; e += 128) keep[e] = tiles[int64_t(tile) * 1024 + e];
  if (threadIdx.x == 0) redo = 0;
  __syncthreads();
  long long total = 0;
  for (int it = 0; it < reps; ++it) {
    for (int e = threadIdx.x; e < 1024; e += 128) a[e] = keep[e];
    __syncthreads();
    const long long t0 = clock64();
    if (V == 0) { if (threadIdx.x < 32) DiagElimWarp<float, 32>(a, keep, b, &redo); __syncthreads(); }
    else if (V == 1) DiagLdltCta32<false>(a, keep, b, &redo);
    else DiagLdltCta32<true>(a, keep, b, &redo);
    __syncthreads();
    total += clock64() - t0;
  }
  if (blockIdx.x < ntiles)
    for (int e = threadIdx.x; e < 1024; e += 128) out[int64_t(blockIdx.x) * 1024 + e] = a[e];
  if (threadIdx.x == 0) cycles[blockIdx.x] = total / reps;
}

static void RefLdltF32(const float* a, int b, double* L, double* D) {
  double w[1024];
  for (int i = 0; i < 1024; ++i) w[i] = a[i];
  for (int k = 0; k < b; ++k) {
    D[k] = w[k * 32 + k];
    for (int r = k + 1; r < b; ++r) L[k * 32 + r] = w[k * 32 + r] / D[k];
    for (int c = k + 1; c < b; ++c)
      for (int r = c; r < b; ++r) w[c * 32 + r] -= L[k * 32 + r] * D[k] * L[k * 32 + c];
  }
}

int RunF32() {
  const int ntiles = 608;
  std::mt19937_64 rng(7);
  std::normal_distribution<double> N(0.0, 1.0);
  std::vector<float> tiles(size_t(ntiles) * 1024);
  for (int t = 0; t < ntiles; ++t) {
    float* A = &tiles[size_t(t) * 1024];
    std::vector<double> M(1024);
    for (auto& x : M) x = N(rng);
    for (int r = 0; r < 32; ++r)
      for (int c = 0; c < 32; ++c) {
        double s = 0;
        for (int q = 0; q < 32; ++q) s += M[q * 32 + r] * M[q * 32 + c];
        A[c * 32 + r] = float(s / 32 + (r == c ? 1.0 : 0.0));
      }
  }
  float* d_t; float* d_o; long long* d_c;
  cudaMalloc(&d_t, sizeof(float) * tiles.size());
  cudaMalloc(&d_o, sizeof(float) * tiles.size());
  cudaMalloc(&d_c, sizeof(long long) * 608);
  cudaMemcpy(d_t, tiles.data(), sizeof(float) * tiles.size(), cudaMemcpyHostToDevice);
  std::vector<float> out(tiles.size());
  std::vector<long long> cyc(608);
  const char* names[3] = {"one warp, rows in registers", "CTA-wide, IEEE reciprocal", "CTA-wide, rcp.approx"};
  for (int b : {32, 21}) {
    for (int V = 0; V < 3; ++V) {
      for (int grid : {1, 608}) {
        if (V == 0) BenchF32<0><<<grid, 128>>>(d_t, ntiles, b, 100, d_o, d_c);
        if (V == 1) BenchF32<1><<<grid, 128>>>(d_t, ntiles, b, 100, d_o, d_c);
        if (V == 2) BenchF32<2><<<grid, 128>>>(d_t, ntiles, b, 100, d_o, d_c);
        cudaDeviceSynchronize();
        cudaMemcpy(cyc.data(), d_c, sizeof(long long) * grid, cudaMemcpyDeviceToHost);
        double mean = 0; for (int g = 0; g < grid; ++g) mean += cyc[g]; mean /= grid;
        printf("b=%2d %-30s grid %3d: %7.0f cycles per tile\n", b, names[V], grid, mean);
      }
      cudaMemcpy(out.data(), d_o, sizeof(float) * out.size(), cudaMemcpyDeviceToHost);
      double worst = 0;
      for (int t = 0; t < ntiles; ++t) {
        std::vector<double> L(1024, 0.0), D(32);
        RefLdltF32(&tiles[size_t(t) * 1024], b, L.data(), D.data());
        const float* o = &out[size_t(t) * 1024];
        for (int k = 0; k < b; ++k) {
          worst = std::fmax(worst, std::fabs((o[k * 33] - D[k]) / D[k]));
          for (int r = k + 1; r < b; ++r) worst = std::fmax(worst, std::fabs(o[k * 32 + r] - L[k * 32 + r]));
        }
      }
      printf("     max err vs double: %.2e\n", worst);
    }
  }
  return 0;
}

int main() {
  RunF64();
  RunF32();
  cudaError_t e = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}
