// Residuals and analytic tangent-space Jacobians of the typed factors, evaluated per factor by one
// thread.  T is the Jacobian / Hessian precision (double for the plain form, float for the mixed
// form); residuals are always returned in double so that the cost reduction stays FP64.
//
// The residual conventions are the reference's generated factors (cited per function).  The
// Jacobians are derived by hand from the chain rule through the same retraction the reference
// linearizes about (gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102: q <- q * exp(w), t <- t + dt;
// gen/cpp/sym/ops/pose2/lie_group_ops.cc:58-82); they are compared against forward-mode
// differentiation in the tests.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "../../include/sfgpu.h"

namespace sfg {

#define SFG_HD __host__ __device__ __forceinline__

// NK keys, NC constants, RD residual rows, TD tangent columns; KT / KS the tangent and storage
// size of key slot k; MK the leading key slots whose entries a warp sums (MergedKeySlots).
template <int KIND>
struct FactorTraits;
template <>
struct FactorTraits<SFG_FACTOR_BEARING_POSE2> {
  static constexpr int NK = 1, NC = 5, RD = 1, TD = 3, MK = 0;
  static constexpr SFG_HD int KT(int k) { return k == 0 ? 3 : (k == 1 ? 0 : 0); }
  static constexpr SFG_HD int KS(int k) { return k == 0 ? 4 : (k == 1 ? 0 : 0); }
};
template <>
struct FactorTraits<SFG_FACTOR_ODOMETRY_POSE2> {
  static constexpr int NK = 2, NC = 3, RD = 1, TD = 6, MK = 0;
  static constexpr SFG_HD int KT(int k) { return k == 0 ? 3 : (k == 1 ? 3 : 0); }
  static constexpr SFG_HD int KS(int k) { return k == 0 ? 4 : (k == 1 ? 4 : 0); }
};
template <>
struct FactorTraits<SFG_FACTOR_SNAVELY_REPROJECTION> {
  static constexpr int NK = 3, NC = 4, RD = 2, TD = 12, MK = 2;
  static constexpr SFG_HD int KT(int k) { return k == 0 ? 6 : (k == 1 ? 3 : 3); }
  static constexpr SFG_HD int KS(int k) { return k == 0 ? 7 : (k == 1 ? 3 : 3); }
};
template <>
struct FactorTraits<SFG_FACTOR_BETWEEN_POSE3> {
  static constexpr int NK = 2, NC = 14, RD = 6, TD = 12, MK = 0;
  static constexpr SFG_HD int KT(int k) { return k == 0 ? 6 : (k == 1 ? 6 : 0); }
  static constexpr SFG_HD int KS(int k) { return k == 0 ? 7 : (k == 1 ? 7 : 0); }
};
template <>
struct FactorTraits<SFG_FACTOR_PRIOR_POSE3> {
  static constexpr int NK = 1, NC = 14, RD = 6, TD = 6, MK = 0;
  static constexpr SFG_HD int KT(int k) { return k == 0 ? 6 : (k == 1 ? 0 : 0); }
  static constexpr SFG_HD int KS(int k) { return k == 0 ? 7 : (k == 1 ? 0 : 0); }
};
template <>
struct FactorTraits<SFG_FACTOR_RANGE_POSE3> {
  static constexpr int NK = 1, NC = 6, RD = 1, TD = 6, MK = 0;
  static constexpr SFG_HD int KT(int k) { return k == 0 ? 6 : (k == 1 ? 0 : 0); }
  static constexpr SFG_HD int KS(int k) { return k == 0 ? 7 : (k == 1 ? 0 : 0); }
};

constexpr double kPiD = 3.14159265358979323846;

// Rotation matrix of a unit [x, y, z, w] quaternion, row-major.
template <typename T>
SFG_HD void QuatToRot(const T* q, T* R) {
  const T x = q[0], y = q[1], z = q[2], w = q[3];
  R[0] = 1 - 2 * (y * y + z * z);
  R[1] = 2 * (x * y - w * z);
  R[2] = 2 * (x * z + w * y);
  R[3] = 2 * (x * y + w * z);
  R[4] = 1 - 2 * (x * x + z * z);
  R[5] = 2 * (y * z - w * x);
  R[6] = 2 * (x * z - w * y);
  R[7] = 2 * (y * z + w * x);
  R[8] = 1 - 2 * (x * x + y * y);
}

template <typename T>
SFG_HD void QuatMulD(const T* p, const T* q, T* o) {
  o[0] = p[3] * q[0] + p[0] * q[3] + p[1] * q[2] - p[2] * q[1];
  o[1] = p[3] * q[1] - p[0] * q[2] + p[1] * q[3] + p[2] * q[0];
  o[2] = p[3] * q[2] + p[0] * q[1] - p[1] * q[0] + p[2] * q[3];
  o[3] = p[3] * q[3] - p[0] * q[0] - p[1] * q[1] - p[2] * q[2];
}

// d(p (x) q)/dq = Lmat(p), 4x4 row-major (rows: output x, y, z, w; cols: q x, y, z, w).
template <typename T>
SFG_HD void QuatLeftMat(const T* p, T* L) {
  const T x = p[0], y = p[1], z = p[2], w = p[3];
  L[0] = w;  L[1] = -z; L[2] = y;  L[3] = x;
  L[4] = z;  L[5] = w;  L[6] = -x; L[7] = y;
  L[8] = -y; L[9] = x;  L[10] = w; L[11] = z;
  L[12] = -x; L[13] = -y; L[14] = -z; L[15] = w;
}

// d(p (x) q)/dp = Rmat(q), 4x4 row-major.
template <typename T>
SFG_HD void QuatRightMat(const T* q, T* Rm) {
  const T x = q[0], y = q[1], z = q[2], w = q[3];
  Rm[0] = w;  Rm[1] = z;  Rm[2] = -y; Rm[3] = x;
  Rm[4] = -z; Rm[5] = w;  Rm[6] = x;  Rm[7] = y;
  Rm[8] = y;  Rm[9] = -x; Rm[10] = w; Rm[11] = z;
  Rm[12] = -x; Rm[13] = -y; Rm[14] = -z; Rm[15] = w;
}

// Rotation part of Pose3 local coordinates (gen/cpp/sym/ops/pose3/lie_group_ops.cc:104-130):
// w = 2 sign(qw) acos(m) / sqrt(1 - m^2) * q.xyz, m = min(|qw|, 1 - eps).  Returns w and
// dw/dq (3x4 row-major).
template <typename T>
SFG_HD void QuatLogWithJacobian(const T* q, double eps, T* w, T* dw) {
  const T aw = q[3] < T(0) ? -q[3] : q[3];
  const T sgn = q[3] < T(0) ? T(-1) : T(1);
  const bool clamped = !(aw < T(1.0 - eps));
  const T m = clamped ? T(1.0 - eps) : aw;
  const T s2 = T(1) - m * m;
  const T sq = sqrt(s2);
  const T ac = acos(m);
  const T k = T(2) * sgn * ac / sq;
  const T dkdm = T(2) * sgn * (T(-1) + m * ac / sq) / s2;
  const T dk = clamped ? T(0) : dkdm * sgn;
  for (int i = 0; i < 3; ++i) {
    w[i] = k * q[i];
    for (int j = 0; j < 3; ++j) dw[i * 4 + j] = (i == j) ? k : T(0);
    dw[i * 4 + 3] = q[i] * dk;
  }
}

// Rot3 retraction (gen/cpp/sym/ops/rot3/lie_group_ops.cc): q <- q * exp(w) with the
// eps-regularised norm, as the rotation part of RetractPose3 below.  a, o: [qx, qy, qz, qw].
SFG_HD void RetractRot3(const double* a, const double* d, double eps, double* o) {
  const double n = sqrt(eps * eps + d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double c = cos(0.5 * n);
  const double s = sin(0.5 * n) / n;
  const double vx = s * d[0], vy = s * d[1], vz = s * d[2];
  const double a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
  o[0] = a3 * vx + a0 * c + a1 * vz - a2 * vy;
  o[1] = a3 * vy - a0 * vz + a1 * c + a2 * vx;
  o[2] = a3 * vz + a0 * vy - a1 * vx + a2 * c;
  o[3] = a3 * c - a0 * vx - a1 * vy - a2 * vz;
}

// Pose3 retraction (gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102): q <- q * exp(w) with the
// eps-regularised norm, t <- t + dt.  a, o: storage [qx, qy, qz, qw, x, y, z]; d: tangent [w, dt].
SFG_HD void RetractPose3(const double* a, const double* d, double eps, double* o) {
  const double n = sqrt(eps * eps + d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double c = cos(0.5 * n);
  const double s = sin(0.5 * n) / n;
  const double vx = s * d[0], vy = s * d[1], vz = s * d[2];
  const double a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
  o[0] = a3 * vx + a0 * c + a1 * vz - a2 * vy;
  o[1] = a3 * vy - a0 * vz + a1 * c + a2 * vx;
  o[2] = a3 * vz + a0 * vy - a1 * vx + a2 * c;
  o[3] = a3 * c - a0 * vx - a1 * vy - a2 * vz;
  o[4] = a[4] + d[3];
  o[5] = a[5] + d[4];
  o[6] = a[6] + d[5];
}

// Values::Retract of one key of any type (symforce/opt/values.cc:315-327): storage a, tangent
// update d, result o.
SFG_HD void RetractKey(int type, const double* a, const double* d, double eps, double* o) {
  switch (type) {
    case SFG_KEY_POSE2: {  // gen/cpp/sym/ops/pose2/lie_group_ops.cc:58-82
      const double c = cos(d[0]), s = sin(d[0]);
      const double re = a[0], im = a[1];
      o[0] = re * c - im * s;
      o[1] = re * s + im * c;
      o[2] = a[2] + d[1];
      o[3] = a[3] + d[2];
      break;
    }
    case SFG_KEY_POSE3:  // gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102
      RetractPose3(a, d, eps, o);
      break;
    case SFG_KEY_ROT3:  // gen/cpp/sym/ops/rot3/lie_group_ops.cc: the rotation part of the above
      RetractRot3(a, d, eps, o);
      break;
    default: {  // VEC1..VEC3 = 1..3, VEC4..VEC6 = 7..9
      const int n = type <= SFG_KEY_VEC3 ? type : type - SFG_KEY_VEC4 + 4;
      for (int i = 0; i < n; ++i) o[i] = a[i] + d[i];
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Factor evaluation: x[slot] points at the key storage, c at the constants (already loaded).
// r: residual (double), J: RD x TD row-major (T).
// ---------------------------------------------------------------------------------------------
template <int KIND, typename T>
struct FactorEval;

// symforce/examples/robot_2d_localization/gen/bearing_factor.h:21-97, whitened by sqrt_info.
template <typename T>
struct FactorEval<SFG_FACTOR_BEARING_POSE2, T> {
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double* p = x[0];
    const double lx = c[0], ly = c[1], angle = c[2], eps = c[3], wgt = c[4];
    const double dx = lx - p[2], dy = ly - p[3];
    const double bx = p[0] * dx + p[1] * dy;
    const double by = p[0] * dy - p[1] * dx;
    const double bxe = bx + (bx < 0 ? -eps : eps);
    const double e = atan2(by, bxe) - angle;
    const double wrapped = e - 2 * kPiD * floor((e + kPiD) / (2 * kPiD));
    r[0] = wgt * wrapped;
    const double inv = wgt / (bxe * bxe + by * by);
    J[0] = T(-(by * by + bxe * bx) * inv);
    J[1] = T((by * p[0] + bxe * p[1]) * inv);
    J[2] = T((by * p[1] - bxe * p[0]) * inv);
  }
};

// symforce/examples/robot_2d_localization/gen/odometry_factor.h:21-98, whitened by sqrt_info.
template <typename T>
struct FactorEval<SFG_FACTOR_ODOMETRY_POSE2, T> {
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double* a = x[0];
    const double* b = x[1];
    const double dx = b[2] - a[2], dy = b[3] - a[3];
    const double n = sqrt(dx * dx + dy * dy + c[1]);
    r[0] = c[2] * (n - c[0]);
    const double gx = c[2] * dx / n, gy = c[2] * dy / n;
    J[0] = T(0);
    J[1] = T(-gx);
    J[2] = T(-gy);
    J[3] = T(0);
    J[4] = T(gx);
    J[5] = T(gy);
  }
};

// symforce/examples/bundle_adjustment_in_the_large/bundle_adjustment_in_the_large.py:18-63 with
// the Cauchy norm whitening (symforce/opt/noise_models.py:318-428, whiten_norm, alpha -> 0).
// The residual is evaluated in double; the Jacobian chain in T.
template <typename T>
struct FactorEval<SFG_FACTOR_SNAVELY_REPROJECTION, T> {
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double* cam = x[0];
    const double* in = x[1];
    const double* X = x[2];
    const double px = c[0], py = c[1], eps = c[2], delta = c[3];
    double R[9];
    QuatToRot(cam, R);
    const double xr0 = R[0] * X[0] + R[1] * X[1] + R[2] * X[2];
    const double xr1 = R[3] * X[0] + R[4] * X[1] + R[5] * X[2];
    const double xr2 = R[6] * X[0] + R[7] * X[1] + R[8] * X[2];
    const double pc0 = xr0 + cam[4], pc1 = xr1 + cam[5], pc2 = xr2 + cam[6];
    const double iz = -1.0 / pc2;
    const double u = pc0 * iz, v = pc1 * iz;
    const double r2 = u * u + v * v;
    const double f = in[0], k1 = in[1], k2 = in[2];
    const double g = 1.0 + k1 * r2 + k2 * r2 * r2;
    const double e0 = f * g * u - px;
    const double e1 = f * g * v - py;
    // whitening
    double s = 1.0;  // dw/de = s I + t e e^T
    T Tt = T(0);
    if (delta > 0) {
      const double n2 = e0 * e0 + e1 * e1 + eps;
      const double n = sqrt(n2);
      const double uu = n2 / (2.0 * delta * delta);
      const double rho2 = 2.0 * delta * delta * log1p(uu);
      const double sq = sqrt(rho2);
      s = sq / n;
      // t only enters the Jacobian: in its precision (two divisions off the FP64 pipe in FP32)
      if constexpr (sizeof(T) == 8) {
        const double dsdn = (n2 / ((1.0 + uu) * sq) - sq) / n2;
        Tt = T(dsdn / n);
      } else {
        const T fn2 = T(n2), fsq = T(sq);
        const T dsdn = (fn2 / ((T(1) + T(uu)) * fsq) - fsq) / fn2;
        Tt = dsdn / T(n);
      }
    }
    r[0] = s * e0;
    r[1] = s * e1;
    // Jacobian chain in T
    const T Ts = T(s), Te0 = T(e0), Te1 = T(e1);
    const T W00 = Ts + Tt * Te0 * Te0, W01 = Tt * Te0 * Te1, W11 = Ts + Tt * Te1 * Te1;
    const T Tu = T(u), Tv = T(v), Tf = T(f), Tg = T(g), Tr2 = T(r2);
    const T dg = T(2) * (T(k1) + T(2) * T(k2) * Tr2);
    // G = de/dp = f (g I + dg p p^T)
    const T G00 = Tf * (Tg + dg * Tu * Tu), G01 = Tf * dg * Tu * Tv, G11 = Tf * (Tg + dg * Tv * Tv);
    // M = dw/dp = W G
    const T M00 = W00 * G00 + W01 * G01, M01 = W00 * G01 + W01 * G11;
    const T M10 = W01 * G00 + W11 * G01, M11 = W01 * G01 + W11 * G11;
    // A = dw/dpc = M * iz [[1, 0, u], [0, 1, v]]
    const T Tiz = T(iz);
    T A[6];
    A[0] = M00 * Tiz;
    A[1] = M01 * Tiz;
    A[2] = (M00 * Tu + M01 * Tv) * Tiz;
    A[3] = M10 * Tiz;
    A[4] = M11 * Tiz;
    A[5] = (M10 * Tu + M11 * Tv) * Tiz;
    T Rt[9];
    for (int i = 0; i < 9; ++i) Rt[i] = T(R[i]);
    // dpc/dw = -[xr]x R ; B = A * (-[xr]x)
    const T a0 = T(xr0), a1 = T(xr1), a2 = T(xr2);
    for (int row = 0; row < 2; ++row) {
      const T* Ar = A + 3 * row;
      // -[a]x = [[0, a2, -a1], [-a2, 0, a0], [a1, -a0, 0]]
      const T b0 = -Ar[1] * a2 + Ar[2] * a1;
      const T b1 = Ar[0] * a2 - Ar[2] * a0;
      const T b2 = -Ar[0] * a1 + Ar[1] * a0;
      T* Jr = J + 12 * row;
      for (int k = 0; k < 3; ++k) {
        Jr[k] = b0 * Rt[k] + b1 * Rt[3 + k] + b2 * Rt[6 + k];      // rotation
        Jr[3 + k] = Ar[k];                                          // translation
        Jr[9 + k] = Ar[0] * Rt[k] + Ar[1] * Rt[3 + k] + Ar[2] * Rt[6 + k];  // point
      }
    }
    // intrinsics: de/d(f, k1, k2) = [g p, f r2 p, f r2^2 p]; dw = W de
    const T Wp0 = W00 * Tu + W01 * Tv, Wp1 = W01 * Tu + W11 * Tv;
    J[6] = Tg * Wp0;
    J[7] = Tf * Tr2 * Wp0;
    J[8] = Tf * Tr2 * Tr2 * Wp0;
    J[18] = Tg * Wp1;
    J[19] = Tf * Tr2 * Wp1;
    J[20] = Tf * Tr2 * Tr2 * Wp1;
  }
};

// local_coordinates(a_T_b, a^-1 b) whitened by diag(s) (symforce/codegen/geo_factors_codegen.py:53-71).
template <typename T>
struct FactorEval<SFG_FACTOR_BETWEEN_POSE3, T> {
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double* a = x[0];
    const double* b = x[1];
    const double* m = c;
    const double* s = c + 7;
    const double eps = c[13];
    const double qa_inv[4] = {-a[0], -a[1], -a[2], a[3]};
    double P[4];
    QuatMulD(qa_inv, b, P);
    const double qm_inv[4] = {-m[0], -m[1], -m[2], m[3]};
    double qe[4];
    QuatMulD(qm_inv, P, qe);
    double Ra[9];
    QuatToRot(a, Ra);
    const double dt[3] = {b[4] - a[4], b[5] - a[5], b[6] - a[6]};
    double tab[3];
    for (int i = 0; i < 3; ++i) tab[i] = Ra[i] * dt[0] + Ra[3 + i] * dt[1] + Ra[6 + i] * dt[2];
    double w[3], dw[12];
    QuatLogWithJacobian(qe, eps, w, dw);
    for (int i = 0; i < 3; ++i) {
      r[i] = s[i] * w[i];
      r[3 + i] = s[3 + i] * (tab[i] - m[4 + i]);
    }
    for (int i = 0; i < 72; ++i) J[i] = T(0);
    // dqe/dwb = Lmat(qe)[:, 0:3] / 2 ; dqe/dwa = -Lmat(qm^-1) Rmat(P)[:, 0:3] / 2
    double Le[16], Lm[16], RP[16];
    QuatLeftMat(qe, Le);
    QuatLeftMat(qm_inv, Lm);
    QuatRightMat(P, RP);
    double dqa[12], dqb[12];  // 4x3
    for (int row = 0; row < 4; ++row)
      for (int k = 0; k < 3; ++k) {
        dqb[row * 3 + k] = 0.5 * Le[row * 4 + k];
        double acc = 0;
        for (int q = 0; q < 4; ++q) acc += Lm[row * 4 + q] * RP[q * 4 + k];
        dqa[row * 3 + k] = -0.5 * acc;
      }
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        double ja = 0, jb = 0;
        for (int q = 0; q < 4; ++q) {
          ja += dw[i * 4 + q] * dqa[q * 3 + k];
          jb += dw[i * 4 + q] * dqb[q * 3 + k];
        }
        J[i * 12 + k] = T(s[i] * ja);
        J[i * 12 + 6 + k] = T(s[i] * jb);
      }
    // translation rows: d tab / d wa = [tab]x, d tab / d ta = -Ra^T, d tab / d tb = Ra^T
    const double cx[9] = {0, -tab[2], tab[1], tab[2], 0, -tab[0], -tab[1], tab[0], 0};
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        J[(3 + i) * 12 + k] = T(s[3 + i] * cx[i * 3 + k]);
        J[(3 + i) * 12 + 3 + k] = T(-s[3 + i] * Ra[k * 3 + i]);
        J[(3 + i) * 12 + 9 + k] = T(s[3 + i] * Ra[k * 3 + i]);
      }
  }
};

// local_coordinates(prior, value) whitened by diag(s) (symforce/codegen/geo_factors_codegen.py:74-86).
template <typename T>
struct FactorEval<SFG_FACTOR_PRIOR_POSE3, T> {
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double* v = x[0];
    const double* p = c;
    const double* s = c + 7;
    const double eps = c[13];
    const double qp_inv[4] = {-p[0], -p[1], -p[2], p[3]};
    double qe[4];
    QuatMulD(qp_inv, v, qe);
    double w[3], dw[12];
    QuatLogWithJacobian(qe, eps, w, dw);
    for (int i = 0; i < 3; ++i) {
      r[i] = s[i] * w[i];
      r[3 + i] = s[3 + i] * (v[4 + i] - p[4 + i]);
    }
    for (int i = 0; i < 36; ++i) J[i] = T(0);
    double Le[16];
    QuatLeftMat(qe, Le);
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        double acc = 0;
        for (int q = 0; q < 4; ++q) acc += dw[i * 4 + q] * 0.5 * Le[q * 4 + k];
        J[i * 6 + k] = T(s[i] * acc);
      }
    for (int i = 0; i < 3; ++i) J[(3 + i) * 6 + 3 + i] = T(s[3 + i]);
  }
};

// 1 / sqrt(x) in FP64: on the device an FP32 seed refined by two Newton steps
// y <- y (3 - x y^2) / 2 (each roughly doubles the correct digits: ~1e-7 -> ~1e-14 -> rounding),
// which avoids the long FP64 square-root and divide sequences.
SFG_HD double RsqrtD(double x) {
#ifdef __CUDA_ARCH__
  if (!(x > 1e-30 && x < 1e30)) return 1.0 / sqrt(x);
  double r = double(rsqrtf(float(x)));
  r = r * (1.5 - 0.5 * x * r * r);
  r = r * (1.5 - 0.5 * x * r * r);
  return r;
#else
  return 1.0 / sqrt(x);
#endif
}

// Range from the Pose3 position to a fixed landmark.
template <typename T>
struct FactorEval<SFG_FACTOR_RANGE_POSE3, T> {
  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {
    const double* v = x[0];
    const double dx = v[4] - c[0], dy = v[5] - c[1], dz = v[6] - c[2];
    const double q = dx * dx + dy * dy + dz * dz + c[5];
    const double inv = RsqrtD(q);
    const double n = q * inv;
    r[0] = c[4] * (n - c[3]);
    J[0] = J[1] = J[2] = T(0);
    const double s = c[4] * inv;
    J[3] = T(s * dx);
    J[4] = T(s * dy);
    J[5] = T(s * dz);
  }
};

// ---------------------------------------------------------------------------------------------
// Factor kinds generated from symbolic residuals (symforce_gb300/factor_defs.py, emitted by
// symforce_gb300/codegen.py): traits and evaluation forward to the generated structs.
// ---------------------------------------------------------------------------------------------
}  // namespace sfg
#include "generated_factor_specs.h"
#include "generated_factors.cuh"
namespace sfg {
#define SFG_GENERATED_KIND(KIND, NKEYS, NCONSTS, RDIM, K0, K1, K2, G)                              \
  template <>                                                                                      \
  struct FactorTraits<KIND> {                                                                      \
    static constexpr int NK = G::NK, NC = G::NC, RD = G::RD, TD = G::TD, MK = 0;                   \
    static constexpr SFG_HD int KT(int k) { return G::KT(k); }                                     \
    static constexpr SFG_HD int KS(int k) { return G::KS(k); }                                     \
  };                                                                                               \
  template <typename T>                                                                            \
  struct FactorEval<KIND, T> {                                                                     \
    static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {             \
      G::template Run<T>(x, c, r, J);                                                              \
    }                                                                                              \
  };
SFG_GENERATED_FACTORS(SFG_GENERATED_KIND)
#undef SFG_GENERATED_KIND

}  // namespace sfg
