// Test infrastructure, not product code.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load the oracle; the GPU library never links it.
//
// CPU restatement of the reference's residual functions and Lie-group retractions, written once
// as templates over the scalar type so that the oracle differentiates them with forward-mode jets
// (jet.h).  Each function cites the reference source it restates.
#pragma once

#include <cmath>

#include "./jet.h"

namespace oracle {

using std::acos;
using std::atan2;
using std::cos;
using std::fabs;
using std::log1p;
using std::sin;
using std::sqrt;

inline double fmin(double x, double c) { return x < c ? x : c; }

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------------------------
// Retractions (Values::Retract -> LieGroupOps<T>::Retract)
// ---------------------------------------------------------------------------------------------

// Pose2 storage [re, im, x, y], tangent [theta, x, y]:
// gen/cpp/sym/ops/pose2/lie_group_ops.cc:58-82 (rotation composed on the right, t += dt).
template <typename S>
void RetractPose2(const double* a, const S* d, S* out) {
  const S c = cos(d[0]);
  const S s = sin(d[0]);
  out[0] = a[0] * c - a[1] * s;
  out[1] = a[0] * s + a[1] * c;
  out[2] = a[2] + d[1];
  out[3] = a[3] + d[2];
}

// Pose3 storage [qx, qy, qz, qw, x, y, z], tangent [w(3), t(3)]:
// gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102.  q <- q * [sin(|w|/2) w/|w|, cos(|w|/2)] with
// |w| = sqrt(eps^2 + w.w); t <- t + dt.
template <typename S>
void RetractPose3(const double* a, const S* d, double eps, S* out) {
  const S n = sqrt(eps * eps + d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const S c = cos(0.5 * n);
  const S s = sin(0.5 * n) / n;
  // q * dq with dq = [s w, c]
  const S vx = s * d[0], vy = s * d[1], vz = s * d[2];
  out[0] = a[3] * vx + a[0] * c + a[1] * vz - a[2] * vy;
  out[1] = a[3] * vy - a[0] * vz + a[1] * c + a[2] * vx;
  out[2] = a[3] * vz + a[0] * vy - a[1] * vx + a[2] * c;
  out[3] = a[3] * c - a[0] * vx - a[1] * vy - a[2] * vz;
  out[4] = a[4] + d[3];
  out[5] = a[5] + d[4];
  out[6] = a[6] + d[5];
}

// ---------------------------------------------------------------------------------------------
// Quaternion helpers, [x, y, z, w] Hamilton convention (sym::Rot3 storage).
// ---------------------------------------------------------------------------------------------
template <typename A, typename B, typename S>
void QuatMul(const A* p, const B* q, S* out) {
  out[0] = p[3] * q[0] + p[0] * q[3] + p[1] * q[2] - p[2] * q[1];
  out[1] = p[3] * q[1] - p[0] * q[2] + p[1] * q[3] + p[2] * q[0];
  out[2] = p[3] * q[2] + p[0] * q[1] - p[1] * q[0] + p[2] * q[3];
  out[3] = p[3] * q[3] - p[0] * q[0] - p[1] * q[1] - p[2] * q[2];
}

template <typename S>
void QuatRotate(const S* q, const S* v, S* out) {
  // R(q) v for unit q
  const S x = q[0], y = q[1], z = q[2], w = q[3];
  out[0] = (1 - 2 * (y * y + z * z)) * v[0] + 2 * (x * y - w * z) * v[1] + 2 * (x * z + w * y) * v[2];
  out[1] = 2 * (x * y + w * z) * v[0] + (1 - 2 * (x * x + z * z)) * v[1] + 2 * (y * z - w * x) * v[2];
  out[2] = 2 * (x * z - w * y) * v[0] + 2 * (y * z + w * x) * v[1] + (1 - 2 * (x * x + y * y)) * v[2];
}

// Rotation part of Pose3 local_coordinates(a, b) = to_tangent(a.R^-1 * b.R):
// gen/cpp/sym/ops/pose3/lie_group_ops.cc:104-130.  q is the relative quaternion a^-1 b.
template <typename S>
void QuatLog(const S* q, double eps, S* out) {
  const S m = fmin(fabs(q[3]), 1.0 - eps);
  const double sgn = Value(q[3]) < 0 ? -1.0 : 1.0;  // copysign(1, w)
  const S k = 2.0 * sgn * acos(m) / sqrt(1.0 - m * m);
  out[0] = k * q[0];
  out[1] = k * q[1];
  out[2] = k * q[2];
}

// ---------------------------------------------------------------------------------------------
// Residuals.  `x` holds the (already retracted) storage of each optimized key in order; `c` the
// per-factor constants in the layout declared in include/sfgpu.h.
// ---------------------------------------------------------------------------------------------

// symforce/examples/robot_2d_localization/gen/bearing_factor.h:21-97 (+ sqrt_info whitening)
template <typename S>
void BearingResidual(const S* pose, const double* c, S* r) {
  const double lx = c[0], ly = c[1], angle = c[2], eps = c[3], w = c[4];
  const S dx = lx - pose[2];
  const S dy = ly - pose[3];
  const S bx = pose[0] * dx + pose[1] * dy;  // R^T (l - t)
  const S by = pose[0] * dy - pose[1] * dx;
  const S bxe = bx + (Value(bx) < 0 ? -eps : eps);  // copysign(eps, x)
  const S e = atan2(by, bxe) - angle;
  // wrap_angle(x) = x - 2 pi floor((x + pi) / (2 pi))
  const double k = std::floor((Value(e) + kPi) / (2 * kPi));
  r[0] = w * (e - 2 * kPi * k);
}

// symforce/examples/robot_2d_localization/gen/odometry_factor.h:21-98 (+ sqrt_info whitening)
template <typename S>
void OdometryResidual(const S* a, const S* b, const double* c, S* r) {
  const double dist = c[0], eps = c[1], w = c[2];
  const S dx = b[2] - a[2];
  const S dy = b[3] - a[3];
  r[0] = w * (sqrt(dx * dx + dy * dy + eps) - dist);
}

// symforce/examples/bundle_adjustment_in_the_large/bundle_adjustment_in_the_large.py:18-63, with the
// optional Cauchy norm whitening (symforce/opt/noise_models.py: ScalarNoiseModel.whiten_norm and
// BarronNoiseModel at alpha = 0, evaluated as its closed-form limit delta^2 log(1 + x^2/(2 delta^2))).
template <typename S>
void SnavelyResidual(const S* cam, const S* intr, const S* pt, const double* c, S* r) {
  const double px = c[0], py = c[1], eps = c[2], delta = c[3];
  S pc[3];
  QuatRotate(cam, pt, pc);
  pc[0] = pc[0] + cam[4];
  pc[1] = pc[1] + cam[5];
  pc[2] = pc[2] + cam[6];
  const S u = pc[0] / (-pc[2]);
  const S v = pc[1] / (-pc[2]);
  const S r2 = u * u + v * v;
  const S g = 1.0 + intr[1] * r2 + intr[2] * r2 * r2;
  S e0 = intr[0] * g * u - px;
  S e1 = intr[0] * g * v - py;
  if (delta > 0) {
    const S n2 = e0 * e0 + e1 * e1 + eps;
    const S n = sqrt(n2);
    const S rho2 = 2.0 * delta * delta * log1p(n2 / (2.0 * delta * delta));  // 2 rho(n)
    const S s = sqrt(rho2) / n;
    e0 = s * e0;
    e1 = s * e1;
  }
  r[0] = e0;
  r[1] = e1;
}

// local_coordinates(a_T_b, between(a, b)) whitened by diag(s):
// symforce/codegen/geo_factors_codegen.py:53-71, gen/cpp/sym/factors/between_factor_pose3.h.
template <typename S>
void BetweenPose3Residual(const S* a, const S* b, const double* c, S* r) {
  const double* m = c;       // a_T_b storage
  const double* s = c + 7;   // sqrt_info diagonal
  const double eps = c[13];
  // a^-1 b : q = qa^* qb, t = Ra^T (tb - ta)
  const S qa_inv[4] = {-a[0], -a[1], -a[2], a[3]};
  S q[4];
  QuatMul(qa_inv, b, q);
  const S dt[3] = {b[4] - a[4], b[5] - a[5], b[6] - a[6]};
  S t[3];
  QuatRotate(qa_inv, dt, t);
  // local_coordinates(m, (q, t)) = [log(qm^* q), t - tm]
  const double qm_inv[4] = {-m[0], -m[1], -m[2], m[3]};
  S qe[4];
  QuatMul(qm_inv, q, qe);
  S w[3];
  QuatLog(qe, eps, w);
  r[0] = s[0] * w[0];
  r[1] = s[1] * w[1];
  r[2] = s[2] * w[2];
  r[3] = s[3] * (t[0] - m[4]);
  r[4] = s[4] * (t[1] - m[5]);
  r[5] = s[5] * (t[2] - m[6]);
}

// local_coordinates(prior, value) whitened by diag(s): symforce/codegen/geo_factors_codegen.py:74-86.
template <typename S>
void PriorPose3Residual(const S* x, const double* c, S* r) {
  const double* p = c;
  const double* s = c + 7;
  const double eps = c[13];
  const double qp_inv[4] = {-p[0], -p[1], -p[2], p[3]};
  S qe[4];
  QuatMul(qp_inv, x, qe);
  S w[3];
  QuatLog(qe, eps, w);
  r[0] = s[0] * w[0];
  r[1] = s[1] * w[1];
  r[2] = s[2] * w[2];
  r[3] = s[3] * (x[4] - p[4]);
  r[4] = s[4] * (x[5] - p[5]);
  r[5] = s[5] * (x[6] - p[6]);
}

// Range from a Pose3 position to a fixed landmark (no reference counterpart; the odometry
// factor's eps-regularised norm is reused).
template <typename S>
void RangePose3Residual(const S* x, const double* c, S* r) {
  const S dx = x[4] - c[0];
  const S dy = x[5] - c[1];
  const S dz = x[6] - c[2];
  r[0] = c[4] * (sqrt(dx * dx + dy * dy + dz * dz + c[5]) - c[3]);
}

// ---------------------------------------------------------------------------------------------
// The factors the library generates from symbolic definitions (restated here by hand, so that the
// oracle checks the generated code independently).
// ---------------------------------------------------------------------------------------------

// Rot3 storage [x, y, z, w], tangent w: gen/cpp/sym/ops/rot3/lie_group_ops.cc, q <- q * exp(w)
// with |w| = sqrt(eps^2 + w.w) (the rotation part of RetractPose3).
template <typename S>
void RetractRot3(const double* a, const S* d, double eps, S* out) {
  const S n = sqrt(eps * eps + d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const S c = cos(0.5 * n);
  const S s = sin(0.5 * n) / n;
  const S vx = s * d[0], vy = s * d[1], vz = s * d[2];
  out[0] = a[3] * vx + a[0] * c + a[1] * vz - a[2] * vy;
  out[1] = a[3] * vy - a[0] * vz + a[1] * c + a[2] * vx;
  out[2] = a[3] * vz + a[0] * vy - a[1] * vx + a[2] * c;
  out[3] = a[3] * c - a[0] * vx - a[1] * vy - a[2] * vz;
}

// prior_factor for Rot3 (symforce/codegen/geo_factors_codegen.py:74-86): diag(s) Log(prior^-1 x);
// consts [prior q (4), s (3), eps].
template <typename S>
void PriorRot3Residual(const S* x, const double* c, S* r) {
  const double qp_inv[4] = {-c[0], -c[1], -c[2], c[3]};
  S qe[4];
  QuatMul(qp_inv, x, qe);
  S w[3];
  QuatLog(qe, c[7], w);
  for (int i = 0; i < 3; ++i) r[i] = c[4 + i] * w[i];
}

// between_factor for Rot3 (symforce/codegen/geo_factors_codegen.py:53-71):
// diag(s) Log(a_T_b^-1 a^-1 b); consts [a_T_b q (4), s (3), eps].
template <typename S>
void BetweenRot3Residual(const S* a, const S* b, const double* c, S* r) {
  const S qa_inv[4] = {-a[0], -a[1], -a[2], a[3]};
  S q[4];
  QuatMul(qa_inv, b, q);
  const double qm_inv[4] = {-c[0], -c[1], -c[2], c[3]};
  S qe[4];
  QuatMul(qm_inv, q, qe);
  S w[3];
  QuatLog(qe, c[7], w);
  for (int i = 0; i < 3; ++i) r[i] = c[4 + i] * w[i];
}

// BarronNoiseModel.whiten of x - y (symforce/opt/noise_models.py:318-428) with delta 1,
// scalar_information 1, x_epsilon = alpha_epsilon = eps and alpha = 2 - 1 / (1 - mu + eps)
// (compute_alpha_from_mu): the factor of test/symforce_gnc_codegen_test.py:24-31;
// consts [y (5), mu, eps].
template <typename S>
void BarronVec5Residual(const S* x, const double* c, S* r) {
  const double mu = c[5], eps = c[6];
  const double alpha = 2.0 - 1.0 / (1.0 - mu + eps);
  const double b = std::fabs(alpha - 2.0) + eps;
  const double d = alpha + (alpha >= 0 ? eps : -eps);
  for (int i = 0; i < 5; ++i) {
    const S e = x[i] - c[i];
    const S barron = (b / d) * (pow(e * e / b + 1.0, d / 2.0) - 1.0);
    r[i] = sqrt(2.0 * barron + eps) - std::sqrt(eps);
  }
}

// r = J x + b (J rows x cols, row-major, then b) over the concatenated key storage.
template <typename S>
void LinearResidual(const S* x, const double* c, int rows, int cols, S* r) {
  for (int i = 0; i < rows; ++i) {
    S acc = S(c[rows * cols + i]);
    for (int j = 0; j < cols; ++j) acc = acc + c[i * cols + j] * x[j];
    r[i] = acc;
  }
}

}  // namespace oracle
