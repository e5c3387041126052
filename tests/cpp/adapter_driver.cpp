// Test driver of the C++ adapters (include/sfgpu_sym.h) over the stand-ins: compiled on the CPU by
// tests/test_library_cpu.py, compiled and run on a GPU by tests/test_gpu_cpp_adapters.py.
//
//  1. GpuSparseCholeskySolver as the LinearSolver concept: Factorize + Solve of a random sparse SPD
//     matrix stored lower (like hessian_lower), residual against the matrix, and L(), D() and
//     Permutation() reassembling P A P^T.
//  2. GpuSparseSchurSolver on a block system, residual.
//  3. GpuLevenbergMarquardtSolver driven the way sym::Optimizer drives its NonlinearSolverType
//     (Reset, then Iterate until a status, symforce/opt/internal/optimizer_utils.h:34-104) on the
//     reference's robot_2d example (symforce/examples/robot_2d_localization/run_localization.cc:
//     27-97): 9 records, initial error in (6.39635, 6.39637), best below 2.2003e-4, SUCCESS.
//  4. ComputeCovariance against the solve of the identity.
// Prints one line per check and returns nonzero on the first failure.
#include <cmath>
#include <cstdio>
#include <random>

#include "symforce_stand_ins.h"
#include "sfgpu_sym.h"

using SparseMat = Eigen::SparseMatrix<double>;

static int Fail(const char* what) {
  std::printf("FAIL %s\n", what);
  return 1;
}

// y = A x for A given by its lower triangle (compressed columns)
static std::vector<double> SymMul(const SparseMat& A, const std::vector<double>& x) {
  std::vector<double> y(x.size(), 0.0);
  for (int64_t c = 0; c < A.cols(); ++c)
    for (int q = A.outerIndexPtr()[c]; q < A.outerIndexPtr()[c + 1]; ++q) {
      const int r = A.innerIndexPtr()[q];
      const double v = A.valuePtr()[q];
      y[size_t(r)] += v * x[size_t(c)];
      if (r != c) y[size_t(c)] += v * x[size_t(r)];
    }
  return y;
}

static SparseMat RandomSpdLower(int n, uint32_t seed, std::vector<std::vector<double>>* dense) {
  std::mt19937 gen(seed);
  std::uniform_real_distribution<double> u(-1, 1);
  std::vector<std::vector<double>> D(size_t(n), std::vector<double>(size_t(n), 0.0));
  for (int k = 0; k < 4 * n; ++k) {
    const int i = int(gen() % n), j = int(gen() % n);
    const double v = u(gen);
    D[i][j] += v;
    D[j][i] += v;
  }
  for (int i = 0; i < n; ++i) D[i][i] = 20.0 + std::fabs(u(gen));
  std::vector<int> outer{0}, inner;
  std::vector<double> vals;
  for (int c = 0; c < n; ++c) {
    for (int r = c; r < n; ++r)
      if (D[r][c] != 0.0 || r == c) {
        inner.push_back(r);
        vals.push_back(D[r][c]);
      }
    outer.push_back(int(inner.size()));
  }
  SparseMat A;
  A.SetCsc(n, n, outer, inner, vals);
  if (dense) *dense = D;
  return A;
}

int main() {
  // ---- 1. LinearSolver concept
  {
    const int n = 60;
    std::vector<std::vector<double>> D;
    SparseMat A = RandomSpdLower(n, 7, &D);
    sfgpu::GpuSparseCholeskySolver<SparseMat> solver;
    solver.AnalyzeSparsityPattern(A);
    if (!solver.Factorize(A)) return Fail("factorize");
    Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic> b(n, 3);
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < n; ++r) b(r, c) = std::sin(0.3 * r + c);
    auto x = solver.Solve(b);
    double rmax = 0;
    for (int c = 0; c < 3; ++c) {
      std::vector<double> xc(n);
      for (int r = 0; r < n; ++r) xc[r] = x(r, c);
      auto y = SymMul(A, xc);
      for (int r = 0; r < n; ++r) rmax = std::fmax(rmax, std::fabs(y[r] - b(r, c)));
    }
    std::printf("linear_solver residual %.3e\n", rmax);
    if (!(rmax < 1e-10)) return Fail("linear solver residual");
    // (I + L) D (I + L)^T == P A P^T
    const auto& L = solver.L();
    const auto& d = solver.D();
    const auto& P = solver.Permutation();
    std::vector<std::vector<double>> Lf(n, std::vector<double>(n, 0.0));
    for (int i = 0; i < n; ++i) Lf[i][i] = 1.0;
    for (int c = 0; c < n; ++c)
      for (int q = L.outerIndexPtr()[c]; q < L.outerIndexPtr()[c + 1]; ++q) {
        if (L.innerIndexPtr()[q] <= c) return Fail("L not strictly lower");
        Lf[L.innerIndexPtr()[q]][c] = L.valuePtr()[q];
      }
    // (P A P^T)(P[a], P[b]) = A(a, b)
    double emax2 = 0;
    for (int a = 0; a < n; ++a)
      for (int bb = 0; bb < n; ++bb) {
        const int i = P.indices()[a], j = P.indices()[bb];
        double s = 0;
        for (int k = 0; k < n; ++k) s += Lf[i][k] * d(k) * Lf[j][k];
        emax2 = std::fmax(emax2, std::fabs(s - D[a][bb]));
      }
    std::printf("linear_solver LDLT reconstruction %.3e\n", emax2);
    if (!(emax2 < 1e-10)) return Fail("L D L^T != P A P^T");
  }
  // ---- 2. Schur solver: B (6 unknowns) coupled to two 3x3 point blocks
  {
    const int nb = 6, n = 12;
    std::vector<std::vector<double>> D(n, std::vector<double>(n, 0.0));
    std::mt19937 gen(3);
    std::uniform_real_distribution<double> u(-1, 1);
    for (int i = 0; i < n; ++i) D[i][i] = 10.0;
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < i; ++j) D[i][j] = D[j][i] = 0.5 * u(gen);
    for (int p = 0; p < 2; ++p)
      for (int a = 0; a < 3; ++a) {
        for (int bb = 0; bb < a; ++bb) D[nb + 3 * p + a][nb + 3 * p + bb] = D[nb + 3 * p + bb][nb + 3 * p + a] = 0.3 * u(gen);
        for (int i = 0; i < nb; ++i) D[nb + 3 * p + a][i] = D[i][nb + 3 * p + a] = 0.4 * u(gen);
      }
    std::vector<int> outer{0}, inner;
    std::vector<double> vals;
    for (int c = 0; c < n; ++c) {
      for (int r = c; r < n; ++r)
        if (D[r][c] != 0.0) {
          inner.push_back(r);
          vals.push_back(D[r][c]);
        }
      outer.push_back(int(inner.size()));
    }
    SparseMat A;
    A.SetCsc(n, n, outer, inner, vals);
    sfgpu::GpuSparseSchurSolver<SparseMat> schur;
    schur.ComputeSymbolicSparsity(A, n - nb);
    schur.Factorize(A);
    Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic> rhs(n, 1);
    for (int r = 0; r < n; ++r) rhs(r, 0) = std::cos(r);
    auto x = schur.Solve(rhs);
    std::vector<double> xv(n);
    for (int r = 0; r < n; ++r) xv[r] = x(r, 0);
    auto y = SymMul(A, xv);
    double rmax = 0;
    for (int r = 0; r < n; ++r) rmax = std::fmax(rmax, std::fabs(y[r] - rhs(r, 0)));
    std::printf("schur residual %.3e\n", rmax);
    if (!(rmax < 1e-10)) return Fail("schur residual");
  }
  // ---- 3. NonlinearSolverType on the robot_2d example
  {
    const double landmarks[3][2] = {{-2, 2}, {1, -3}, {5, 2}};
    const double distances[2] = {1.7, 1.4};
    const double angles[3][3] = {{55, 245, -35}, {95, 220, -20}, {125, 220, -20}};
    const double eps = 10 * 2.220446049250313e-16;
    std::vector<int32_t> bkeys, okeys;
    std::vector<double> bconsts, oconsts;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        bkeys.push_back(i);
        for (double v : {landmarks[j][0], landmarks[j][1], angles[i][j] * M_PI / 180, eps, 1.0}) bconsts.push_back(v);
      }
    for (int i = 0; i < 2; ++i) {
      okeys.push_back(i);
      okeys.push_back(i + 1);
      for (double v : {distances[i], eps, 1.0}) oconsts.push_back(v);
    }
    const int32_t key_types[3] = {SFG_KEY_POSE2, SFG_KEY_POSE2, SFG_KEY_POSE2};
    sfg_factor_batch_t batches[2] = {{SFG_FACTOR_BEARING_POSE2, 9, bkeys.data(), bconsts.data()},
                                     {SFG_FACTOR_ODOMETRY_POSE2, 2, okeys.data(), oconsts.data()}};
    sfg_problem_t problem{3, key_types, 2, batches, 0};
    sfg_form_params_t form;
    sfg_default_form_params(&form);
    sym::optimizer_params_t params;  // DefaultOptimizerParams
    sfgpu::GpuLevenbergMarquardtSolver<double> solver(params, "robot_2d", eps, problem, form);
    // Values: a leading non-optimized scalar, then the three poses (identity); the index names
    // the poses' storage
    sym::Values<double> values;
    values.Data() = {42.0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    sym::index_t index;
    for (int i = 0; i < 3; ++i) index.entries.push_back({1 + 4 * i, 4, 3});
    solver.SetIndex(index);
    // OptimizeImpl / IterateToConvergenceImpl (symforce/opt/internal/optimizer_utils.h:34-104)
    sym::OptimizationStats<SparseMat> stats;
    solver.Reset(values);
    const int num_iterations = params.iterations;
    int i = 0;
    for (; i < num_iterations; ++i) {
      const auto st = solver.Iterate({}, stats);
      if (st) {
        stats.status = st->first;
        stats.failure_reason = st->second.int_value();
        break;
      }
    }
    if (i == num_iterations) stats.status = sym::optimization_status_t::from_int(SFG_STATUS_HIT_ITERATION_LIMIT);
    values = solver.GetBestValues();
    const double first = stats.iterations.front().new_error;
    const double best = stats.iterations[size_t(stats.best_index)].new_error;
    std::printf("nonlinear_solver records %zu first %.15g best %.6e status %d\n", stats.iterations.size(), first,
                best, stats.status.int_value());
    if (stats.iterations.size() != 9) return Fail("robot_2d records");
    if (!(first > 6.39635 && first < 6.39637)) return Fail("robot_2d initial error");
    if (!(best < 2.2003e-4)) return Fail("robot_2d best error");
    if (stats.status.int_value() != SFG_STATUS_SUCCESS) return Fail("robot_2d status");
    if (values.Data()[0] != 42.0) return Fail("non-optimized entry changed");
    const double pose0[4] = {0.477063, 0.878869, -0.583038, -0.824491};
    for (int k = 0; k < 4; ++k)
      if (std::fabs(values.Data()[1 + k] - pose0[k]) > 1e-6) return Fail("robot_2d pose 0");
    const auto& lin = solver.GetBestLinearization();
    double err = 0;
    for (int64_t r = 0; r < lin.residual.rows(); ++r) err += 0.5 * lin.residual(r) * lin.residual(r);
    std::printf("best linearization error %.6e rows %lld hessian nnz %lld\n", err, (long long)lin.residual.rows(),
                (long long)lin.hessian_lower.nonZeros());
    if (std::fabs(err - best) > 1e-12 * std::fmax(1.0, best)) return Fail("best linearization error");
    // 4. ComputeCovariance: covariance * H == I
    Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic> cov;
    solver.ComputeCovariance(lin.hessian_lower, cov);
    double cmax = 0;
    const int64_t n = lin.hessian_lower.rows();
    for (int64_t c = 0; c < n; ++c) {
      std::vector<double> col(static_cast<size_t>(n));
      for (int64_t r = 0; r < n; ++r) col[size_t(r)] = cov(r, c);
      auto y = SymMul(lin.hessian_lower, col);
      for (int64_t r = 0; r < n; ++r) cmax = std::fmax(cmax, std::fabs(y[size_t(r)] - (r == c ? 1.0 : 0.0)));
    }
    std::printf("covariance H residual %.3e\n", cmax);
    if (!(cmax < 1e-8)) return Fail("covariance");
  }
  std::printf("ALL OK\n");
  return 0;
}
