/*
 * sfgpu_sym.h - C++ adapters that plug the GB300 back end (sfgpu.h) into SymForce's template plug
 * points, header-only, over the C ABI:
 *
 *   sfgpu::GpuSparseCholeskySolver<MatrixType>   the LinearSolver concept of
 *       sym::LevenbergMarquardtSolver<Scalar, LinearSolverType> (used at
 *       symforce/opt/levenberg_marquardt_solver.tcc:191, 202, 210-211, 217, 351-355; the interface of
 *       symforce/opt/sparse_cholesky/sparse_cholesky_solver.h:28-163): AnalyzeSparsityPattern,
 *       Factorize, Solve, SolveInPlace, L(), D(), Permutation().  The factorization and solves run on
 *       the GPU; the linearization stays the caller's (any sym::Factor).
 *
 *       sym::LevenbergMarquardtSolver<double, sfgpu::GpuSparseCholeskySolver<Eigen::SparseMatrix<double>>>
 *
 *   sfgpu::GpuSparseSchurSolver<MatrixType>      SparseSchurSolver (symforce/opt/sparse_schur_solver.h:
 *       62-135): ComputeSymbolicSparsity(A, C_dim), Factorize(A), Solve(rhs).
 *
 *   sfgpu::GpuLevenbergMarquardtSolver<Scalar>   the NonlinearSolverType of
 *       sym::Optimizer<Scalar, NonlinearSolverType> (symforce/opt/optimizer.h:72-111, the interface of
 *       symforce/opt/levenberg_marquardt_solver.h:131-215).  The whole Levenberg-Marquardt loop runs
 *       on the device over typed factor batches (sfg_problem_t), which the Optimizer forwards to the
 *       solver's constructor as its extra arguments:
 *
 *       sym::Optimizer<double, sfgpu::GpuLevenbergMarquardtSolver<double>> opt(
 *           params, factors, "gpu", keys, epsilon, problem, form);
 *
 *       The device kernels evaluate the typed batches, not the sym::Factor std::functions (a GPU
 *       cannot call those), so `problem` must describe the same factors; Iterate ignores the
 *       LinearizeFunc.  The first Iterate after Reset runs the whole loop (params.iterations) and
 *       appends every record; later Iterates of that run return without work.
 *
 * Include this header after the Eigen and SymForce headers (it names Eigen::SparseMatrix,
 * Eigen::Matrix, Eigen::PermutationMatrix, Eigen::Map, sym::Values, sym::index_t, sym::Linearization,
 * sym::OptimizationStats, sym::optimizer_params_t and the LCM enums, and includes none of them).
 * Errors of the C ABI are rethrown as std::runtime_error, where the reference asserts
 * (symforce/opt/assert.h:41-47).
 */
#ifndef SFGPU_SYM_H_
#define SFGPU_SYM_H_

#include <cstdint>
#include <functional>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "sfgpu.h"

namespace sfgpu {

inline void Check(int32_t rc, const char* what) {
  if (rc != SFG_OK)
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " + sfg_last_error());
}

// Lower-triangle compressed columns of a column-major sparse matrix (only entries with row >= col;
// a full symmetric matrix gives its lower half).  `src` maps every kept entry to its position in
// the matrix's value array, so later value arrays of the same pattern are gathered without search.
template <typename MatrixType>
void LowerPattern(const MatrixType& A, std::vector<int32_t>& col_ptr, std::vector<int32_t>& row_idx,
                  std::vector<int64_t>& src) {
  const int64_t n = A.cols();
  const auto* outer = A.outerIndexPtr();
  const auto* inner = A.innerIndexPtr();
  const auto* nnz = A.innerNonZeroPtr();  // null when compressed
  col_ptr.assign(static_cast<size_t>(n) + 1, 0);
  row_idx.clear();
  src.clear();
  for (int64_t c = 0; c < n; ++c) {
    const int64_t b = outer[c], e = nnz ? outer[c] + nnz[c] : outer[c + 1];
    for (int64_t q = b; q < e; ++q)
      if (inner[q] >= c) {
        row_idx.push_back(int32_t(inner[q]));
        src.push_back(q);
      }
    col_ptr[static_cast<size_t>(c) + 1] = int32_t(row_idx.size());
  }
}

// ---------------------------------------------------------------------------------------------
// SparseCholeskySolver on the GPU (LDL^T, unit L, no pivoting; block ordering of the library).
// ---------------------------------------------------------------------------------------------
template <typename _MatrixType>
class GpuSparseCholeskySolver {
 public:
  using MatrixType = _MatrixType;
  using Scalar = typename MatrixType::Scalar;
  using StorageIndex = typename MatrixType::StorageIndex;
  using CholMatrixType = Eigen::SparseMatrix<Scalar, Eigen::ColMajor, StorageIndex>;
  using VectorType = Eigen::Matrix<Scalar, Eigen::Dynamic, 1>;
  using RhsType = Eigen::Matrix<Scalar, Eigen::Dynamic, Eigen::Dynamic>;
  using PermutationMatrixType = Eigen::PermutationMatrix<Eigen::Dynamic, Eigen::Dynamic, StorageIndex>;

  explicit GpuSparseCholeskySolver(int32_t ordering = SFG_ORDERING_NESTED_DISSECTION, int32_t device = 0)
      : ordering_(ordering), device_(device) {}
  GpuSparseCholeskySolver(const GpuSparseCholeskySolver& o) : ordering_(o.ordering_), device_(o.device_) {}
  GpuSparseCholeskySolver& operator=(const GpuSparseCholeskySolver& o) {
    if (this != &o) {
      Release();
      ordering_ = o.ordering_;
      device_ = o.device_;
    }
    return *this;
  }
  ~GpuSparseCholeskySolver() { Release(); }

  bool IsInitialized() const { return handle_ != nullptr && factored_; }

  // ComputeSymbolicSparsity on the lower triangle of A (symforce/opt/sparse_cholesky/
  // sparse_cholesky_solver.tcc:26-106): the ordering, elimination tree and supernodes, on the host.
  void ComputeSymbolicSparsity(const MatrixType& A) {
    Release();
    LowerPattern(A, col_ptr_, row_idx_, src_);
    n_ = int32_t(A.cols());
    Check(sfg_ldlt_create(n_, col_ptr_.data(), row_idx_.data(), ordering_, device_, &handle_),
          "sfg_ldlt_create");
  }
  void AnalyzeSparsityPattern(const MatrixType& A) { ComputeSymbolicSparsity(A); }

  // Numeric factorization of A (same pattern as analyzed) on the GPU.
  bool Factorize(const MatrixType& A) {
    if (!handle_) ComputeSymbolicSparsity(A);
    vals_.resize(src_.size());
    const Scalar* v = A.valuePtr();
    for (size_t q = 0; q < src_.size(); ++q) vals_[q] = double(v[src_[q]]);
    Check(sfg_ldlt_factorize(handle_, vals_.data()), "sfg_ldlt_factorize");
    factored_ = true;
    have_factors_ = false;
    return true;
  }

  template <typename Rhs>
  RhsType Solve(const Rhs& b) const {
    RhsType x(b.rows(), b.cols());
    for (int64_t c = 0; c < int64_t(b.cols()); ++c)
      for (int64_t r = 0; r < int64_t(b.rows()); ++r) x(r, c) = b(r, c);
    SolveInPlace(x);
    return x;
  }

  template <typename Rhs>
  void SolveInPlace(Rhs& b) const {
    if (!factored_) throw std::runtime_error("GpuSparseCholeskySolver: Factorize first");
    const int64_t n = b.rows(), k = b.cols();
    std::vector<double> in(static_cast<size_t>(n * k)), out(static_cast<size_t>(n * k));
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < n; ++r) in[static_cast<size_t>(c * n + r)] = double(b(r, c));
    Check(sfg_ldlt_solve(handle_, in.data(), out.data(), int32_t(k)), "sfg_ldlt_solve");
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < n; ++r) b(r, c) = Scalar(out[static_cast<size_t>(c * n + r)]);
  }

  // L (unit lower, strictly lower part stored), D and the permutation (new index of old index i)
  // of the last factorization, copied back from the device on first use.
  const CholMatrixType& L() const {
    Fetch();
    return L_;
  }
  const VectorType& D() const {
    Fetch();
    return D_;
  }
  const PermutationMatrixType& Permutation() const {
    Fetch();
    return perm_;
  }

 private:
  void Release() {
    if (handle_) sfg_ldlt_destroy(handle_);
    handle_ = nullptr;
    factored_ = false;
    have_factors_ = false;
  }
  void Fetch() const {
    if (!factored_) throw std::runtime_error("GpuSparseCholeskySolver: Factorize first");
    if (have_factors_) return;
    int64_t nnz = 0;
    Check(sfg_ldlt_lower(handle_, &nnz, nullptr, nullptr, nullptr), "sfg_ldlt_lower");
    std::vector<int32_t> cp(static_cast<size_t>(n_) + 1), ri(static_cast<size_t>(nnz));
    std::vector<double> lv(static_cast<size_t>(nnz));
    Check(sfg_ldlt_lower(handle_, &nnz, cp.data(), ri.data(), lv.data()), "sfg_ldlt_lower");
    std::vector<StorageIndex> outer(cp.begin(), cp.end()), inner(ri.begin(), ri.end());
    std::vector<Scalar> vals(lv.begin(), lv.end());
    L_ = Eigen::Map<const CholMatrixType>(n_, n_, StorageIndex(nnz), outer.data(), inner.data(), vals.data());
    std::vector<double> d(static_cast<size_t>(n_));
    Check(sfg_ldlt_diagonal(handle_, d.data()), "sfg_ldlt_diagonal");
    D_.resize(n_);
    for (int32_t i = 0; i < n_; ++i) D_(i) = Scalar(d[static_cast<size_t>(i)]);
    std::vector<int32_t> p(static_cast<size_t>(n_));
    Check(sfg_ldlt_permutation(handle_, p.data()), "sfg_ldlt_permutation");
    perm_.resize(n_);
    for (int32_t i = 0; i < n_; ++i) perm_.indices()[i] = StorageIndex(p[static_cast<size_t>(i)]);
    have_factors_ = true;
  }

  int32_t ordering_, device_;
  int32_t n_ = 0;
  sfg_ldlt* handle_ = nullptr;
  bool factored_ = false;
  std::vector<int32_t> col_ptr_, row_idx_;
  std::vector<int64_t> src_;
  std::vector<double> vals_;
  mutable bool have_factors_ = false;
  mutable CholMatrixType L_;
  mutable VectorType D_;
  mutable PermutationMatrixType perm_;
};

// ---------------------------------------------------------------------------------------------
// SparseSchurSolver on the GPU: A = [[B, E^T], [E, C]] with C 3 x 3 block diagonal.
// ---------------------------------------------------------------------------------------------
template <typename _MatrixType>
class GpuSparseSchurSolver {
 public:
  using MatrixType = _MatrixType;
  using Scalar = typename MatrixType::Scalar;
  using MatrixX = Eigen::Matrix<Scalar, Eigen::Dynamic, Eigen::Dynamic>;

  explicit GpuSparseSchurSolver(int32_t device = 0) : device_(device) {}
  GpuSparseSchurSolver(const GpuSparseSchurSolver&) = delete;
  GpuSparseSchurSolver& operator=(const GpuSparseSchurSolver&) = delete;
  ~GpuSparseSchurSolver() {
    if (handle_) sfg_schur_destroy(handle_);
  }

  bool IsInitialized() const { return handle_ != nullptr; }

  void ComputeSymbolicSparsity(const MatrixType& A, int C_dim) {
    if (handle_) sfg_schur_destroy(handle_);
    handle_ = nullptr;
    LowerPattern(A, col_ptr_, row_idx_, src_);
    n_ = int32_t(A.cols());
    Check(sfg_schur_create(n_, col_ptr_.data(), row_idx_.data(), C_dim, device_, &handle_),
          "sfg_schur_create");
  }

  void Factorize(const MatrixType& A) {
    std::vector<double> v(src_.size());
    for (size_t q = 0; q < src_.size(); ++q) v[q] = double(A.valuePtr()[src_[q]]);
    Check(sfg_schur_factorize(handle_, v.data()), "sfg_schur_factorize");
  }

  template <typename RhsType>
  MatrixX Solve(const RhsType& rhs) const {
    const int64_t n = rhs.rows(), k = rhs.cols();
    std::vector<double> in(static_cast<size_t>(n * k)), out(static_cast<size_t>(n * k));
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < n; ++r) in[static_cast<size_t>(c * n + r)] = double(rhs(r, c));
    Check(sfg_schur_solve(handle_, in.data(), out.data(), int32_t(k)), "sfg_schur_solve");
    MatrixX x(n, k);
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < n; ++r) x(r, c) = Scalar(out[static_cast<size_t>(c * n + r)]);
    return x;
  }

 private:
  int32_t device_;
  int32_t n_ = 0;
  sfg_schur* handle_ = nullptr;
  std::vector<int32_t> col_ptr_, row_idx_;
  std::vector<int64_t> src_;
};

// ---------------------------------------------------------------------------------------------
// NonlinearSolverType for sym::Optimizer: the Levenberg-Marquardt loop on the device.
// ---------------------------------------------------------------------------------------------
template <typename ScalarType>
class GpuLevenbergMarquardtSolver {
 public:
  using Scalar = ScalarType;
  using MatrixType = Eigen::SparseMatrix<Scalar>;
  using LinearSolverType = GpuSparseCholeskySolver<MatrixType>;
  using ValuesType = sym::Values<Scalar>;
  using LinearizationType = sym::Linearization<MatrixType>;
  using FailureReason = sym::levenberg_marquardt_solver_failure_reason_t;
  using LinearizeFunc = std::function<void(const ValuesType&, LinearizationType&)>;

  // `problem`: the typed factor batches over the optimized keys in index order (the order of
  // sym::Values::CreateIndex(keys)); `form`: precision / linear solver of the device loop.  The
  // problem's arrays are copied by sfg_create.
  GpuLevenbergMarquardtSolver(const sym::optimizer_params_t& p, const std::string& id, const Scalar epsilon,
                              const sfg_problem_t& problem, sfg_form_params_t form)
      : p_(p), id_(id) {
    form.epsilon = double(epsilon);
    Check(sfg_create(&problem, &form, &handle_), "sfg_create");
    int64_t s = 0, n = 0, m = 0;
    Check(sfg_storage_dim(handle_, &s, &n, &m), "sfg_storage_dim");
    storage_.resize(static_cast<size_t>(s));
  }
  GpuLevenbergMarquardtSolver(const GpuLevenbergMarquardtSolver&) = delete;
  GpuLevenbergMarquardtSolver& operator=(const GpuLevenbergMarquardtSolver&) = delete;
  ~GpuLevenbergMarquardtSolver() {
    if (handle_) sfg_destroy(handle_);
  }

  // The optimized entries of the Values, in order (symforce/opt/levenberg_marquardt_solver.h:158-160).
  void SetIndex(const sym::index_t& index) {
    entries_.clear();
    int64_t total = 0;
    for (const auto& e : index.entries) {
      entries_.push_back({int64_t(e.offset), int64_t(e.storage_dim)});
      total += e.storage_dim;
    }
    if (total != int64_t(storage_.size()))
      throw std::runtime_error("GpuLevenbergMarquardtSolver: index storage does not match the problem's keys");
  }

  // Reset / ResetState (levenberg_marquardt_solver.h:163-183): the next Iterate starts a new run.
  void Reset(const ValuesType& values) {
    best_ = values;
    Gather(values);
    Check(sfg_set_values(handle_, storage_.data(), int64_t(storage_.size())), "sfg_set_values");
    ran_ = false;
    continue_ = false;
  }
  void ResetState(const ValuesType& values) {
    Reset(values);
    continue_ = started_;
  }
  void RelaxDampingToInitial() { relax_ = true; }

  const sym::optimizer_params_t& Params() const { return p_; }
  void UpdateParams(const sym::optimizer_params_t& p) { p_ = p; }

  // The first call after Reset runs the device loop for Params().iterations and appends its records;
  // it returns the final status unless the loop ended on the iteration limit, which the caller's
  // loop reports itself (symforce/opt/internal/optimizer_utils.h:43-64).
  std::optional<std::pair<sym::optimization_status_t, FailureReason>> Iterate(
      const LinearizeFunc& /*func*/, sym::OptimizationStats<MatrixType>& stats) {
    if (ran_) return {};
    sfg_optimizer_params_t dp;
    ToDevice(p_, &dp);
    std::vector<sfg_iteration_t> recs(static_cast<size_t>(dp.iterations) + 1);
    sfg_stats_t st{recs.data(), int32_t(recs.size()), 0, 0, 0, 0, 0, 0.0};
    if (continue_) {
      Check(sfg_optimize_continue(handle_, &dp, -1, relax_ ? 1 : 0, &st), "sfg_optimize_continue");
    } else {
      Check(sfg_optimize(handle_, &dp, -1, &st), "sfg_optimize");
    }
    relax_ = false;
    ran_ = true;
    started_ = true;
    const size_t base = stats.iterations.size();
    for (int32_t i = 0; i < st.num_iterations; ++i) {
      const sfg_iteration_t& r = recs[static_cast<size_t>(i)];
      stats.iterations.emplace_back();
      auto& o = stats.iterations.back();
      o.iteration = int16_t(r.iteration);
      o.current_lambda = r.current_lambda;
      o.new_error = r.new_error;
      o.new_error_linear = r.new_error_linear;
      o.relative_reduction = r.relative_reduction;
      o.update_angle_change = r.update_angle_change;
      o.update_accepted = r.update_accepted != 0;
    }
    if (st.best_index >= 0) stats.best_index = int32_t(base) + st.best_index;
    if (p_.debug_stats) FillDebugStats(stats);
    Check(sfg_get_values(handle_, storage_.data(), int64_t(storage_.size())), "sfg_get_values");
    Scatter(best_);
    if (st.status == SFG_STATUS_HIT_ITERATION_LIMIT) return {};
    return {{sym::optimization_status_t::from_int(st.status), FailureReason::from_int(st.failure_reason)}};
  }

  const ValuesType& GetBestValues() const { return best_; }

  // The linearization at the best values (the reference keeps the Best state block's; the device
  // relinearizes there, which gives the same numbers).
  const LinearizationType& GetBestLinearization() const {
    const int64_t m = ResidualDim(), n = TangentDim();
    std::vector<double> res(static_cast<size_t>(m)), rhs(static_cast<size_t>(n));
    double err = 0;
    Check(sfg_set_values(handle_, storage_.data(), int64_t(storage_.size())), "sfg_set_values");
    Check(sfg_linearize(handle_, res.data(), rhs.data(), &err), "sfg_linearize");
    int64_t nnz = 0;
    Check(sfg_hessian_lower(handle_, &nnz, nullptr, nullptr, nullptr), "sfg_hessian_lower");
    std::vector<int32_t> cp(static_cast<size_t>(n) + 1), ri(static_cast<size_t>(nnz));
    std::vector<double> hv(static_cast<size_t>(nnz));
    Check(sfg_hessian_lower(handle_, &nnz, cp.data(), ri.data(), hv.data()), "sfg_hessian_lower");
    best_lin_.residual.resize(m);
    for (int64_t i = 0; i < m; ++i) best_lin_.residual(i) = Scalar(res[static_cast<size_t>(i)]);
    best_lin_.rhs.resize(n);
    for (int64_t i = 0; i < n; ++i) best_lin_.rhs(i) = Scalar(rhs[static_cast<size_t>(i)]);
    std::vector<typename MatrixType::StorageIndex> outer(cp.begin(), cp.end()), inner(ri.begin(), ri.end());
    std::vector<Scalar> vals(hv.begin(), hv.end());
    best_lin_.hessian_lower = Eigen::Map<const MatrixType>(n, n, nnz, outer.data(), inner.data(), vals.data());
    best_lin_.SetInitialized(true);
    return best_lin_;
  }

  // ComputeCovariance (symforce/opt/levenberg_marquardt_solver.tcc:344-355) with the GPU LDL^T.
  void ComputeCovariance(const MatrixType& hessian_lower, Eigen::Matrix<Scalar, Eigen::Dynamic, Eigen::Dynamic>& covariance) {
    LinearSolverType solver;
    solver.ComputeSymbolicSparsity(hessian_lower);
    solver.Factorize(hessian_lower);
    const int64_t n = hessian_lower.rows();
    covariance = Eigen::Matrix<Scalar, Eigen::Dynamic, Eigen::Dynamic>::Identity(n, n);
    solver.SolveInPlace(covariance);
  }

  sfg_handle* Handle() const { return handle_; }

 private:
  struct Entry {
    int64_t offset, size;
  };
  int64_t ResidualDim() const {
    int64_t s, n, m;
    Check(sfg_storage_dim(handle_, &s, &n, &m), "sfg_storage_dim");
    return m;
  }
  int64_t TangentDim() const {
    int64_t s, n, m;
    Check(sfg_storage_dim(handle_, &s, &n, &m), "sfg_storage_dim");
    return n;
  }
  void Gather(const ValuesType& values) {
    const auto& data = values.Data();
    size_t q = 0;
    for (const Entry& e : entries_)
      for (int64_t i = 0; i < e.size; ++i) storage_[q++] = double(data[static_cast<size_t>(e.offset + i)]);
  }
  void Scatter(ValuesType& values) const {
    Scalar* data = values.DataPointer();
    size_t q = 0;
    for (const Entry& e : entries_)
      for (int64_t i = 0; i < e.size; ++i) data[e.offset + i] = Scalar(storage_[q++]);
  }
  void FillDebugStats(sym::OptimizationStats<MatrixType>& stats) const {
    const int64_t n = TangentDim();
    std::vector<int32_t> perm(static_cast<size_t>(n));
    if (sfg_permutation(handle_, perm.data(), n) == SFG_OK) {
      stats.linear_solver_ordering.resize(n);
      for (int64_t i = 0; i < n; ++i) stats.linear_solver_ordering(i) = perm[static_cast<size_t>(i)];
    }
    int64_t nnz = 0;
    if (sfg_factor_lower(handle_, &nnz, nullptr, nullptr, nullptr) == SFG_OK) {
      std::vector<int32_t> cp(static_cast<size_t>(n) + 1), ri(static_cast<size_t>(nnz));
      Check(sfg_factor_lower(handle_, &nnz, cp.data(), ri.data(), nullptr), "sfg_factor_lower");
      stats.cholesky_factor_sparsity.row_indices.assign(ri.begin(), ri.end());
      stats.cholesky_factor_sparsity.column_pointers.assign(cp.begin(), cp.end());
      stats.cholesky_factor_sparsity.shape = {int32_t(n), int32_t(n)};
    }
  }
  static void ToDevice(const sym::optimizer_params_t& p, sfg_optimizer_params_t* o) {
    sfg_default_optimizer_params(o);
    o->verbose = p.verbose;
    o->debug_stats = p.debug_stats;
    o->check_derivatives = p.check_derivatives;
    o->include_jacobians = p.include_jacobians;
    o->debug_checks = p.debug_checks;
    o->initial_lambda = p.initial_lambda;
    o->lambda_lower_bound = p.lambda_lower_bound;
    o->lambda_upper_bound = p.lambda_upper_bound;
    o->lambda_update_type = int32_t(p.lambda_update_type.int_value());
    o->lambda_up_factor = p.lambda_up_factor;
    o->lambda_down_factor = p.lambda_down_factor;
    o->dynamic_lambda_update_beta = p.dynamic_lambda_update_beta;
    o->dynamic_lambda_update_gamma = p.dynamic_lambda_update_gamma;
    o->dynamic_lambda_update_p = p.dynamic_lambda_update_p;
    o->use_diagonal_damping = p.use_diagonal_damping;
    o->use_unit_damping = p.use_unit_damping;
    o->keep_max_diagonal_damping = p.keep_max_diagonal_damping;
    o->diagonal_damping_min = p.diagonal_damping_min;
    o->iterations = p.iterations;
    o->early_exit_min_reduction = p.early_exit_min_reduction;
    o->early_exit_min_absolute_error = p.early_exit_min_absolute_error;
    o->enable_bold_updates = p.enable_bold_updates;
  }

  sym::optimizer_params_t p_;
  std::string id_;
  sfg_handle* handle_ = nullptr;
  std::vector<double> storage_;
  std::vector<Entry> entries_;
  ValuesType best_;
  mutable LinearizationType best_lin_;
  bool ran_ = false, continue_ = false, started_ = false, relax_ = false;
};

}  // namespace sfgpu

#endif  // SFGPU_SYM_H_
