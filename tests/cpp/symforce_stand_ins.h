// Test infrastructure: minimal stand-ins for the parts of Eigen and SymForce that
// include/sfgpu_sym.h names (neither library is installed here).  They follow the real types'
// interfaces for the members the adapters use (Eigen::SparseMatrix compressed-column storage and
// Map construction, dense column-major matrices, PermutationMatrix::indices; sym::Values storage,
// sym::index_t entries, sym::Linearization, sym::OptimizationStats and the LCM enum helpers) and
// nothing else.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace Eigen {
constexpr int Dynamic = -1;
enum { ColMajor = 0 };

template <typename ScalarT, int Rows, int Cols>
class Matrix {
 public:
  using Scalar = ScalarT;
  Matrix() = default;
  explicit Matrix(int64_t n) { resize(n); }
  Matrix(int64_t r, int64_t c) { resize(r, c); }
  void resize(int64_t n) { resize(n, 1); }
  void resize(int64_t r, int64_t c) {
    r_ = r;
    c_ = c;
    d_.assign(size_t(r * c), Scalar(0));
  }
  int64_t rows() const { return r_; }
  int64_t cols() const { return c_; }
  Scalar& operator()(int64_t i, int64_t j) { return d_[size_t(j * r_ + i)]; }
  const Scalar& operator()(int64_t i, int64_t j) const { return d_[size_t(j * r_ + i)]; }
  Scalar& operator()(int64_t i) { return d_[size_t(i)]; }
  const Scalar& operator()(int64_t i) const { return d_[size_t(i)]; }
  Scalar* data() { return d_.data(); }
  static Matrix Identity(int64_t r, int64_t c) {
    Matrix m(r, c);
    for (int64_t i = 0; i < r && i < c; ++i) m(i, i) = Scalar(1);
    return m;
  }

 private:
  int64_t r_ = 0, c_ = 0;
  std::vector<Scalar> d_;
};
using VectorXi = Matrix<int, Dynamic, 1>;

template <typename T>
class Map;

template <typename ScalarT, int Options = 0, typename StorageIndexT = int>
class SparseMatrix {
 public:
  using Scalar = ScalarT;
  using StorageIndex = StorageIndexT;
  SparseMatrix() = default;
  SparseMatrix(int64_t r, int64_t c) : r_(r), c_(c), outer_(size_t(c) + 1, 0) {}
  SparseMatrix& operator=(const Map<const SparseMatrix>& m);
  int64_t rows() const { return r_; }
  int64_t cols() const { return c_; }
  int64_t nonZeros() const { return int64_t(inner_.size()); }
  const StorageIndex* outerIndexPtr() const { return outer_.data(); }
  const StorageIndex* innerIndexPtr() const { return inner_.data(); }
  const StorageIndex* innerNonZeroPtr() const { return nullptr; }
  const Scalar* valuePtr() const { return vals_.data(); }
  Scalar* valuePtr() { return vals_.data(); }
  // test helper: build from compressed columns
  void SetCsc(int64_t r, int64_t c, std::vector<StorageIndex> outer, std::vector<StorageIndex> inner,
              std::vector<Scalar> vals) {
    r_ = r;
    c_ = c;
    outer_ = std::move(outer);
    inner_ = std::move(inner);
    vals_ = std::move(vals);
  }

 private:
  int64_t r_ = 0, c_ = 0;
  std::vector<StorageIndex> outer_{0}, inner_;
  std::vector<Scalar> vals_;
};

template <typename ScalarT, int Options, typename StorageIndexT>
class Map<const SparseMatrix<ScalarT, Options, StorageIndexT>> {
 public:
  Map(int64_t r, int64_t c, int64_t nnz, const StorageIndexT* outer, const StorageIndexT* inner,
      const ScalarT* vals)
      : r(r), c(c), outer(outer, outer + c + 1), inner(inner, inner + nnz), vals(vals, vals + nnz) {}
  int64_t r, c;
  std::vector<StorageIndexT> outer, inner;
  std::vector<ScalarT> vals;
};

template <typename S, int O, typename I>
SparseMatrix<S, O, I>& SparseMatrix<S, O, I>::operator=(const Map<const SparseMatrix<S, O, I>>& m) {
  SetCsc(m.r, m.c, m.outer, m.inner, m.vals);
  return *this;
}

template <int Size, int MaxSize, typename StorageIndex>
class PermutationMatrix {
 public:
  void resize(int64_t n) { idx_.assign(size_t(n), 0); }
  std::vector<StorageIndex>& indices() { return idx_; }
  const std::vector<StorageIndex>& indices() const { return idx_; }

 private:
  std::vector<StorageIndex> idx_;
};
}  // namespace Eigen

namespace sym {
// LCM enums: from_int / int_value, compared by value
#define SFGPU_STAND_IN_ENUM(NAME)                                      \
  struct NAME {                                                        \
    int32_t v = 0;                                                     \
    static NAME from_int(int32_t x) { return NAME{x}; }                \
    int32_t int_value() const { return v; }                            \
    bool operator==(const NAME& o) const { return v == o.v; }          \
  };
SFGPU_STAND_IN_ENUM(optimization_status_t)
SFGPU_STAND_IN_ENUM(levenberg_marquardt_solver_failure_reason_t)
SFGPU_STAND_IN_ENUM(lambda_update_type_t)
#undef SFGPU_STAND_IN_ENUM

struct optimizer_params_t {
  bool verbose = false, debug_stats = false, check_derivatives = false, include_jacobians = false,
       debug_checks = false;
  double initial_lambda = 1.0, lambda_lower_bound = 0.0, lambda_upper_bound = 1e6;
  lambda_update_type_t lambda_update_type{1};
  double lambda_up_factor = 4.0, lambda_down_factor = 1.0 / 4.0;
  double dynamic_lambda_update_beta = 2.0, dynamic_lambda_update_gamma = 3.0;
  int32_t dynamic_lambda_update_p = 3;
  bool use_diagonal_damping = false, use_unit_damping = true, keep_max_diagonal_damping = false;
  double diagonal_damping_min = 1e-6;
  int32_t iterations = 50;
  double early_exit_min_reduction = 1e-6, early_exit_min_absolute_error = 1e-10;
  bool enable_bold_updates = false;
};

struct optimization_iteration_t {
  int16_t iteration = 0;
  double current_lambda = 0, new_error = 0, new_error_linear = 0, relative_reduction = 0,
         update_angle_change = 0;
  bool update_accepted = false;
};

struct sparse_matrix_structure_t {
  std::vector<int32_t> row_indices, column_pointers, shape;
};

struct index_entry_t {
  int64_t offset = 0;
  int32_t storage_dim = 0, tangent_dim = 0;
};
struct index_t {
  int32_t storage_dim = 0, tangent_dim = 0;
  std::vector<index_entry_t> entries;
};

template <typename Scalar>
class Values {
 public:
  std::vector<Scalar>& Data() { return data_; }
  const std::vector<Scalar>& Data() const { return data_; }
  Scalar* DataPointer() { return data_.data(); }

 private:
  std::vector<Scalar> data_;
};

template <typename MatrixType>
struct Linearization {
  using Scalar = typename MatrixType::Scalar;
  Eigen::Matrix<Scalar, Eigen::Dynamic, 1> residual, rhs;
  MatrixType hessian_lower, jacobian;
  bool initialized = false;
  void SetInitialized(bool b) { initialized = b; }
};

template <typename MatrixType>
struct OptimizationStats {
  std::vector<optimization_iteration_t> iterations;
  int32_t best_index = 0;
  optimization_status_t status{};
  int32_t failure_reason = 0;
  Eigen::VectorXi linear_solver_ordering;
  sparse_matrix_structure_t cholesky_factor_sparsity;
};
}  // namespace sym
