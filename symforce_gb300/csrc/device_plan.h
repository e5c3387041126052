// Device-side resources shared by the optimizer handle and the standalone solvers: a simple
// device allocation arena and the device copy of a multifrontal factorization plan.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"
#include "layout.h"

namespace sfg {

struct DeviceArena {
  std::vector<void*> ptrs;
  DeviceArena() = default;
  DeviceArena(const DeviceArena&) = delete;
  DeviceArena& operator=(const DeviceArena&) = delete;
  ~DeviceArena() {
    for (void* p : ptrs) cudaFree(p);
  }
  void* Alloc(size_t bytes);
  template <typename T>
  T* Upload(const std::vector<T>& v) {
    T* p = static_cast<T*>(Alloc(v.size() * sizeof(T)));
    if (!v.empty()) SFG_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
  }
  template <typename T>
  T* Zeros(size_t n) {
    if (n == 0) n = 1;
    T* p = static_cast<T*>(Alloc(n * sizeof(T)));
    SFG_CUDA(cudaMemset(p, 0, n * sizeof(T)));
    return p;
  }
};

// Device copy of a symbolic factorization and its task plan, plus the numeric buffers.
struct FactorPlan {
  Symbolic sym;
  TaskPlan plan;
  FactorDev f{};
  int grid_factor = 1, grid_solve = 1;
  size_t elem = 8;
  void* F = nullptr;       // front pool
  void* Linv = nullptr;    // inverses of the diagonal tiles
  void* ycon = nullptr;
  void* ysave = nullptr;
  void* xperm = nullptr;
  void* xb = nullptr;      // backward exchange values of split solves (ysave's size, right after it)
  int64_t nsave = 0;       // scalars of ysave (and of xb)
  int nflags = 0;
};

// Analyze `pat` with the given ordering and upload everything the factor / solve kernels need.
// `damping_by_scalar`: diagonal entries get damping[original scalar index] added at assembly.
void BuildFactorPlan(DeviceArena& A, FactorPlan& fp, const BlockPattern& pat, int ordering,
                     size_t elem, int* error_word, const LmState* st, int64_t a_stride,
                     int64_t b_stride, int num_sms, bool trace);

// The unit lower factor of a factorization plan as a compressed-column strict-lower matrix in the
// solver's ordering (the L() of SparseCholeskySolver, symforce/opt/sparse_cholesky/
// sparse_cholesky_solver.h:128-131): the supernodal pattern (every entry below the diagonal of a
// front's pivot columns, explicit zeros included).  With `front` (the front pool on the host, FP64
// or FP32 per elem) the values are gathered too.
void FactorLowerCsc(const FactorPlan& fp, const void* front, std::vector<int32_t>& col_ptr,
                    std::vector<int32_t>& row_idx, std::vector<double>* values);

// Per-row segments of the symmetric product with a block pattern (lower blocks stored row-major).
SpmvDev BuildSpmv(DeviceArena& A, const BlockPattern& pat, int64_t a_stride, int64_t b_stride);

// Device copy of a Schur layout for elements of `elem` bytes, with the S-block terms cut into
// chunks (128 terms in FP64, 256 in FP32: measured best on GB300 across the 50- and 1,000-camera
// workloads) and the chunks' partial-sum buffer.
SchurDev UploadSchur(DeviceArena& A, const SchurLayout& S, int elem);

// `gate` (optional): the launched kernels do nothing unless *gate != 0.
template <typename T>
void EnqueueFactor(const FactorPlan& fp, const void* A, const double* damping, cudaStream_t s,
                   const int* gate = nullptr);
// b is read at the Init block's offset (b + init_idx * b_stride) unless fixed_b, which the
// refinement's correction solves use for their single right-hand-side buffer.
template <typename T>
void EnqueueSolve(const FactorPlan& fp, const void* b, void* x, cudaStream_t s, bool fixed_b = false,
                  const int* gate = nullptr);

}  // namespace sfg
