// Standalone linear solvers of the C ABI: the LinearSolver concept on a user CSC matrix
// (SparseCholeskySolver, symforce/opt/sparse_cholesky/sparse_cholesky_solver.h:28-163) and the
// Schur-complement solver (SparseSchurSolver, symforce/opt/sparse_schur_solver.h:62-135), both
// running the same device kernels as the optimizer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "device_plan.h"
#include "kernels.h"
#include "layout.h"

namespace sfg {
extern thread_local std::string g_last_error;
}

namespace {

using sfg::Error;

using Arena = sfg::DeviceArena;

template <typename F>
int32_t Guard(F&& fn) {
  try {
    fn();
    return SFG_OK;
  } catch (const Error& e) {
    sfg::g_last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    sfg::g_last_error = e.what();
    return SFG_ERR_INVALID_ARGUMENT;
  }
}

void SelectDevice(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    throw Error(SFG_ERR_NO_DEVICE, "no CUDA device is visible; this library has no CPU fallback");
  if (device < 0 || device >= n) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad device ordinal");
  SFG_CUDA(cudaSetDevice(device));
}

using Plan = sfg::FactorPlan;

void CheckError(const sfg::LmState* st) {
  int e = 0;
  SFG_CUDA(cudaMemcpy(&e, &st->device_error, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) throw Error(SFG_ERR_DEVICE_STATUS, "device factorization hit its wait cap");
}

sfg::LmState* MakeState(Arena& A) {
  sfg::LmState s0{};
  auto* st = static_cast<sfg::LmState*>(A.Alloc(sizeof(sfg::LmState)));
  SFG_CUDA(cudaMemcpy(st, &s0, sizeof(s0), cudaMemcpyHostToDevice));
  return st;
}

// Validate a lower CSC structure.
void CheckCsc(int32_t n, const int32_t* col_ptr, const int32_t* row_idx) {
  if (n <= 0 || !col_ptr || !row_idx) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad CSC arguments");
  if (col_ptr[0] != 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "col_ptr[0] must be 0");
  for (int c = 0; c < n; ++c) {
    if (col_ptr[c + 1] < col_ptr[c]) throw Error(SFG_ERR_INVALID_ARGUMENT, "col_ptr not monotone");
    for (int32_t q = col_ptr[c]; q < col_ptr[c + 1]; ++q)
      if (row_idx[q] < c || row_idx[q] >= n)
        throw Error(SFG_ERR_INVALID_ARGUMENT, "CSC must hold the lower triangle only");
  }
}

}  // namespace

struct sfg_ldlt {
  Arena A;
  int device = 0;
  cudaStream_t stream = nullptr;
  int32_t n = 0;
  sfg::BlockPattern pat;
  Plan plan;
  sfg::LmState* st = nullptr;
  std::vector<int64_t> csc_to_val;
  double* vals = nullptr;
  double* b = nullptr;
  double* x = nullptr;
  bool factored = false;
  ~sfg_ldlt() {
    if (stream) cudaStreamDestroy(stream);
  }
};

struct sfg_schur {
  Arena A;
  int device = 0;
  cudaStream_t stream = nullptr;
  int32_t n = 0, c_dim = 0;
  sfg::HostProblem P;
  sfg::LinLayout L;
  sfg::SchurLayout SL;
  sfg::SchurDev sd{};
  Plan plan;
  sfg::LmState* st = nullptr;
  std::vector<int64_t> csc_to_val;
  double *hess = nullptr, *rhs = nullptr, *damping = nullptr, *cinv = nullptr, *W = nullptr,
         *tp = nullptr, *S = nullptr, *v = nullptr, *y = nullptr, *update = nullptr;
  bool factored = false;
  ~sfg_schur() {
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int32_t sfg_ldlt_create(int32_t n, const int32_t* col_ptr, const int32_t* row_idx, int32_t ordering,
                        int32_t device, sfg_ldlt** out) {
  if (!out) return SFG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto s = std::make_unique<sfg_ldlt>();
  const int32_t rc = Guard([&] {
    CheckCsc(n, col_ptr, row_idx);
    SelectDevice(device);
    s->device = device;
    s->n = n;
    std::vector<std::pair<int, int>> pairs;
    for (int c = 0; c < n; ++c)
      for (int32_t q = col_ptr[c]; q < col_ptr[c + 1]; ++q) pairs.push_back({row_idx[q], c});
    s->pat = sfg::MakePattern(std::vector<int>(n, 1), pairs);
    s->csc_to_val.resize(col_ptr[n]);
    for (int c = 0; c < n; ++c)
      for (int32_t q = col_ptr[c]; q < col_ptr[c + 1]; ++q)
        s->csc_to_val[q] = s->pat.boff[s->pat.Find(row_idx[q], c)];
    SFG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->st = MakeState(s->A);
    int sms = 0;
    SFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    sfg::BuildFactorPlan(s->A, s->plan, s->pat, ordering, 8, &s->st->device_error, s->st, 0, 0, sms,
                         false);
    s->vals = s->A.Zeros<double>(size_t(s->pat.nvals()));
    s->b = s->A.Zeros<double>(size_t(n));
    s->x = s->A.Zeros<double>(size_t(n));
  });
  if (rc == SFG_OK) *out = s.release();
  return rc;
}

int32_t sfg_ldlt_factorize(sfg_ldlt* s, const double* values) {
  return Guard([&] {
    if (!s || !values) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    SFG_CUDA(cudaSetDevice(s->device));
    std::vector<double> v(s->pat.nvals(), 0.0);
    for (size_t q = 0; q < s->csc_to_val.size(); ++q) v[s->csc_to_val[q]] += values[q];
    SFG_CUDA(cudaMemcpy(s->vals, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
    sfg::EnqueueFactor<double>(s->plan, s->vals, nullptr, s->stream);
    SFG_CUDA(cudaStreamSynchronize(s->stream));
    SFG_CUDA(cudaGetLastError());
    CheckError(s->st);
    s->factored = true;
  });
}

int32_t sfg_ldlt_solve(sfg_ldlt* s, const double* b, double* x, int32_t nrhs) {
  return Guard([&] {
    if (!s || !b || !x || nrhs < 1) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad argument");
    if (!s->factored) throw Error(SFG_ERR_INVALID_ARGUMENT, "factorize first");
    SFG_CUDA(cudaSetDevice(s->device));
    const Plan& p = s->plan;
    for (int r = 0; r < nrhs; ++r) {
      SFG_CUDA(cudaMemcpyAsync(s->b, b + size_t(r) * s->n, sizeof(double) * s->n, cudaMemcpyHostToDevice,
                               s->stream));
      sfg::EnqueueSolve<double>(p, s->b, s->x, s->stream);
      SFG_CUDA(cudaMemcpyAsync(x + size_t(r) * s->n, s->x, sizeof(double) * s->n, cudaMemcpyDeviceToHost,
                               s->stream));
      SFG_CUDA(cudaStreamSynchronize(s->stream));
      CheckError(s->st);
    }
  });
}

int32_t sfg_ldlt_diagonal(sfg_ldlt* s, double* d) {
  return Guard([&] {
    if (!s || !d) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (!s->factored) throw Error(SFG_ERR_INVALID_ARGUMENT, "factorize first");
    const auto& S = s->plan.sym;
    std::vector<double> F(S.front_pool);
    SFG_CUDA(cudaMemcpy(F.data(), s->plan.F, sizeof(double) * F.size(), cudaMemcpyDeviceToHost));
    for (int q = 0; q < S.ns; ++q)
      for (int c = 0; c < S.sn_w[q]; ++c)
        d[S.idx[S.idx_off[q] + c]] = F[S.sn_foff[q] + int64_t(c) * (S.sn_m[q] + 1)];
  });
}

int32_t sfg_ldlt_lower(sfg_ldlt* s, int64_t* nnz, int32_t* col_ptr, int32_t* row_idx, double* values) {
  return Guard([&] {
    if (!s || !nnz) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (!s->factored) throw Error(SFG_ERR_INVALID_ARGUMENT, "factorize first");
    SFG_CUDA(cudaSetDevice(s->device));
    std::vector<double> F;
    if (values) {
      F.resize(size_t(s->plan.sym.front_pool));
      SFG_CUDA(cudaMemcpy(F.data(), s->plan.F, sizeof(double) * F.size(), cudaMemcpyDeviceToHost));
    }
    std::vector<int32_t> cp, ri;
    std::vector<double> v;
    sfg::FactorLowerCsc(s->plan, values ? F.data() : nullptr, cp, ri, values ? &v : nullptr);
    if (!col_ptr && !row_idx && !values) {
      *nnz = int64_t(ri.size());
      return;
    }
    if (*nnz < int64_t(ri.size())) throw Error(SFG_ERR_CAPACITY, "nnz capacity too small");
    *nnz = int64_t(ri.size());
    if (col_ptr) std::copy(cp.begin(), cp.end(), col_ptr);
    if (row_idx) std::copy(ri.begin(), ri.end(), row_idx);
    if (values) std::copy(v.begin(), v.end(), values);
  });
}

int32_t sfg_ldlt_permutation(sfg_ldlt* s, int32_t* perm) {
  return Guard([&] {
    if (!s || !perm) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    const auto& S = s->plan.sym;
    for (int q = 0; q < S.nb; ++q) perm[S.border[q]] = int32_t(S.pstart[q]);
  });
}

int32_t sfg_ldlt_destroy(sfg_ldlt* s) {
  if (s) {
    cudaSetDevice(s->device);
    delete s;
  }
  return SFG_OK;
}

int32_t sfg_schur_create(int32_t n, const int32_t* col_ptr, const int32_t* row_idx, int32_t c_dim,
                         int32_t device, sfg_schur** out) {
  if (!out) return SFG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto s = std::make_unique<sfg_schur>();
  const int32_t rc = Guard([&] {
    CheckCsc(n, col_ptr, row_idx);
    if (c_dim <= 0 || c_dim >= n || c_dim % 3 != 0)
      throw Error(SFG_ERR_STRUCTURE, "C must be made of 3x3 diagonal blocks");
    SelectDevice(device);
    s->device = device;
    s->n = n;
    s->c_dim = c_dim;
    const int nb = n - c_dim, npts = c_dim / 3;
    sfg::HostProblem& P = s->P;
    P.nkeys = nb + npts;
    P.tdim.assign(nb, 1);
    P.tdim.insert(P.tdim.end(), npts, 3);
    P.sdim = P.tdim;
    P.key_type.assign(P.nkeys, SFG_KEY_VEC1);
    for (int k = nb; k < P.nkeys; ++k) P.key_type[k] = SFG_KEY_VEC3;
    P.toff.assign(P.nkeys + 1, 0);
    for (int k = 0; k < P.nkeys; ++k) P.toff[k + 1] = P.toff[k] + P.tdim[k];
    P.soff = P.toff;
    P.N = P.S = n;
    P.num_schur = npts;
    auto key_of = [&](int i) { return i < nb ? i : nb + (i - nb) / 3; };
    std::vector<std::pair<int, int>> pairs;
    for (int c = 0; c < n; ++c)
      for (int32_t q = col_ptr[c]; q < col_ptr[c + 1]; ++q) pairs.push_back({key_of(row_idx[q]), key_of(c)});
    s->L.H = sfg::MakePattern(P.tdim, pairs);
    s->L.nvals = s->L.H.nvals();
    s->L.N = n;
    s->csc_to_val.resize(col_ptr[n]);
    for (int c = 0; c < n; ++c)
      for (int32_t q = col_ptr[c]; q < col_ptr[c + 1]; ++q) {
        const int r = row_idx[q];
        const int kr = key_of(r), kc = key_of(c);
        const int64_t blk = s->L.H.Find(kr, kc);
        s->csc_to_val[q] = s->L.H.boff[blk] + int64_t(r - P.toff[kr]) * P.tdim[kc] + (c - P.toff[kc]);
      }
    s->SL = sfg::BuildSchurLayout(P, s->L, /*g_at_e=*/true);
    SFG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    Arena& A = s->A;
    s->st = MakeState(A);
    const auto& S = s->SL;
    s->sd = sfg::UploadSchur(A, S, 8);
    s->hess = A.Zeros<double>(size_t(s->L.nvals));
    s->rhs = A.Zeros<double>(size_t(n));
    s->damping = A.Zeros<double>(size_t(n));
    s->cinv = A.Zeros<double>(9 * size_t(npts));
    s->W = A.Zeros<double>(size_t(std::max<int64_t>(S.nG, 1)));  // G = L^-1 E
    s->tp = A.Zeros<double>(3 * size_t(npts));
    s->S = A.Zeros<double>(size_t(S.Spat.nvals()));
    s->v = A.Zeros<double>(size_t(S.nB));
    s->y = A.Zeros<double>(size_t(S.nB));
    s->update = A.Zeros<double>(size_t(n));
    int sms = 0;
    SFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    sfg::BuildFactorPlan(A, s->plan, S.Spat, SFG_ORDERING_NESTED_DISSECTION, 8, &s->st->device_error,
                         s->st, 0, 0, sms, false);
  });
  if (rc == SFG_OK) *out = s.release();
  return rc;
}

int32_t sfg_schur_factorize(sfg_schur* s, const double* values) {
  return Guard([&] {
    if (!s || !values) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    SFG_CUDA(cudaSetDevice(s->device));
    std::vector<double> v(s->L.nvals, 0.0);
    for (size_t q = 0; q < s->csc_to_val.size(); ++q) v[s->csc_to_val[q]] += values[q];
    SFG_CUDA(cudaMemcpy(s->hess, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
    cudaStream_t st = s->stream;
    // L^-1 and G = L^-1 E only depend on the matrix; the rhs-dependent t_p is recomputed in solve
    sfg::LaunchSchurPoints<double>(s->sd, s->hess, s->rhs, s->L.nvals, s->n, s->damping, s->cinv, s->W,
                                   s->tp, s->st, st);
    sfg::LaunchSchurBuildS<double>(s->sd, s->hess, s->L.nvals, s->damping, s->W, s->S, s->st, st);
    sfg::EnqueueFactor<double>(s->plan, s->S, nullptr, st);
    SFG_CUDA(cudaStreamSynchronize(st));
    SFG_CUDA(cudaGetLastError());
    CheckError(s->st);
    s->factored = true;
  });
}

int32_t sfg_schur_solve(sfg_schur* s, const double* b, double* x, int32_t nrhs) {
  return Guard([&] {
    if (!s || !b || !x || nrhs < 1) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad argument");
    if (!s->factored) throw Error(SFG_ERR_INVALID_ARGUMENT, "factorize first");
    SFG_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = s->stream;
    const Plan& p = s->plan;
    std::vector<double> u(s->n);
    for (int r = 0; r < nrhs; ++r) {
      SFG_CUDA(cudaMemcpyAsync(s->rhs, b + size_t(r) * s->n, sizeof(double) * s->n, cudaMemcpyHostToDevice, st));
      sfg::LaunchSchurPoints<double>(s->sd, s->hess, s->rhs, s->L.nvals, s->n, s->damping, s->cinv, s->W,
                                     s->tp, s->st, st);
      sfg::LaunchSchurRhs<double>(s->sd, s->hess, s->L.nvals, s->rhs, s->n, s->tp, s->v, s->st, st);
      sfg::EnqueueSolve<double>(p, s->v, s->y, st);
      sfg::LaunchSchurBackSub<double>(s->sd, s->y, s->W, s->tp, s->cinv, s->update, st);
      SFG_CUDA(cudaMemcpyAsync(u.data(), s->update, sizeof(double) * s->n, cudaMemcpyDeviceToHost, st));
      SFG_CUDA(cudaStreamSynchronize(st));
      CheckError(s->st);
      for (int i = 0; i < s->n; ++i) x[size_t(r) * s->n + i] = -u[i];
    }
  });
}

int32_t sfg_schur_destroy(sfg_schur* s) {
  if (s) {
    cudaSetDevice(s->device);
    delete s;
  }
  return SFG_OK;
}

int32_t sfg_selftest_wait_cap(int32_t device, int32_t* device_status, double* ms) {
  return Guard([&] {
    if (!device_status) throw Error(SFG_ERR_INVALID_ARGUMENT, "device_status is null");
    SelectDevice(device);
    int* buf = nullptr;  // [0]: the flag nothing sets, [1]: the error word
    SFG_CUDA(cudaMalloc(&buf, 2 * sizeof(int)));
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&] {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (st) cudaStreamDestroy(st);
      cudaFree(buf);
    };
    try {
      SFG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      SFG_CUDA(cudaEventCreate(&e0));
      SFG_CUDA(cudaEventCreate(&e1));
      SFG_CUDA(cudaMemsetAsync(buf, 0, 2 * sizeof(int), st));
      SFG_CUDA(cudaEventRecord(e0, st));
      SFG_CUDA(sfg::LaunchWaitCapSelfTest(buf, buf + 1, st));
      SFG_CUDA(cudaEventRecord(e1, st));
      SFG_CUDA(cudaStreamSynchronize(st));
      int err = 0;
      SFG_CUDA(cudaMemcpy(&err, buf + 1, sizeof(int), cudaMemcpyDeviceToHost));
      float t = 0.f;
      SFG_CUDA(cudaEventElapsedTime(&t, e0, e1));
      *device_status = err;
      if (ms) *ms = double(t);
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

}  // extern "C"
