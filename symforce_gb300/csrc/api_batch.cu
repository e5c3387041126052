// C ABI of the batched form: many independent problems solved by one persistent kernel launch
// (kernels_batch.cu), captured in a CUDA graph, with a launch-shape autotuner.  Batches of Pose3
// chains take the block-tridiagonal path; any other batch the dense path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "device_plan.h"
#include "kernels.h"

namespace sfg {
extern thread_local std::string g_last_error;
}

struct sfg_batch {
  sfg::DeviceArena arena;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int nprob = 0;
  int nmax = 0;
  int64_t total_poses = 0;
  int64_t total_storage = 0;  // doubles of all problems' values
  std::vector<int32_t> n_host;
  std::vector<int64_t> pose0_host;
  sfg::BatchLmDev d{};
  sfg::LmParams* params = nullptr;
  double epsilon = 0;
  int shape = 0;  // kernel instantiation (warps per CTA x register budget)
  int ctas = 0;
  size_t ws_slots = 0;
  int rec_cap = 0;
  bool values_set = false;
  // graph of one optimize launch for the current shape / record capacity
  cudaGraphExec_t exec = nullptr;
  int graph_shape = -1, graph_ctas = -1, graph_rec = -1;

  ~sfg_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace sfg {
namespace {

template <typename F>
int32_t GuardB(F&& fn) {
  try {
    fn();
    return SFG_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host out of memory";
    return SFG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return SFG_ERR_INVALID_ARGUMENT;
  }
}

void ToParams(const sfg_optimizer_params_t& p, int iterations, double eps, LmParams* o) {
  o->initial_lambda = p.initial_lambda;
  o->lambda_lower_bound = p.lambda_lower_bound;
  o->lambda_upper_bound = p.lambda_upper_bound;
  o->lambda_up_factor = p.lambda_up_factor;
  o->lambda_down_factor = p.lambda_down_factor;
  o->dynamic_beta = p.dynamic_lambda_update_beta;
  o->dynamic_gamma = p.dynamic_lambda_update_gamma;
  o->diagonal_damping_min = p.diagonal_damping_min;
  o->early_exit_min_reduction = p.early_exit_min_reduction;
  o->early_exit_min_absolute_error = p.early_exit_min_absolute_error;
  o->epsilon = eps;
  o->lambda_update_type = p.lambda_update_type;
  o->dynamic_p = p.dynamic_lambda_update_p;
  o->use_diagonal_damping = p.use_diagonal_damping;
  o->use_unit_damping = p.use_unit_damping;
  o->keep_max_diagonal_damping = p.keep_max_diagonal_damping;
  o->enable_bold_updates = p.enable_bold_updates;
  o->iterations = iterations;
}

void CreateChain(const sfg_problem_t* problems, int32_t num_problems, sfg_batch* b);
void CreateDense(const sfg_problem_t* problems, int32_t num_problems, sfg_batch* b);

void Create(const sfg_problem_t* problems, int32_t num_problems, const sfg_form_params_t* form,
            sfg_batch* b) {
  if (!problems || num_problems <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "no problems");
  sfg_form_params_t fm;
  sfg_default_form_params(&fm);
  if (form) fm = *form;
  if (fm.precision != SFG_PRECISION_FP64)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "the batched form solves in FP64");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    throw Error(SFG_ERR_NO_DEVICE, "no CUDA device is visible; this library has no CPU fallback");
  if (fm.device < 0 || fm.device >= ndev) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad device ordinal");
  SFG_CUDA(cudaSetDevice(fm.device));
  b->device = fm.device;
  b->epsilon = fm.epsilon;
  SFG_CUDA(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, fm.device));
  b->nprob = num_problems;
  try {
    CreateChain(problems, num_problems, b);
  } catch (const Error& e) {
    if (e.code != SFG_ERR_STRUCTURE) throw;
    CreateDense(problems, num_problems, b);
  }
  SFG_CUDA(cudaDeviceSynchronize());
}

// Pose3 chains (throws SFG_ERR_STRUCTURE, before allocating anything, for any other problem).
void CreateChain(const sfg_problem_t* problems, int32_t num_problems, sfg_batch* b) {
  // validate and flatten
  std::vector<int32_t> n(num_problems);
  std::vector<int64_t> pose0(num_problems);
  int64_t total = 0;
  for (int p = 0; p < num_problems; ++p) {
    const sfg_problem_t& P = problems[p];
    if (P.num_keys <= 0 || !P.key_types) throw Error(SFG_ERR_INVALID_ARGUMENT, "problem without keys");
    if (P.num_schur_keys != 0) throw Error(SFG_ERR_STRUCTURE, "batched problems have no Schur keys");
    for (int k = 0; k < P.num_keys; ++k)
      if (P.key_types[k] != SFG_KEY_POSE3)
        throw Error(SFG_ERR_STRUCTURE, "batched problems have POSE3 keys only");
    n[p] = P.num_keys;
    pose0[p] = total;
    total += P.num_keys;
  }
  b->total_poses = total;
  b->total_storage = total * 7;
  b->nmax = *std::max_element(n.begin(), n.end());
  std::vector<std::vector<std::pair<int, int64_t>>> un(total);   // (kind, const offset)
  std::vector<std::vector<std::pair<int, int64_t>>> bw(total);   // (rev, const offset)
  std::vector<double> consts;
  for (int p = 0; p < num_problems; ++p) {
    const sfg_problem_t& P = problems[p];
    for (int bi = 0; bi < P.num_batches; ++bi) {
      const sfg_factor_batch_t& B = P.batches[bi];
      if (B.count == 0) continue;
      if (B.count < 0 || !B.keys || !B.consts) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad factor batch");
      const FactorSpec spec = Spec(B.kind);
      if (B.kind != SFG_FACTOR_PRIOR_POSE3 && B.kind != SFG_FACTOR_RANGE_POSE3 &&
          B.kind != SFG_FACTOR_BETWEEN_POSE3)
        throw Error(SFG_ERR_STRUCTURE, "batched problems take PRIOR_POSE3, RANGE_POSE3 and BETWEEN_POSE3");
      for (int f = 0; f < B.count; ++f) {
        const int32_t* k = B.keys + size_t(f) * spec.nkeys;
        for (int q = 0; q < spec.nkeys; ++q)
          if (k[q] < 0 || k[q] >= P.num_keys) throw Error(SFG_ERR_INVALID_ARGUMENT, "factor key out of range");
        const int64_t off = int64_t(consts.size());
        consts.insert(consts.end(), B.consts + size_t(f) * spec.nconsts,
                      B.consts + size_t(f + 1) * spec.nconsts);
        if (spec.nkeys == 1) {
          un[pose0[p] + k[0]].push_back({B.kind, off});
        } else {
          const int lo = std::min(k[0], k[1]), hi = std::max(k[0], k[1]);
          if (hi != lo + 1)
            throw Error(SFG_ERR_STRUCTURE, "batched between factors must join consecutive keys");
          bw[pose0[p] + lo].push_back({k[0] > k[1] ? 1 : 0, off});
        }
      }
    }
  }
  std::vector<int64_t> un_ptr(total + 1, 0), un_coff, bw_ptr(total + 1, 0), bw_coff;
  std::vector<int8_t> un_kind, bw_rev;
  for (int64_t g = 0; g < total; ++g) {
    for (auto& e : un[g]) {
      un_kind.push_back(int8_t(e.first));
      un_coff.push_back(e.second);
    }
    un_ptr[g + 1] = int64_t(un_kind.size());
    for (auto& e : bw[g]) {
      bw_rev.push_back(int8_t(e.first));
      bw_coff.push_back(e.second);
    }
    bw_ptr[g + 1] = int64_t(bw_rev.size());
  }
  // work estimate per problem: factors + poses; largest first
  std::vector<int64_t> work(num_problems);
  for (int p = 0; p < num_problems; ++p)
    work[p] = (un_ptr[pose0[p] + n[p]] - un_ptr[pose0[p]]) + 40 * n[p];
  std::vector<int32_t> order(num_problems);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work[a] > work[c]; });
  SFG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  DeviceArena& A = b->arena;
  BatchLmDev& d = b->d;
  d.nprob = num_problems;
  d.nmax = b->nmax;
  d.order = A.Upload(order);
  d.n = A.Upload(n);
  d.pose0 = A.Upload(pose0);
  d.un_ptr = A.Upload(un_ptr);
  d.un_kind = A.Upload(un_kind);
  d.un_coff = A.Upload(un_coff);
  d.bw_ptr = A.Upload(bw_ptr);
  d.bw_rev = A.Upload(bw_rev);
  d.bw_coff = A.Upload(bw_coff);
  d.consts = A.Upload(consts);
  d.values_in = A.Zeros<double>(size_t(total) * 7);
  d.values_out = A.Zeros<double>(size_t(total) * 7);
  d.st = A.Zeros<LmState>(size_t(num_problems));
  d.counter = A.Zeros<int>(1);
  b->params = static_cast<LmParams*>(A.Alloc(sizeof(LmParams)));
  b->n_host = n;
  b->pose0_host = pose0;
  d.dense = 0;
  d.ws_stride = int64_t(kBatchWsPerPose) * b->nmax;
  // launch shape until the autotuner picks one: 8 warps per CTA, as many CTAs as fit
  b->shape = 0;
  b->ctas = std::max(1, BatchMaxCtasPerSm(b->shape, false)) * b->num_sms;
}

// Any keys and factor kinds, tangent dimension up to kBatchDenseMaxN a problem, every factor's keys
// distinct: the dense path.
void CreateDense(const sfg_problem_t* problems, int32_t num_problems, sfg_batch* b) {
  std::vector<int32_t> dn_n(num_problems), dn_s(num_problems), dn_k0(num_problems), dn_nk(num_problems);
  std::vector<int64_t> dn_s0(num_problems), f_ptr(num_problems + 1, 0), f_coff, work(num_problems);
  std::vector<int8_t> key_type, f_kind;
  std::vector<int32_t> key_soff, key_toff, f_key;
  std::vector<double> consts;
  int64_t total_s = 0;
  int nmax_t = 1, smax = 1;
  for (int p = 0; p < num_problems; ++p) {
    const sfg_problem_t& P = problems[p];
    if (P.num_keys <= 0 || !P.key_types) throw Error(SFG_ERR_INVALID_ARGUMENT, "problem without keys");
    dn_k0[p] = int32_t(key_type.size());
    dn_nk[p] = P.num_keys;
    dn_s0[p] = total_s;
    int so = 0, to = 0;
    for (int k = 0; k < P.num_keys; ++k) {
      int sd = 0, td = 0;
      KeyDims(P.key_types[k], &sd, &td);
      key_type.push_back(int8_t(P.key_types[k]));
      key_soff.push_back(so);
      key_toff.push_back(to);
      so += sd;
      to += td;
    }
    if (to > kBatchDenseMaxN)
      throw Error(SFG_ERR_STRUCTURE, "batched problem " + std::to_string(p) + " has tangent dimension " +
                                         std::to_string(to) + ", more than the batched form's " +
                                         std::to_string(kBatchDenseMaxN));
    dn_n[p] = to;
    dn_s[p] = so;
    total_s += so;
    nmax_t = std::max(nmax_t, to);
    smax = std::max(smax, so);
    int64_t nf = 0;
    for (int bi = 0; bi < P.num_batches; ++bi) {
      const sfg_factor_batch_t& B = P.batches[bi];
      if (B.count == 0) continue;
      if (B.count < 0 || !B.keys || (!B.consts && Spec(B.kind).nconsts > 0))
        throw Error(SFG_ERR_INVALID_ARGUMENT, "bad factor batch");
      const FactorSpec spec = Spec(B.kind);
      if (spec.nkeys > kBatchDenseKeys) throw Error(SFG_ERR_STRUCTURE, "factor with too many keys");
      for (int f = 0; f < B.count; ++f) {
        const int32_t* k = B.keys + size_t(f) * spec.nkeys;
        for (int q = 0; q < spec.nkeys; ++q) {
          if (k[q] < 0 || k[q] >= P.num_keys) throw Error(SFG_ERR_INVALID_ARGUMENT, "factor key out of range");
          if (P.key_types[k[q]] != spec.key_types[q])
            throw Error(SFG_ERR_INVALID_ARGUMENT, "factor key of the wrong type");
          for (int r = 0; r < q; ++r)
            if (k[r] == k[q]) throw Error(SFG_ERR_STRUCTURE, "batched factors take distinct keys");
        }
        f_kind.push_back(int8_t(B.kind));
        for (int q = 0; q < kBatchDenseKeys; ++q) f_key.push_back(q < spec.nkeys ? dn_k0[p] + k[q] : -1);
        f_coff.push_back(int64_t(consts.size()));
        consts.insert(consts.end(), B.consts + size_t(f) * spec.nconsts,
                      B.consts + size_t(f + 1) * spec.nconsts);
        ++nf;
      }
    }
    f_ptr[p + 1] = int64_t(f_kind.size());
    work[p] = int64_t(to) * to * to / 6 + 64 * nf;  // factorization + linearization
  }
  std::vector<int32_t> order(num_problems);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work[a] > work[c]; });
  SFG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  DeviceArena& A = b->arena;
  BatchLmDev& d = b->d;
  d.nprob = num_problems;
  d.nmax = 1;
  d.dense = 1;
  d.nmax_t = nmax_t;
  d.smax = smax;
  d.ws_stride = BatchDenseWsStride(nmax_t, smax);
  d.order = A.Upload(order);
  d.dn_n = A.Upload(dn_n);
  d.dn_s = A.Upload(dn_s);
  d.dn_s0 = A.Upload(dn_s0);
  d.dn_k0 = A.Upload(dn_k0);
  d.dn_nk = A.Upload(dn_nk);
  d.key_type = A.Upload(key_type);
  d.key_soff = A.Upload(key_soff);
  d.key_toff = A.Upload(key_toff);
  d.f_ptr = A.Upload(f_ptr);
  d.f_kind = A.Upload(f_kind);
  d.f_key = A.Upload(f_key);
  d.f_coff = A.Upload(f_coff);
  d.consts = A.Upload(consts);
  d.values_in = A.Zeros<double>(size_t(total_s));
  d.values_out = A.Zeros<double>(size_t(total_s));
  d.st = A.Zeros<LmState>(size_t(num_problems));
  d.counter = A.Zeros<int>(1);
  b->params = static_cast<LmParams*>(A.Alloc(sizeof(LmParams)));
  b->nmax = 1;
  b->total_storage = total_s;
  b->shape = 0;
  b->ctas = std::max(1, BatchMaxCtasPerSm(b->shape, true)) * b->num_sms;
}

void EnsureWorkspace(sfg_batch* b, int ctas, int shape) {
  const size_t slots = size_t(ctas) * BatchShapeWarps(shape);
  if (slots <= b->ws_slots) return;
  b->d.ws = static_cast<double*>(b->arena.Alloc(slots * size_t(b->d.ws_stride) * sizeof(double)));
  b->ws_slots = slots;
  b->graph_shape = -1;
}

void EnsureRecords(sfg_batch* b, int cap) {
  if (cap <= b->rec_cap) return;
  b->d.records = static_cast<sfg_iteration_t*>(
      b->arena.Alloc(size_t(b->nprob) * cap * sizeof(sfg_iteration_t)));
  b->rec_cap = cap;
  b->d.rec_cap = cap;
  b->graph_shape = -1;
}

// One optimize launch of the current shape as a CUDA graph (queue reset + persistent kernel).
void RunGraph(sfg_batch* b) {
  if (b->graph_shape != b->shape || b->graph_ctas != b->ctas || b->graph_rec != b->rec_cap) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    cudaGraph_t g;
    SFG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    LaunchBatchLm(b->d, b->params, b->ctas, b->shape, b->stream);
    SFG_CUDA(cudaStreamEndCapture(b->stream, &g));
    const cudaError_t e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    SFG_CUDA(e);
    b->graph_shape = b->shape;
    b->graph_ctas = b->ctas;
    b->graph_rec = b->rec_cap;
  }
  SFG_CUDA(cudaGraphLaunch(b->exec, b->stream));
}

double Optimize(sfg_batch* b, const sfg_optimizer_params_t& params, int iters) {
  LmParams lp{};
  ToParams(params, iters, b->epsilon, &lp);
  EnsureRecords(b, iters + 1);
  EnsureWorkspace(b, b->ctas, b->shape);
  SFG_CUDA(cudaMemcpyAsync(b->params, &lp, sizeof(lp), cudaMemcpyHostToDevice, b->stream));
  cudaEvent_t e0, e1;
  SFG_CUDA(cudaEventCreate(&e0));
  SFG_CUDA(cudaEventCreate(&e1));
  SFG_CUDA(cudaEventRecord(e0, b->stream));
  RunGraph(b);
  SFG_CUDA(cudaEventRecord(e1, b->stream));
  SFG_CUDA(cudaStreamSynchronize(b->stream));
  SFG_CUDA(cudaGetLastError());
  float ms = 0.f;
  SFG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return double(ms);
}

}  // namespace
}  // namespace sfg

using sfg::Error;

extern "C" {

int32_t sfg_batch_create(const sfg_problem_t* problems, int32_t num_problems,
                         const sfg_form_params_t* form, sfg_batch** out) {
  if (!out) {
    sfg::g_last_error = "out is null";
    return SFG_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  auto b = std::make_unique<sfg_batch>();
  const int32_t rc = sfg::GuardB([&] { sfg::Create(problems, num_problems, form, b.get()); });
  if (rc == SFG_OK) *out = b.release();
  return rc;
}

int32_t sfg_batch_destroy(sfg_batch* b) {
  if (!b) return SFG_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  delete b;
  return SFG_OK;
}

int32_t sfg_batch_storage_dim(const sfg_batch* b, int64_t* storage_dim) {
  if (!b || !storage_dim) return SFG_ERR_INVALID_ARGUMENT;
  *storage_dim = b->total_storage;
  return SFG_OK;
}

int32_t sfg_batch_set_values(sfg_batch* b, const double* storage, int64_t n) {
  return sfg::GuardB([&] {
    if (!b || !storage) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (n != b->total_storage) throw Error(SFG_ERR_INVALID_ARGUMENT, "values size mismatch");
    SFG_CUDA(cudaSetDevice(b->device));
    SFG_CUDA(cudaMemcpyAsync(const_cast<double*>(b->d.values_in), storage, size_t(n) * 8,
                             cudaMemcpyHostToDevice, b->stream));
    SFG_CUDA(cudaStreamSynchronize(b->stream));
    b->values_set = true;
  });
}

int32_t sfg_batch_get_values(sfg_batch* b, double* storage, int64_t n) {
  return sfg::GuardB([&] {
    if (!b || !storage) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (n != b->total_storage) throw Error(SFG_ERR_INVALID_ARGUMENT, "values size mismatch");
    SFG_CUDA(cudaSetDevice(b->device));
    SFG_CUDA(cudaMemcpyAsync(storage, b->d.values_out, size_t(n) * 8, cudaMemcpyDeviceToHost, b->stream));
    SFG_CUDA(cudaStreamSynchronize(b->stream));
  });
}

int32_t sfg_batch_optimize(sfg_batch* b, const sfg_optimizer_params_t* params, int32_t num_iterations,
                           sfg_batch_result_t* results, double* device_ms) {
  return sfg::GuardB([&] {
    if (!b || !params) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->values_set) throw Error(SFG_ERR_INVALID_ARGUMENT, "sfg_batch_set_values was not called");
    if (params->lambda_update_type != SFG_LAMBDA_UPDATE_STATIC &&
        params->lambda_update_type != SFG_LAMBDA_UPDATE_DYNAMIC)
      throw Error(SFG_ERR_INVALID_ARGUMENT, "Invalid lambda update type");
    const int iters = num_iterations < 0 ? params->iterations : num_iterations;
    if (iters <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "num_iterations must be positive");
    SFG_CUDA(cudaSetDevice(b->device));
    const double ms = sfg::Optimize(b, *params, iters);
    if (device_ms) *device_ms = ms;
    if (results) {
      std::vector<sfg::LmState> st(b->nprob);
      SFG_CUDA(cudaMemcpy(st.data(), b->d.st, st.size() * sizeof(sfg::LmState), cudaMemcpyDeviceToHost));
      std::vector<sfg_iteration_t> first(b->nprob);
      SFG_CUDA(cudaMemcpy2D(first.data(), sizeof(sfg_iteration_t), b->d.records,
                            sizeof(sfg_iteration_t) * b->rec_cap, sizeof(sfg_iteration_t), b->nprob,
                            cudaMemcpyDeviceToHost));
      for (int p = 0; p < b->nprob; ++p) {
        results[p].num_iterations = st[p].num_records;
        results[p].best_index = st[p].best_index;
        results[p].status = st[p].status;
        results[p].failure_reason = st[p].failure_reason;
        results[p].initial_error = first[p].new_error;
        results[p].best_error = st[p].error[st[p].best_idx];
      }
    }
  });
}

int32_t sfg_batch_records(sfg_batch* b, int32_t problem, sfg_iteration_t* records, int32_t capacity,
                          int32_t* count) {
  return sfg::GuardB([&] {
    if (!b || !count) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (problem < 0 || problem >= b->nprob) throw Error(SFG_ERR_INVALID_ARGUMENT, "problem out of range");
    SFG_CUDA(cudaSetDevice(b->device));
    sfg::LmState st;
    SFG_CUDA(cudaMemcpy(&st, b->d.st + problem, sizeof(st), cudaMemcpyDeviceToHost));
    *count = st.num_records;
    if (!records) return;
    if (capacity < st.num_records) throw Error(SFG_ERR_CAPACITY, "records buffer too small");
    SFG_CUDA(cudaMemcpy(records, b->d.records + size_t(problem) * b->rec_cap,
                        sizeof(sfg_iteration_t) * st.num_records, cudaMemcpyDeviceToHost));
  });
}

int32_t sfg_batch_autotune(sfg_batch* b, const sfg_optimizer_params_t* params, int32_t* warps_per_cta,
                           int32_t* ctas) {
  return sfg::GuardB([&] {
    if (!b || !params) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->values_set) throw Error(SFG_ERR_INVALID_ARGUMENT, "sfg_batch_set_values was not called");
    SFG_CUDA(cudaSetDevice(b->device));
    double best = 1e300;
    int bs = b->shape, bc = b->ctas;
    for (int shape = 0; shape < sfg::BatchShapes(); ++shape) {
      const int per_sm = sfg::BatchMaxCtasPerSm(shape, b->d.dense != 0);
      if (per_sm <= 0) continue;
      for (int frac : {1, 2}) {  // every resident CTA, or half of them
        if (frac == 2 && per_sm < 2) continue;
        const int c = std::max(1, per_sm / frac) * b->num_sms;
        b->shape = shape;
        b->ctas = c;
        sfg::Optimize(b, *params, params->iterations);  // warm-up of this shape
        const double ms = sfg::Optimize(b, *params, params->iterations);
        if (ms < best) {
          best = ms;
          bs = shape;
          bc = c;
        }
      }
    }
    b->shape = bs;
    b->ctas = bc;
    if (warps_per_cta) *warps_per_cta = sfg::BatchShapeWarps(bs);
    if (ctas) *ctas = bc;
  });
}

}  // extern "C"
