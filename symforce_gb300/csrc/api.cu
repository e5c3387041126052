// The C ABI (include/sfgpu.h): handle lifetime, device buffers, and the CUDA graph that runs the
// whole Levenberg-Marquardt loop on the device (a prologue, then a conditional while node whose
// body is one LevenbergMarquardtSolver::Iterate).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "device_plan.h"
#include "kernels.h"
#include "layout.h"

namespace sfg {

thread_local std::string g_last_error;

namespace {

bool TraceOn() {
  const char* tr = std::getenv("SFG_TRACE_FACTOR");
  return tr && tr[0] == '1';
}

void CheckDevice(int device) {
  int n = 0;
  const cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    throw Error(SFG_ERR_NO_DEVICE, "no CUDA device is visible; this library has no CPU fallback");
  if (device < 0 || device >= n) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad device ordinal");
  SFG_CUDA(cudaSetDevice(device));
}

}  // namespace
}  // namespace sfg

// =============================================================================================
// Handle
// =============================================================================================
struct sfg_handle {
  sfg::DeviceArena arena;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  sfg::HostProblem P;
  sfg::LinLayout L;
  bool schur = false;
  sfg::SchurLayout SL;
  int precision = SFG_PRECISION_FP64;
  size_t elem = 8;
  double epsilon = 10 * DBL_EPSILON;
  sfg::FactorPlan fp;
  // buffers
  double* values = nullptr;     // [3][S]
  double* values_in = nullptr;  // [S]
  double* residual = nullptr;   // [3][M]
  void* hess = nullptr;         // [3][nvals]
  void* rhs = nullptr;          // [3][N]
  void* stage = nullptr;
  double* cost_partials = nullptr;
  int ncost = 0;
  int64_t* key_soff = nullptr;
  int64_t* key_toff = nullptr;
  int32_t* key_type = nullptr;
  std::vector<sfg::BatchDev> batches;
  std::vector<int> batch_kind;
  sfg::ReduceDev red{};
  sfg::DampDev damp{};
  double* update = nullptr;
  double* last_update = nullptr;
  double* delta_partials = nullptr;
  sfg::LmState* st = nullptr;
  sfg::LmParams* params = nullptr;
  sfg_iteration_t* records = nullptr;
  int records_cap = 0;
  // schur
  sfg::SchurDev sd{};
  void *cinv = nullptr, *W = nullptr, *tp = nullptr, *S = nullptr, *v = nullptr, *y = nullptr;
  void* xsol = nullptr;
  // FP64 refinement of a low-precision solve (mixed form)
  int refine_steps = 0;
  sfg::SpmvDev spmv{};
  double* ydbl = nullptr;
  double* rres = nullptr;
  void* rlo = nullptr;
  void* dy = nullptr;
  // PCG forms and training-sample collection
  int pcg_mode = 0;  // 0: exact solve, 1: block-Jacobi PCG, 2: learned PCG
  bool have_precond = false;
  sfg::PrecondLayout PL;
  sfg::PrecondDev pd{};
  float* rho = nullptr;
  float* feats = nullptr;
  float* fac = nullptr;
  float* zout = nullptr;
  float *mlp_h1 = nullptr, *mlp_h2 = nullptr;  // hidden activations of the network's inference
  void* Pblk = nullptr;
  int64_t* blk_off = nullptr;  // [nbl][81] S offsets of the group blocks
  void* Sb = nullptr;          // [nbl][81] group blocks of S
  float* net = nullptr;
  sfg::PcgState* ps = nullptr;
  sfg::PcgDev pcg{};
  sfg::BandDev band{};  // band preconditioner (band.band > 0)
  void* Mband = nullptr;
  int pcg_grid = 1, pcg_threads = 32;
  int collect_cap = 0;
  float* samples = nullptr;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool have_graph = false;
  bool values_set = false;
  bool optimized = false;   // an sfg_optimize call has run (sfg_optimize_continue needs one)
  int last_linearized_block = -1;

  ~sfg_handle() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace sfg {
namespace {

LinOut MakeLinOut(sfg_handle* h, int which) {
  LinOut o;
  o.values = h->values;
  o.key_soff = h->key_soff;
  o.residual = h->residual;
  o.hess = h->hess;
  o.rhs = h->rhs;
  o.stage = h->stage;
  o.cost_partials = h->cost_partials;
  o.S = h->P.S;
  o.M = h->P.M;
  o.N = h->P.N;
  o.nvals = h->L.nvals;
  o.st = h->st;
  o.which = which;
  return o;
}

template <typename T>
void EnqueueLinearize(sfg_handle* h, int which, cudaStream_t s) {
  const LinOut o = MakeLinOut(h, which);
  for (size_t b = 0; b < h->batches.size(); ++b) LaunchLinearize<T>(h->batch_kind[b], o, h->batches[b], s);
  LaunchReduceStage<T>(h->red, o, s);
  LaunchFinishCost(h->cost_partials, h->ncost, h->st, which, s);
}

// Mixed form: widen the low-precision solution and refine it in FP64 a fixed number of times
// against the matrix that was factored (r = b - A y in FP64, correction solved with the factors).
template <typename T>
void EnqueueRefinement(sfg_handle* h, const void* A, const double* damping, const void* b,
                       const void* x_lo, cudaStream_t s, const int* gate = nullptr) {
  if (sizeof(T) == 8) return;
  const int64_t n = h->spmv.n;
  LaunchWiden<T>(x_lo, h->ydbl, n, s, gate);
  for (int k = 0; k < h->refine_steps; ++k) {
    LaunchRefineResidual<T>(h->spmv, A, damping, b, h->ydbl, h->rres, h->rlo, h->st, s, gate);
    EnqueueSolve<T>(h->fp, h->rlo, h->dy, s, /*fixed_b=*/true, gate);
    LaunchAccumulate<T>(h->dy, h->ydbl, n, s, gate);
  }
}

// Preconditioner blocks of the current reduced system (features, network, assembly).
template <typename T>
void EnqueuePrecond(sfg_handle* h, cudaStream_t s) {
  LaunchGroupBlocks<T>(h->blk_off, int64_t(h->pcg.nbl) * kPrecondBlock * kPrecondBlock, h->S, h->Sb, s);
  LaunchPrecondFeatures<T>(h->pd, h->spmv, h->S, h->rho, h->feats, h->fac, s);
  if (h->pcg_mode == 2)
    SFG_CUDA(LaunchMlpInferTc(h->feats, kPrecondFeatures, h->pd.ng, h->net, h->mlp_h1, h->mlp_h2, h->zout,
                              &h->st->device_error, s));
  if (h->band.band > 0) {
    LaunchBandFactor<T>(h->band, h->Sb, s);
    LaunchBandAssemble<T>(h->band, h->pcg_mode == 2 ? h->zout : nullptr, h->Mband, s);
  } else {
    LaunchPrecondAssemble<T>(h->pd.ng, h->fac, h->pcg_mode == 2 ? h->zout : nullptr, h->Pblk, s);
  }
}

// Reduced-system solve of the PCG forms: PCG into ydbl; the exact factorization and solve (with
// FP64 refinement in the mixed form) run only when the PCG missed its tolerance.
template <typename T>
void EnqueuePcgSolve(sfg_handle* h, cudaStream_t s, bool gated) {
  EnqueuePrecond<T>(h, s);
  if (h->pcg.coarse) LaunchGaugeBasis<T>(h->pcg, h->values, h->P.S, h->st, s);
  SFG_CUDA(LaunchPcg<T>(h->pcg, h->pcg_grid, h->pcg_threads, s));
  const int* gate = gated ? &h->ps->need_fallback : nullptr;
  EnqueueFactor<T>(h->fp, h->S, nullptr, s, gate);
  EnqueueSolve<T>(h->fp, h->v, h->y, s, false, gate);
  if (sizeof(T) == 8) LaunchWiden<double>(h->y, h->ydbl, h->sd.nB, s, gate);
  else EnqueueRefinement<T>(h, h->S, nullptr, h->v, h->y, s, gate);
}

template <typename T>
void EnqueueIterationBody(sfg_handle* h, cudaGraphConditionalHandle cond, int use_cond,
                          cudaStream_t s) {
  const int64_t N = h->P.N;
  LaunchDamping<T>(h->damp, h->hess, h->L.nvals, h->params, h->st, s);
  if (h->schur) {
    LaunchSchurPoints<T>(h->sd, h->hess, h->rhs, h->L.nvals, N, h->damp.damping, h->cinv, h->W, h->tp,
                         h->st, s);
    LaunchSchurBuildS<T>(h->sd, h->hess, h->L.nvals, h->damp.damping, h->W, h->S, h->st, s);
    LaunchSchurRhs<T>(h->sd, h->hess, h->L.nvals, h->rhs, N, h->tp, h->v, h->st, s);
    const double* ysol;
    if (h->pcg_mode) {
      EnqueuePcgSolve<T>(h, s, /*gated=*/true);
      ysol = h->ydbl;
    } else {
      EnqueueFactor<T>(h->fp, h->S, nullptr, s);
      EnqueueSolve<T>(h->fp, h->v, h->y, s);
      EnqueueRefinement<T>(h, h->S, nullptr, h->v, h->y, s);
      ysol = sizeof(T) == 8 ? static_cast<const double*>(h->y) : h->ydbl;
    }
    if (h->collect_cap > 0) {
      if (!h->pcg_mode) LaunchPrecondFeatures<T>(h->pd, h->spmv, h->S, h->rho, h->feats, h->fac, s);
      LaunchCollectSamples<T>(h->pd, h->feats, h->fac, h->v, ysol, h->samples, h->collect_cap, h->ps,
                              h->st, s);
    }
    LaunchSchurBackSub<T>(h->sd, ysol, h->W, h->tp, h->cinv, h->update, s);
  } else {
    EnqueueFactor<T>(h->fp, h->hess, h->damp.damping, s);
    EnqueueSolve<T>(h->fp, h->rhs, h->xsol, s);
    EnqueueRefinement<T>(h, h->hess, h->damp.damping, h->rhs, h->xsol, s);
    if (sizeof(T) == 8) LaunchNegate<T>(h->xsol, h->update, N, s);
    else LaunchNegate<double>(h->ydbl, h->update, N, s);
  }
  RetractDev r;
  r.nkeys = h->P.nkeys;
  r.key_type = h->key_type;
  r.soff = h->key_soff;
  r.toff = h->key_toff;
  r.values = h->values;
  r.S = h->P.S;
  r.update = h->update;
  LaunchRetract(r, h->params, h->st, s);
  EnqueueLinearize<T>(h, 1, s);
  LaunchLinearDelta<T>(h->update, h->rhs, h->damp.damping, h->last_update, N, h->delta_partials,
                       h->st, 1, s);
  LaunchDecide(h->params, h->st, h->records, h->update, h->last_update, N, h->delta_partials,
               DeltaPartials(), cond, use_cond, s);
}

template <typename T>
void BuildGraph(sfg_handle* h) {
  if (h->exec) {
    cudaGraphExecDestroy(h->exec);
    h->exec = nullptr;
  }
  if (h->graph) {
    cudaGraphDestroy(h->graph);
    h->graph = nullptr;
  }
  cudaGraph_t g;
  SFG_CUDA(cudaGraphCreate(&g, 0));
  h->graph = g;
  cudaGraphConditionalHandle cond;
  SFG_CUDA(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
  cudaStream_t s = h->stream;
  SFG_CUDA(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  // prologue: Reset, Step, relinearize Init, initial record
  LaunchCopyValues(h->values_in, h->values, h->P.S, h->st, 1, s);
  LaunchBegin(h->params, h->st, 0, s);
  if (h->ps) LaunchPcgBegin(h->ps, s);
  EnqueueLinearize<T>(h, 0, s);
  LaunchFirstRecord(h->params, h->st, h->records, cond, 1, s);
  // conditional while node
  cudaStreamCaptureStatus status;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  SFG_CUDA(cudaStreamGetCaptureInfo(s, &status, nullptr, nullptr, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  std::vector<cudaGraphNode_t> dv(deps, deps + ndeps);
  SFG_CUDA(cudaGraphAddNode(&cnode, g, dv.data(), nullptr, dv.size(), &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  SFG_CUDA(cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  // epilogue: best values back into the input buffer
  LaunchCopyBest(h->values, h->values_in, h->P.S, h->st, s);
  SFG_CUDA(cudaStreamEndCapture(s, &g));
  // body
  cudaStream_t bs;
  SFG_CUDA(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
  SFG_CUDA(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  EnqueueIterationBody<T>(h, cond, 1, bs);
  cudaGraph_t body_out;
  SFG_CUDA(cudaStreamEndCapture(bs, &body_out));
  cudaStreamDestroy(bs);
  SFG_CUDA(cudaGraphInstantiate(&h->exec, g, 0));
  h->have_graph = true;
}

// The same work as the graph, launched one kernel at a time from the host (the loop condition is
// read back after every iteration).  Used for per-kernel profiling, since profilers do not
// attribute kernels inside graphs that contain conditional nodes.
template <typename T>
void RunEager(sfg_handle* h) {
  cudaStream_t s = h->stream;
  LaunchCopyValues(h->values_in, h->values, h->P.S, h->st, 1, s);
  LaunchBegin(h->params, h->st, 0, s);
  if (h->ps) LaunchPcgBegin(h->ps, s);
  EnqueueLinearize<T>(h, 0, s);
  LaunchFirstRecord(h->params, h->st, h->records, 0, 0, s);
  for (;;) {
    int done = 0;
    SFG_CUDA(cudaMemcpyAsync(&done, &h->st->done, sizeof(int), cudaMemcpyDeviceToHost, s));
    SFG_CUDA(cudaStreamSynchronize(s));
    if (done) break;
    EnqueueIterationBody<T>(h, 0, 0, s);
  }
  LaunchCopyBest(h->values, h->values_in, h->P.S, h->st, s);
}

void ToLmParams(const sfg_optimizer_params_t& p, int iterations, double eps, LmParams* o) {
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
  o->continue_state = 0;
  o->relax_damping = 0;
}

template <typename F>
int32_t Guard(F&& fn) {
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

// Camera blocks, feature buffers and the PCG state (PCG forms, sample collection).
void EnsurePrecond(sfg_handle* h) {
  if (h->have_precond) return;
  if (!h->schur) throw Error(SFG_ERR_INVALID_ARGUMENT, "camera blocks need a Schur-form handle");
  DeviceArena& A = h->arena;
  h->PL = BuildPrecondLayout(h->P, h->SL);
  const PrecondLayout& L = h->PL;
  PrecondDev& d = h->pd;
  d.ng = L.ng;
  d.nB = int(h->SL.nB);
  d.gidx = A.Upload(L.gidx);
  d.goff = A.Upload(L.goff);
  d.degree = A.Upload(L.degree);
  d.scalar_group = A.Upload(L.scalar_group);
  d.sdiag_off = A.Upload(L.sdiag_off);
  if (!h->spmv.row_ptr) h->spmv = BuildSpmv(A, h->SL.Spat, 0, 0);
  const size_t ng = size_t(std::max(L.ng, 1));
  h->rho = A.Zeros<float>(size_t(std::max<int64_t>(h->SL.nB, 1)));
  h->feats = A.Zeros<float>(ng * kPrecondFeatures);
  h->fac = A.Zeros<float>(ng * kPrecondFac);
  h->zout = A.Zeros<float>(ng * kPrecondTri);
  h->mlp_h1 = A.Zeros<float>(ng * kPrecondHidden);
  h->mlp_h2 = A.Zeros<float>(ng * kPrecondHidden);
  h->Pblk = A.Alloc(ng * kPrecondBlock * kPrecondBlock * h->elem);
  if (!h->ps) h->ps = A.Zeros<PcgState>(1);
  h->have_precond = true;
}

void CreateHandle(const sfg_problem_t* problem, const sfg_form_params_t* form, sfg_handle* h) {
  sfg_form_params_t fm;
  sfg_default_form_params(&fm);
  if (form) fm = *form;
  if (fm.precision != SFG_PRECISION_FP64 && fm.precision != SFG_PRECISION_MIXED)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "unknown precision");
  CheckDevice(fm.device);
  h->device = fm.device;
  SFG_CUDA(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, fm.device));
  h->P = ParseProblem(problem);
  h->precision = fm.precision;
  h->elem = fm.precision == SFG_PRECISION_MIXED ? 4 : 8;
  if (fm.pcg_band < 0 || fm.pcg_band > kPcgMaxBand)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "pcg_band must be in 0.." + std::to_string(kPcgMaxBand));
  if (fm.pcg_band > 0 && fm.pcg_coarse != 0)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "pcg_band and pcg_coarse cannot be combined");
  if (fm.refine_steps < 0 || fm.refine_steps > 64)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "refine_steps must be in 0..64");
  h->refine_steps = fm.precision == SFG_PRECISION_MIXED ? fm.refine_steps : 0;
  h->epsilon = fm.epsilon;
  if (fm.linear_solver < SFG_LINEAR_SOLVER_SPARSE_LDLT || fm.linear_solver > SFG_LINEAR_SOLVER_PCG_LEARNED)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "unknown linear solver");
  h->pcg_mode = fm.linear_solver == SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI ? 1
                : fm.linear_solver == SFG_LINEAR_SOLVER_PCG_LEARNED  ? 2
                                                                     : 0;
  h->schur = fm.linear_solver != SFG_LINEAR_SOLVER_SPARSE_LDLT;
  if (h->schur && h->P.num_schur == 0)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "Schur and PCG solvers require num_schur_keys > 0");
  h->L = BuildLinLayout(h->P);
  if (h->schur) {
    // G = L^-1 E at E's offsets (SFG_SCHUR_G_AT_E=0: point-major, for layout measurements)
    bool g_at_e = true;
    if (const char* e = std::getenv("SFG_SCHUR_G_AT_E")) g_at_e = std::atoi(e) != 0;
    h->SL = BuildSchurLayout(h->P, h->L, g_at_e);
  }
  SFG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  DeviceArena& A = h->arena;
  const HostProblem& P = h->P;
  const size_t E = h->elem;
  h->values = A.Zeros<double>(3 * size_t(P.S));
  h->values_in = A.Zeros<double>(size_t(P.S));
  h->residual = A.Zeros<double>(3 * size_t(std::max<int64_t>(P.M, 1)));
  h->hess = A.Alloc(3 * size_t(h->L.nvals) * E);
  SFG_CUDA(cudaMemset(h->hess, 0, 3 * size_t(h->L.nvals) * E));
  h->rhs = A.Alloc(3 * size_t(P.N) * E);
  h->stage = A.Alloc(size_t(std::max<int64_t>(h->L.nstage, 1)) * E);
  std::vector<int64_t> soff(P.soff.begin(), P.soff.begin() + P.nkeys);
  std::vector<int64_t> toff(P.toff.begin(), P.toff.begin() + P.nkeys);
  h->key_soff = A.Upload(soff);
  h->key_toff = A.Upload(toff);
  h->key_type = A.Upload(std::vector<int32_t>(P.key_type.begin(), P.key_type.end()));
  // batches
  int partial = 0;
  const int lb = LinearizeBlockSize();
  for (size_t b = 0; b < P.batches.size(); ++b) {
    const HostBatch& B = P.batches[b];
    BatchDev d{};
    d.count = B.count;
    d.nent = h->L.maps[b].nent;
    // structure-of-arrays in the layout's device order of the factors
    const std::vector<int32_t>& order = h->L.maps[b].order;
    std::vector<int32_t> keys(size_t(B.count) * B.nk);
    for (int f = 0; f < B.count; ++f)
      for (int k = 0; k < B.nk; ++k) keys[size_t(k) * B.count + f] = B.keys[size_t(order[f]) * B.nk + k];
    std::vector<double> consts(size_t(B.count) * B.nc);
    for (int f = 0; f < B.count; ++f)
      for (int c = 0; c < B.nc; ++c)
        consts[size_t(c) * B.count + f] = B.consts[size_t(order[f]) * B.nc + c];
    d.keys = A.Upload(keys);
    d.consts = A.Upload(consts);
    d.dest = A.Upload(h->L.maps[b].dest);
    d.roff = B.roff;
    d.partial_base = partial;
    partial += (B.count + lb - 1) / lb;
    h->batches.push_back(d);
    h->batch_kind.push_back(B.kind);
  }
  h->ncost = std::max(partial, 1);
  h->cost_partials = A.Zeros<double>(h->ncost);
  h->red.ngroups = int(h->L.red_dst.size());
  h->red.dst = A.Upload(h->L.red_dst);
  h->red.ptr = A.Upload(h->L.red_ptr);
  h->damp.N = P.N;
  h->damp.diag_off = A.Upload(h->L.diag_off);
  h->damp.damping = A.Zeros<double>(size_t(P.N));
  h->damp.max_diagonal = A.Zeros<double>(size_t(P.N));
  h->update = A.Zeros<double>(size_t(P.N));
  h->last_update = A.Zeros<double>(size_t(P.N));
  h->delta_partials = A.Zeros<double>(4 * size_t(DeltaPartials()));
  h->st = static_cast<LmState*>(A.Alloc(sizeof(LmState)));
  {
    LmState s0{};
    s0.init_idx = 0;
    s0.new_idx = 1;
    s0.best_idx = 0;
    s0.free_idx = 2;
    s0.iteration = -1;
    SFG_CUDA(cudaMemcpy(h->st, &s0, sizeof(LmState), cudaMemcpyHostToDevice));
  }
  h->params = static_cast<LmParams*>(A.Alloc(sizeof(LmParams)));
  int* err_word = &h->st->device_error;
  if (h->schur) {
    const SchurLayout& S = h->SL;
    h->sd = UploadSchur(A, S, E);
    h->cinv = A.Alloc(9 * size_t(std::max(S.npoints, 1)) * E);
    h->W = A.Alloc(size_t(std::max<int64_t>(S.nG, 1)) * E);  // G = L^-1 E
    h->tp = A.Alloc(3 * size_t(std::max(S.npoints, 1)) * E);
    h->S = A.Alloc(size_t(std::max<int64_t>(S.Spat.nvals(), 1)) * E);
    h->v = A.Alloc(size_t(std::max<int64_t>(S.nB, 1)) * E);
    h->y = A.Alloc(size_t(std::max<int64_t>(S.nB, 1)) * E);
    BuildFactorPlan(A, h->fp, S.Spat, fm.ordering, E, err_word, h->st, 0, 0, h->num_sms, TraceOn());
    if (h->elem == 4 || h->pcg_mode) h->spmv = BuildSpmv(A, S.Spat, 0, 0);
  } else {
    h->xsol = A.Alloc(size_t(P.N) * E);
    BuildFactorPlan(A, h->fp, h->L.H, fm.ordering, E, err_word, h->st, h->L.nvals, P.N, h->num_sms,
                    TraceOn());
    if (h->elem == 4) h->spmv = BuildSpmv(A, h->L.H, h->L.nvals, P.N);
  }
  if (h->elem == 4) {
    const size_t n = size_t(std::max(h->spmv.n, 1));
    h->ydbl = A.Zeros<double>(n);
    h->rres = A.Zeros<double>(n);
    h->rlo = A.Alloc(n * E);
    h->dy = A.Alloc(n * E);
    if (!h->ydbl || !h->rres || !h->rlo || !h->dy || !h->spmv.row_ptr)
      throw Error(SFG_ERR_OUT_OF_MEMORY, "refinement buffers were not allocated");
  }
  if (h->pcg_mode) {
    const int64_t nB = std::max<int64_t>(h->SL.nB, 1);
    if (!h->ydbl) h->ydbl = A.Zeros<double>(size_t(nB));
    EnsurePrecond(h);
    h->net = A.Zeros<float>(kPrecondParams);  // zero weights: L = I, block Jacobi
    int split = 1;
    if (E == 8) PcgShape<double>(h->pd.ng, h->num_sms, &h->pcg_grid, &h->pcg_threads, &split);
    else PcgShape<float>(h->pd.ng, h->num_sms, &h->pcg_grid, &h->pcg_threads, &split);
    PcgDev& c = h->pcg;
    c.split = split;
    const PrecondLayout& PL = h->PL;
    c.pd = h->pd;
    c.gptr = A.Upload(PL.gptr);
    c.gent = reinterpret_cast<const int2*>(A.Upload(PL.gent));
    c.nbl = int(PL.blk_row.size());
    h->blk_off = A.Upload(PL.blk_off);
    h->Sb = A.Alloc(PL.blk_off.size() * E);
    c.Sb = h->Sb;
    c.v = h->v;
    c.P = h->Pblk;
    c.y = h->ydbl;
    c.yg = A.Zeros<double>(size_t(std::max(h->pd.ng, 1)) * kPrecondBlock);
    c.z = A.Zeros<char>(size_t(std::max(h->pd.ng, 1)) * kPrecondBlock * E);
    c.staged = 0;
    if (h->pcg_grid == 1) {
      const int nent = PL.gptr.back();
      const size_t smem = E == 8 ? PcgStagedSmem<double>(h->pd.ng, c.nbl, nent)
                                 : PcgStagedSmem<float>(h->pd.ng, c.nbl, nent);
      if (smem > 0) {
        if (E == 8) ConfigurePcg<double>();
        else ConfigurePcg<float>();
        c.staged = int(smem);
      }
    }
    c.partials = A.Zeros<double>(2 * size_t(kPcgReduceMax) * size_t(h->pcg_grid));
    // the gauge coarse correction needs at least two cameras' poses (otherwise Z^T S Z is singular)
    c.coarse = (fm.pcg_coarse != 0 && PL.gauge_rows >= 12) ? 1 : 0;
    if (fm.pcg_band > 0) {
      const BandPattern BP = BuildBandPattern(PL, fm.pcg_band);
      BandDev& bd = h->band;
      bd.ng = h->pd.ng;
      bd.band = fm.pcg_band;
      bd.nj = A.Upload(BP.nj);
      bd.jgrp = A.Upload(BP.jgrp);
      bd.jblk = A.Upload(BP.jblk);
      bd.gidx = h->pd.gidx;
      const size_t blocks = size_t(std::max(h->pd.ng, 1)) * (fm.pcg_band + 1);
      bd.G = A.Zeros<char>(blocks * kPrecondBlock * kPrecondBlock * E);
      h->Mband = A.Zeros<char>(blocks * kPrecondBlock * kPrecondBlock * E);
      c.band = fm.pcg_band;
      c.Mb = h->Mband;
      c.RQ = A.Zeros<char>(size_t(std::max(h->pd.ng, 1)) * kPrecondBlock * 2 * E);
    }
    if (c.coarse) {
      const size_t rows = size_t(std::max(h->pd.ng, 1)) * kPrecondBlock;
      c.zg = A.Zeros<char>(size_t(kGaugeDim) * rows * E);
      c.szg = A.Zeros<char>(size_t(kGaugeDim) * rows * E);
      c.gauge_soff = A.Upload(PL.gauge_soff);
      c.gauge_comp = A.Upload(PL.gauge_comp);
    }
    if (const char* tr = std::getenv("SFG_TRACE_PCG"); tr && tr[0] == '1') {
      c.trace_cap = 4096;
      c.trace = A.Zeros<unsigned long long>(1 + 4 * size_t(c.trace_cap));
    }
    c.bar = A.Zeros<unsigned>(2);
    c.ps = h->ps;
    c.err = err_word;
    c.tol = fm.pcg_tol > 0 ? fm.pcg_tol : 1e-8;
    c.inner_floor = E == 4 ? 1e-5 : 0.0;
    c.max_iters = fm.pcg_max_iters > 0 ? fm.pcg_max_iters : 500;
    c.max_outer = E == 4 ? 8 : 4;
  }
  SFG_CUDA(cudaDeviceSynchronize());
}

int PrologueKernels(const sfg_handle* h) {
  int n = 0;
  for (const auto& b : h->batches) n += b.count > 0 ? 1 : 0;
  n += h->red.ngroups > 0 ? 1 : 0;
  return n + 1 /*cost*/ + 1 /*copy*/ + 1 /*begin*/ + 1 /*first record*/ + 1 /*copy best*/;
}

int BodyKernels(const sfg_handle* h) {
  int n = 0;
  for (const auto& b : h->batches) n += b.count > 0 ? 1 : 0;
  n += h->red.ngroups > 0 ? 1 : 0;
  n += 1;  // cost
  n += 1 /*damping*/ + 1 /*retract*/ + 1 /*delta*/ + 1 /*decide*/ + 3 /*reset, factor, solve*/;
  n += h->schur ? 6 /*points, W, S chunks, S, rhs, back-substitution*/ : 1 /*negate*/;
  if (h->elem == 4) n += 1 + 4 * h->refine_steps;  // widen; residual, reset, solve, accumulate
  if (h->pcg_mode) {
    n += 1 /*group blocks*/ + 2 /*row coupling, features*/ + (h->pcg_mode == 2 ? 1 : 0) +
         (h->band.band > 0 ? 2 /*band factor, band assembly*/ : 1 /*assemble*/) + 1 /*PCG*/ +
         (h->pcg.coarse ? 1 : 0) /*gauge basis*/;
    if (h->elem == 8) n += 1;  // widen of the fallback solution
  }
  if (h->collect_cap > 0) n += (h->pcg_mode ? 0 : 2) + 1;
  return n;
}

void EnsureRecords(sfg_handle* h, int cap) {
  if (cap <= h->records_cap) return;
  int c = std::max(cap, 64);
  h->records = static_cast<sfg_iteration_t*>(h->arena.Alloc(size_t(c) * sizeof(sfg_iteration_t)));
  h->records_cap = c;
  h->have_graph = false;
}

}  // namespace
}  // namespace sfg

// =============================================================================================
// extern "C"
// =============================================================================================
using sfg::Error;
using sfg::Guard;

extern "C" {

int32_t sfg_abi_version(void) { return SFG_ABI_VERSION; }

const char* sfg_last_error(void) { return sfg::g_last_error.c_str(); }

void sfg_default_optimizer_params(sfg_optimizer_params_t* o) {
  // sym::DefaultOptimizerParams (symforce/opt/optimizer.cc:8-56)
  std::memset(o, 0, sizeof(*o));
  o->initial_lambda = 1.0;
  o->lambda_lower_bound = 0.0;
  o->lambda_upper_bound = 1000000.0;
  o->lambda_update_type = SFG_LAMBDA_UPDATE_STATIC;
  o->lambda_up_factor = 4.0;
  o->lambda_down_factor = 1 / 4.0;
  o->dynamic_lambda_update_beta = 2.0;
  o->dynamic_lambda_update_gamma = 3.0;
  o->dynamic_lambda_update_p = 3;
  o->use_diagonal_damping = 0;
  o->use_unit_damping = 1;
  o->keep_max_diagonal_damping = 0;
  o->diagonal_damping_min = 1e-6;
  o->iterations = 50;
  o->early_exit_min_reduction = 1e-6;
  o->early_exit_min_absolute_error = 0.0;
  o->enable_bold_updates = 0;
}

void sfg_default_form_params(sfg_form_params_t* o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = SFG_PRECISION_FP64;
  o->linear_solver = SFG_LINEAR_SOLVER_SPARSE_LDLT;
  o->ordering = SFG_ORDERING_NESTED_DISSECTION;
  o->device = 0;
  o->epsilon = 10 * DBL_EPSILON;
  o->refine_steps = 1;
  o->pcg_max_iters = 500;
  o->pcg_tol = 1e-8;
  o->pcg_coarse = 0;
}

int32_t sfg_key_dims(int32_t key_type, int32_t* storage_dim, int32_t* tangent_dim) {
  return Guard([&] {
    int s, t;
    sfg::KeyDims(key_type, &s, &t);
    if (storage_dim) *storage_dim = s;
    if (tangent_dim) *tangent_dim = t;
  });
}

int32_t sfg_factor_dims(int32_t kind, int32_t* num_keys, int32_t* num_consts, int32_t* residual_dim) {
  return Guard([&] {
    const sfg::FactorSpec s = sfg::Spec(kind);
    if (num_keys) *num_keys = s.nkeys;
    if (num_consts) *num_consts = s.nconsts;
    if (residual_dim) *residual_dim = s.rdim;
  });
}

int32_t sfg_create(const sfg_problem_t* problem, const sfg_form_params_t* form, sfg_handle** out) {
  if (!out) {
    sfg::g_last_error = "out is null";
    return SFG_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  auto h = std::make_unique<sfg_handle>();
  const int32_t rc = Guard([&] { sfg::CreateHandle(problem, form, h.get()); });
  if (rc == SFG_OK) *out = h.release();
  return rc;
}

int32_t sfg_destroy(sfg_handle* h) {
  if (!h) return SFG_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
  return SFG_OK;
}

int32_t sfg_storage_dim(const sfg_handle* h, int64_t* storage_dim, int64_t* tangent_dim,
                        int64_t* residual_dim) {
  if (!h) return SFG_ERR_INVALID_ARGUMENT;
  if (storage_dim) *storage_dim = h->P.S;
  if (tangent_dim) *tangent_dim = h->P.N;
  if (residual_dim) *residual_dim = h->P.M;
  return SFG_OK;
}

int32_t sfg_set_values(sfg_handle* h, const double* storage, int64_t n) {
  return Guard([&] {
    if (!h || !storage) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (n != h->P.S) throw Error(SFG_ERR_INVALID_ARGUMENT, "values size mismatch");
    SFG_CUDA(cudaSetDevice(h->device));
    SFG_CUDA(cudaMemcpyAsync(h->values_in, storage, size_t(n) * sizeof(double), cudaMemcpyHostToDevice,
                             h->stream));
    SFG_CUDA(cudaStreamSynchronize(h->stream));
    h->values_set = true;
  });
}

namespace sfg {
namespace {
int32_t OptimizeImpl(sfg_handle* h, const sfg_optimizer_params_t* params, int32_t num_iterations,
                     sfg_stats_t* stats, int continue_state, int relax_damping);
}
}  // namespace sfg

int32_t sfg_optimize(sfg_handle* h, const sfg_optimizer_params_t* params, int32_t num_iterations,
                     sfg_stats_t* stats) {
  return sfg::OptimizeImpl(h, params, num_iterations, stats, 0, 0);
}

int32_t sfg_optimize_continue(sfg_handle* h, const sfg_optimizer_params_t* params,
                              int32_t num_iterations, int32_t relax_damping, sfg_stats_t* stats) {
  return Guard([&] {
    if (!h) throw Error(SFG_ERR_INVALID_ARGUMENT, "null handle");
    if (!h->optimized) throw Error(SFG_ERR_INVALID_ARGUMENT, "sfg_optimize_continue needs a prior sfg_optimize");
    const int32_t rc = sfg::OptimizeImpl(h, params, num_iterations, stats, 1, relax_damping ? 1 : 0);
    if (rc != SFG_OK) throw Error(rc, sfg::g_last_error);
  });
}

int32_t sfg_set_factor_consts(sfg_handle* h, int32_t batch, const double* consts, int64_t n) {
  return Guard([&] {
    if (!h || !consts) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (batch < 0 || batch >= int32_t(h->P.batches.size()))
      throw Error(SFG_ERR_INVALID_ARGUMENT, "batch index out of range");
    sfg::HostBatch& B = h->P.batches[size_t(batch)];
    if (n != int64_t(B.count) * B.nc) throw Error(SFG_ERR_INVALID_ARGUMENT, "consts size mismatch");
    B.consts.assign(consts, consts + n);
    const std::vector<int32_t>& order = h->L.maps[size_t(batch)].order;
    std::vector<double> soa(static_cast<size_t>(n));
    for (int f = 0; f < B.count; ++f)
      for (int c = 0; c < B.nc; ++c) soa[size_t(c) * B.count + f] = consts[size_t(order[f]) * B.nc + c];
    SFG_CUDA(cudaSetDevice(h->device));
    if (n > 0)
      SFG_CUDA(cudaMemcpyAsync(const_cast<double*>(h->batches[size_t(batch)].consts), soa.data(),
                               sizeof(double) * size_t(n), cudaMemcpyHostToDevice, h->stream));
    SFG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

namespace sfg {
namespace {
int32_t OptimizeImpl(sfg_handle* h, const sfg_optimizer_params_t* params, int32_t num_iterations,
                     sfg_stats_t* stats, int continue_state, int relax_damping) {
  return Guard([&] {
    if (!h || !params) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (!h->values_set) throw Error(SFG_ERR_INVALID_ARGUMENT, "sfg_set_values was not called");
    if (params->lambda_update_type != SFG_LAMBDA_UPDATE_STATIC &&
        params->lambda_update_type != SFG_LAMBDA_UPDATE_DYNAMIC)
      throw Error(SFG_ERR_INVALID_ARGUMENT, "Invalid lambda update type");
    const int iters = num_iterations < 0 ? params->iterations : num_iterations;
    if (iters <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "num_iterations must be positive");
    SFG_CUDA(cudaSetDevice(h->device));
    sfg::EnsureRecords(h, iters + 1);
    if (!h->have_graph) {
      if (h->elem == 8) sfg::BuildGraph<double>(h);
      else sfg::BuildGraph<float>(h);
    }
    sfg::LmParams lp;
    sfg::ToLmParams(*params, iters, h->epsilon, &lp);
    lp.continue_state = continue_state;
    lp.relax_damping = relax_damping;
    SFG_CUDA(cudaMemcpyAsync(h->params, &lp, sizeof(lp), cudaMemcpyHostToDevice, h->stream));
    cudaEvent_t e0, e1;
    SFG_CUDA(cudaEventCreate(&e0));
    SFG_CUDA(cudaEventCreate(&e1));
    SFG_CUDA(cudaEventRecord(e0, h->stream));
    const char* eager = std::getenv("SFG_EAGER");
    if (eager && eager[0] == '1') {
      if (h->elem == 8) sfg::RunEager<double>(h);
      else sfg::RunEager<float>(h);
    } else {
      SFG_CUDA(cudaGraphLaunch(h->exec, h->stream));
    }
    SFG_CUDA(cudaEventRecord(e1, h->stream));
    SFG_CUDA(cudaStreamSynchronize(h->stream));
    float ms = 0.f;
    SFG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sfg::LmState st;
    SFG_CUDA(cudaMemcpy(&st, h->st, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.device_error)
      throw Error(SFG_ERR_DEVICE_STATUS, "device loop hit its cap (code " + std::to_string(st.device_error) + ")");
    if (stats) {
      stats->device_ms = double(ms);
      stats->kernel_launches = sfg::PrologueKernels(h) +
                               std::max(st.num_records - (continue_state ? 0 : 1), 0) * sfg::BodyKernels(h);
      stats->num_iterations = st.num_records;
      stats->best_index = st.best_index;
      stats->status = st.status;
      stats->failure_reason = st.failure_reason;
      if (stats->iterations) {
        if (stats->capacity < st.num_records)
          throw Error(SFG_ERR_CAPACITY, "stats->iterations too small");
        SFG_CUDA(cudaMemcpy(stats->iterations, h->records, sizeof(sfg_iteration_t) * st.num_records,
                            cudaMemcpyDeviceToHost));
      }
    }
    h->optimized = true;
  });
}
}  // namespace
}  // namespace sfg

int32_t sfg_factor_lower(sfg_handle* h, int64_t* nnz, int32_t* col_ptr, int32_t* row_idx, double* values) {
  return Guard([&] {
    if (!h || !nnz) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (!h->fp.F) throw Error(SFG_ERR_STRUCTURE, "this form has no sparse factorization");
    SFG_CUDA(cudaSetDevice(h->device));
    SFG_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<unsigned char> F;
    if (values) {
      F.resize(size_t(h->fp.sym.front_pool) * h->fp.elem);
      SFG_CUDA(cudaMemcpy(F.data(), h->fp.F, F.size(), cudaMemcpyDeviceToHost));
    }
    std::vector<int32_t> cp, ri;
    std::vector<double> v;
    sfg::FactorLowerCsc(h->fp, values ? F.data() : nullptr, cp, ri, values ? &v : nullptr);
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

int32_t sfg_get_values(sfg_handle* h, double* storage, int64_t n) {
  return Guard([&] {
    if (!h || !storage) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (n != h->P.S) throw Error(SFG_ERR_INVALID_ARGUMENT, "values size mismatch");
    SFG_CUDA(cudaSetDevice(h->device));
    SFG_CUDA(cudaMemcpyAsync(storage, h->values_in, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
    SFG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int32_t sfg_linearize(sfg_handle* h, double* residual, double* rhs, double* error) {
  return Guard([&] {
    if (!h) throw Error(SFG_ERR_INVALID_ARGUMENT, "null handle");
    if (!h->values_set) throw Error(SFG_ERR_INVALID_ARGUMENT, "sfg_set_values was not called");
    SFG_CUDA(cudaSetDevice(h->device));
    sfg::LmState st;
    SFG_CUDA(cudaMemcpy(&st, h->st, sizeof(st), cudaMemcpyDeviceToHost));
    const int blk = st.best_idx == 2 ? 1 : 2;  // any block that does not hold the best values
    const int which = 2 + blk;
    cudaStream_t s = h->stream;
    sfg::LaunchCopyValues(h->values_in, h->values, h->P.S, h->st, which, s);
    if (h->elem == 8) sfg::EnqueueLinearize<double>(h, which, s);
    else sfg::EnqueueLinearize<float>(h, which, s);
    SFG_CUDA(cudaStreamSynchronize(s));
    SFG_CUDA(cudaGetLastError());
    h->last_linearized_block = blk;
    if (residual) {
      // the device holds each batch's residuals in its device factor order
      std::vector<double> dev(size_t(h->P.M));
      SFG_CUDA(cudaMemcpy(dev.data(), h->residual + size_t(blk) * h->P.M, sizeof(double) * h->P.M,
                          cudaMemcpyDeviceToHost));
      for (size_t b = 0; b < h->P.batches.size(); ++b) {
        const sfg::HostBatch& B = h->P.batches[b];
        const std::vector<int32_t>& order = h->L.maps[b].order;
        for (int f = 0; f < B.count; ++f)
          for (int i = 0; i < B.rdim; ++i)
            residual[B.roff + int64_t(order[f]) * B.rdim + i] = dev[B.roff + int64_t(f) * B.rdim + i];
      }
    }
    if (rhs) {
      if (h->elem == 8) {
        SFG_CUDA(cudaMemcpy(rhs, static_cast<double*>(h->rhs) + size_t(blk) * h->P.N,
                            sizeof(double) * h->P.N, cudaMemcpyDeviceToHost));
      } else {
        std::vector<float> tmp(h->P.N);
        SFG_CUDA(cudaMemcpy(tmp.data(), static_cast<float*>(h->rhs) + size_t(blk) * h->P.N,
                            sizeof(float) * h->P.N, cudaMemcpyDeviceToHost));
        std::copy(tmp.begin(), tmp.end(), rhs);
      }
    }
    if (error) {
      SFG_CUDA(cudaMemcpy(&st, h->st, sizeof(st), cudaMemcpyDeviceToHost));
      *error = st.error[blk];
    }
  });
}

int32_t sfg_hessian_lower(sfg_handle* h, int64_t* nnz, int32_t* col_ptr, int32_t* row_idx,
                          double* values) {
  return Guard([&] {
    if (!h || !nnz) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    sfg::BuildCscExport(h->L, h->P);
    const auto& L = h->L;
    *nnz = int64_t(L.csc_rowidx.size());
    if (col_ptr) std::copy(L.csc_colptr.begin(), L.csc_colptr.end(), col_ptr);
    if (row_idx) std::copy(L.csc_rowidx.begin(), L.csc_rowidx.end(), row_idx);
    if (values) {
      if (h->last_linearized_block < 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "call sfg_linearize first");
      std::vector<double> hv(L.nvals);
      SFG_CUDA(cudaSetDevice(h->device));
      if (h->elem == 8) {
        SFG_CUDA(cudaMemcpy(hv.data(), static_cast<double*>(h->hess) + size_t(h->last_linearized_block) * L.nvals,
                            sizeof(double) * L.nvals, cudaMemcpyDeviceToHost));
      } else {
        std::vector<float> tmp(L.nvals);
        SFG_CUDA(cudaMemcpy(tmp.data(), static_cast<float*>(h->hess) + size_t(h->last_linearized_block) * L.nvals,
                            sizeof(float) * L.nvals, cudaMemcpyDeviceToHost));
        std::copy(tmp.begin(), tmp.end(), hv.begin());
      }
      for (size_t q = 0; q < L.csc_src.size(); ++q) values[q] = hv[L.csc_src[q]];
    }
  });
}

int32_t sfg_permutation(sfg_handle* h, int32_t* perm, int64_t n) {
  return Guard([&] {
    if (!h || !perm) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    const sfg::Symbolic& S = h->fp.sym;
    if (n != S.n) throw Error(SFG_ERR_INVALID_ARGUMENT, "size mismatch");
    const sfg::BlockPattern& pat = h->schur ? h->SL.Spat : h->L.H;
    for (int q = 0; q < S.nb; ++q) {
      const int old = S.border[q];
      for (int t = 0; t < pat.dim[old]; ++t) perm[pat.off[old] + t] = int32_t(S.pstart[q] + t);
    }
  });
}

int32_t sfg_fronts(sfg_handle* h, int32_t* count, int32_t* width, int32_t* size) {
  return Guard([&] {
    if (!h || !count) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    const sfg::Symbolic& S = h->fp.sym;
    const int32_t cap = *count;
    *count = S.ns;
    if (cap == 0) return;
    if (cap < S.ns || !width || !size) throw Error(SFG_ERR_INVALID_ARGUMENT, "capacity too small");
    for (int q = 0; q < S.ns; ++q) {
      width[q] = S.sn_w[q];
      size[q] = S.sn_m[q];
    }
  });
}

int32_t sfg_time_stage(sfg_handle* h, int32_t stage, int32_t reps, double* ms_per_launch,
                       double* algorithmic_bytes, double* fmas) {
  return Guard([&] {
    if (!h || reps < 1) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad argument");
    if (!h->have_graph) throw Error(SFG_ERR_INVALID_ARGUMENT, "call sfg_optimize first");
    SFG_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const auto& P = h->P;
    double bytes = 0, fma = 0;
    std::function<void()> launch;
    switch (stage) {
      case SFG_STAGE_LINEARIZE: {
        launch = [&] {
          if (h->elem == 8) sfg::EnqueueLinearize<double>(h, 1, s);
          else sfg::EnqueueLinearize<float>(h, 1, s);
        };
        int64_t consts = 0;
        for (const auto& b : P.batches) consts += int64_t(b.count) * b.nc;
        bytes = 8.0 * double(P.S + consts + P.M + h->L.nnz_lower + P.N);
        for (const auto& b : P.batches) {
          const double td = b.tdim, rd = b.rdim;
          fma += double(b.count) * (rd * td * (td + 1) / 2 + rd * td);
        }
        break;
      }
      case SFG_STAGE_SCHUR: {
        if (!h->schur) throw Error(SFG_ERR_INVALID_ARGUMENT, "handle has no Schur stage");
        const auto& S = h->SL;
        launch = [&] {
          if (h->elem == 8) {
            sfg::LaunchSchurPoints<double>(h->sd, h->hess, h->rhs, h->L.nvals, P.N, h->damp.damping,
                                           h->cinv, h->W, h->tp, h->st, s);
            sfg::LaunchSchurBuildS<double>(h->sd, h->hess, h->L.nvals, h->damp.damping, h->W, h->S,
                                           h->st, s);
            sfg::LaunchSchurRhs<double>(h->sd, h->hess, h->L.nvals, h->rhs, P.N, h->tp, h->v, h->st, s);
          } else {
            sfg::LaunchSchurPoints<float>(h->sd, h->hess, h->rhs, h->L.nvals, P.N, h->damp.damping,
                                          h->cinv, h->W, h->tp, h->st, s);
            sfg::LaunchSchurBuildS<float>(h->sd, h->hess, h->L.nvals, h->damp.damping, h->W, h->S,
                                          h->st, s);
            sfg::LaunchSchurRhs<float>(h->sd, h->hess, h->L.nvals, h->rhs, P.N, h->tp, h->v, h->st, s);
          }
        };
        // read E and C blocks + rhs, write W and S; E is re-read for the rhs
        int64_t ne = 0;
        for (size_t e = 0; e < S.pt_eoff.size(); ++e) ne += 3 * S.pt_ekey_dim[e];
        bytes = 8.0 * double(2 * ne + 2 * ne + 9 * S.npoints + S.Spat.nvals() + P.N);
        for (size_t b = 0; b + 1 < S.sb_ptr.size(); ++b)
          fma += 3.0 * S.sb_dk[b] * S.sb_dl[b] * double(S.sb_ptr[b + 1] - S.sb_ptr[b]);
        fma += 9.0 * double(ne) / 3.0 * 3.0;
        break;
      }
      case SFG_STAGE_FACTOR: {
        const sfg::FactorPlan& fp = h->fp;
        const void* A = h->schur ? h->S : h->hess;
        const double* damping = h->schur ? nullptr : h->damp.damping;
        launch = [&, A, damping] {
          if (h->elem == 8) sfg::EnqueueFactor<double>(fp, A, damping, s);
          else sfg::EnqueueFactor<float>(fp, A, damping, s);
        };
        bytes = 8.0 * 2.0 * double(fp.sym.front_pool);
        fma = fp.sym.flops;
        break;
      }
      case SFG_STAGE_SOLVE: {
        const sfg::FactorPlan& fp = h->fp;
        const void* b = h->schur ? h->v : h->rhs;
        void* x = h->schur ? h->y : h->xsol;
        launch = [&, b, x] {
          if (h->elem == 8) sfg::EnqueueSolve<double>(fp, b, x, s);
          else sfg::EnqueueSolve<float>(fp, b, x, s);
        };
        bytes = 8.0 * double(fp.sym.nnz_L + fp.sym.n) * 2.0;
        fma = 2.0 * double(fp.sym.nnz_L);
        break;
      }
      default:
        throw Error(SFG_ERR_INVALID_ARGUMENT, "unknown stage");
    }
    launch();
    cudaEvent_t e0, e1;
    SFG_CUDA(cudaEventCreate(&e0));
    SFG_CUDA(cudaEventCreate(&e1));
    SFG_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; ++r) launch();
    SFG_CUDA(cudaEventRecord(e1, s));
    SFG_CUDA(cudaStreamSynchronize(s));
    SFG_CUDA(cudaGetLastError());
    float ms = 0.f;
    SFG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sfg::LmState st;
    SFG_CUDA(cudaMemcpy(&st, h->st, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.device_error) throw Error(SFG_ERR_DEVICE_STATUS, "device loop hit its cap");
    if (stage == SFG_STAGE_FACTOR && h->fp.f.trace) {
      if (const char* path = std::getenv("SFG_TRACE_FACTOR_FILE")) {
        const auto& tasks = h->fp.plan.tasks;
        std::vector<unsigned long long> tr(8 * tasks.size());
        SFG_CUDA(cudaMemcpy(tr.data(), h->fp.f.trace, tr.size() * 8, cudaMemcpyDeviceToHost));
        if (FILE* fo = std::fopen(path, "wb")) {
          const int64_t n = int64_t(tasks.size());
          std::fwrite(&n, 8, 1, fo);
          std::fwrite(tasks.data(), sizeof(int4), tasks.size(), fo);
          std::fwrite(tr.data(), 8, tr.size(), fo);
          std::fclose(fo);
        }
      }
    }
    if (ms_per_launch) *ms_per_launch = double(ms) / reps;
    if (algorithmic_bytes) *algorithmic_bytes = bytes;
    if (fmas) *fmas = fma;
  });
}

int32_t sfg_fp64_diag_tiles(sfg_handle* h, int64_t* count) {
  return Guard([&] {
    if (!h || !count) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    int c = 0;
    if (h->fp.f.fp64_tiles) {
      SFG_CUDA(cudaSetDevice(h->device));
      SFG_CUDA(cudaStreamSynchronize(h->stream));
      SFG_CUDA(cudaMemcpy(&c, h->fp.f.fp64_tiles, sizeof(int), cudaMemcpyDeviceToHost));
    }
    *count = c;
  });
}

int32_t sfg_get_pcg_stats(sfg_handle* h, sfg_pcg_stats_t* out) {
  return Guard([&] {
    if (!h || !out) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    if (!h->ps) return;
    SFG_CUDA(cudaSetDevice(h->device));
    sfg::PcgState ps;
    SFG_CUDA(cudaMemcpy(&ps, h->ps, sizeof(ps), cudaMemcpyDeviceToHost));
    out->solves = ps.solves;
    out->fallbacks = ps.fallbacks;
    out->iterations = ps.total_iterations;
    out->max_iterations = ps.max_iterations;
    out->last_iterations = ps.iterations;
    out->max_rel_residual = ps.max_rel_residual;
    out->last_rel_residual = ps.rel_residual;
    // the iteration trace of the last solve (SFG_TRACE_PCG=1), written to SFG_TRACE_PCG_FILE
    const char* path = std::getenv("SFG_TRACE_PCG_FILE");
    if (h->pcg.trace && path) {
      std::vector<unsigned long long> tr(1 + 4 * size_t(h->pcg.trace_cap));
      SFG_CUDA(cudaMemcpy(tr.data(), h->pcg.trace, tr.size() * 8, cudaMemcpyDeviceToHost));
      if (FILE* fo = std::fopen(path, "wb")) {
        std::fwrite(tr.data(), 8, tr.size(), fo);
        std::fclose(fo);
      }
    }
  });
}

}  // extern "C"

namespace sfg {
namespace {
template <typename T>
void StepError(sfg_handle* h, double* rel_step_error, int32_t* iterations, double* rel_residual) {
  cudaStream_t s = h->stream;
  const int64_t N = h->P.N, nB = h->SL.nB;
  PcgState saved;
  SFG_CUDA(cudaMemcpy(&saved, h->ps, sizeof(saved), cudaMemcpyDeviceToHost));
  LaunchDamping<T>(h->damp, h->hess, h->L.nvals, h->params, h->st, s);
  LaunchSchurPoints<T>(h->sd, h->hess, h->rhs, h->L.nvals, N, h->damp.damping, h->cinv, h->W, h->tp,
                       h->st, s);
  LaunchSchurBuildS<T>(h->sd, h->hess, h->L.nvals, h->damp.damping, h->W, h->S, h->st, s);
  LaunchSchurRhs<T>(h->sd, h->hess, h->L.nvals, h->rhs, N, h->tp, h->v, h->st, s);
  EnqueuePrecond<T>(h, s);
  if (h->pcg.coarse) LaunchGaugeBasis<T>(h->pcg, h->values, h->P.S, h->st, s);
  SFG_CUDA(LaunchPcg<T>(h->pcg, h->pcg_grid, h->pcg_threads, s));
  std::vector<double> ypcg(nB), yex(nB);
  SFG_CUDA(cudaMemcpyAsync(ypcg.data(), h->ydbl, nB * 8, cudaMemcpyDeviceToHost, s));
  PcgState ps;
  SFG_CUDA(cudaMemcpyAsync(&ps, h->ps, sizeof(ps), cudaMemcpyDeviceToHost, s));
  SFG_CUDA(cudaStreamSynchronize(s));
  EnqueueFactor<T>(h->fp, h->S, nullptr, s);
  EnqueueSolve<T>(h->fp, h->v, h->y, s);
  if (sizeof(T) == 8) LaunchWiden<double>(h->y, h->ydbl, nB, s);
  else EnqueueRefinement<T>(h, h->S, nullptr, h->v, h->y, s);
  SFG_CUDA(cudaMemcpyAsync(yex.data(), h->ydbl, nB * 8, cudaMemcpyDeviceToHost, s));
  SFG_CUDA(cudaMemcpyAsync(h->ps, &saved, sizeof(saved), cudaMemcpyHostToDevice, s));
  SFG_CUDA(cudaStreamSynchronize(s));
  SFG_CUDA(cudaGetLastError());
  LmState st;
  SFG_CUDA(cudaMemcpy(&st, h->st, sizeof(st), cudaMemcpyDeviceToHost));
  if (st.device_error) throw Error(SFG_ERR_DEVICE_STATUS, "device loop hit its cap");
  double num = 0, den = 0;
  for (int64_t i = 0; i < nB; ++i) {
    num += (ypcg[i] - yex[i]) * (ypcg[i] - yex[i]);
    den += yex[i] * yex[i];
  }
  if (rel_step_error) *rel_step_error = den > 0 ? std::sqrt(num / den) : std::sqrt(num);
  if (iterations) *iterations = ps.iterations;
  if (rel_residual) *rel_residual = ps.rel_residual;
}
}  // namespace
}  // namespace sfg

extern "C" {

int32_t sfg_pcg_step_error(sfg_handle* h, double* rel_step_error, int32_t* iterations,
                           double* rel_residual) {
  return Guard([&] {
    if (!h) throw Error(SFG_ERR_INVALID_ARGUMENT, "null handle");
    if (!h->pcg_mode) throw Error(SFG_ERR_INVALID_ARGUMENT, "handle is not a PCG form");
    if (!h->have_graph) throw Error(SFG_ERR_INVALID_ARGUMENT, "call sfg_optimize first");
    SFG_CUDA(cudaSetDevice(h->device));
    if (h->elem == 8) sfg::StepError<double>(h, rel_step_error, iterations, rel_residual);
    else sfg::StepError<float>(h, rel_step_error, iterations, rel_residual);
  });
}

int32_t sfg_set_preconditioner_weights(sfg_handle* h, const float* weights, int64_t n) {
  return Guard([&] {
    if (!h || !weights) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    if (n != sfg::kPrecondParams)
      throw Error(SFG_ERR_INVALID_ARGUMENT, "expected " + std::to_string(sfg::kPrecondParams) + " weights");
    if (h->pcg_mode != 2) throw Error(SFG_ERR_INVALID_ARGUMENT, "handle is not the learned PCG form");
    SFG_CUDA(cudaSetDevice(h->device));
    SFG_CUDA(cudaMemcpyAsync(h->net, weights, size_t(n) * 4, cudaMemcpyHostToDevice, h->stream));
    SFG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int32_t sfg_collect_samples(sfg_handle* h, int32_t max_systems) {
  return Guard([&] {
    if (!h) throw Error(SFG_ERR_INVALID_ARGUMENT, "null handle");
    if (max_systems < 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "max_systems must be >= 0");
    SFG_CUDA(cudaSetDevice(h->device));
    if (max_systems > h->collect_cap) {
      sfg::EnsurePrecond(h);
      h->samples = static_cast<float*>(h->arena.Alloc(size_t(max_systems) * std::max(h->pd.ng, 1) *
                                                      sfg::kSampleFloats * 4));
    }
    h->collect_cap = max_systems;
    h->have_graph = false;
  });
}

int32_t sfg_get_samples(sfg_handle* h, float* samples, int64_t cap, int64_t* count) {
  return Guard([&] {
    if (!h || !count) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    *count = 0;
    if (h->collect_cap == 0) return;
    SFG_CUDA(cudaSetDevice(h->device));
    sfg::LmState st;
    SFG_CUDA(cudaMemcpy(&st, h->st, sizeof(st), cudaMemcpyDeviceToHost));
    const int systems = std::min(std::max(st.num_records - 1, 0), h->collect_cap);
    const int64_t n = int64_t(systems) * h->pd.ng;
    *count = n;
    if (!samples) return;
    if (cap < n) throw Error(SFG_ERR_CAPACITY, "samples buffer too small");
    SFG_CUDA(cudaMemcpy(samples, h->samples, size_t(n) * sfg::kSampleFloats * 4, cudaMemcpyDeviceToHost));
  });
}

// ---- standalone SparseCholeskySolver / SparseSchurSolver: provided by api_solvers.cu
}  // extern "C"
