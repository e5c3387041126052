// sfg_dense_ldlt_solve_noalloc: a dense LDL^T solve that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a solve: code running
// under an allocator that forbids cudaMalloc (a custom pool, or a real-time loop that must not
// synchronize the device the way cudaMalloc / cudaFree can), and plugins that only ever receive
// pointers from their host application.  This entry point keeps its working memory in fixed-size
// file-scope device arrays (below) instead: the factor front, the diagonal-tile inverses, the tile
// version counters, the task list and the solve vectors.  Every GPU that loads the library holds
// these arrays (about 2.2 MB) until the process exits.
//
// It runs the same persistent tile-task factorization and triangular-solve kernels as
// sfg_ldlt_factorize / sfg_ldlt_solve, on one dense front (no ordering, no assembly lists).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "kernels.h"

namespace sfg {
extern thread_local std::string g_last_error;
}

namespace {

constexpr int kMaxN = 512;                       // largest system this entry point accepts
constexpr int kTile = sfg::kFactorTileF64;       // the FP64 tile of the factorization kernel
constexpr int kMaxTiles = kMaxN / kTile;
constexpr int kMaxStates = kMaxTiles * (kMaxTiles + 1) / 2;
constexpr int kMaxTasks = kMaxTiles * (kMaxTiles + 1) * (kMaxTiles + 2) / 6 + kMaxTiles;

// ---- the scratch: one copy per device, shared by every call ------------------------------------
struct NoAllocMeta {
  sfg::LmState st;          // the kernels read init_idx from a state block (always 0 here)
  int counters[2];
  int front_flags[2];
  int error;
  int32_t sn_w[1], sn_m[1], tile_base[2], npiv[1], ntiles[1], col_base[2], child_ptr[2], parent[1];
  int32_t child_list[1], rel[1];
  int64_t sn_foff[1], a_ptr[2], e_rptr[2], e_round[1], linv_base[2], rel_off[2], idx_off[2];
  int64_t a_src[1], e_src[1];
  int32_t a_dst[1], a_damp[1], e_dst[1];
};
static __device__ __align__(256) double g_front[kMaxN * kMaxN];
static __device__ __align__(256) double g_linv[kMaxTiles * kTile * kTile];
static __device__ __align__(256) double g_vec[3 * kMaxN];  // ysave, xperm, ycon
static __device__ __align__(256) int g_tile_state[kMaxStates];
static __device__ __align__(256) int4 g_tasks[kMaxTasks];
static __device__ __align__(256) int32_t g_ident[kMaxN];
static __device__ __align__(256) NoAllocMeta g_meta;

// Device addresses of the scratch, looked up once per device.
struct Scratch {
  bool ready = false;
  double* front;
  double* linv;
  double* vec;
  int* tile_state;
  int4* tasks;
  int32_t* ident;
  NoAllocMeta* meta;
};
constexpr int kMaxDevices = 64;
Scratch g_scratch[kMaxDevices];
std::mutex g_scratch_mutex;

int SetupScratch(int device, Scratch** out) {
  if (device < 0 || device >= kMaxDevices) {
    sfg::g_last_error = "device ordinal out of range";
    return SFG_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  Scratch& s = g_scratch[device];
  if (!s.ready) {
    struct Entry {
      void** dst;
      const void* symbol;
    } entries[] = {
        {reinterpret_cast<void**>(&s.front), reinterpret_cast<const void*>(&g_front)},
        {reinterpret_cast<void**>(&s.linv), reinterpret_cast<const void*>(&g_linv)},
        {reinterpret_cast<void**>(&s.vec), reinterpret_cast<const void*>(&g_vec)},
        {reinterpret_cast<void**>(&s.tile_state), reinterpret_cast<const void*>(&g_tile_state)},
        {reinterpret_cast<void**>(&s.tasks), reinterpret_cast<const void*>(&g_tasks)},
        {reinterpret_cast<void**>(&s.ident), reinterpret_cast<const void*>(&g_ident)},
        {reinterpret_cast<void**>(&s.meta), reinterpret_cast<const void*>(&g_meta)},
    };
    for (const Entry& e : entries) {
      const cudaError_t rc = cudaGetSymbolAddress(e.dst, e.symbol);
      if (rc != cudaSuccess) {
        sfg::g_last_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(rc);
        return SFG_ERR_CUDA;
      }
    }
    s.ready = true;
  }
  *out = &s;
  return SFG_OK;
}

// Copy the lower triangle of A into the front, reset the counters, and write the task list of one
// dense front (panels: diagonal tile, panel solves, trailing updates; no assembly tasks, since the
// tiles start out assembled).  One block per column of A (n blocks): block c copies column c's lower
// part and, for c < nt, writes panel c's tasks from its closed-form offset in the list; block 0
// also writes the plan's scalars.
__global__ void PrepareKernel(int n, const double* A, int64_t lda) {
  const int nt = (n + kTile - 1) / kTile;
  const int c = blockIdx.x;
  for (int r = c + threadIdx.x; r < n; r += blockDim.x) g_front[r + int64_t(c) * n] = A[r + int64_t(c) * lda];
  if (c < nt && threadIdx.x == 0) {
    // tasks of the panels before k: 1 + (nt - k' - 1) + (nt - k' - 1)(nt - k') / 2 each
    int t = 0;
    for (int k = 0; k < c; ++k) t += 1 + (nt - k - 1) + (nt - k - 1) * (nt - k) / 2;
    const int k = c;
    g_tasks[t++] = make_int4(sfg::kTaskDiag, 0, k * 65536 + k, k);
    for (int i = k + 1; i < nt; ++i) g_tasks[t++] = make_int4(sfg::kTaskTrsm, 0, i * 65536 + k, k);
    for (int j = k + 1; j < nt; ++j)
      for (int i = j; i < nt; ++i) g_tasks[t++] = make_int4(sfg::kTaskUpdate, 0, i * 65536 + j, k);
  }
  if (c != 0) return;
  for (int q = threadIdx.x; q < nt * (nt + 1) / 2; q += blockDim.x) g_tile_state[q] = 1;
  for (int q = threadIdx.x; q < n; q += blockDim.x) g_ident[q] = q;
  if (threadIdx.x == 0) {
    NoAllocMeta& m = g_meta;
    m.st = sfg::LmState{};
    m.counters[0] = m.counters[1] = 0;
    m.front_flags[0] = m.front_flags[1] = 0;
    m.error = 0;
    m.sn_w[0] = n;
    m.sn_m[0] = n;
    m.sn_foff[0] = 0;
    m.tile_base[0] = 0;
    m.tile_base[1] = nt * (nt + 1) / 2;
    m.npiv[0] = nt;
    m.ntiles[0] = nt;
    m.col_base[0] = 0;
    m.col_base[1] = nt;
    m.child_ptr[0] = m.child_ptr[1] = 0;
    m.parent[0] = -1;
    m.a_ptr[0] = m.a_ptr[1] = 0;
    m.e_rptr[0] = m.e_rptr[1] = 0;
    m.e_round[0] = 0;
    m.linv_base[0] = 0;
    m.linv_base[1] = int64_t(nt) * kTile * kTile;
    m.rel_off[0] = m.rel_off[1] = 0;
    m.idx_off[0] = 0;
    m.idx_off[1] = n;
  }
}

// After the solve: a zero or non-finite pivot (D, on the front's diagonal) or a non-finite solution
// entry marks the factorization as failed (error word 3; the capped waits use 1 and 2).  The
// unpivoted LDL^T then divided by zero or carried an overflow into x.
constexpr int kNoAllocBadPivot = 3;
__global__ void CheckPivotsKernel(int n, const double* x) {
  bool bad = false;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const double d = g_front[q + int64_t(q) * n];
    bad = bad || d == 0.0 || !isfinite(d) || !isfinite(x[q]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0 && g_meta.error == 0) g_meta.error = kNoAllocBadPivot;
}

int TaskCount(int nt) {
  int t = 0;
  for (int k = 0; k < nt; ++k) t += 1 + (nt - k - 1) + (nt - k - 1) * (nt - k) / 2;
  return t;
}

}  // namespace

extern "C" int32_t sfg_dense_ldlt_solve_noalloc(int32_t n, const double* A, int64_t lda,
                                                const double* b, double* x, void* stream) {
  if (n <= 0 || n > kMaxN) {
    sfg::g_last_error = "sfg_dense_ldlt_solve_noalloc: n = " + std::to_string(n) +
                        " is outside 1.." + std::to_string(kMaxN) + " (the size of its fixed scratch)";
    return SFG_ERR_INVALID_ARGUMENT;
  }
  if (!A || !b || !x || lda < n) {
    sfg::g_last_error = "sfg_dense_ldlt_solve_noalloc: null pointer or lda < n";
    return SFG_ERR_INVALID_ARGUMENT;
  }
  int device = 0;
  cudaError_t rc = cudaGetDevice(&device);
  if (rc != cudaSuccess) {
    sfg::g_last_error = std::string("cudaGetDevice: ") + cudaGetErrorString(rc);
    return SFG_ERR_NO_DEVICE;
  }
  Scratch* s = nullptr;
  const int32_t setup = SetupScratch(device, &s);
  if (setup != SFG_OK) return setup;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nt = (n + kTile - 1) / kTile;
  const int ntasks = TaskCount(nt);
  NoAllocMeta* m = s->meta;
  sfg::FactorDev f{};
  f.ns = 1;
  f.ntasks = ntasks;
  f.tile = kTile;
  f.tasks = s->tasks;
  f.sn_w = m->sn_w;
  f.sn_m = m->sn_m;
  f.sn_foff = m->sn_foff;
  f.tile_base = m->tile_base;
  f.npiv = m->npiv;
  f.ntiles = m->ntiles;
  f.col_base = m->col_base;
  f.a_ptr = m->a_ptr;
  f.a_src = m->a_src;
  f.a_dst = m->a_dst;
  f.a_damp = m->a_damp;
  f.e_rptr = m->e_rptr;
  f.e_round = m->e_round;
  f.e_src = m->e_src;
  f.e_dst = m->e_dst;
  f.linv_base = m->linv_base;
  f.trace = nullptr;
  f.rel_off = m->rel_off;
  f.rel = m->rel;
  f.child_ptr = m->child_ptr;
  f.child_list = m->child_list;
  f.parent = m->parent;
  f.idx_off = m->idx_off;
  f.idx = s->ident;
  f.scalar_old = s->ident;
  f.tile_state = s->tile_state;
  f.counters = m->counters;
  f.front_flags = m->front_flags;
  f.error = &m->error;
  f.max_m = n;
  f.st = &m->st;
  f.a_stride = 0;
  f.b_stride = 0;
  if (ntasks > kMaxTasks) {
    sfg::g_last_error = "sfg_dense_ldlt_solve_noalloc: task list exceeds its scratch";
    return SFG_ERR_CAPACITY;
  }
  PrepareKernel<<<n, 128, 0, st>>>(n, A, lda);
  sfg::LaunchFactor<double>(f, s->front, nullptr, s->front, s->linv,
                            std::max(1, std::min(ntasks, sms * 8)), st);
  sfg::LaunchSolve<double>(f, s->front, s->linv, b, s->vec + 2 * kMaxN, s->vec, s->vec + kMaxN, x, nullptr,
                           std::max(1, std::min(2, sms)), st);
  CheckPivotsKernel<<<1, 256, 0, st>>>(n, x);
  rc = cudaGetLastError();
  if (rc != cudaSuccess) {
    sfg::g_last_error = std::string("sfg_dense_ldlt_solve_noalloc launch: ") + cudaGetErrorString(rc);
    return SFG_ERR_CUDA;
  }
  // The call is synchronous: it copies the device status word to the host and waits for `stream`
  // before it returns, so that a capped dependency wait or a failed pivot is reported as a status.
  int err = 0;
  rc = cudaMemcpyAsync(&err, &m->error, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (rc == cudaSuccess) rc = cudaStreamSynchronize(st);
  if (rc != cudaSuccess) {
    sfg::g_last_error = std::string("sfg_dense_ldlt_solve_noalloc: ") + cudaGetErrorString(rc);
    return SFG_ERR_CUDA;
  }
  if (err == kNoAllocBadPivot) {
    sfg::g_last_error = "sfg_dense_ldlt_solve_noalloc: zero or non-finite pivot (A is singular or "
                        "not factorizable without pivoting)";
    return SFG_ERR_NUMERICAL;
  }
  if (err != 0) {
    sfg::g_last_error = "sfg_dense_ldlt_solve_noalloc: a device wait hit its cap";
    return SFG_ERR_DEVICE_STATUS;
  }
  return SFG_OK;
}
