// Shared definitions of the GB300 LM back end: problem layout on the host, device-side plain
// structs, and error helpers.  Host code is C++17; device code is CUDA for sm_103a.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sfgpu.h"
#include "device.cuh"
#include "generated_factor_specs.h"

namespace sfg {

// Error carried from host helpers to the C ABI boundary, where it becomes a status code.
struct Error : std::runtime_error {
  int32_t code;
  Error(int32_t c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define SFG_CUDA(call)                                                                         \
  do {                                                                                         \
    cudaError_t e__ = (call);                                                                  \
    if (e__ != cudaSuccess)                                                                    \
      throw ::sfg::Error(SFG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__) +   \
                                           " (" + __FILE__ + ":" + std::to_string(__LINE__) + ")"); \
  } while (0)

inline void KeyDims(int type, int* sdim, int* tdim) {
  switch (type) {
    case SFG_KEY_VEC1: *sdim = 1; *tdim = 1; return;
    case SFG_KEY_VEC2: *sdim = 2; *tdim = 2; return;
    case SFG_KEY_VEC3: *sdim = 3; *tdim = 3; return;
    case SFG_KEY_POSE2: *sdim = 4; *tdim = 3; return;
    case SFG_KEY_POSE3: *sdim = 7; *tdim = 6; return;
    case SFG_KEY_ROT3: *sdim = 4; *tdim = 3; return;
    case SFG_KEY_VEC4: *sdim = 4; *tdim = 4; return;
    case SFG_KEY_VEC5: *sdim = 5; *tdim = 5; return;
    case SFG_KEY_VEC6: *sdim = 6; *tdim = 6; return;
  }
  throw Error(SFG_ERR_INVALID_ARGUMENT, "unknown key type " + std::to_string(type));
}

struct FactorSpec {
  int nkeys, nconsts, rdim;
  int key_types[3];
};

inline FactorSpec Spec(int kind) {
  switch (kind) {
    case SFG_FACTOR_BEARING_POSE2: return {1, 5, 1, {SFG_KEY_POSE2, 0, 0}};
    case SFG_FACTOR_ODOMETRY_POSE2: return {2, 3, 1, {SFG_KEY_POSE2, SFG_KEY_POSE2, 0}};
    case SFG_FACTOR_SNAVELY_REPROJECTION: return {3, 4, 2, {SFG_KEY_POSE3, SFG_KEY_VEC3, SFG_KEY_VEC3}};
    case SFG_FACTOR_BETWEEN_POSE3: return {2, 14, 6, {SFG_KEY_POSE3, SFG_KEY_POSE3, 0}};
    case SFG_FACTOR_PRIOR_POSE3: return {1, 14, 6, {SFG_KEY_POSE3, 0, 0}};
    case SFG_FACTOR_RANGE_POSE3: return {1, 6, 1, {SFG_KEY_POSE3, 0, 0}};
#define SFG_GENERATED_SPEC(KIND, NKEYS, NCONSTS, RDIM, K0, K1, K2, G) \
    case KIND: return {NKEYS, NCONSTS, RDIM, {K0, K1, K2}};
    SFG_GENERATED_FACTORS(SFG_GENERATED_SPEC)
#undef SFG_GENERATED_SPEC
  }
  throw Error(SFG_ERR_INVALID_ARGUMENT, "unknown factor kind " + std::to_string(kind));
}

// Leading key slots whose J^T J / J^T r entries a warp of the linearization kernel sums before
// storing, when all 32 of its factors share those keys (the factors of such a kind are ordered by
// these keys on the device).  Snavely reprojection: the camera's pose and calibration, seen by
// hundreds of observations each.  The factor traits of the kernel carry the same number.
constexpr int MergedKeySlots(int kind) { return kind == SFG_FACTOR_SNAVELY_REPROJECTION ? 2 : 0; }

// ---------------------------------------------------------------------------------------------
// Host problem
// ---------------------------------------------------------------------------------------------
struct HostBatch {
  int kind = 0, count = 0, nk = 0, nc = 0, rdim = 0, tdim = 0;
  std::vector<int32_t> keys;     // [count * nk] factor-major (as given)
  std::vector<double> consts;    // [count * nc] factor-major (as given)
  std::vector<int> key_tdim;     // tangent dim of each key slot
  int64_t roff = 0;              // first residual row of the batch
  int64_t first_factor = 0;      // global index of the first factor of the batch
};

struct HostProblem {
  int nkeys = 0;
  std::vector<int> key_type, sdim, tdim;
  std::vector<int64_t> soff, toff;
  int64_t S = 0, N = 0, M = 0, F = 0;
  std::vector<HostBatch> batches;
  int num_schur = 0;  // trailing keys eliminated by Schur complement
};

HostProblem ParseProblem(const sfg_problem_t* p);

// ---------------------------------------------------------------------------------------------
// Block-sparse symmetric matrix structure: key blocks (i >= j) stored dense row-major d_i x d_j,
// blocks ordered by column then row.  Diagonal blocks are stored full.
// ---------------------------------------------------------------------------------------------
struct BlockPattern {
  int nb = 0;
  std::vector<int> dim;            // [nb]
  std::vector<int64_t> off;        // scalar offset of each block row/col [nb + 1]
  std::vector<int64_t> colptr;     // [nb + 1] into rows/boff
  std::vector<int32_t> rows;       // block row index of each stored block
  std::vector<int64_t> boff;       // value offset of each stored block (+1 sentinel)
  int64_t Find(int i, int j) const;  // stored block index of (i, j), i >= j, or -1
  int64_t nvals() const { return boff.empty() ? 0 : boff.back(); }
  int64_t nblocks() const { return int64_t(rows.size()); }
};

// Build a pattern from a list of (i, j) lower block pairs (duplicates allowed); all diagonal
// blocks are included.
BlockPattern MakePattern(const std::vector<int>& dims, std::vector<std::pair<int, int>> pairs);

// ---------------------------------------------------------------------------------------------
// Supernodal symbolic factorization of a BlockPattern (block level), consumed by the device
// multifrontal LDL^T.  Fronts are dense, column-major, m x m, first w columns pivots.
// ---------------------------------------------------------------------------------------------
struct Symbolic {
  int nb = 0;
  int64_t n = 0;                       // scalar dimension
  std::vector<int32_t> border;         // block order: border[new] = old block
  std::vector<int32_t> bperm;          // bperm[old] = new
  std::vector<int64_t> pstart;         // scalar start of each NEW block [nb + 1]
  // supernodes in postorder (children before parents)
  int ns = 0;
  std::vector<int32_t> sn_first, sn_last;  // new block range [first, last]
  std::vector<int32_t> sn_parent;          // -1 for roots
  std::vector<int32_t> sn_w, sn_h, sn_m;   // scalar pivot width, below height, front size
  std::vector<int64_t> sn_foff;            // front offset in the front pool (entries)
  std::vector<std::vector<int32_t>> sn_rows;  // row blocks below (new indices), ascending
  std::vector<std::vector<int32_t>> sn_children;
  int64_t front_pool = 0;
  // scalar index list of each front (new scalar indices), length m
  std::vector<int64_t> idx_off;        // [ns + 1] into idx
  std::vector<int32_t> idx;
  // relative positions of each child's update rows inside its parent front
  std::vector<int64_t> rel_off;        // [ns + 1] into rel (length h of the child)
  std::vector<int32_t> rel;
  // original matrix blocks assembled into each front
  struct Asm {
    int64_t src;   // value offset of the stored block (row-major d_i x d_j)
    int32_t row0, col0;  // position of the block inside the front (scalar)
    int16_t di, dj;      // stored block dims (rows, cols) as stored
    int16_t transpose;   // 1: place block^T (stored block is above the diagonal after ordering)
    int16_t diag;        // 1: diagonal block (lower triangle only)
    int32_t oi, oj;      // original block row / column
  };
  std::vector<int64_t> asm_off;        // [ns + 1]
  std::vector<Asm> asms;
  int64_t nnz_L = 0;                   // scalar nonzeros of L below the diagonal (incl. explicit zeros)
  double flops = 0;                    // multiply-add count of the numeric factorization
};

Symbolic Analyze(const BlockPattern& A, int ordering);

// Tile task list for the persistent factorization kernel.
struct TaskPlan {
  int tile = 16;
  std::vector<int32_t> tile_base;   // [ns + 1] first tile-state index of each front
  std::vector<int32_t> ntiles;      // tiles per front dimension
  std::vector<int32_t> npiv;        // pivot tiles per front
  std::vector<int4> tasks;          // {type, front, i << 16 | j, k}
  int32_t nstates = 0;
  std::vector<int32_t> asm_col_base;  // [ns + 1]
  std::vector<int64_t> asm_col_off;   // per (front, tile column)
  std::vector<int32_t> asm_col_list;
};
// separate_inverse: FP64 chains leave the diagonal tiles' inverses to kTaskInverse tasks;
// tc_updates: runs of trailing updates go to tensor-core tasks (FP32 tiles of 32).
TaskPlan PlanTasks(const Symbolic& sym, int tile, bool separate_inverse, bool tc_updates);

// Split of the front triangular solves over CTAs: a front with more tiles than a solve CTA has
// warps gets kp pivot-block CTAs of block_tiles pivot tiles and ku CTAs of as many update-row tiles
// (kp = 0: one CTA per direction).  Tasks are (front, sub-task): forward ones in front order (a
// front's blocks in order, then its update CTAs), then backward ones in reverse front order (a
// front's blocks from the last one down), so that every sub-task waits only on lower task numbers.
// Empty task lists when no front is split.
struct SolveSplit {
  std::vector<int32_t> kp, ku, task_front, task_sub;
  int nf = 0;  // forward tasks
};
SolveSplit PlanSolveSplit(const TaskPlan& plan, int ns, int warps, int block_tiles, bool split);

// Flattened per-(front, tile column) assembly lists, extend-add rounds and solve maps of a
// symbolic factorization and its task plan, as the device kernels read them.
struct FactorMaps {
  std::vector<int64_t> a_ptr, a_src;   // [slots + 1]; source value of each assembled entry
  std::vector<int32_t> a_dst, a_damp;  // front position (r + c m); damping index or -1
  std::vector<int64_t> e_rptr;         // [slots + 1] rounds of each slot
  std::vector<int64_t> e_round;        // [rounds + 1] entries of each round
  std::vector<int64_t> e_src;          // child front entry (front pool index)
  std::vector<int32_t> e_dst;          // parent front position
  std::vector<int64_t> linv_base;      // [ns + 1] pivot-tile inverses of each front
  std::vector<int32_t> child_ptr, child_list;
  std::vector<int32_t> scalar_old;     // [n] original scalar of each new scalar
};
FactorMaps BuildFactorMaps(const Symbolic& S, const TaskPlan& T, const BlockPattern& pat);

}  // namespace sfg
