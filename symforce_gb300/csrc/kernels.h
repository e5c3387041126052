// Host-callable launchers of the device kernels (one definition per .cu file).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/sfgpu.h"
#include "device.cuh"

namespace sfg {

// Resident CTAs per SM the persistent factorization kernel is compiled for (its register budget:
// 65,536 / (CTAs x 128 threads) a thread): 4 (128 registers; FP32, and FP64 plans of few fronts,
// whose chains set the time), and 8 for FP64 plans of many fronts (FactorDev::wide: 64
// registers, twice the trailing updates in flight; 1,000 cameras, 32 fronts: 3.34 -> 3.07 ms; one
// 450-wide front: 0.343 -> 0.353 ms).
constexpr int kFactorCtasPerSm = 4;
constexpr int kFactorCtasPerSmWide = 8;
constexpr int kFactorWideFronts = 8;  // FP64 plans of at least this many fronts run wide
// Tile edge of the factorization.  The critical path of a front is pivots x pivot latency (a chain
// of dependent FP64 operations, 64 cycles each on this GPU) plus panels x per-panel hand-offs;
// measured on the 450-unknown reduced system, FP64 tiles of 8 and 16 give the same factor time
// (0.66 ms), and 16 keeps the task list 7x shorter.
constexpr int kFactorTileF64 = 16;
constexpr int kFactorTileF32 = 32;

// ---------------------------------------------------------------- linearization (kernels_lin.cu)
// Evaluate every factor of a batch at the Init or New values, writing residual rows, packed
// Gauss-Newton Hessian / rhs entries (directly, or into staging when shared), and per-CTA cost
// partial sums.  T = double (plain form) or float (mixed form).
template <typename T>
void LaunchLinearize(int kind, const LinOut& out, const BatchDev& b, cudaStream_t s);
int LinearizeBlockSize();

// Sum staged contributions into shared Hessian / rhs destinations in a fixed order.
struct ReduceDev {
  int ngroups;
  const int32_t* dst;   // sink index (< nvals + N) of each group
  const int64_t* ptr;   // [ngroups + 1] range of the group's staging slots
};
template <typename T>
void LaunchReduceStage(const ReduceDev& r, const LinOut& out, cudaStream_t s);

// Cost of a state block: 0.5 * sum of the cost partials (fixed order, deterministic).
void LaunchFinishCost(const double* partials, int npartials, LmState* st, int which,
                      cudaStream_t s);

// ---------------------------------------------------------------- LM bookkeeping (kernels_lm.cu)
struct DampDev {
  int64_t N;
  const int64_t* diag_off;  // value offset of each tangent scalar's diagonal entry in H
  double* damping;          // [N]
  double* max_diagonal;     // [N]
};
template <typename T>
void LaunchDamping(const DampDev& d, const void* hess, int64_t nvals, const LmParams* p,
                   LmState* st, cudaStream_t s);

struct RetractDev {
  int nkeys;
  const int32_t* key_type;
  const int64_t* soff;
  const int64_t* toff;
  double* values;   // [3][S]
  int64_t S;
  const double* update;  // [N]
};
void LaunchRetract(const RetractDev& r, const LmParams* p, LmState* st, cudaStream_t s);

// Per-CTA partial sums of u.(rhs - d.u) (rhs of the Init block) and, for bold updates, of u.last,
// u.u and last.last; the decide kernel adds the partials in a fixed order.
template <typename T>
void LaunchLinearDelta(const double* update, const void* rhs, const double* damping,
                       const double* last_update, int64_t N, double* partials, LmState* st,
                       int bold, cudaStream_t s);
int DeltaPartials();

// The end of LevenbergMarquardtSolver::Iterate: stats record, accept / reject, lambda update,
// best tracking, state-index juggling, early exit; sets the graph's loop condition when use_cond
// (launched inside the optimize graph) and only the state's done flag otherwise.
void LaunchDecide(const LmParams* p, LmState* st, sfg_iteration_t* records, const double* update,
                  double* last_update, int64_t N, const double* delta_partials, int nparts,
                  cudaGraphConditionalHandle h, int use_cond, cudaStream_t s);
// Start of an optimize call: Reset + the first half of the first Iterate (Step).
void LaunchBegin(const LmParams* p, LmState* st, int reset_indices, cudaStream_t s);
// After the Init block has been linearized for the first time: initial record and the
// non-finite check (INITIAL_ERROR_NOT_FINITE).
void LaunchFirstRecord(const LmParams* p, LmState* st, sfg_iteration_t* records,
                       cudaGraphConditionalHandle h, int use_cond, cudaStream_t s);
void LaunchCopyValues(const double* src, double* values, int64_t S, const LmState* st, int which,
                      cudaStream_t s);
void LaunchCopyBest(const double* values, double* dst, int64_t S, const LmState* st, cudaStream_t s);

// ---------------------------------------------------------------- Schur + LDL^T (kernels_solve.cu)
struct SchurDev {
  int npoints;
  int nB;                       // scalar dimension of the reduced system
  int nBk;                      // keys of the reduced system
  const int32_t* bkey_toff;     // [nBk + 1] their tangent offsets
  int64_t c_toff;               // tangent offset of the first point
  const int64_t* pt_diag;       // H value offset of each point's 3x3 block
  const int64_t* pt_eptr;       // [np + 1] E blocks of each point
  const int32_t* pt_ekey_toff;  // tangent offset of the B key of each E block
  const int32_t* pt_ekey_dim;   // dim of that key
  const int64_t* pt_eoff;       // H value offset of E block (3 x d_k, row-major)
  const int64_t* pt_woff;       // G = L^-1 E offset (3 x d_k) of each E block in the G buffer
  const int64_t* e_order;       // optional: the order the G kernel takes the E blocks in (null: 0, 1, ...)
  int64_t nE;                   // E blocks (pt_eptr[npoints])
  const int32_t* pt_of_e;       // [nE] point of each E block
  int nsblocks;
  const int64_t* sb_ptr;        // [nsblocks + 1] terms of each S block
  const int64_t* sb_eoff;       // G_pk offset (G buffer, E's layout) per term
  const int64_t* sb_woff;       // G_pl offset (G buffer, E's layout) per term
  const int64_t* sb_hoff;       // H value offset of the B block (-1: none)
  const int64_t* sb_soff;       // S value offset of the block
  const int32_t* sb_dk;         // rows of the block
  const int32_t* sb_dl;         // cols
  const int32_t* sb_diag_toff;  // tangent offset of the key if diagonal block, else -1
  // the S-block terms cut into chunks of at most chunk_terms (one warp each), partial sums per chunk
  int nchunks;
  int chunk_terms;
  const int32_t* ch_block;      // [nchunks] S block of the chunk
  const int64_t* ch_begin;      // [nchunks] first term of the chunk
  const int64_t* sb_chunk_ptr;  // [nsblocks + 1] chunks of each S block
  void* partials;               // T [nchunks][36] chunk sums (row-major 6 x 6)
  const int64_t* r_ptr;         // [nB + 1] points of each B scalar
  const int64_t* r_eoff;        // E block offset per entry (column of the scalar inside E)
  const int32_t* r_ecol;        // column inside the E block
  const int32_t* r_dk;          // E block column count
  const int32_t* r_pt;          // point index
};
template <typename T>
void LaunchSchurPoints(const SchurDev& d, const void* hess, const void* rhs, int64_t nvals,
                       int64_t N, const double* damping, void* cinv, void* W, void* tp,
                       const LmState* st, cudaStream_t s);
template <typename T>
void LaunchSchurBuildS(const SchurDev& d, const void* hess, int64_t nvals, const double* damping,
                       const void* W, void* S, const LmState* st, cudaStream_t s);
template <typename T>
void LaunchSchurRhs(const SchurDev& d, const void* hess, int64_t nvals, const void* rhs, int64_t N,
                    const void* tp, void* v, const LmState* st, cudaStream_t s);
// y: the reduced-system solution in FP64.
template <typename T>
void LaunchSchurBackSub(const SchurDev& d, const void* y, const void* W, const void* tp, const void* cinv,
                        double* update, cudaStream_t s);

// Symmetric block-sparse matrix-vector product layout (per scalar row: segments of a stored block
// row, or of a stored block column for the mirrored upper part).
struct SpmvDev {
  int n;
  const int64_t* row_ptr;     // [n + 1]
  const int64_t* seg_base;    // value offset of the segment's first entry
  const int32_t* seg_stride;  // distance between consecutive entries (1: along a row)
  const int32_t* seg_len;
  const int32_t* seg_x;       // x index of the segment's first entry
  int64_t a_stride, b_stride; // per-state-block strides of the matrix / rhs (0: fixed buffers)
};
// `gate` (optional): the kernels do nothing unless *gate != 0 (the PCG forms run the exact
// solve only as a fallback).
template <typename T>
void LaunchRefineResidual(const SpmvDev& m, const void* A, const double* damping, const void* b,
                          const double* y, double* r, void* r_lo, const LmState* st, cudaStream_t s,
                          const int* gate = nullptr);
template <typename T>
void LaunchWiden(const void* x, double* y, int64_t n, cudaStream_t s, const int* gate = nullptr);
template <typename T>
void LaunchAccumulate(const void* dx, double* y, int64_t n, cudaStream_t s, const int* gate = nullptr);

struct FactorDev {
  int ns, ntasks, tile;
  const int4* tasks;
  const int32_t* sn_w;
  const int32_t* sn_m;
  const int64_t* sn_foff;
  const int32_t* tile_base;
  const int32_t* npiv;
  const int32_t* ntiles;
  // assembly, flattened per (front, tile column) slot; slot = col_base[front] + tile column
  const int32_t* col_base;       // [ns + 1]
  const int64_t* a_ptr;          // [nslots + 1] original entries of each slot
  const int64_t* a_src;          // value index in the assembled matrix
  const int32_t* a_dst;          // position inside the front (row + col * m)
  const int32_t* a_damp;         // scalar index into the damping vector, or -1
  const int64_t* e_rptr;         // [nslots + 1] rounds of child update entries of each slot
  const int64_t* e_round;        // round boundaries (entry indices), one past per slot's last
  const int64_t* e_src;          // absolute index into the front pool (child update entry)
  const int32_t* e_dst;          // position inside the front
  const int64_t* linv_base;      // [ns] offset of the front's pivot-tile inverses
  unsigned long long* trace;     // optional per-task timestamps (null: off)
  const int64_t* rel_off;
  const int32_t* rel;
  const int32_t* child_ptr;
  const int32_t* child_list;
  const int32_t* parent;
  const int64_t* idx_off;
  const int32_t* idx;         // new scalar indices of each front
  const int32_t* scalar_old;  // new scalar -> old scalar
  int* tile_state;
  int* counters;              // [0]: factor task counter, [1]: solve task counter
  int* front_flags;           // [2 * ns]: forward done, backward done
  int* error;                 // device error word
  int* fp64_tiles;            // optional: FP32 diagonal tiles factored again in FP64 (near-singular)
  int max_m;                  // largest front (solve kernel shared memory)
  const LmState* st;          // state whose Init block the matrix / rhs are read from
  int64_t a_stride;           // per-state-block stride of the matrix values (0: fixed)
  int64_t b_stride;           // per-state-block stride of the rhs (0: fixed)
  const int* gate;            // optional: the kernels return at once unless *gate != 0
  // optional: [kSmFlagSlots] per-SM flags (1: the SM is given to a chain task; its other CTAs
  // leave the kernel) followed by the count of SMs so given, at most iso_limit
  int* sm_flags = nullptr;
  int iso_limit = 0;
  int wide = 0;  // FP64: the build for kFactorCtasPerSmWide resident CTAs (the grid is sized to it)
  // optional: solves of wide fronts shared by several CTAs (null solve_front: one CTA per front and
  // direction).  Tasks [0, solve_nf) are forward (fronts in order), [solve_nf, solve_nf +
  // solve_nb) backward (fronts in reverse order); each is (front, sub-task).  Per front: solve_kp
  // pivot-block CTAs (0: the front is solved by one CTA) and solve_ku update-row CTAs.
  const int32_t* solve_front = nullptr;
  const int32_t* solve_sub = nullptr;
  const int32_t* solve_kp = nullptr;
  const int32_t* solve_ku = nullptr;
  int solve_nf = 0, solve_nb = 0;
};
constexpr int kSmFlagSlots = 512;
// Pivot tiles of one CTA of a split front solve (one per warp).
constexpr int kSolveBlockTiles = 4;
// Warps of a solve CTA.
int SolveWarps();
template <typename T>
void LaunchFactor(const FactorDev& f, const void* A, const double* damping, void* F, void* Linv,
                  int grid, cudaStream_t s);
// Solve (L D L^T) x = b for b in the original scalar order; x in the original order.  Linv: the
// inverses of the pivot tiles' unit lower factors that LaunchFactor wrote.
// xb: the backward exchange buffer (as large as ysave) of split solves, else unused.
template <typename T>
void LaunchSolve(const FactorDev& f, const void* F, const void* Linv, const void* b, void* ycon,
                 void* ysave, void* xperm, void* x, void* xb, int grid, cudaStream_t s);
int FactorThreads();
// One CTA waits (capped) for *flag >= 1 while nothing sets it; the cap sets *err.
cudaError_t LaunchWaitCapSelfTest(const int* flag, int* err, cudaStream_t s);
// `unset` (optional): n_unset values of elem bytes set to the split solves' unset pattern.
void LaunchResetFactorState(int* tile_state, int nstates, int* front_flags, int nflags,
                            int* counters, cudaStream_t s, const int* gate = nullptr,
                            void* unset = nullptr, int64_t n_unset = 0, int elem = 8);
template <typename T>
void LaunchNegate(const void* x, double* u, int64_t n, cudaStream_t s);
// Opt the solve kernel into the shared memory its largest front needs (call once per device).
template <typename T>
void ConfigureSolve(int max_m);

// ---------------------------------------------------------------- PCG forms (kernels_pcg.cu)
constexpr int kPrecondBlock = 9;
constexpr int kPrecondFeatures = 96;
constexpr int kPrecondHidden = 256;
constexpr int kPrecondTri = 45;
constexpr int kPrecondFac = kPrecondTri + kPrecondBlock;   // C (lower, packed) + D^-1/2
constexpr int kSampleFloats = kPrecondFeatures + 2 * kPrecondBlock;
constexpr int kPrecondParams = kPrecondFeatures * kPrecondHidden + kPrecondHidden +
                               kPrecondHidden * kPrecondHidden + kPrecondHidden +
                               kPrecondHidden * kPrecondTri + kPrecondTri;

// Camera blocks of the reduced system (groups of B keys that share factors).
struct PrecondDev {
  int ng;                       // blocks
  int nB;                       // scalar dimension of the reduced system
  const int32_t* gidx;          // [ng][9] reduced-system scalar of each block row, -1: padding
  const int64_t* goff;          // [ng][81] S value offset of (a, b); -1 padding, -2 not stored
  const float* degree;          // [ng] neighbouring blocks
  const int32_t* scalar_group;  // [nB] block of each scalar
  const int64_t* sdiag_off;     // [nB] S value offset of each diagonal entry
};
// Features of every block (and its scaled Cholesky factor); `rho` is scratch [nB].
template <typename T>
void LaunchPrecondFeatures(const PrecondDev& pd, const SpmvDev& m, const void* S, float* rho,
                           float* feats, float* fac, cudaStream_t s);
// Preconditioner blocks P_g (T, [ng][81]) from the factors and the network outputs (null: L = I).
template <typename T>
void LaunchPrecondAssemble(int ng, const float* fac, const float* z, void* P, cudaStream_t s);
// The network's inference pass on the tensor cores (tcgen05, TF32 with a three-pass split for FP32
// accuracy): z[n][45] from x[n][96] (row stride ldx floats), 96 -> 256 -> 256 -> 45 with ReLU;
// h1, h2: [n][256] scratch; a capped wait that gives up sets *err.
cudaError_t LaunchMlpInferTc(const float* x, int64_t ldx, int64_t n, const float* weights, float* h1, float* h2,
                             float* z, int* err, cudaStream_t s);
// Training samples of one system: [ng][114] at samples + slot * ng * 114, slot = the LM record
// index of the iteration, skipped when slot >= max_systems.
template <typename T>
void LaunchCollectSamples(const PrecondDev& pd, const float* feats, const float* fac, const void* v,
                          const double* y, float* samples, int max_systems, PcgState* ps,
                          const LmState* st, cudaStream_t s);

struct PcgDev {
  PrecondDev pd;
  const int32_t* gptr;      // [ng + 1] entries of each group row
  const int2* gent;         // {stored group block, neighbour << 1 | transposed}
  int nbl;                  // stored (lower) 9 x 9 group blocks
  const void* Sb;           // T [nbl][81] group blocks of S, row-major
  const void* v;            // T [nB] rhs (reduced-system order)
  const void* P;            // T [ng][81]
  double* y;                // [nB] FP64 solution (reduced-system order)
  double* yg;               // [ng][9] FP64 solution by group (read by the residual passes)
  void* z;                  // T [ng][9] preconditioned residual by group (read by the product)
  int staged;               // one CTA holding blocks, entries, z and y in shared memory: its
                            // dynamic shared memory bytes (0: blocks read from L2)
  double* partials;         // [2][grid][2] per-CTA partial sums (double buffered)
  unsigned* bar;            // [2] grid barrier arrival count (zeroed before each launch)
  PcgState* ps;
  int* err;                 // device error word
  double tol;               // FP64 relative residual target
  double inner_floor;       // smallest relative reduction asked of one inner solve
  int max_iters, max_outer;
  int split;                // lanes per row of a multi-CTA launch (1 or 3)
  // coarse correction on the camera poses' similarity gauge (coarse != 0): basis Z and S Z by
  // group row, column-major T [7][ng * 9] (Z from the current values, S Z by the PCG launch)
  int coarse;
  void* zg;
  void* szg;
  const int64_t* gauge_soff;  // [ng * 9] POSE3 storage offset of a pose row, -1 otherwise
  const int32_t* gauge_comp;  // [ng * 9] tangent component of a pose row
  // factorized sparse approximate inverse over `band` neighbouring groups (band > 0): the lower
  // band blocks of M = G^T Lambda G, T [ng][band + 1][81] (slot d: M_{g, g - d}, row-major), and
  // the residual and product of every row, interleaved (T2 [ng][9]), that the rows of M read from
  // the other CTAs
  int band = 0;
  const void* Mb = nullptr;
  void* RQ = nullptr;
  // optional iteration trace of CTA 0 (SFG_TRACE_PCG): [0] inner iterations of the last solve,
  // then per inner iteration (up to trace_cap) the %globaltimer after the product with S, after
  // the first grid reduction, after the preconditioner, after the second grid reduction
  unsigned long long* trace = nullptr;
  int trace_cap = 0;
};
constexpr int kGaugeDim = 7;      // world translation 3, rotation 3, scale 1
constexpr int kPcgMaxBand = 6;    // neighbouring groups of a band preconditioner row (9 (k + 1) <= 63)
// Pattern of the band preconditioner: per group row l the groups J_l (ascending, the last one l
// itself; nj[l] of them) and the stored S group block of every pair (J_l[s1], J_l[s2]), s1 >= s2,
// at jblk[l][s1 * (band + 1) + s2] (-1: a zero block).
struct BandDev {
  int ng = 0, band = 0;
  const int32_t* nj = nullptr;    // [ng]
  const int32_t* jgrp = nullptr;  // [ng][band + 1]
  const int32_t* jblk = nullptr;  // [ng][(band + 1)^2]
  const int32_t* gidx = nullptr;  // [ng][9] reduced-system scalar of each group row, -1 padding
  void* G = nullptr;              // T [ng][band + 1][81]: block (l, l - band + slot) of G
};
// G (block rows of the factorized approximate inverse) from the group blocks Sb of S.
template <typename T>
void LaunchBandFactor(const BandDev& b, const void* Sb, cudaStream_t s);
// The band blocks of M = G^T Lambda G (Lambda_l = L L^T from the network outputs z, or I when z
// is null) into Mb (T [ng][band + 1][81]).
template <typename T>
void LaunchBandAssemble(const BandDev& b, const float* z, void* Mb, cudaStream_t s);
constexpr int kPcgReduceMax = 32; // values one PCG grid reduction can carry
// Gather the 9 x 9 group blocks of S: Sb[q][e] = S[off[q][e]] (0 where off < 0).
template <typename T>
void LaunchGroupBlocks(const int64_t* off, int64_t n, const void* S, void* Sb, cudaStream_t s);
// The similarity-gauge basis Z (T [7][ng * 9]) of the camera poses at the state block init_idx of
// `values` (storage size `S` per block).
template <typename T>
void LaunchGaugeBasis(const PcgDev& d, const double* values, int64_t S, const LmState* st, cudaStream_t s);
// Shared memory of a staged (one CTA) PCG launch; 0 if the blocks do not fit.
template <typename T>
size_t PcgStagedSmem(int ng, int nbl, int nent);
// Opt the staged PCG kernel into its shared memory (once per device).
template <typename T>
void ConfigurePcg();
// Launch shape of the PCG kernel for ng camera blocks: grid (cooperative when > 1, all CTAs
// resident), threads and lanes per row (1 or 3); throws if the CTAs do not fit on the device.
template <typename T>
void PcgShape(int ng, int num_sms, int* grid, int* threads, int* split);
template <typename T>
cudaError_t LaunchPcg(const PcgDev& d, int grid, int threads, cudaStream_t s);
void LaunchPcgBegin(PcgState* ps, cudaStream_t s);

// ---------------------------------------------------------------- batched problems (kernels_batch.cu)
// Doubles of one warp slot's workspace per pose of the largest problem.
constexpr int kBatchWsPerPose = 3 * 7 + 3 * 36 + 3 * 36 + 3 * 6 + 27 + 27 + 6 + 6 + 6 + 6 + 36 + 36 + 6;

struct BatchLmDev {
  int nprob;
  int nmax;                    // poses of the largest problem
  const int32_t* order;        // problems, largest first
  const int32_t* n;            // poses per problem
  const int64_t* pose0;        // first pose (global index) of each problem
  const int64_t* un_ptr;       // [total poses + 1] unary factors of each pose
  const int8_t* un_kind;       // SFG_FACTOR_PRIOR_POSE3 / SFG_FACTOR_RANGE_POSE3
  const int64_t* un_coff;      // offset of the factor's constants
  const int64_t* bw_ptr;       // [total poses + 1] between factors from pose k to k + 1
  const int8_t* bw_rev;        // 1: the factor's keys are (k + 1, k)
  const int64_t* bw_coff;
  const double* consts;
  const double* values_in;     // [total poses][7]
  double* values_out;          // best values
  LmState* st;                 // [nprob]
  sfg_iteration_t* records;    // [nprob][rec_cap] (null: none)
  int rec_cap;
  double* ws;                  // [slots][ws_stride]
  int* counter;                // problem queue head (zero before launch)
  // Dense path (dense = 1: problems of any key and factor kinds that are not Pose3 chains; the
  // chain arrays above are then unused): problem p has dn_nk[p] keys from global key dn_k0[p],
  // tangent dimension dn_n[p] (at most kBatchDenseMaxN), storage dn_s[p] doubles at dn_s0[p] of
  // the values, and factors f_ptr[p] .. f_ptr[p + 1] - 1 (kind, up to kBatchDenseKeys global key
  // indices, -1 past the factor's keys, constants offset).
  int dense;
  int nmax_t, smax;            // largest tangent dimension / storage of a problem
  int64_t ws_stride;           // doubles of one workspace slot
  const int32_t* dn_n;
  const int32_t* dn_s;
  const int64_t* dn_s0;
  const int32_t* dn_k0;
  const int32_t* dn_nk;
  const int8_t* key_type;      // [total keys]
  const int32_t* key_soff;     // storage offset of the key within its problem
  const int32_t* key_toff;     // tangent offset of the key within its problem
  const int64_t* f_ptr;        // [nprob + 1]
  const int8_t* f_kind;
  const int32_t* f_key;        // [factors][kBatchDenseKeys]
  const int64_t* f_coff;
};
constexpr int kBatchDenseMaxN = 128;  // largest tangent dimension of a dense-path problem
constexpr int kBatchDenseKeys = 4;    // keys of a factor
constexpr int kBatchDenseRd = 12;     // residual rows of a factor
constexpr int kBatchDenseTd = 16;     // tangent columns of a factor
// Doubles of one dense-path workspace slot for problems up to n tangent / s storage dimensions.
inline int64_t BatchDenseWsStride(int n, int s) {
  return 3 * int64_t(s) + 4 * int64_t(n) * n + 9 * int64_t(n) + 32 * (int64_t(kBatchDenseRd) * (kBatchDenseTd + 1) + 1);
}
// Launch shapes (kernel instantiations): warps per CTA x register budget.
int BatchShapes();
int BatchShapeWarps(int shape);
int BatchMaxCtasPerSm(int shape, bool dense);
void LaunchBatchLm(const BatchLmDev& d, const LmParams* p, int ctas, int shape, cudaStream_t s);

// ---------------------------------------------------------------- network training (kernels_mlp.cu)
// Epilogues of the network's GEMMs: C = A B, + bias[n], ReLU(+ bias[n]), or times (mask[m][n] > 0).
enum GemmEpilogue { kEpiNone = 0, kEpiBiasRelu = 1, kEpiBias = 2, kEpiMask = 3 };
// C[M x N] = epilogue(A B) on the tensor cores (kernels_tc.cu); element (m, k) of A at
// A[m a_rs + k a_cs], (k, n) of B at B[k b_rs + n b_cs], C row-major with leading dimension ldc;
// a capped wait that gives up sets *err.
cudaError_t LaunchGemmTc(int M, int N, int K, const float* A, int64_t a_rs, int64_t a_cs, const float* B,
                         int64_t b_rs, int64_t b_cs, float* C, int64_t ldc, int epilogue, const float* bias,
                         const float* mask, int64_t ldmask, int* err, cudaStream_t s);
// out[n] = sum_m A[m][n] (fixed order).
void LaunchColSum(int M, int N, const float* A, int64_t lda, float* out, cudaStream_t s);
// Loss head: per sample (row of z, g_hat / x_hat at sample + 96 / + 105 with row stride lds)
// the loss and d loss / d z scaled by `scale`; loss_sum receives scale * sum of the losses.
void LaunchHead(int n, const float* z, const float* samples, int64_t lds, float scale, float kaporin,
                float* dz, float* loss, double* loss_sum, cudaStream_t s);
// rows[i] = samples[idx[i]] (kSampleFloats floats each).
void LaunchGather(int n, const float* samples, const int32_t* idx, float* rows, cudaStream_t s);
void LaunchAdam(int64_t n, float* w, const float* g, float* m, float* v, float lr, float beta1,
                float beta2, float eps, float c1, float c2, cudaStream_t s);

}  // namespace sfg
