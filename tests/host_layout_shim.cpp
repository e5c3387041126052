// Test shim: the host scatter plan of the linearization (LinLayout) for the CPU tests, so that the
// plan can be checked against an independent count of every Hessian entry's contributions without
// a GPU.  tests/test_host_layout.py compiles it with g++ together with the library's host sources.
#include <algorithm>
#include <cstdint>

#include "layout.h"

namespace {
sfg::HostProblem g_problem;
sfg::LinLayout g_layout;
sfg::SchurLayout g_schur;
sfg::Symbolic g_sym;
sfg::TaskPlan g_plan;
sfg::FactorMaps g_maps;
sfg::PrecondLayout g_pre;

template <typename V, typename O>
void Put(const std::vector<V>& v, O* out) {
  std::copy(v.begin(), v.end(), out);
}
}  // namespace

extern "C" {

// Build the plan of a problem; 0 on success.
int shim_build(const sfg_problem_t* p) {
  try {
    g_problem = sfg::ParseProblem(p);
    g_layout = sfg::BuildLinLayout(g_problem);
    return 0;
  } catch (...) {
    return 1;
  }
}

// nvals, N, nstage, staged groups, batches, stored key blocks, keys
void shim_sizes(int64_t* out) {
  out[0] = g_layout.nvals;
  out[1] = g_layout.N;
  out[2] = g_layout.nstage;
  out[3] = int64_t(g_layout.red_dst.size());
  out[4] = int64_t(g_layout.maps.size());
  out[5] = g_layout.H.nblocks();
  out[6] = g_problem.nkeys;
}

// entries per factor, tangent dims of the merged key slots, factor count
void shim_batch(int b, int32_t* out) {
  out[0] = g_layout.maps[b].nent;
  out[1] = g_layout.maps[b].merged_dims;
  out[2] = g_problem.batches[b].count;
}

void shim_batch_arrays(int b, int32_t* dest, int32_t* order) {
  const auto& m = g_layout.maps[b];
  std::copy(m.dest.begin(), m.dest.end(), dest);
  std::copy(m.order.begin(), m.order.end(), order);
}

void shim_groups(int32_t* red_dst, int64_t* red_ptr) {
  std::copy(g_layout.red_dst.begin(), g_layout.red_dst.end(), red_dst);
  std::copy(g_layout.red_ptr.begin(), g_layout.red_ptr.end(), red_ptr);
}

// block pattern of the Hessian: colptr [nkeys + 1], rows / boff [nblocks], and the tangent offset
// of every key [nkeys + 1]
void shim_pattern(int64_t* colptr, int32_t* rows, int64_t* boff, int64_t* toff) {
  const auto& H = g_layout.H;
  std::copy(H.colptr.begin(), H.colptr.end(), colptr);
  std::copy(H.rows.begin(), H.rows.end(), rows);
  std::copy(H.boff.begin(), H.boff.end() - 1, boff);
  std::copy(g_problem.toff.begin(), g_problem.toff.end(), toff);
}

// The Schur plan of the problem built last (points = the trailing num_schur keys); 0 on success.
int shim_build_schur() {
  try {
    g_schur = sfg::BuildSchurLayout(g_problem, g_layout);
    return 0;
  } catch (...) {
    return 1;
  }
}

// The same with G = L^-1 E at E's offsets (the library's default); e_order into out ([nE]).
int shim_build_schur_g_at_e(int64_t* e_order) {
  try {
    g_schur = sfg::BuildSchurLayout(g_problem, g_layout, true);
    if (e_order) Put(g_schur.e_order, e_order);
    return 0;
  } catch (...) {
    return 1;
  }
}

// nB_keys, npoints, nB, c_toff, E blocks, S blocks, terms, rhs entries, S values
void shim_schur_sizes(int64_t* out) {
  const auto& S = g_schur;
  out[0] = S.nB_keys;
  out[1] = S.npoints;
  out[2] = S.nB;
  out[3] = S.c_toff;
  out[4] = int64_t(S.pt_eoff.size());
  out[5] = S.Spat.nblocks();
  out[6] = int64_t(S.sb_eoff.size());
  out[7] = int64_t(S.r_eoff.size());
  out[8] = S.Spat.nvals();
}

// 64-bit arrays: 0 pt_diag, 1 pt_eptr, 2 pt_eoff, 3 pt_woff, 4 sb_ptr, 5 sb_eoff, 6 sb_woff,
// 7 sb_hoff, 8 sb_soff, 9 r_ptr, 10 r_eoff, 11 Spat colptr, 12 Spat boff
void shim_schur_i64(int which, int64_t* out) {
  const auto& S = g_schur;
  switch (which) {
    case 0: Put(S.pt_diag, out); break;
    case 1: Put(S.pt_eptr, out); break;
    case 2: Put(S.pt_eoff, out); break;
    case 3: Put(S.pt_woff, out); break;
    case 4: Put(S.sb_ptr, out); break;
    case 5: Put(S.sb_eoff, out); break;
    case 6: Put(S.sb_woff, out); break;
    case 7: Put(S.sb_hoff, out); break;
    case 8: Put(S.sb_soff, out); break;
    case 9: Put(S.r_ptr, out); break;
    case 10: Put(S.r_eoff, out); break;
    case 11: Put(S.Spat.colptr, out); break;
    case 12: std::copy(S.Spat.boff.begin(), S.Spat.boff.end() - 1, out); break;
  }
}

// 32-bit arrays: 0 pt_ekey_dim, 1 sb_dk, 2 sb_dl, 3 r_ecol, 4 r_dk, 5 r_pt, 6 Spat rows
void shim_schur_i32(int which, int32_t* out) {
  const auto& S = g_schur;
  switch (which) {
    case 0: Put(S.pt_ekey_dim, out); break;
    case 1: Put(S.sb_dk, out); break;
    case 2: Put(S.sb_dl, out); break;
    case 3: Put(S.r_ecol, out); break;
    case 4: Put(S.r_dk, out); break;
    case 5: Put(S.r_pt, out); break;
    case 6: Put(S.Spat.rows, out); break;
  }
}

// Symbolic factorization and tile task plan of the Hessian pattern (which 0) or of the reduced
// system of the Schur plan (which 1), nested-dissection ordering; 0 on success.
int shim_build_factor_plan(int which, int tile) {
  try {
    g_sym = sfg::Analyze(which == 0 ? g_layout.H : g_schur.Spat, SFG_ORDERING_NESTED_DISSECTION);
    g_plan = sfg::PlanTasks(g_sym, tile, tile == 16, tile == 32);  // FP64 tiles 16 wide, FP32 32
    g_maps = sfg::BuildFactorMaps(g_sym, g_plan, which == 0 ? g_layout.H : g_schur.Spat);
    return 0;
  } catch (...) {
    return 1;
  }
}

// fronts, tasks, children in all
void shim_factor_sizes(int64_t* out) {
  out[0] = g_sym.ns;
  out[1] = int64_t(g_plan.tasks.size());
  int64_t nc = 0;
  for (const auto& c : g_sym.sn_children) nc += int64_t(c.size());
  out[2] = nc;
}

// tasks [ntasks][4] = {type, front, i << 16 | j, k}; per front: pivot tiles, tiles, parent, pivot
// width, front size; children of every front (child_ptr [ns + 1], child_list)
void shim_factor_arrays(int32_t* tasks, int32_t* npiv, int32_t* ntiles, int32_t* parent, int32_t* w,
                        int32_t* m, int32_t* child_ptr, int32_t* child_list) {
  for (size_t t = 0; t < g_plan.tasks.size(); ++t) {
    const int4 v = g_plan.tasks[t];
    tasks[4 * t] = v.x;
    tasks[4 * t + 1] = v.y;
    tasks[4 * t + 2] = v.z;
    tasks[4 * t + 3] = v.w;
  }
  Put(g_plan.npiv, npiv);
  Put(g_plan.ntiles, ntiles);
  Put(g_sym.sn_parent, parent);
  Put(g_sym.sn_w, w);
  Put(g_sym.sn_m, m);
  child_ptr[0] = 0;
  int32_t q = 0;
  for (int s = 0; s < g_sym.ns; ++s) {
    for (int c : g_sym.sn_children[s]) child_list[q++] = c;
    child_ptr[s + 1] = q;
  }
}

// sizes of the maps arrays: 0 a_ptr, 1 a_src, 2 e_rptr, 3 e_round, 4 e_src, 5 idx_off, 6 idx,
// 7 rel_off, 8 rel, 9 sn_foff, 10 scalar_old, 11 col_base; 12 front pool entries, 13 n
void shim_maps_sizes(int64_t* out) {
  out[0] = int64_t(g_maps.a_ptr.size());
  out[1] = int64_t(g_maps.a_src.size());
  out[2] = int64_t(g_maps.e_rptr.size());
  out[3] = int64_t(g_maps.e_round.size());
  out[4] = int64_t(g_maps.e_src.size());
  out[5] = int64_t(g_sym.idx_off.size());
  out[6] = int64_t(g_sym.idx.size());
  out[7] = int64_t(g_sym.rel_off.size());
  out[8] = int64_t(g_sym.rel.size());
  out[9] = int64_t(g_sym.sn_foff.size());
  out[10] = int64_t(g_maps.scalar_old.size());
  out[11] = int64_t(g_plan.asm_col_base.size());
  out[12] = g_sym.front_pool;
  out[13] = g_sym.n;
}

// 64-bit: 0 a_ptr, 1 a_src, 2 e_rptr, 3 e_round, 4 e_src, 5 idx_off, 7 rel_off, 9 sn_foff;
// 32-bit: 21 a_dst, 22 a_damp, 24 e_dst, 26 idx, 28 rel, 30 scalar_old, 31 col_base
void shim_maps_i64(int which, int64_t* out) {
  switch (which) {
    case 0: Put(g_maps.a_ptr, out); break;
    case 1: Put(g_maps.a_src, out); break;
    case 2: Put(g_maps.e_rptr, out); break;
    case 3: Put(g_maps.e_round, out); break;
    case 4: Put(g_maps.e_src, out); break;
    case 5: Put(g_sym.idx_off, out); break;
    case 7: Put(g_sym.rel_off, out); break;
    case 9: Put(g_sym.sn_foff, out); break;
  }
}
void shim_maps_i32(int which, int32_t* out) {
  switch (which) {
    case 21: Put(g_maps.a_dst, out); break;
    case 22: Put(g_maps.a_damp, out); break;
    case 24: Put(g_maps.e_dst, out); break;
    case 26: Put(g_sym.idx, out); break;
    case 28: Put(g_sym.rel, out); break;
    case 30: Put(g_maps.scalar_old, out); break;
    case 31: Put(g_plan.asm_col_base, out); break;
  }
}

// Camera blocks of the reduced system (the PCG forms) of the Schur plan built last; 0 on success.
int shim_build_precond() {
  try {
    g_pre = sfg::BuildPrecondLayout(g_problem, g_schur);
    return 0;
  } catch (...) {
    return 1;
  }
}

// camera blocks, stored 9 x 9 group blocks, group-row entries
void shim_precond_sizes(int64_t* out) {
  out[0] = g_pre.ng;
  out[1] = int64_t(g_pre.blk_row.size());
  out[2] = int64_t(g_pre.gent.size() / 2);
}

void shim_precond_arrays(int32_t* gidx, int64_t* blk_off, int32_t* gptr, int32_t* gent) {
  Put(g_pre.gidx, gidx);
  Put(g_pre.blk_off, blk_off);
  Put(g_pre.gptr, gptr);
  Put(g_pre.gent, gent);
}

// Band preconditioner pattern over `band` neighbouring groups of the camera blocks built last:
// nj [ng], jgrp [ng][band + 1], jblk [ng][band + 1][band + 1].
void shim_band_pattern(int band, int32_t* nj, int32_t* jgrp, int32_t* jblk) {
  const sfg::BandPattern B = sfg::BuildBandPattern(g_pre, band);
  Put(B.nj, nj);
  Put(B.jgrp, jgrp);
  Put(B.jblk, jblk);
}

// Split of the front solves (block_tiles pivot tiles a CTA, `warps` warps a CTA) of the factor
// plan built last: out = {forward tasks, all tasks}; then shim_solve_split_arrays.
static sfg::SolveSplit g_split;
void shim_solve_split(int warps, int block_tiles, int64_t* out) {
  g_split = sfg::PlanSolveSplit(g_plan, g_sym.ns, warps, block_tiles, true);
  out[0] = g_split.nf;
  out[1] = int64_t(g_split.task_front.size());
}
void shim_solve_split_arrays(int32_t* kp, int32_t* ku, int32_t* task_front, int32_t* task_sub) {
  Put(g_split.kp, kp);
  Put(g_split.ku, ku);
  Put(g_split.task_front, task_front);
  Put(g_split.task_sub, task_sub);
}

}  // extern "C"
