// Host-computed layouts: where every factor's linearization lands in the block-sparse Hessian,
// the Schur complement term lists, and the reference CSC export map.
#pragma once

#include <cstdint>
#include <vector>

#include "common.h"

namespace sfg {

struct LinLayout {
  BlockPattern H;                  // key blocks of hessian_lower (tangent dims)
  std::vector<int64_t> diag_off;   // [N] value offset of each diagonal scalar
  struct BatchMap {
    int nent = 0;                  // packed H entries + rhs entries per factor
    int merged_dims = 0;           // tangent dims of the merged key slots (0: no warp merging)
    std::vector<int32_t> dest;     // [nent][count] sink index, device order
    std::vector<int32_t> order;    // [count] device factor -> the user's factor index
  };
  std::vector<BatchMap> maps;
  int64_t nvals = 0, N = 0, nstage = 0;
  // groups of staged contributions: destination and [ptr, ptr+1) range of staging slots
  std::vector<int32_t> red_dst;
  std::vector<int64_t> red_ptr;
  int64_t nnz_lower = 0;            // scalar entries of the reference CSC lower layout
  // reference CSC lower layout (symforce/opt/linearizer.cc:324-353): values come from csc_src;
  // built on first use (BuildCscExport), it is as large as the Hessian itself
  std::vector<int32_t> csc_colptr, csc_rowidx;
  std::vector<int64_t> csc_src;
};

LinLayout BuildLinLayout(const HostProblem& P);
// Fill L's CSC export arrays (once; a no-op when they exist).
void BuildCscExport(LinLayout& L, const HostProblem& P);

struct SchurLayout {
  int nB_keys = 0, npoints = 0;
  int64_t nB = 0, c_toff = 0;
  std::vector<int64_t> pt_diag, pt_eptr, pt_eoff, pt_woff;
  std::vector<int32_t> pt_ekey_toff, pt_ekey_dim;
  std::vector<int32_t> pt_of_e;    // point of each E block
  int64_t nW = 0;
  BlockPattern Spat;               // pattern of the reduced system over B keys
  // terms of S block q: [sb_ptr[q], sb_ptr[q + 1]); each term's two blocks G_pk, G_pl
  // (G = L_p^-1 E, L_p the Cholesky factor of the point block) at offsets sb_eoff, sb_woff of the
  // G buffer; pt_goff: the G offset of each E block (pt_eoff or pt_woff, see BuildSchurLayout)
  std::vector<int64_t> sb_ptr, sb_eoff, sb_woff, sb_hoff, sb_soff;
  bool g_at_e = false;
  int64_t nG = 0;                  // G buffer size
  std::vector<int64_t> e_order;    // g_at_e: E blocks in Hessian-offset order (else empty)
  std::vector<int32_t> sb_dk, sb_dl, sb_diag_toff;
  std::vector<int32_t> bkey_toff;  // [nB_keys + 1] tangent offsets of the reduced system's keys
  std::vector<int64_t> r_ptr, r_eoff;
  std::vector<int32_t> r_ecol, r_dk, r_pt;
};

// g_at_e: the G = L^-1 E blocks sit at E's offsets in a Hessian-sized buffer (a key's blocks
// contiguous over its points, for both operands of every S term; the kernel forming G takes the
// blocks in that order); otherwise point-major in a compact buffer.
SchurLayout BuildSchurLayout(const HostProblem& P, const LinLayout& L, bool g_at_e = false);

// Camera blocks of the reduced system for the PCG forms: B keys joined when they share a factor
// (pose + intrinsics of a camera), at most 9 scalars per block, ordered by their first key.
struct PrecondLayout {
  int ng = 0;
  std::vector<int32_t> gidx;          // [ng][9] reduced-system scalar, -1 padding
  std::vector<int64_t> goff;          // [ng][81] S value offset of (a, b); -1 padding, -2 zero
  std::vector<float> degree;          // [ng] neighbouring blocks
  std::vector<int32_t> scalar_group;  // [nB]
  std::vector<int64_t> sdiag_off;     // [nB]
  // 9 x 9 group blocks of S (lower: column group <= row group), row-major, 81 entries each
  std::vector<int32_t> blk_row, blk_col;
  std::vector<int64_t> blk_off;       // [nblocks][81] S value offset; -1 padding, -2 zero
  std::vector<int32_t> gptr;          // [ng + 1] entries of each group row
  std::vector<int32_t> gent;          // [entries][2] {stored block, neighbour << 1 | transposed}
  // similarity gauge of the camera poses: per group row, the storage offset of its POSE3 key in the
  // values (-1: not a pose row) and its tangent component (0..2 rotation, 3..5 translation)
  std::vector<int64_t> gauge_soff;    // [ng][9]
  std::vector<int32_t> gauge_comp;    // [ng][9]
  int gauge_rows = 0;                 // pose rows
};
PrecondLayout BuildPrecondLayout(const HostProblem& P, const SchurLayout& SL);

// Pattern of the band preconditioner over `band` neighbouring groups: per group row l the groups
// J_l = {h : l - band <= h < l, S_lh stored} + {l} (ascending) and the stored group block of
// every pair (J_l[s1], J_l[s2]), s1 >= s2 (-1: structurally zero).
struct BandPattern {
  int band = 0;
  std::vector<int32_t> nj;    // [ng]
  std::vector<int32_t> jgrp;  // [ng][band + 1], -1 past nj
  std::vector<int32_t> jblk;  // [ng][band + 1][band + 1]
};
BandPattern BuildBandPattern(const PrecondLayout& L, int band);

}  // namespace sfg
