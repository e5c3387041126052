// Test shim: the host scatter plan of the linearization (LinLayout) for the CPU tests, so that the
// plan can be checked against an independent count of every Hessian entry's contributions without
// a GPU.  tests/test_host_layout.py compiles it with g++ together with the library's host sources.
#include <algorithm>
#include <cstdint>

#include "layout.h"

namespace {
sfg::HostProblem g_problem;
sfg::LinLayout g_layout;
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

}  // extern "C"
