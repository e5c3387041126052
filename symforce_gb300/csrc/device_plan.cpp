// Device factorization plans: flattening of the host symbolic structure into the per-tile-column
// assembly lists and task tables the persistent factorization kernel consumes.
#include "device_plan.h"

#include <algorithm>
#include <cstdlib>
#include <array>
#include <unordered_map>

namespace sfg {

void* DeviceArena::Alloc(size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) bytes = 16;
  const cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess)
    throw Error(e == cudaErrorMemoryAllocation ? SFG_ERR_OUT_OF_MEMORY : SFG_ERR_CUDA,
                std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
  ptrs.push_back(p);
  return p;
}

void BuildFactorPlan(DeviceArena& A, FactorPlan& fp, const BlockPattern& pat, int ordering,
                     size_t elem, int* error_word, const LmState* st, int64_t a_stride,
                     int64_t b_stride, int num_sms, bool trace) {
  fp.elem = elem;
  fp.sym = Analyze(pat, ordering);
  const Symbolic& S = fp.sym;
  const int tile = elem == 8 ? kFactorTileF64 : kFactorTileF32;
  // FP64 chains leave the inverses of their diagonal factors to separate tasks; FP32 fronts take
  // runs of trailing updates on the tensor cores (SFG_FACTOR_TC=0: SIMT tile updates only)
  bool tc = elem == 4;
  if (const char* e = std::getenv("SFG_FACTOR_TC")) tc = tc && std::atoi(e) != 0;
  fp.plan = PlanTasks(S, tile, elem == 8, tc);
  const TaskPlan& T = fp.plan;
  FactorDev& f = fp.f;
  f.ns = S.ns;
  f.ntasks = int(T.tasks.size());
  f.tile = T.tile;
  f.tasks = A.Upload(T.tasks);
  f.sn_w = A.Upload(S.sn_w);
  f.sn_m = A.Upload(S.sn_m);
  f.sn_foff = A.Upload(S.sn_foff);
  f.tile_base = A.Upload(T.tile_base);
  f.npiv = A.Upload(T.npiv);
  f.ntiles = A.Upload(T.ntiles);
  // ---- flattened assembly per (front, tile column), tree and solve maps
  const FactorMaps M = BuildFactorMaps(S, T, pat);
  const std::vector<int64_t>& linv_base = M.linv_base;
  f.col_base = A.Upload(T.asm_col_base);
  f.a_ptr = A.Upload(M.a_ptr);
  f.a_src = A.Upload(M.a_src);
  f.a_dst = A.Upload(M.a_dst);
  f.a_damp = A.Upload(M.a_damp);
  f.e_rptr = A.Upload(M.e_rptr);
  f.e_round = A.Upload(M.e_round);
  f.e_src = A.Upload(M.e_src);
  f.e_dst = A.Upload(M.e_dst);
  f.linv_base = A.Upload(linv_base);
  f.trace = trace ? A.Zeros<unsigned long long>(8 * T.tasks.size()) : nullptr;  // start, ready, end, SM, 4 phase stamps
  f.rel_off = A.Upload(S.rel_off);
  f.rel = A.Upload(S.rel);
  f.child_ptr = A.Upload(M.child_ptr);
  f.child_list = A.Upload(M.child_list);
  f.parent = A.Upload(S.sn_parent);
  f.idx_off = A.Upload(S.idx_off);
  f.idx = A.Upload(S.idx);
  f.scalar_old = A.Upload(M.scalar_old);
  f.tile_state = A.Zeros<int>(size_t(T.nstates));
  f.counters = A.Zeros<int>(2);
  fp.nflags = 2 * S.ns + kSmFlagSlots + 1;
  f.front_flags = A.Zeros<int>(size_t(fp.nflags));
  f.sm_flags = f.front_flags + 2 * S.ns;
  // chains may take at most half of the SMs for themselves
  f.iso_limit = std::max(1, num_sms / 2);
  f.error = error_word;
  f.fp64_tiles = A.Zeros<int>(1);
  int maxm = 1;
  for (int s = 0; s < S.ns; ++s) maxm = std::max(maxm, S.sn_m[s]);
  f.max_m = maxm;
  f.st = st;
  f.a_stride = a_stride;
  f.b_stride = b_stride;
  fp.F = A.Alloc(size_t(S.front_pool) * elem);
  fp.Linv = A.Alloc(size_t(std::max<int64_t>(linv_base[S.ns], 1)) * elem);
  fp.ycon = A.Alloc(size_t(std::max<int64_t>(S.rel_off[S.ns], 1)) * elem);
  fp.nsave = std::max<int64_t>(S.idx_off[S.ns], 1);
  fp.ysave = A.Alloc(size_t(2 * fp.nsave) * elem);
  fp.xb = static_cast<char*>(fp.ysave) + size_t(fp.nsave) * elem;
  fp.xperm = A.Alloc(size_t(std::max<int64_t>(S.n, 1)) * elem);
  // FP64 solves of fronts with more tiles than a solve CTA has warps are split over CTAs of
  // kSolveBlockTiles pivot tiles (and, forward, CTAs of as many update tiles): one SM's FP64 pipe
  // caps a front's solve.  FP32 solves keep one CTA per front and direction, as does
  // SFG_SOLVE_SPLIT=0.
  bool split = elem == 8;
  if (const char* e = std::getenv("SFG_SOLVE_SPLIT")) split = split && std::atoi(e) != 0;
  const SolveSplit sp = PlanSolveSplit(T, S.ns, SolveWarps(), kSolveBlockTiles, split);
  int ntasks_solve = 2 * S.ns;
  if (!sp.task_front.empty()) {
    f.solve_front = A.Upload(sp.task_front);
    f.solve_sub = A.Upload(sp.task_sub);
    f.solve_kp = A.Upload(sp.kp);
    f.solve_ku = A.Upload(sp.ku);
    f.solve_nf = sp.nf;
    f.solve_nb = int(sp.task_front.size()) - sp.nf;
    ntasks_solve = int(sp.task_front.size());
  }
  const int per_sm = 8;
  // the factorization kernel is built for kFactorCtasPerSm (or, FP64 plans of many fronts,
  // kFactorCtasPerSmWide) resident CTAs of 128 threads per SM; SFG_FACTOR_WIDE=0 / 1 overrides
  // SFG_FACTOR_CTAS_PER_SM (1..that) narrows the grid for launch-shape measurements
  f.wide = (elem == 8 && S.ns >= kFactorWideFronts) ? 1 : 0;
  if (const char* e = std::getenv("SFG_FACTOR_WIDE")) f.wide = (elem == 8 && std::atoi(e) != 0) ? 1 : 0;
  const int max_per_sm = f.wide ? kFactorCtasPerSmWide : kFactorCtasPerSm;
  int factor_per_sm = max_per_sm;
  if (const char* e = std::getenv("SFG_FACTOR_CTAS_PER_SM"))
    factor_per_sm = std::max(1, std::min(max_per_sm, std::atoi(e)));
  fp.grid_factor = std::max(1, std::min<int>(f.ntasks, num_sms * factor_per_sm));
  fp.grid_solve = std::max(1, std::min<int>(ntasks_solve, num_sms * per_sm));
  if (elem == 8) ConfigureSolve<double>(maxm);
  else ConfigureSolve<float>(maxm);
}

void FactorLowerCsc(const FactorPlan& fp, const void* front, std::vector<int32_t>& col_ptr,
                    std::vector<int32_t>& row_idx, std::vector<double>* values) {
  const Symbolic& S = fp.sym;
  const int64_t n = S.n;
  std::vector<std::vector<std::pair<int32_t, double>>> cols(static_cast<size_t>(n));
  for (int s = 0; s < S.ns; ++s) {
    const int w = S.sn_w[s], m = S.sn_m[s];
    const int32_t* idx = S.idx.data() + S.idx_off[s];
    for (int q = 0; q < w; ++q) {
      auto& col = cols[size_t(idx[q])];
      for (int r = q + 1; r < m; ++r) {
        double v = 0.0;
        if (front) {
          const int64_t at = S.sn_foff[s] + r + int64_t(q) * m;
          v = fp.elem == 8 ? static_cast<const double*>(front)[at] : double(static_cast<const float*>(front)[at]);
        }
        col.push_back({idx[r], v});
      }
    }
  }
  col_ptr.assign(size_t(n) + 1, 0);
  row_idx.clear();
  if (values) values->clear();
  for (int64_t c = 0; c < n; ++c) {
    auto& col = cols[size_t(c)];
    std::sort(col.begin(), col.end());
    for (const auto& e : col) {
      row_idx.push_back(e.first);
      if (values) values->push_back(e.second);
    }
    col_ptr[size_t(c) + 1] = int32_t(row_idx.size());
  }
}

SpmvDev BuildSpmv(DeviceArena& A, const BlockPattern& pat, int64_t a_stride, int64_t b_stride) {
  const int64_t n = pat.off[pat.nb];
  std::vector<std::vector<std::array<int64_t, 4>>> rows(n);  // base, stride, len, x
  for (int j = 0; j < pat.nb; ++j)
    for (int64_t q = pat.colptr[j]; q < pat.colptr[j + 1]; ++q) {
      const int i = pat.rows[q];
      const int di = pat.dim[i], dj = pat.dim[j];
      const int64_t b = pat.boff[q];
      if (i == j) {
        for (int r = 0; r < di; ++r) {
          rows[pat.off[i] + r].push_back({b + int64_t(r) * dj, 1, r + 1, pat.off[j]});
          if (r + 1 < di)
            rows[pat.off[i] + r].push_back({b + int64_t(r + 1) * dj + r, dj, di - r - 1, pat.off[j] + r + 1});
        }
      } else {
        for (int r = 0; r < di; ++r) rows[pat.off[i] + r].push_back({b + int64_t(r) * dj, 1, dj, pat.off[j]});
        for (int c = 0; c < dj; ++c) rows[pat.off[j] + c].push_back({b + c, dj, di, pat.off[i]});
      }
    }
  std::vector<int64_t> ptr(n + 1, 0), base;
  std::vector<int32_t> stride, len, x;
  for (int64_t r = 0; r < n; ++r) {
    for (auto& sg : rows[r]) {
      base.push_back(sg[0]);
      stride.push_back(int32_t(sg[1]));
      len.push_back(int32_t(sg[2]));
      x.push_back(int32_t(sg[3]));
    }
    ptr[r + 1] = int64_t(base.size());
  }
  SpmvDev m{};
  m.n = int(n);
  m.row_ptr = A.Upload(ptr);
  m.seg_base = A.Upload(base);
  m.seg_stride = A.Upload(stride);
  m.seg_len = A.Upload(len);
  m.seg_x = A.Upload(x);
  m.a_stride = a_stride;
  m.b_stride = b_stride;
  return m;
}

template <typename T>
void EnqueueFactor(const FactorPlan& fp, const void* A, const double* damping, cudaStream_t s,
                   const int* gate) {
  LaunchResetFactorState(fp.f.tile_state, fp.plan.nstates, fp.f.front_flags, fp.nflags,
                         fp.f.counters, s, gate);
  FactorDev f = fp.f;
  f.gate = gate;
  LaunchFactor<T>(f, A, damping, fp.F, fp.Linv, fp.grid_factor, s);
}

template <typename T>
void EnqueueSolve(const FactorPlan& fp, const void* b, void* x, cudaStream_t s, bool fixed_b,
                  const int* gate) {
  // split solves: the exchange values (ysave, xb) back to the unset pattern
  const bool split = fp.f.solve_front != nullptr;
  LaunchResetFactorState(fp.f.tile_state, 0, fp.f.front_flags, fp.nflags, fp.f.counters, s, gate,
                         split ? fp.ysave : nullptr, split ? 2 * fp.nsave : 0, int(sizeof(T)));
  FactorDev f = fp.f;
  f.gate = gate;
  if (fixed_b) f.b_stride = 0;
  LaunchSolve<T>(f, fp.F, fp.Linv, b, fp.ycon, fp.ysave, fp.xperm, x, fp.xb, fp.grid_solve, s);
}

template void EnqueueFactor<double>(const FactorPlan&, const void*, const double*, cudaStream_t,
                                    const int*);
template void EnqueueFactor<float>(const FactorPlan&, const void*, const double*, cudaStream_t,
                                   const int*);
template void EnqueueSolve<double>(const FactorPlan&, const void*, void*, cudaStream_t, bool, const int*);
template void EnqueueSolve<float>(const FactorPlan&, const void*, void*, cudaStream_t, bool, const int*);

SchurDev UploadSchur(DeviceArena& A, const SchurLayout& S, int elem) {
  SchurDev d{};
  d.npoints = S.npoints;
  d.nB = int(S.nB);
  d.c_toff = S.c_toff;
  d.pt_diag = A.Upload(S.pt_diag);
  d.pt_eptr = A.Upload(S.pt_eptr);
  d.pt_ekey_toff = A.Upload(S.pt_ekey_toff);
  d.pt_ekey_dim = A.Upload(S.pt_ekey_dim);
  d.pt_eoff = A.Upload(S.pt_eoff);
  d.nE = int64_t(S.pt_eoff.size());
  d.pt_of_e = A.Upload(S.pt_of_e);
  d.pt_woff = S.g_at_e ? d.pt_eoff : A.Upload(S.pt_woff);  // where each block's G lives
  d.e_order = S.e_order.empty() ? nullptr : A.Upload(S.e_order);
  d.nsblocks = int(S.Spat.nblocks());
  d.sb_ptr = A.Upload(S.sb_ptr);
  d.sb_eoff = A.Upload(S.sb_eoff);
  d.sb_woff = A.Upload(S.sb_woff);
  d.sb_hoff = A.Upload(S.sb_hoff);
  d.sb_soff = A.Upload(S.sb_soff);
  d.sb_dk = A.Upload(S.sb_dk);
  d.sb_dl = A.Upload(S.sb_dl);
  d.sb_diag_toff = A.Upload(S.sb_diag_toff);
  int64_t ct = elem == 8 ? 128 : 256;
  if (const char* e = std::getenv("SFG_SCHUR_CHUNK")) {  // tuning override: terms per chunk
    const long v = std::atol(e);
    if (v >= 1 && v <= (1 << 20)) ct = v;
  }
  std::vector<int32_t> ch_block;
  std::vector<int64_t> ch_begin, chunk_ptr(1, 0);
  for (int b = 0; b < d.nsblocks; ++b) {
    for (int64_t t = S.sb_ptr[b]; t < S.sb_ptr[b + 1]; t += ct) {
      ch_block.push_back(b);
      ch_begin.push_back(t);
    }
    chunk_ptr.push_back(int64_t(ch_block.size()));
  }
  if (ch_block.size() > size_t(INT32_MAX)) throw Error(SFG_ERR_STRUCTURE, "too many Schur term chunks");
  d.nchunks = int(ch_block.size());
  d.chunk_terms = int(ct);
  d.ch_block = A.Upload(ch_block);
  d.ch_begin = A.Upload(ch_begin);
  d.sb_chunk_ptr = A.Upload(chunk_ptr);
  d.partials = A.Alloc(std::max<size_t>(ch_block.size(), 1) * 36 * size_t(elem));
  d.r_ptr = A.Upload(S.r_ptr);
  d.r_eoff = A.Upload(S.r_eoff);
  d.r_ecol = A.Upload(S.r_ecol);
  d.r_dk = A.Upload(S.r_dk);
  d.nBk = S.nB_keys;
  d.bkey_toff = A.Upload(S.bkey_toff);
  d.r_pt = A.Upload(S.r_pt);
  return d;
}

}  // namespace sfg
