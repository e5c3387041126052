// Linearization and Schur layouts (host, once per problem structure).
//
// BuildLinLayout is the block analogue of Linearizer::BuildInitialLinearization
// (symforce/opt/linearizer.cc:148-356): it fixes the hessian_lower pattern (every entry of every
// co-occurring lower key block plus the full diagonal) and, for every factor, where each entry of
// its packed J^T J / J^T r goes.  Entries with a single contributor are written in place by the
// linearization kernel; shared entries get staging slots grouped per destination in factor order
// and are summed by a second kernel, which makes the result independent of thread scheduling.
//
// Factors of a kind with merged key slots (MergedKeySlots: the camera of a reprojection factor)
// are put in device order by those keys.  A warp of 32 consecutive device factors that all share
// them sums the entries among those keys across its lanes (a shuffle reduce-scatter) and makes one
// contribution per entry, at the sink index of its first factor; every other entry stays one
// contribution per factor.  The staged work of a camera block falls from one slot per observation
// to one per warp.
#include <algorithm>
#include <numeric>

#include "layout.h"

namespace sfg {

LinLayout BuildLinLayout(const HostProblem& P) {
  LinLayout L;
  // key pairs
  std::vector<std::pair<int, int>> pairs;
  for (const auto& B : P.batches)
    for (int f = 0; f < B.count; ++f)
      for (int a = 0; a < B.nk; ++a)
        for (int b = 0; b < a; ++b) {
          const int ka = B.keys[size_t(f) * B.nk + a], kb = B.keys[size_t(f) * B.nk + b];
          pairs.push_back({std::max(ka, kb), std::min(ka, kb)});
        }
  L.H = MakePattern(P.tdim, std::move(pairs));
  L.nvals = L.H.nvals();
  L.N = P.N;
  L.diag_off.resize(P.N);
  for (int k = 0; k < P.nkeys; ++k) {
    const int64_t blk = L.H.Find(k, k);
    for (int r = 0; r < P.tdim[k]; ++r) L.diag_off[P.toff[k] + r] = L.H.boff[blk] + r * P.tdim[k] + r;
  }
  // device order of every batch and the warps that merge their leading key slots
  std::vector<std::vector<int32_t>> order(P.batches.size());
  std::vector<std::vector<char>> warp_merged(P.batches.size());
  std::vector<int> merged_dims(P.batches.size(), 0);
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    const int ms = MergedKeySlots(B.kind);
    auto& ord = order[bi];
    ord.resize(B.count);
    std::iota(ord.begin(), ord.end(), 0);
    if (ms == 0) continue;
    for (int s = 0; s < ms; ++s) merged_dims[bi] += B.key_tdim[s];
    auto key = [&](int32_t f, int s) { return B.keys[size_t(f) * B.nk + s]; };
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t x, int32_t y) {
      for (int s = 0; s < ms; ++s)
        if (key(x, s) != key(y, s)) return key(x, s) < key(y, s);
      return false;
    });
    const int nwarps = B.count / 32;  // full warps only
    warp_merged[bi].assign(size_t(nwarps), 0);
    for (int w = 0; w < nwarps; ++w) {
      bool same = true;
      for (int l = 1; l < 32 && same; ++l)
        for (int s = 0; s < ms; ++s) same = same && key(ord[32 * w + l], s) == key(ord[32 * w], s);
      warp_merged[bi][w] = same;
    }
  }
  // Whether device factor f of batch bi contributes entry e itself (false: its warp's first
  // factor carries the warp's sum).
  auto contributes = [&](size_t bi, int f, int e, int nh) {
    const int mt = merged_dims[bi];
    if (mt == 0 || (f & 31) == 0) return true;
    const size_t w = size_t(f) / 32;
    if (w >= warp_merged[bi].size() || !warp_merged[bi][w]) return true;
    const bool merged_entry = e < nh ? e < mt * (mt + 1) / 2 : e - nh < mt;
    return !merged_entry;
  };
  // slot (H value index or nvals + tangent index) of every factor entry; f is the user's index
  auto entry_slot = [&](const HostBatch& B, int f, int e, int* kslot_of, int* local_of) -> int64_t {
    const int td = B.tdim;
    const int nh = td * (td + 1) / 2;
    const int32_t* keys = &B.keys[size_t(f) * B.nk];
    if (e >= nh) {
      const int a = e - nh;
      return L.nvals + P.toff[keys[kslot_of[a]]] + local_of[a];
    }
    // packed lower index e -> (a, b), a >= b
    int a = 0;
    while ((a + 1) * (a + 2) / 2 <= e) ++a;
    const int b = e - a * (a + 1) / 2;
    const int ka = keys[kslot_of[a]], kb = keys[kslot_of[b]];
    const int ra = local_of[a], rb = local_of[b];
    if (ka == kb) return L.H.boff[L.H.Find(ka, ka)] + int64_t(ra) * P.tdim[ka] + rb;
    if (ka > kb) return L.H.boff[L.H.Find(ka, kb)] + int64_t(ra) * P.tdim[kb] + rb;
    return L.H.boff[L.H.Find(kb, ka)] + int64_t(rb) * P.tdim[ka] + ra;
  };
  const int64_t nslots = L.nvals + P.N;
  std::vector<int32_t> cnt(nslots, 0);
  std::vector<std::vector<int>> kslot(P.batches.size()), local(P.batches.size());
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    for (int s = 0; s < B.nk; ++s)
      for (int r = 0; r < B.key_tdim[s]; ++r) {
        kslot[bi].push_back(s);
        local[bi].push_back(r);
      }
  }
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    const int nh = B.tdim * (B.tdim + 1) / 2;
    const int nent = nh + B.tdim;
    for (int f = 0; f < B.count; ++f)
      for (int e = 0; e < nent; ++e)
        if (contributes(bi, f, e, nh)) cnt[entry_slot(B, order[bi][f], e, kslot[bi].data(), local[bi].data())]++;
  }
  for (int64_t s = 0; s < nslots; ++s)
    if (cnt[s] == 0) {
      // every stored value must receive at least one contribution (the reference sets explicit
      // zeros from the first linearization; the block pattern never has untouched entries except
      // the strictly upper part of diagonal blocks, which is not a slot)
      const bool upper_of_diag = [&] {
        if (s >= L.nvals) return false;
        const auto it = std::upper_bound(L.H.boff.begin(), L.H.boff.end(), s) - 1;
        const int64_t blk = it - L.H.boff.begin();
        int j = int(std::upper_bound(L.H.colptr.begin(), L.H.colptr.end(), blk) - L.H.colptr.begin()) - 1;
        const int i = L.H.rows[blk];
        if (i != j) return false;
        const int64_t o = s - L.H.boff[blk];
        return (o % P.tdim[i]) > (o / P.tdim[i]);
      }();
      if (!upper_of_diag) throw Error(SFG_ERR_STRUCTURE, "Hessian entry without a contributor");
    }
  // staging groups in slot order
  std::vector<int64_t> group_base(nslots, -1);
  L.red_ptr.push_back(0);
  for (int64_t s = 0; s < nslots; ++s)
    if (cnt[s] > 1) {
      group_base[s] = L.red_ptr.back();
      L.red_dst.push_back(int32_t(s));
      L.red_ptr.push_back(L.red_ptr.back() + cnt[s]);
    }
  L.nstage = L.red_ptr.back();
  if (nslots + L.nstage >= (int64_t(1) << 31))
    throw Error(SFG_ERR_STRUCTURE, "problem too large for 32-bit sink indices");
  std::vector<int32_t> seen(nslots, 0);
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    LinLayout::BatchMap M;
    const int nh = B.tdim * (B.tdim + 1) / 2;
    M.nent = nh + B.tdim;
    M.merged_dims = merged_dims[bi];
    M.dest.resize(size_t(M.nent) * B.count);
    for (int f = 0; f < B.count; ++f)
      for (int e = 0; e < M.nent; ++e) {
        const size_t at = size_t(e) * B.count + f;
        if (!contributes(bi, f, e, nh)) {
          M.dest[at] = M.dest[at - (f & 31)];  // never read: the warp's first factor stores
          continue;
        }
        const int64_t s = entry_slot(B, order[bi][f], e, kslot[bi].data(), local[bi].data());
        int64_t d;
        if (cnt[s] == 1) {
          d = s;
        } else {
          d = nslots + group_base[s] + seen[s];
          seen[s]++;
        }
        M.dest[at] = int32_t(d);
      }
    M.order = std::move(order[bi]);
    L.maps.push_back(std::move(M));
  }
  // CSC export
  L.csc_colptr.assign(P.N + 1, 0);
  for (int kc = 0; kc < P.nkeys; ++kc)
    for (int cc = 0; cc < P.tdim[kc]; ++cc) {
      const int64_t col = P.toff[kc] + cc;
      for (int64_t q = L.H.colptr[kc]; q < L.H.colptr[kc + 1]; ++q) {
        const int kr = L.H.rows[q];
        for (int lr = (kr == kc ? cc : 0); lr < P.tdim[kr]; ++lr) {
          L.csc_rowidx.push_back(int32_t(P.toff[kr] + lr));
          L.csc_src.push_back(L.H.boff[q] + int64_t(lr) * P.tdim[kc] + cc);
        }
      }
      L.csc_colptr[col + 1] = int32_t(L.csc_rowidx.size());
    }
  return L;
}

SchurLayout BuildSchurLayout(const HostProblem& P, const LinLayout& L) {
  SchurLayout S;
  S.nB_keys = P.nkeys - P.num_schur;
  S.npoints = P.num_schur;
  S.nB = P.toff[S.nB_keys];
  S.c_toff = S.nB;
  for (int k = S.nB_keys; k < P.nkeys; ++k)
    if (P.tdim[k] != 3) throw Error(SFG_ERR_STRUCTURE, "Schur keys must be 3-dimensional");
  // E lists per point, sorted by B key
  std::vector<std::vector<std::pair<int, int64_t>>> pe(S.npoints);
  for (int j = 0; j < P.nkeys; ++j)
    for (int64_t q = L.H.colptr[j]; q < L.H.colptr[j + 1]; ++q) {
      const int i = L.H.rows[q];
      if (i < S.nB_keys) continue;
      if (j >= S.nB_keys) {
        if (i != j)
          throw Error(SFG_ERR_STRUCTURE,
                      "Submatrix C of A is not block diagonal, cannot use a Schur complement solver");
        continue;
      }
      pe[i - S.nB_keys].push_back({j, L.H.boff[q]});
    }
  S.pt_eptr.push_back(0);
  for (int p = 0; p < S.npoints; ++p) {
    const int kp = S.nB_keys + p;
    S.pt_diag.push_back(L.H.boff[L.H.Find(kp, kp)]);
    for (auto& e : pe[p]) {
      S.pt_eoff.push_back(e.second);
      S.pt_woff.push_back(S.nW);
      S.pt_ekey_toff.push_back(int32_t(P.toff[e.first]));
      S.pt_ekey_dim.push_back(P.tdim[e.first]);
      S.nW += 3 * P.tdim[e.first];
    }
    S.pt_eptr.push_back(int64_t(S.pt_eoff.size()));
  }
  // reduced pattern
  std::vector<std::pair<int, int>> pairs;
  for (int j = 0; j < S.nB_keys; ++j)
    for (int64_t q = L.H.colptr[j]; q < L.H.colptr[j + 1]; ++q)
      if (L.H.rows[q] < S.nB_keys) pairs.push_back({L.H.rows[q], j});
  for (int p = 0; p < S.npoints; ++p)
    for (size_t a = 0; a < pe[p].size(); ++a)
      for (size_t b = 0; b <= a; ++b) pairs.push_back({pe[p][a].first, pe[p][b].first});
  std::vector<int> bdims(P.tdim.begin(), P.tdim.begin() + S.nB_keys);
  S.Spat = MakePattern(bdims, pairs);
  const int64_t nsb = S.Spat.nblocks();
  std::vector<std::vector<std::pair<int64_t, int64_t>>> terms(nsb);
  for (int p = 0; p < S.npoints; ++p) {
    const int64_t e0 = S.pt_eptr[p];
    for (size_t a = 0; a < pe[p].size(); ++a)
      for (size_t b = 0; b <= a; ++b) {
        // pe sorted ascending: a >= b => key_a >= key_b
        const int64_t blk = S.Spat.Find(pe[p][a].first, pe[p][b].first);
        terms[blk].push_back({S.pt_eoff[e0 + a], S.pt_woff[e0 + b]});
      }
  }
  S.sb_ptr.push_back(0);
  for (int j = 0; j < S.nB_keys; ++j)
    for (int64_t q = S.Spat.colptr[j]; q < S.Spat.colptr[j + 1]; ++q) {
      const int i = S.Spat.rows[q];
      for (auto& t : terms[q]) {
        S.sb_eoff.push_back(t.first);
        S.sb_woff.push_back(t.second);
      }
      S.sb_ptr.push_back(int64_t(S.sb_eoff.size()));
      const int64_t hb = L.H.Find(i, j);
      S.sb_hoff.push_back(hb >= 0 ? L.H.boff[hb] : -1);
      S.sb_soff.push_back(S.Spat.boff[q]);
      S.sb_dk.push_back(P.tdim[i]);
      S.sb_dl.push_back(P.tdim[j]);
      S.sb_diag_toff.push_back(i == j ? int32_t(P.toff[i]) : -1);
    }
  // reduced rhs lists
  std::vector<std::vector<int64_t>> rl(S.nB);  // per B scalar: indices into (eoff, col, dk, pt)
  S.r_ptr.assign(S.nB + 1, 0);
  std::vector<int64_t> cntr(S.nB, 0);
  for (int p = 0; p < S.npoints; ++p)
    for (auto& e : pe[p])
      for (int c = 0; c < P.tdim[e.first]; ++c) cntr[P.toff[e.first] + c]++;
  for (int64_t i = 0; i < S.nB; ++i) S.r_ptr[i + 1] = S.r_ptr[i] + cntr[i];
  const int64_t nr = S.r_ptr[S.nB];
  S.r_eoff.resize(nr);
  S.r_ecol.resize(nr);
  S.r_dk.resize(nr);
  S.r_pt.resize(nr);
  std::vector<int64_t> fill(S.r_ptr.begin(), S.r_ptr.end() - 1);
  for (int p = 0; p < S.npoints; ++p)
    for (auto& e : pe[p])
      for (int c = 0; c < P.tdim[e.first]; ++c) {
        const int64_t i = P.toff[e.first] + c;
        const int64_t q = fill[i]++;
        S.r_eoff[q] = e.second;
        S.r_ecol[q] = c;
        S.r_dk[q] = P.tdim[e.first];
        S.r_pt[q] = p;
      }
  return S;
}

}  // namespace sfg
