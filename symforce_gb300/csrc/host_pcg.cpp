// Camera blocks of the reduced camera system for the PCG forms (host, once per structure).
#include <algorithm>
#include <numeric>
#include <set>

#include "kernels.h"
#include "layout.h"

namespace sfg {

namespace {
int Find(std::vector<int>& parent, int a) {
  while (parent[a] != a) a = parent[a] = parent[parent[a]];
  return a;
}
}  // namespace

PrecondLayout BuildPrecondLayout(const HostProblem& P, const SchurLayout& SL) {
  constexpr int kB = kPrecondBlock;
  const int nbk = SL.nB_keys;
  std::vector<int> parent(nbk);
  std::iota(parent.begin(), parent.end(), 0);
  for (const HostBatch& b : P.batches)
    for (int f = 0; f < b.count; ++f) {
      int first = -1;
      for (int k = 0; k < b.nk; ++k) {
        const int key = b.keys[size_t(f) * b.nk + k];
        if (key >= nbk) continue;
        if (first < 0) {
          first = key;
        } else {
          const int ra = Find(parent, first), rb = Find(parent, key);
          if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
        }
      }
    }
  // blocks in order of their first key; keys inside a block in key order
  std::vector<int> group_of_root(nbk, -1), key_group(nbk);
  std::vector<std::vector<int>> members;
  for (int k = 0; k < nbk; ++k) {
    const int r = Find(parent, k);
    if (group_of_root[r] < 0) {
      group_of_root[r] = int(members.size());
      members.emplace_back();
    }
    key_group[k] = group_of_root[r];
    members[key_group[k]].push_back(k);
  }
  PrecondLayout L;
  L.ng = int(members.size());
  L.gidx.assign(size_t(L.ng) * kB, -1);
  L.goff.assign(size_t(L.ng) * kB * kB, -1);
  L.degree.assign(L.ng, 0.f);
  L.scalar_group.assign(SL.nB, -1);
  L.sdiag_off.assign(SL.nB, -1);
  L.gauge_soff.assign(size_t(L.ng) * kB, -1);
  L.gauge_comp.assign(size_t(L.ng) * kB, 0);
  const BlockPattern& S = SL.Spat;
  // the reduced system keeps only the lower triangle of its diagonal key blocks up to date
  auto entry_offset = [&](int ka, int ta, int kb, int tb) -> int64_t {
    if (ka < kb || (ka == kb && ta < tb)) {
      std::swap(ka, kb);
      std::swap(ta, tb);
    }
    const int64_t q = S.Find(ka, kb);
    if (q < 0) return -1;
    return S.boff[q] + int64_t(ta) * S.dim[kb] + tb;
  };
  for (int g = 0; g < L.ng; ++g) {
    std::vector<std::pair<int, int>> dims;  // (key, tangent index)
    for (int k : members[g])
      for (int t = 0; t < S.dim[k]; ++t) dims.push_back({k, t});
    if (int(dims.size()) > kB)
      throw Error(SFG_ERR_STRUCTURE, "a camera block of the reduced system has " +
                                         std::to_string(dims.size()) +
                                         " scalars; the PCG forms support at most 9");
    for (size_t a = 0; a < dims.size(); ++a) {
      const int64_t s = S.off[dims[a].first] + dims[a].second;
      L.gidx[size_t(g) * kB + a] = int32_t(s);
      L.scalar_group[s] = g;
      if (P.key_type[dims[a].first] == SFG_KEY_POSE3) {
        L.gauge_soff[size_t(g) * kB + a] = P.soff[dims[a].first];
        L.gauge_comp[size_t(g) * kB + a] = dims[a].second;
        ++L.gauge_rows;
      }
      for (size_t b = 0; b < dims.size(); ++b) {
        const int64_t o = entry_offset(dims[a].first, dims[a].second, dims[b].first, dims[b].second);
        L.goff[(size_t(g) * kB + a) * kB + b] = o < 0 ? -2 : o;  // -2: structurally zero
      }
    }
  }
  for (int k = 0; k < nbk; ++k) {
    const int64_t q = S.Find(k, k);
    for (int t = 0; t < S.dim[k]; ++t) L.sdiag_off[S.off[k] + t] = S.boff[q] + int64_t(t) * S.dim[k] + t;
  }
  std::vector<std::set<int>> nbr(L.ng);
  for (int j = 0; j < nbk; ++j)
    for (int64_t q = S.colptr[j]; q < S.colptr[j + 1]; ++q) {
      const int gi = key_group[S.rows[q]], gj = key_group[j];
      if (gi != gj) {
        nbr[gi].insert(gj);
        nbr[gj].insert(gi);
      }
    }
  for (int g = 0; g < L.ng; ++g) L.degree[g] = float(nbr[g].size());
  // 9 x 9 group blocks of S: stored lower blocks (g, h <= g) with the S offset of each entry, and
  // per group row its entries (stored block, neighbour, transposed) in neighbour order
  std::vector<std::vector<int>> lower(L.ng);
  for (int g = 0; g < L.ng; ++g) {
    lower[g].push_back(g);
    for (int h : nbr[g])
      if (h < g) lower[g].push_back(h);
    std::sort(lower[g].begin(), lower[g].end());
  }
  std::vector<std::vector<std::pair<int, int>>> row_entries(L.ng);  // (neighbour, block)
  for (int g = 0; g < L.ng; ++g)
    for (int h : lower[g]) {
      const int q = int(L.blk_row.size());
      L.blk_row.push_back(g);
      L.blk_col.push_back(h);
      for (int a = 0; a < kB; ++a)
        for (int b = 0; b < kB; ++b) {
          const int32_t sa = L.gidx[size_t(g) * kB + a], sb = L.gidx[size_t(h) * kB + b];
          int64_t o = -1;
          if (sa >= 0 && sb >= 0) {
            const int ka = int(std::upper_bound(S.off.begin(), S.off.end(), int64_t(sa)) - S.off.begin()) - 1;
            const int kb2 = int(std::upper_bound(S.off.begin(), S.off.end(), int64_t(sb)) - S.off.begin()) - 1;
            o = entry_offset(ka, int(sa - S.off[ka]), kb2, int(sb - S.off[kb2]));
            if (o < 0) o = -2;
          }
          L.blk_off.push_back(o);
        }
      row_entries[g].push_back({h, q});
      if (h != g) row_entries[h].push_back({g, q});
    }
  L.gptr.assign(L.ng + 1, 0);
  for (int g = 0; g < L.ng; ++g) {
    std::sort(row_entries[g].begin(), row_entries[g].end());
    for (auto& e : row_entries[g]) {
      L.gent.push_back(e.second);
      L.gent.push_back((e.first << 1) | (e.first > g ? 1 : 0));
    }
    L.gptr[g + 1] = int32_t(L.gent.size() / 2);
  }
  return L;
}

BandPattern BuildBandPattern(const PrecondLayout& L, int band) {
  BandPattern B;
  B.band = band;
  const int K1 = band + 1;
  // stored lower group blocks by row: (column, block), ascending (blk_row is nondecreasing)
  std::vector<std::vector<std::pair<int, int>>> lower(L.ng);
  for (size_t q = 0; q < L.blk_row.size(); ++q) lower[L.blk_row[q]].push_back({L.blk_col[q], int(q)});
  for (auto& r : lower) std::sort(r.begin(), r.end());
  auto find = [&](int g, int h) {
    auto it = std::lower_bound(lower[g].begin(), lower[g].end(), std::make_pair(h, -1));
    return (it != lower[g].end() && it->first == h) ? it->second : -1;
  };
  B.nj.assign(L.ng, 0);
  B.jgrp.assign(size_t(L.ng) * K1, -1);
  B.jblk.assign(size_t(L.ng) * K1 * K1, -1);
  for (int l = 0; l < L.ng; ++l) {
    std::vector<int> J;
    for (const auto& e : lower[l])
      if (e.first >= l - band && e.first < l) J.push_back(e.first);
    J.push_back(l);
    B.nj[l] = int32_t(J.size());
    for (size_t s1 = 0; s1 < J.size(); ++s1) {
      B.jgrp[size_t(l) * K1 + s1] = J[s1];
      for (size_t s2 = 0; s2 <= s1; ++s2) B.jblk[(size_t(l) * K1 + s1) * K1 + s2] = find(J[s1], J[s2]);
    }
  }
  return B;
}

}  // namespace sfg
