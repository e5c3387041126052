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
  // row-major index of the stored blocks, so that a block is found in the shorter of its row and
  // its column (a point's row holds a few camera blocks; a camera's column, every point it sees)
  std::vector<int64_t> hr_ptr(size_t(L.H.nb) + 1, 0);
  for (int64_t q = 0; q < L.H.nblocks(); ++q) hr_ptr[size_t(L.H.rows[q]) + 1]++;
  for (int i = 0; i < L.H.nb; ++i) hr_ptr[i + 1] += hr_ptr[i];
  std::vector<int32_t> hr_col(static_cast<size_t>(L.H.nblocks()));
  std::vector<int64_t> hr_blk(hr_col.size());
  {
    std::vector<int64_t> fill(hr_ptr.begin(), hr_ptr.end() - 1);
    for (int j = 0; j < L.H.nb; ++j)
      for (int64_t q = L.H.colptr[j]; q < L.H.colptr[j + 1]; ++q) {
        const int64_t at = fill[L.H.rows[q]]++;
        hr_col[at] = j;  // ascending: columns are visited in order
        hr_blk[at] = q;
      }
  }
  auto find_block = [&](int i, int j) -> int64_t {  // i >= j, the block must exist
    if (hr_ptr[i + 1] - hr_ptr[i] < L.H.colptr[j + 1] - L.H.colptr[j]) {
      const auto b = hr_col.begin() + hr_ptr[i], e = hr_col.begin() + hr_ptr[i + 1];
      return hr_blk[std::lower_bound(b, e, j) - hr_col.begin()];
    }
    return L.H.Find(i, j);
  };
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
  // Device factor f of batch bi is a later factor of a merged warp: its merged entries are carried
  // by the warp's first factor, and it contributes only the others.
  auto merged_tail = [&](size_t bi, int f) {
    if (merged_dims[bi] == 0 || (f & 31) == 0) return false;
    const size_t w = size_t(f) / 32;
    return w < warp_merged[bi].size() && warp_merged[bi][w] != 0;
  };
  // the merged entries of a batch's packing: the packed prefix and the rhs prefix of its merged
  // key slots
  auto merged_entries = [&](size_t bi, int nh, int nent) {
    const int mt = merged_dims[bi];
    std::vector<char> m(size_t(nent), 0);
    for (int e = 0; e < nent; ++e) m[e] = e < nh ? e < mt * (mt + 1) / 2 : e - nh < mt;
    return m;
  };
  // Packed entries by key-slot pair: a factor's keys are distinct (ParseProblem), so the entries
  // of one pair of its key slots fill one stored block (the lower triangle of a diagonal block, a
  // whole off-diagonal block), and every value of a block has the same contributors.  The counts
  // and the staging ranks below are therefore kept per block, and an entry's slot is its block's
  // offset plus its place inside the block, stored (max key, min key) row-major.
  struct EntryPlace {
    std::vector<int32_t> pair;    // key-slot pair sa * (sa + 1) / 2 + sb (sa >= sb) of entry e < nh
    std::vector<int32_t> off;     // place in the block stored as (key of sa, key of sb)
    std::vector<int32_t> off_sw;  // place in the block stored as (key of sb, key of sa)
    std::vector<int32_t> lidx;    // diagonal pair (sa == sb): rank of the entry in the lower
                                  // triangle (row-major); -1 for other pairs
    std::vector<int32_t> rslot, rloc;  // rhs entry: key slot and row inside the key
  };
  std::vector<EntryPlace> places(P.batches.size());
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    std::vector<int> ks, lo;
    for (int sl = 0; sl < B.nk; ++sl)
      for (int r = 0; r < B.key_tdim[sl]; ++r) {
        ks.push_back(sl);
        lo.push_back(r);
      }
    EntryPlace& E = places[bi];
    for (int a = 0; a < B.tdim; ++a)
      for (int b = 0; b <= a; ++b) {
        const int sa = ks[a], sb = ks[b], ra = lo[a], rb = lo[b];
        E.pair.push_back(sa * (sa + 1) / 2 + sb);
        E.off.push_back(ra * B.key_tdim[sb] + rb);
        E.off_sw.push_back(rb * B.key_tdim[sa] + ra);
        E.lidx.push_back(sa == sb ? ra * (ra + 1) / 2 + rb : -1);
      }
    for (int a = 0; a < B.tdim; ++a) {
      E.rslot.push_back(ks[a]);
      E.rloc.push_back(lo[a]);
    }
  }
  // the stored block of each key-slot pair of the user's factor f (swapped: stored as (kb, ka))
  auto factor_blocks = [&](const HostBatch& B, int f, int64_t* blk, char* swapped) {
    const int32_t* keys = &B.keys[size_t(f) * B.nk];
    for (int sa = 0; sa < B.nk; ++sa)
      for (int sb = 0; sb <= sa; ++sb) {
        const int ka = keys[sa], kb = keys[sb], pr = sa * (sa + 1) / 2 + sb;
        swapped[pr] = ka < kb;
        blk[pr] = ka >= kb ? find_block(ka, kb) : find_block(kb, ka);
      }
  };
  constexpr int kMaxPairs = 6;  // factors have at most three keys
  const int64_t nslots = L.nvals + P.N;
  std::vector<int32_t> cnt_blk(static_cast<size_t>(L.H.nblocks()), 0), cnt_key(P.nkeys, 0);
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    if (B.nk * (B.nk + 1) / 2 > kMaxPairs) throw Error(SFG_ERR_STRUCTURE, "factor with more than three keys");
    const int ms = MergedKeySlots(B.kind);
    int64_t blk[kMaxPairs];
    char swapped[kMaxPairs];
    for (int f = 0; f < B.count; ++f) {
      const int uf = order[bi][f];
      factor_blocks(B, uf, blk, swapped);
      const bool tail = merged_tail(bi, f);
      for (int sa = 0; sa < B.nk; ++sa) {
        if (tail && sa < ms) continue;  // carried by the warp's first factor
        for (int sb = 0; sb <= sa; ++sb) cnt_blk[blk[sa * (sa + 1) / 2 + sb]]++;
        cnt_key[B.keys[size_t(uf) * B.nk + sa]]++;
      }
    }
  }
  // Every stored value must receive at least one contribution (the reference sets explicit zeros
  // from the first linearization; the block pattern never has untouched entries except the strict
  // upper part of diagonal blocks, which is not a slot).
  for (int64_t q = 0; q < L.H.nblocks(); ++q)
    if (cnt_blk[q] == 0) throw Error(SFG_ERR_STRUCTURE, "Hessian entry without a contributor");
  for (int k = 0; k < P.nkeys; ++k)
    if (cnt_key[k] == 0) throw Error(SFG_ERR_STRUCTURE, "Hessian entry without a contributor");
  // Staging groups in slot order: every slot of a block (the lower triangle of a diagonal block)
  // with more than one contributor gets as many consecutive staging slots as its block has
  // contributors.  base_blk / base_key: the first staging slot of the block's (the key's rhs's)
  // first slot, or -1 when its slots have one contributor each and are written in place.
  constexpr int64_t kSinkLimit = int64_t(1) << 31;
  if (nslots >= kSinkLimit) throw Error(SFG_ERR_STRUCTURE, "problem too large for 32-bit sink indices");
  std::vector<int32_t> base_blk(cnt_blk.size(), -1), base_key(P.nkeys, -1);
  L.red_ptr.push_back(0);
  auto stage = [&](int64_t slot, int32_t c) {
    if (nslots + L.red_ptr.back() + c >= kSinkLimit)
      throw Error(SFG_ERR_STRUCTURE, "problem too large for 32-bit sink indices");
    L.red_dst.push_back(int32_t(slot));
    L.red_ptr.push_back(L.red_ptr.back() + c);
  };
  for (int kc = 0; kc < P.nkeys; ++kc)
    for (int64_t q = L.H.colptr[kc]; q < L.H.colptr[kc + 1]; ++q) {
      const int32_t c = cnt_blk[q];
      if (c <= 1) continue;
      base_blk[q] = int32_t(nslots + L.red_ptr.back());
      const int dc = P.tdim[kc], dr = P.tdim[L.H.rows[q]];
      const bool diag = L.H.rows[q] == kc;
      for (int r = 0; r < dr; ++r)
        for (int cc = 0; cc < (diag ? r + 1 : dc); ++cc) stage(L.H.boff[q] + int64_t(r) * dc + cc, c);
    }
  for (int k = 0; k < P.nkeys; ++k) {
    const int32_t c = cnt_key[k];
    if (c <= 1) continue;
    base_key[k] = int32_t(nslots + L.red_ptr.back());
    for (int r = 0; r < P.tdim[k]; ++r) stage(L.nvals + P.toff[k] + r, c);
  }
  L.nstage = L.red_ptr.back();
  // Sink of the contribution of rank k (device factor order) in its block: the slot itself for a
  // single contributor, else base + (place of the slot among the block's slots) * count + k.
  std::vector<int32_t> count_blk(cnt_blk), count_key(cnt_key);
  std::fill(cnt_blk.begin(), cnt_blk.end(), 0);
  std::fill(cnt_key.begin(), cnt_key.end(), 0);
  std::vector<int32_t>& rank_blk = cnt_blk;
  std::vector<int32_t>& rank_key = cnt_key;
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    const EntryPlace& E = places[bi];
    const int ms = MergedKeySlots(B.kind);
    LinLayout::BatchMap M;
    const int nh = B.tdim * (B.tdim + 1) / 2;
    M.nent = nh + B.tdim;
    M.merged_dims = merged_dims[bi];
    M.dest.resize(size_t(M.nent) * B.count);
    // factors in runs of 32 (a warp): sink indices in factor order, then written entry-major
    constexpr int kRun = 32;
    std::vector<int32_t> run(size_t(kRun) * M.nent);
    const std::vector<char> merged = merged_entries(bi, nh, M.nent);
    int64_t blk[kMaxPairs], base[kMaxPairs];
    char swapped[kMaxPairs];
    int32_t rank[kMaxPairs], sbase[kMaxPairs], scount[kMaxPairs];
    int32_t rank_rhs[3], rbase[3], rcount[3];
    for (int f0 = 0; f0 < B.count; f0 += kRun) {
      const int nf = std::min(kRun, B.count - f0);
      for (int j = 0; j < nf; ++j) {
        const int f = f0 + j, uf = order[bi][f];
        const int32_t* keys = &B.keys[size_t(uf) * B.nk];
        factor_blocks(B, uf, blk, swapped);
        const bool tail = merged_tail(bi, f);
        for (int sa = 0; sa < B.nk; ++sa) {
          const bool skip = tail && sa < ms;
          for (int sb = 0; sb <= sa; ++sb) {
            const int pr = sa * (sa + 1) / 2 + sb;
            const int64_t q = blk[pr];
            base[pr] = L.H.boff[q];
            sbase[pr] = base_blk[q];
            scount[pr] = count_blk[q];
            rank[pr] = skip ? 0 : rank_blk[q]++;
          }
          const int kk = keys[sa];
          rbase[sa] = base_key[kk];
          rcount[sa] = count_key[kk];
          rank_rhs[sa] = skip ? 0 : rank_key[kk]++;
        }
        for (int e = 0; e < M.nent; ++e) {
          int32_t& out = run[size_t(e) * kRun + j];
          if (tail && merged[e]) {
            out = run[size_t(e) * kRun];  // never read: the warp's first factor stores
            continue;
          }
          if (e < nh) {
            const int pr = E.pair[e];
            const int32_t o = swapped[pr] ? E.off_sw[e] : E.off[e];
            if (sbase[pr] < 0) out = int32_t(base[pr] + o);
            else out = sbase[pr] + (E.lidx[e] >= 0 ? E.lidx[e] : o) * scount[pr] + rank[pr];
          } else {
            const int a = e - nh, sl = E.rslot[a];
            out = rbase[sl] < 0 ? int32_t(L.nvals + P.toff[keys[sl]] + E.rloc[a])
                                : rbase[sl] + E.rloc[a] * rcount[sl] + rank_rhs[sl];
          }
        }
      }
      for (int e = 0; e < M.nent; ++e)
        std::copy(run.begin() + size_t(e) * kRun, run.begin() + size_t(e) * kRun + nf,
                  M.dest.begin() + size_t(e) * B.count + f0);
    }
    M.order = std::move(order[bi]);
    L.maps.push_back(std::move(M));
  }
  // scalar entries of the CSC lower layout: full off-diagonal blocks, lower diagonal blocks
  for (int kc = 0; kc < P.nkeys; ++kc)
    for (int64_t q = L.H.colptr[kc]; q < L.H.colptr[kc + 1]; ++q) {
      const int64_t dr = P.tdim[L.H.rows[q]], dc = P.tdim[kc];
      L.nnz_lower += L.H.rows[q] == kc ? dc * (dc + 1) / 2 : dr * dc;
    }
  return L;
}

void BuildCscExport(LinLayout& L, const HostProblem& P) {
  if (!L.csc_colptr.empty()) return;
  L.csc_colptr.assign(P.N + 1, 0);
  L.csc_rowidx.reserve(size_t(L.nnz_lower));
  L.csc_src.reserve(size_t(L.nnz_lower));
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
      S.pt_of_e.push_back(p);
      S.pt_ekey_toff.push_back(int32_t(P.toff[e.first]));
      S.pt_ekey_dim.push_back(P.tdim[e.first]);
      S.nW += 3 * P.tdim[e.first];
    }
    S.pt_eptr.push_back(int64_t(S.pt_eoff.size()));
  }
  // points of every B key, in point order, with the offset of the point's E block for the key
  std::vector<int64_t> kp_ptr(size_t(S.nB_keys) + 1, 0);
  for (int p = 0; p < S.npoints; ++p)
    for (const auto& e : pe[p]) kp_ptr[size_t(e.first) + 1]++;
  for (int k = 0; k < S.nB_keys; ++k) kp_ptr[k + 1] += kp_ptr[k];
  std::vector<int32_t> kp(static_cast<size_t>(kp_ptr[S.nB_keys]));
  std::vector<int64_t> kp_eoff(kp.size());
  {
    std::vector<int64_t> fill(kp_ptr.begin(), kp_ptr.end() - 1);
    for (int p = 0; p < S.npoints; ++p)
      for (const auto& e : pe[p]) {
        const int64_t q = fill[e.first]++;
        kp[q] = p;
        kp_eoff[q] = e.second;
      }
  }
  // reduced pattern: the B-B blocks of H and every pair of B keys that share a point, found per
  // column key through its points (a stamp per row key keeps each pair once)
  std::vector<std::pair<int, int>> pairs;
  for (int j = 0; j < S.nB_keys; ++j)
    for (int64_t q = L.H.colptr[j]; q < L.H.colptr[j + 1]; ++q)
      if (L.H.rows[q] < S.nB_keys) pairs.push_back({L.H.rows[q], j});
  {
    std::vector<int> stamp(size_t(S.nB_keys), -1);
    for (int kb = 0; kb < S.nB_keys; ++kb)
      for (int64_t q = kp_ptr[kb]; q < kp_ptr[kb + 1]; ++q)
        for (const auto& e : pe[kp[q]])
          if (e.first >= kb && stamp[e.first] != kb) {
            stamp[e.first] = kb;
            pairs.push_back({e.first, kb});
          }
  }
  std::vector<int> bdims(P.tdim.begin(), P.tdim.begin() + S.nB_keys);
  S.Spat = MakePattern(bdims, pairs);
  const int64_t nsb = S.Spat.nblocks();
  // terms of every S block in point order (a counting sort by block over the terms in the order
  // points and their E pairs are visited)
  int64_t nterms = 0;
  for (int p = 0; p < S.npoints; ++p) nterms += int64_t(pe[p].size()) * (pe[p].size() + 1) / 2;
  std::vector<int32_t> tblk(static_cast<size_t>(nterms));
  S.sb_ptr.assign(size_t(nsb) + 1, 0);
  {
    int64_t t = 0;
    for (int p = 0; p < S.npoints; ++p)
      for (size_t a = 0; a < pe[p].size(); ++a)
        for (size_t b = 0; b <= a; ++b) {
          // pe sorted ascending: a >= b => key_a >= key_b
          const int64_t blk = S.Spat.Find(pe[p][a].first, pe[p][b].first);
          tblk[t++] = int32_t(blk);
          S.sb_ptr[blk + 1]++;
        }
  }
  for (int64_t q = 0; q < nsb; ++q) S.sb_ptr[q + 1] += S.sb_ptr[q];
  S.sb_eoff.resize(size_t(nterms));
  S.sb_woff.resize(size_t(nterms));
  {
    std::vector<int64_t> fill(S.sb_ptr.begin(), S.sb_ptr.end() - 1);
    int64_t t = 0;
    for (int p = 0; p < S.npoints; ++p) {
      const int64_t e0 = S.pt_eptr[p];
      for (size_t a = 0; a < pe[p].size(); ++a)
        for (size_t b = 0; b <= a; ++b) {
          const int64_t k = fill[tblk[t++]]++;
          S.sb_eoff[k] = S.pt_eoff[e0 + a];
          S.sb_woff[k] = S.pt_woff[e0 + b];
        }
    }
  }
  for (int j = 0; j < S.nB_keys; ++j)
    for (int64_t q = S.Spat.colptr[j]; q < S.Spat.colptr[j + 1]; ++q) {
      const int i = S.Spat.rows[q];
      const int64_t hb = L.H.Find(i, j);
      S.sb_hoff.push_back(hb >= 0 ? L.H.boff[hb] : -1);
      S.sb_soff.push_back(S.Spat.boff[q]);
      S.sb_dk.push_back(P.tdim[i]);
      S.sb_dl.push_back(P.tdim[j]);
      S.sb_diag_toff.push_back(i == j ? int32_t(P.toff[i]) : -1);
    }
  // reduced rhs lists: per B scalar, the points that see its key in point order
  S.r_ptr.assign(S.nB + 1, 0);
  for (int k = 0; k < S.nB_keys; ++k)
    for (int c = 0; c < P.tdim[k]; ++c) {
      const int64_t i = P.toff[k] + c;
      S.r_ptr[i + 1] = S.r_ptr[i] + (kp_ptr[k + 1] - kp_ptr[k]);
    }
  const int64_t nr = S.r_ptr[S.nB];
  S.r_eoff.resize(nr);
  S.r_ecol.resize(nr);
  S.r_dk.resize(nr);
  S.r_pt.resize(nr);
  for (int k = 0; k < S.nB_keys; ++k)
    for (int c = 0; c < P.tdim[k]; ++c) {
      int64_t q = S.r_ptr[P.toff[k] + c];
      for (int64_t u = kp_ptr[k]; u < kp_ptr[k + 1]; ++u, ++q) {
        S.r_eoff[q] = kp_eoff[u];
        S.r_ecol[q] = c;
        S.r_dk[q] = P.tdim[k];
        S.r_pt[q] = kp[u];
      }
    }
  return S;
}

}  // namespace sfg
