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
//
// Counts and staging ranks are kept per stored block (all values of a block have the same
// contributors), and the passes whose items are independent (factors' block lookups and sink
// indices, the Schur complement's columns) run on host threads; every array is the same as a
// sequential pass gives.
#include <algorithm>
#include <numeric>
#include <thread>

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
    // stable sort by the merged key slots, lexicographic: counting sorts from the last slot
    {
      std::vector<int32_t> tmp(ord.size());
      std::vector<int64_t> cnt(size_t(P.nkeys) + 1);
      for (int s = ms - 1; s >= 0; --s) {
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int32_t f : ord) cnt[size_t(key(f, s)) + 1]++;
        for (int k = 0; k < P.nkeys; ++k) cnt[k + 1] += cnt[k];
        for (int32_t f : ord) tmp[size_t(cnt[key(f, s)]++)] = f;
        ord.swap(tmp);
      }
    }
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
  if (L.H.nblocks() >= (int64_t(1) << 31)) throw Error(SFG_ERR_STRUCTURE, "too many Hessian blocks");
  const unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  // run fn(i0, i1) over [0, n) in contiguous parts on host threads
  auto parallel = [&](int64_t n, int64_t min_part, auto&& fn) {
    const int nt = int(std::min<int64_t>(nthreads, std::max<int64_t>(1, n / min_part)));
    if (nt <= 1) {
      fn(int64_t(0), n);
      return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
    for (auto& th : pool) th.join();
  };
  // the stored block of every key-slot pair of every factor (device order) and its orientation
  std::vector<std::vector<int32_t>> fblk(P.batches.size());
  std::vector<std::vector<uint8_t>> fswap(P.batches.size());
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    const int npair = B.nk * (B.nk + 1) / 2;
    if (npair > kMaxPairs) throw Error(SFG_ERR_STRUCTURE, "factor with more than three keys");
    fblk[bi].resize(size_t(B.count) * npair);
    fswap[bi].resize(B.count);
    parallel(B.count, 4096, [&](int64_t f0, int64_t f1) {
      int64_t blk[kMaxPairs];
      char swapped[kMaxPairs];
      for (int64_t f = f0; f < f1; ++f) {
        factor_blocks(B, order[bi][f], blk, swapped);
        uint8_t bits = 0;
        for (int pr = 0; pr < npair; ++pr) {
          fblk[bi][size_t(f) * npair + pr] = int32_t(blk[pr]);
          bits |= uint8_t(swapped[pr] ? 1 : 0) << pr;
        }
        fswap[bi][f] = bits;
      }
    });
  }
  // Contributors per block and per key (rhs) in device factor order; the count before a factor's
  // contribution is that contribution's rank, kept per factor for the sink pass (key-slot pairs,
  // then the key slots' rhs).
  std::vector<int32_t> cnt_blk(static_cast<size_t>(L.H.nblocks()), 0), cnt_key(P.nkeys, 0);
  std::vector<std::vector<int32_t>> ranks(P.batches.size());
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    const int npair = B.nk * (B.nk + 1) / 2, nr = npair + B.nk;
    const int ms = MergedKeySlots(B.kind);
    ranks[bi].resize(size_t(B.count) * nr);
    for (int f = 0; f < B.count; ++f) {
      const int uf = order[bi][f];
      int32_t* rk = &ranks[bi][size_t(f) * nr];
      const int32_t* blk = &fblk[bi][size_t(f) * npair];
      const bool tail = merged_tail(bi, f);
      for (int sa = 0; sa < B.nk; ++sa) {
        const bool skip = tail && sa < ms;  // carried by the warp's first factor
        for (int sb = 0; sb <= sa; ++sb) {
          const int pr = sa * (sa + 1) / 2 + sb;
          rk[pr] = skip ? 0 : cnt_blk[blk[pr]]++;
        }
        rk[npair + sa] = skip ? 0 : cnt_key[B.keys[size_t(uf) * B.nk + sa]]++;
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
  // Factors are independent here, so runs of them are spread over host threads.
  for (size_t bi = 0; bi < P.batches.size(); ++bi) {
    const auto& B = P.batches[bi];
    const EntryPlace& E = places[bi];
    const int npair = B.nk * (B.nk + 1) / 2, nr = npair + B.nk;
    LinLayout::BatchMap M;
    const int nh = B.tdim * (B.tdim + 1) / 2;
    M.nent = nh + B.tdim;
    M.merged_dims = merged_dims[bi];
    M.dest.resize(size_t(M.nent) * B.count);
    // factors in runs of 32 (a warp): sink indices in factor order, then written entry-major
    constexpr int kRun = 32;
    const std::vector<char> merged = merged_entries(bi, nh, M.nent);
    const int nruns = (B.count + kRun - 1) / kRun;
    auto work = [&](int64_t run0, int64_t run1) {
      std::vector<int32_t> run(size_t(kRun) * M.nent);
      int64_t base[kMaxPairs];
      char swapped[kMaxPairs];
      int32_t sbase[kMaxPairs], scount[kMaxPairs], rbase[3], rcount[3];
      for (int64_t ru = run0; ru < run1; ++ru) {
        const int f0 = int(ru) * kRun, nf = std::min(kRun, B.count - f0);
        for (int j = 0; j < nf; ++j) {
          const int f = f0 + j, uf = order[bi][f];
          const int32_t* keys = &B.keys[size_t(uf) * B.nk];
          const int32_t* rk = &ranks[bi][size_t(f) * nr];
          const int32_t* blk = &fblk[bi][size_t(f) * npair];
          const uint8_t bits = fswap[bi][f];
          const bool tail = merged_tail(bi, f);
          for (int pr = 0; pr < npair; ++pr) {
            base[pr] = L.H.boff[blk[pr]];
            sbase[pr] = base_blk[blk[pr]];
            scount[pr] = cnt_blk[blk[pr]];
            swapped[pr] = (bits >> pr) & 1;
          }
          for (int sa = 0; sa < B.nk; ++sa) {
            rbase[sa] = base_key[keys[sa]];
            rcount[sa] = cnt_key[keys[sa]];
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
              else out = sbase[pr] + (E.lidx[e] >= 0 ? E.lidx[e] : o) * scount[pr] + rk[pr];
            } else {
              const int a = e - nh, sl = E.rslot[a];
              out = rbase[sl] < 0 ? int32_t(L.nvals + P.toff[keys[sl]] + E.rloc[a])
                                  : rbase[sl] + E.rloc[a] * rcount[sl] + rk[npair + sl];
            }
          }
        }
        for (int e = 0; e < M.nent; ++e)
          std::copy(run.begin() + size_t(e) * kRun, run.begin() + size_t(e) * kRun + nf,
                    M.dest.begin() + size_t(e) * B.count + f0);
      }
    };
    parallel(nruns, 64, work);
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

SchurLayout BuildSchurLayout(const HostProblem& P, const LinLayout& L, bool g_at_e) {
  SchurLayout S;
  S.nB_keys = P.nkeys - P.num_schur;
  S.npoints = P.num_schur;
  S.nB = P.toff[S.nB_keys];
  S.c_toff = S.nB;
  for (int k = S.nB_keys; k < P.nkeys; ++k)
    if (P.tdim[k] != 3) throw Error(SFG_ERR_STRUCTURE, "Schur keys must be 3-dimensional");
  const unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  // run fn(i0, i1) over [0, n) in contiguous parts on host threads
  auto parallel = [&](int64_t n, int64_t min_part, auto&& fn) {
    const int nt = int(std::min<int64_t>(nthreads, std::max<int64_t>(1, n / min_part)));
    if (nt <= 1) {
      fn(int64_t(0), n);
      return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
    for (auto& th : pool) th.join();
  };
  // E lists per point (compressed rows), sorted by B key: the points' rows of the B columns of H
  std::vector<int64_t> pe_ptr(size_t(S.npoints) + 1, 0);
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
      pe_ptr[size_t(i - S.nB_keys) + 1]++;
    }
  for (int p = 0; p < S.npoints; ++p) pe_ptr[p + 1] += pe_ptr[p];
  const int64_t ne = pe_ptr[S.npoints];
  std::vector<int32_t> pe_key(static_cast<size_t>(ne));
  std::vector<int64_t> pe_boff(static_cast<size_t>(ne));
  // e_order (G at E's offsets): the E blocks in the order of their Hessian offsets (key-major), so
  // that the kernel forming G = L^-1 E writes (and reads) consecutive addresses
  if (g_at_e) S.e_order.resize(size_t(ne));
  {
    std::vector<int64_t> fill(pe_ptr.begin(), pe_ptr.end() - 1);
    int64_t km = 0;
    for (int j = 0; j < S.nB_keys; ++j)  // ascending B keys: each point's list comes out sorted
      for (int64_t q = L.H.colptr[j]; q < L.H.colptr[j + 1]; ++q) {
        const int i = L.H.rows[q];
        if (i < S.nB_keys) continue;
        const int64_t at = fill[i - S.nB_keys]++;
        pe_key[at] = j;
        pe_boff[at] = L.H.boff[q];
        if (g_at_e) S.e_order[size_t(km++)] = at;
      }
  }
  S.pt_diag.resize(S.npoints);
  S.pt_eptr.assign(pe_ptr.begin(), pe_ptr.end());
  S.pt_eoff.resize(ne);
  S.pt_woff.resize(ne);
  S.pt_of_e.resize(ne);
  S.pt_ekey_toff.resize(ne);
  S.pt_ekey_dim.resize(ne);
  for (int p = 0; p < S.npoints; ++p) {
    const int kp = S.nB_keys + p;
    S.pt_diag[p] = L.H.boff[L.H.Find(kp, kp)];
    for (int64_t e = pe_ptr[p]; e < pe_ptr[p + 1]; ++e) {
      S.pt_eoff[e] = pe_boff[e];
      S.pt_woff[e] = S.nW;
      S.pt_of_e[e] = p;
      S.pt_ekey_toff[e] = int32_t(P.toff[pe_key[e]]);
      S.pt_ekey_dim[e] = P.tdim[pe_key[e]];
      S.nW += 3 * P.tdim[pe_key[e]];
    }
  }
  // points of every B key, in point order, with the offset of the point's E block for the key and
  // the key's place in the point's list
  std::vector<int64_t> kp_ptr(size_t(S.nB_keys) + 1, 0);
  for (int64_t e = 0; e < ne; ++e) kp_ptr[size_t(pe_key[e]) + 1]++;
  for (int k = 0; k < S.nB_keys; ++k) kp_ptr[k + 1] += kp_ptr[k];
  std::vector<int32_t> kp(static_cast<size_t>(kp_ptr[S.nB_keys])), kp_pos(kp.size());
  std::vector<int64_t> kp_eoff(kp.size());
  {
    std::vector<int64_t> fill(kp_ptr.begin(), kp_ptr.end() - 1);
    for (int p = 0; p < S.npoints; ++p)
      for (int64_t e = pe_ptr[p]; e < pe_ptr[p + 1]; ++e) {
        const int64_t q = fill[pe_key[e]]++;
        kp[q] = p;
        kp_pos[q] = int32_t(e - pe_ptr[p]);
        kp_eoff[q] = pe_boff[e];
      }
  }
  // reduced pattern: the B-B blocks of H and every pair of B keys that share a point, found per
  // column key through its points (a stamp per row key keeps each pair once)
  std::vector<std::pair<int, int>> pairs;
  for (int j = 0; j < S.nB_keys; ++j)
    for (int64_t q = L.H.colptr[j]; q < L.H.colptr[j + 1]; ++q)
      if (L.H.rows[q] < S.nB_keys) pairs.push_back({L.H.rows[q], j});
  {
    std::vector<std::vector<std::pair<int, int>>> found(nthreads);
    std::vector<int64_t> part_start;
    {
      const int nt = int(std::min<int64_t>(nthreads, std::max<int64_t>(1, S.nB_keys / 16)));
      for (int t = 0; t <= nt; ++t) part_start.push_back(int64_t(S.nB_keys) * t / nt);
    }
    const int nparts = int(part_start.size()) - 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < nparts; ++t)
      pool.emplace_back([&, t] {
        std::vector<int> stamp(size_t(S.nB_keys), -1);
        for (int kb = int(part_start[t]); kb < int(part_start[t + 1]); ++kb)
          for (int64_t q = kp_ptr[kb]; q < kp_ptr[kb + 1]; ++q) {
            const int p = kp[q];
            for (int64_t e = pe_ptr[p]; e < pe_ptr[p + 1]; ++e) {
              const int ka = pe_key[e];
              if (ka >= kb && stamp[ka] != kb) {
                stamp[ka] = kb;
                found[t].push_back({ka, kb});
              }
            }
          }
      });
    for (auto& th : pool) th.join();
    for (int t = 0; t < nparts; ++t) pairs.insert(pairs.end(), found[t].begin(), found[t].end());
  }
  std::vector<int> bdims(P.tdim.begin(), P.tdim.begin() + S.nB_keys);
  S.Spat = MakePattern(bdims, pairs);
  const int64_t nsb = S.Spat.nblocks();
  // Terms of every S block in point order.  The blocks of column key kb take their terms from the
  // points that see kb (in point order, so each block's terms come out in point order), one term
  // per E pair (a >= b) of the point with kb at b; a dense row map per column finds the blocks.
  // Columns are independent (disjoint blocks): counted, then filled, in parallel.
  auto for_columns = [&](auto&& fn) {
    const int nt = int(std::min<int64_t>(nthreads, std::max(1, S.nB_keys / 16)));
    auto part = [&](int t) {
      std::vector<int64_t> row_blk(size_t(S.nB_keys), -1);
      for (int kb = int(int64_t(S.nB_keys) * t / nt); kb < int(int64_t(S.nB_keys) * (t + 1) / nt); ++kb) {
        for (int64_t q = S.Spat.colptr[kb]; q < S.Spat.colptr[kb + 1]; ++q) row_blk[S.Spat.rows[q]] = q;
        for (int64_t u = kp_ptr[kb]; u < kp_ptr[kb + 1]; ++u) {
          const int p = kp[u], b = kp_pos[u];
          const int64_t e0 = pe_ptr[p], n = pe_ptr[p + 1] - e0;
          for (int64_t a = b; a < n; ++a) fn(row_blk[pe_key[e0 + a]], e0 + a, e0 + b);  // pair in the pattern
        }
      }
    };
    if (nt <= 1) {
      part(0);
    } else {
      std::vector<std::thread> pool;
      for (int t = 0; t < nt; ++t) pool.emplace_back(part, t);
      for (auto& th : pool) th.join();
    }
  };
  S.g_at_e = g_at_e;
  S.nG = g_at_e ? L.nvals : S.nW;
  S.sb_ptr.assign(size_t(nsb) + 1, 0);
  for_columns([&](int64_t blk, int64_t, int64_t) { S.sb_ptr[blk + 1]++; });
  for (int64_t q = 0; q < nsb; ++q) S.sb_ptr[q + 1] += S.sb_ptr[q];
  const int64_t nterms = S.sb_ptr[nsb];
  S.sb_eoff.resize(size_t(nterms));
  S.sb_woff.resize(size_t(nterms));
  {
    std::vector<int64_t> fill(S.sb_ptr.begin(), S.sb_ptr.end() - 1);
    for_columns([&](int64_t blk, int64_t ea, int64_t eb) {
      const int64_t k = fill[blk]++;
      // both operands are G = L^-1 E blocks (at E's offsets or at W's)
      S.sb_eoff[k] = g_at_e ? S.pt_eoff[ea] : S.pt_woff[ea];
      S.sb_woff[k] = g_at_e ? S.pt_eoff[eb] : S.pt_woff[eb];
    });
  }
  S.sb_hoff.resize(size_t(nsb));
  S.sb_soff.resize(size_t(nsb));
  S.sb_dk.resize(size_t(nsb));
  S.sb_dl.resize(size_t(nsb));
  S.sb_diag_toff.resize(size_t(nsb));
  parallel(S.nB_keys, 16, [&](int64_t j0, int64_t j1) {
    for (int j = int(j0); j < int(j1); ++j)
      for (int64_t q = S.Spat.colptr[j]; q < S.Spat.colptr[j + 1]; ++q) {
        const int i = S.Spat.rows[q];
        const int64_t hb = L.H.Find(i, j);
        S.sb_hoff[q] = hb >= 0 ? L.H.boff[hb] : -1;
        S.sb_soff[q] = S.Spat.boff[q];
        S.sb_dk[q] = P.tdim[i];
        S.sb_dl[q] = P.tdim[j];
        S.sb_diag_toff[q] = i == j ? int32_t(P.toff[i]) : -1;
      }
  });
  S.bkey_toff.resize(size_t(S.nB_keys) + 1);
  for (int k = 0; k <= S.nB_keys; ++k) S.bkey_toff[size_t(k)] = int32_t(k < S.nB_keys ? P.toff[k] : S.nB);
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
  parallel(S.nB_keys, 16, [&](int64_t k0, int64_t k1) {
    for (int k = int(k0); k < int(k1); ++k)
      for (int c = 0; c < P.tdim[k]; ++c) {
        int64_t q = S.r_ptr[P.toff[k] + c];
        for (int64_t u = kp_ptr[k]; u < kp_ptr[k + 1]; ++u, ++q) {
          S.r_eoff[q] = kp_eoff[u];
          S.r_ecol[q] = c;
          S.r_dk[q] = P.tdim[k];
          S.r_pt[q] = kp[u];
        }
      }
  });
  return S;
}

}  // namespace sfg
