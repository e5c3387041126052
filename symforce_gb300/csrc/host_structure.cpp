// Host-side structure analysis, run once per problem structure (the reference does the same once:
// Linearizer::BuildInitialLinearization, symforce/opt/linearizer.cc:148-356, and
// SparseCholeskySolver::ComputeSymbolicSparsity, symforce/opt/sparse_cholesky/
// sparse_cholesky_solver.tcc:26-106).
//
//  - ParseProblem: validates a sfg_problem_t and lays out keys in state-vector order.
//  - MakePattern: block-sparse lower pattern (every co-occurring key pair, plus every diagonal
//    block), the block analogue of the reference's CSC hessian_lower pattern.
//  - Analyze: block fill-reducing ordering (nested dissection / minimum degree / natural),
//    elimination tree, block column structures, postorder, fundamental + relaxed supernodes,
//    and the assembly / extend-add maps of a multifrontal LDL^T.
//  - PlanTasks: the tile task list of the persistent factorization kernel.
#include <algorithm>
#include <cstring>
#include <deque>
#include <numeric>
#include <queue>
#include <set>
#include <unordered_map>

#include "common.h"

namespace sfg {

HostProblem ParseProblem(const sfg_problem_t* p) {
  if (!p) throw Error(SFG_ERR_INVALID_ARGUMENT, "problem is null");
  if (p->num_keys <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "problem has no keys");
  if (p->num_batches < 0 || (p->num_batches > 0 && !p->batches))
    throw Error(SFG_ERR_INVALID_ARGUMENT, "bad factor batches");
  if (!p->key_types) throw Error(SFG_ERR_INVALID_ARGUMENT, "key_types is null");
  HostProblem P;
  P.nkeys = p->num_keys;
  P.key_type.assign(p->key_types, p->key_types + p->num_keys);
  P.sdim.resize(P.nkeys);
  P.tdim.resize(P.nkeys);
  P.soff.resize(P.nkeys + 1);
  P.toff.resize(P.nkeys + 1);
  for (int k = 0; k < P.nkeys; ++k) {
    KeyDims(P.key_type[k], &P.sdim[k], &P.tdim[k]);
    P.soff[k] = P.S;
    P.toff[k] = P.N;
    P.S += P.sdim[k];
    P.N += P.tdim[k];
  }
  P.soff[P.nkeys] = P.S;
  P.toff[P.nkeys] = P.N;
  std::vector<char> touched(P.nkeys, 0);
  for (int b = 0; b < p->num_batches; ++b) {
    const sfg_factor_batch_t& B = p->batches[b];
    const FactorSpec s = Spec(B.kind);
    if (B.count < 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "negative factor count");
    if (B.count > 0 && (!B.keys || !B.consts))
      throw Error(SFG_ERR_INVALID_ARGUMENT, "factor batch arrays are null");
    HostBatch H;
    H.kind = B.kind;
    H.count = B.count;
    H.nk = s.nkeys;
    H.nc = s.nconsts;
    H.rdim = s.rdim;
    H.keys.assign(B.keys, B.keys + size_t(B.count) * s.nkeys);
    H.consts.assign(B.consts, B.consts + size_t(B.count) * s.nconsts);
    for (int j = 0; j < s.nkeys; ++j) {
      int sd, td;
      KeyDims(s.key_types[j], &sd, &td);
      H.key_tdim.push_back(td);
      H.tdim += td;
    }
    for (int f = 0; f < B.count; ++f)
      for (int j = 0; j < s.nkeys; ++j) {
        const int k = H.keys[size_t(f) * s.nkeys + j];
        if (k < 0 || k >= P.nkeys)
          throw Error(SFG_ERR_INVALID_ARGUMENT, "factor key index out of range");
        if (P.key_type[k] != s.key_types[j])
          throw Error(SFG_ERR_INVALID_ARGUMENT, "factor key has the wrong type");
        for (int q = 0; q < j; ++q)
          if (H.keys[size_t(f) * s.nkeys + q] == k)
            throw Error(SFG_ERR_INVALID_ARGUMENT, "a key appears twice in one factor");
        touched[k] = 1;
      }
    H.roff = P.M;
    H.first_factor = P.F;
    P.M += int64_t(B.count) * s.rdim;
    P.F += B.count;
    P.batches.push_back(std::move(H));
  }
  // The reference throws when a key of the state vector is not touched by any factor
  // (symforce/opt/linearizer.cc:264-272).
  for (int k = 0; k < P.nkeys; ++k)
    if (!touched[k])
      throw Error(SFG_ERR_INVALID_ARGUMENT,
                  "Key " + std::to_string(k) + " is in the state vector but is not optimized by any factor.");
  P.num_schur = p->num_schur_keys;
  if (P.num_schur < 0 || P.num_schur >= P.nkeys)
    throw Error(SFG_ERR_INVALID_ARGUMENT, "num_schur_keys out of range");
  return P;
}

int64_t BlockPattern::Find(int i, int j) const {
  auto b = rows.begin() + colptr[j], e = rows.begin() + colptr[j + 1];
  auto it = std::lower_bound(b, e, i);
  if (it == e || *it != i) return -1;
  return it - rows.begin();
}

BlockPattern MakePattern(const std::vector<int>& dims, std::vector<std::pair<int, int>> pairs) {
  BlockPattern P;
  P.nb = int(dims.size());
  P.dim = dims;
  P.off.assign(P.nb + 1, 0);
  for (int b = 0; b < P.nb; ++b) P.off[b + 1] = P.off[b] + dims[b];
  for (int b = 0; b < P.nb; ++b) pairs.push_back({b, b});
  for (auto& pr : pairs)
    if (pr.first < pr.second) std::swap(pr.first, pr.second);
  // sort by column then row: a counting sort by row, then a stable one by column
  {
    std::vector<std::pair<int, int>> tmp(pairs.size());
    std::vector<int64_t> cnt(size_t(P.nb) + 1, 0);
    for (const auto& pr : pairs) cnt[size_t(pr.first) + 1]++;
    for (int b = 0; b < P.nb; ++b) cnt[b + 1] += cnt[b];
    for (const auto& pr : pairs) tmp[size_t(cnt[pr.first]++)] = pr;
    std::fill(cnt.begin(), cnt.end(), 0);
    for (const auto& pr : tmp) cnt[size_t(pr.second) + 1]++;
    for (int b = 0; b < P.nb; ++b) cnt[b + 1] += cnt[b];
    for (const auto& pr : tmp) pairs[size_t(cnt[pr.second]++)] = pr;
  }
  pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
  P.colptr.assign(P.nb + 1, 0);
  P.rows.resize(pairs.size());
  P.boff.resize(pairs.size() + 1);
  int64_t v = 0;
  for (size_t q = 0; q < pairs.size(); ++q) {
    P.rows[q] = pairs[q].first;
    P.colptr[pairs[q].second + 1]++;
    P.boff[q] = v;
    v += int64_t(dims[pairs[q].first]) * dims[pairs[q].second];
  }
  P.boff[pairs.size()] = v;
  for (int b = 0; b < P.nb; ++b) P.colptr[b + 1] += P.colptr[b];
  return P;
}

// ---------------------------------------------------------------------------------------------
// Orderings on the block graph.  Each returns order[new] = old.
// ---------------------------------------------------------------------------------------------
namespace {

using Adj = std::vector<std::vector<int>>;

Adj BuildAdjacency(const BlockPattern& A) {
  Adj adj(A.nb);
  for (int j = 0; j < A.nb; ++j)
    for (int64_t q = A.colptr[j]; q < A.colptr[j + 1]; ++q) {
      const int i = A.rows[q];
      if (i == j) continue;
      adj[i].push_back(j);
      adj[j].push_back(i);
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  return adj;
}

// Minimum (weighted external) degree with an explicit elimination graph; ties by index.
std::vector<int32_t> MinDegree(const Adj& adj0, const std::vector<int>& dims,
                               const std::vector<int>& nodes) {
  // local relabel
  const int n = int(nodes.size());
  std::vector<int> local(adj0.size(), -1);
  for (int q = 0; q < n; ++q) local[nodes[q]] = q;
  std::vector<std::set<int>> adj(n);
  for (int q = 0; q < n; ++q)
    for (int u : adj0[nodes[q]])
      if (local[u] >= 0) adj[q].insert(local[u]);
  std::vector<int64_t> deg(n);
  auto degree = [&](int v) {
    int64_t d = 0;
    for (int u : adj[v]) d += dims[nodes[u]];
    return d;
  };
  using Item = std::pair<int64_t, int>;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
  for (int v = 0; v < n; ++v) {
    deg[v] = degree(v);
    pq.push({deg[v], v});
  }
  std::vector<char> done(n, 0);
  std::vector<int32_t> order;
  order.reserve(n);
  while (!pq.empty()) {
    auto [d, v] = pq.top();
    pq.pop();
    if (done[v] || d != deg[v]) continue;
    done[v] = 1;
    order.push_back(nodes[v]);
    std::vector<int> nb(adj[v].begin(), adj[v].end());
    for (int u : nb) adj[u].erase(v);
    for (size_t a = 0; a < nb.size(); ++a)
      for (size_t b = a + 1; b < nb.size(); ++b) {
        adj[nb[a]].insert(nb[b]);
        adj[nb[b]].insert(nb[a]);
      }
    for (int u : nb) {
      deg[u] = degree(u);
      pq.push({deg[u], u});
    }
    adj[v].clear();
  }
  return order;
}

// BFS levels inside the node subset marked by `in` (value == tag), from `src`.
int Bfs(const Adj& adj, const std::vector<int>& in, int tag, int src, std::vector<int>& level,
        std::vector<int>& visit_order) {
  visit_order.clear();
  level[src] = 0;
  visit_order.push_back(src);
  int maxl = 0;
  for (size_t h = 0; h < visit_order.size(); ++h) {
    const int v = visit_order[h];
    for (int u : adj[v])
      if (in[u] == tag && level[u] < 0) {
        level[u] = level[v] + 1;
        maxl = std::max(maxl, level[u]);
        visit_order.push_back(u);
      }
  }
  return maxl;
}

// Nested dissection by BFS level-structure bisection from a pseudo-peripheral node.  Small parts
// are ordered by minimum degree; separators come after both halves.
void NestedDissection(const Adj& adj, const std::vector<int>& dims, std::vector<int> nodes,
                      std::vector<int>& in, int& next_tag, std::vector<int32_t>& out) {
  const int kLeaf = 24;
  if (int(nodes.size()) <= kLeaf) {
    auto o = MinDegree(adj, dims, nodes);
    out.insert(out.end(), o.begin(), o.end());
    return;
  }
  const int tag = next_tag++;
  for (int v : nodes) in[v] = tag;
  std::vector<int> level(adj.size(), -1), vo;
  // connected components first
  std::vector<std::vector<int>> comps;
  for (int v : nodes) {
    if (level[v] >= 0) continue;
    Bfs(adj, in, tag, v, level, vo);
    comps.push_back(vo);
  }
  if (comps.size() > 1) {
    for (auto& c : comps) NestedDissection(adj, dims, c, in, next_tag, out);
    return;
  }
  // pseudo-peripheral node: repeat BFS from the farthest node a few times
  int src = nodes[0];
  int ecc = -1;
  for (int it = 0; it < 4; ++it) {
    for (int v : nodes) level[v] = -1;
    const int e = Bfs(adj, in, tag, src, level, vo);
    if (e <= ecc) break;
    ecc = e;
    src = vo.back();
  }
  for (int v : nodes) level[v] = -1;
  const int maxl = Bfs(adj, in, tag, src, level, vo);
  if (maxl < 2) {
    auto o = MinDegree(adj, dims, nodes);
    out.insert(out.end(), o.begin(), o.end());
    return;
  }
  // choose the separator level that splits the weight in half
  std::vector<int64_t> wl(maxl + 1, 0);
  int64_t total = 0;
  for (int v : nodes) {
    wl[level[v]] += dims[v];
    total += dims[v];
  }
  int sep = 1;
  int64_t acc = 0;
  for (int l = 0; l <= maxl; ++l) {
    acc += wl[l];
    if (2 * acc >= total) {
      sep = std::min(std::max(l, 1), maxl - 1);
      break;
    }
  }
  std::vector<int> left, right, separator;
  for (int v : nodes) {
    if (level[v] < sep) left.push_back(v);
    else if (level[v] > sep) right.push_back(v);
    else separator.push_back(v);
  }
  // Thin the separator: keep only nodes adjacent to the right side.
  {
    std::vector<int> keep;
    const int rtag = next_tag++;
    for (int v : right) in[v] = rtag;
    for (int v : separator) {
      bool touches_right = false;
      for (int u : adj[v])
        if (in[u] == rtag) {
          touches_right = true;
          break;
        }
      if (touches_right) keep.push_back(v);
      else left.push_back(v);
    }
    separator.swap(keep);
  }
  std::sort(left.begin(), left.end());
  std::sort(right.begin(), right.end());
  std::sort(separator.begin(), separator.end());
  NestedDissection(adj, dims, left, in, next_tag, out);
  NestedDissection(adj, dims, right, in, next_tag, out);
  out.insert(out.end(), separator.begin(), separator.end());
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Symbolic analysis
// ---------------------------------------------------------------------------------------------
Symbolic Analyze(const BlockPattern& A, int ordering) {
  Symbolic S;
  const int nb = A.nb;
  S.nb = nb;
  S.n = A.off[nb];
  const Adj adj = BuildAdjacency(A);
  std::vector<int32_t> order;
  if (ordering == SFG_ORDERING_NATURAL) {
    order.resize(nb);
    std::iota(order.begin(), order.end(), 0);
  } else if (ordering == SFG_ORDERING_MIN_DEGREE) {
    std::vector<int> all(nb);
    std::iota(all.begin(), all.end(), 0);
    order = MinDegree(adj, A.dim, all);
  } else if (ordering == SFG_ORDERING_NESTED_DISSECTION) {
    std::vector<int> all(nb);
    std::iota(all.begin(), all.end(), 0);
    std::vector<int> in(nb, -1);
    int tag = 0;
    NestedDissection(adj, A.dim, all, in, tag, order);
  } else {
    throw Error(SFG_ERR_INVALID_ARGUMENT, "unknown ordering");
  }
  if (int(order.size()) != nb) throw Error(SFG_ERR_STRUCTURE, "ordering lost nodes");

  // elimination tree + postorder, then final order = order o postorder
  auto etree = [&](const std::vector<int32_t>& ord, std::vector<int32_t>& parent,
                   std::vector<std::vector<int32_t>>& lower_rows) {
    std::vector<int32_t> perm(nb);
    for (int q = 0; q < nb; ++q) perm[ord[q]] = q;
    // lower_rows[j] = new rows i > j with A(i, j) != 0 (new indices)
    lower_rows.assign(nb, {});
    std::vector<std::vector<int32_t>> upper(nb);  // upper[i] = new cols j < i
    for (int oj = 0; oj < nb; ++oj)
      for (int u : adj[oj]) {
        const int ni = perm[u], nj = perm[oj];
        if (ni > nj) {
          lower_rows[nj].push_back(ni);
          upper[ni].push_back(nj);
        }
      }
    parent.assign(nb, -1);
    std::vector<int32_t> ancestor(nb, -1);
    for (int j = 0; j < nb; ++j)
      for (int i : upper[j]) {
        int r = i;
        while (ancestor[r] != -1 && ancestor[r] != j) {
          const int nx = ancestor[r];
          ancestor[r] = j;
          r = nx;
        }
        if (ancestor[r] == -1) {
          ancestor[r] = j;
          parent[r] = j;
        }
      }
    for (auto& v : lower_rows) std::sort(v.begin(), v.end());
  };
  std::vector<int32_t> parent;
  std::vector<std::vector<int32_t>> lower_rows;
  etree(order, parent, lower_rows);
  {
    std::vector<std::vector<int32_t>> kids(nb);
    std::vector<int32_t> roots;
    for (int j = 0; j < nb; ++j) (parent[j] < 0 ? roots : kids[parent[j]]).push_back(j);
    std::vector<int32_t> post;
    post.reserve(nb);
    std::vector<std::pair<int, size_t>> stack;
    for (int r : roots) {
      stack.push_back({r, 0});
      while (!stack.empty()) {
        auto& [v, c] = stack.back();
        if (c < kids[v].size()) {
          const int ch = kids[v][c++];
          stack.push_back({ch, 0});
        } else {
          post.push_back(v);
          stack.pop_back();
        }
      }
    }
    std::vector<int32_t> final_order(nb);
    for (int q = 0; q < nb; ++q) final_order[q] = order[post[q]];
    order.swap(final_order);
  }
  etree(order, parent, lower_rows);
  S.border = order;
  S.bperm.assign(nb, 0);
  for (int q = 0; q < nb; ++q) S.bperm[order[q]] = q;
  S.pstart.assign(nb + 1, 0);
  for (int q = 0; q < nb; ++q) S.pstart[q + 1] = S.pstart[q] + A.dim[order[q]];
  std::vector<int> ndim(nb);
  for (int q = 0; q < nb; ++q) ndim[q] = A.dim[order[q]];

  // block column structures of L
  std::vector<std::vector<int32_t>> kids(nb);
  for (int j = 0; j < nb; ++j)
    if (parent[j] >= 0) kids[parent[j]].push_back(j);
  std::vector<std::vector<int32_t>> colstruct(nb);
  for (int j = 0; j < nb; ++j) {
    std::vector<int32_t> s = lower_rows[j];
    for (int c : kids[j])
      for (int r : colstruct[c])
        if (r != j) s.push_back(r);
    std::sort(s.begin(), s.end());
    s.erase(std::unique(s.begin(), s.end()), s.end());
    colstruct[j].swap(s);
    // children structures are no longer needed past their parent
    for (int c : kids[j]) std::vector<int32_t>().swap(colstruct[c]);
  }
  // recompute structures kept for supernode detection: we need |struct(j)| and struct of the
  // first column of each supernode; recompute fully (kept this time).
  std::vector<std::vector<int32_t>> cs(nb);
  for (int j = 0; j < nb; ++j) {
    std::vector<int32_t> s = lower_rows[j];
    for (int c : kids[j])
      for (int r : cs[c])
        if (r != j) s.push_back(r);
    std::sort(s.begin(), s.end());
    s.erase(std::unique(s.begin(), s.end()), s.end());
    cs[j].swap(s);
  }

  // fundamental supernodes
  struct Sn {
    int first, last;
    std::vector<int32_t> rows;  // row blocks below last
    int parent = -1;
    bool alive = true;
  };
  std::vector<Sn> sns;
  std::vector<int> sn_of(nb, -1);
  for (int j = 0; j < nb; ++j) {
    const bool join = j > 0 && parent[j - 1] == j && kids[j].size() == 1 &&
                      cs[j - 1].size() == cs[j].size() + 1;
    if (join) {
      sns.back().last = j;
      sns.back().rows = cs[j];
    } else {
      sns.push_back({j, j, cs[j], -1, true});
    }
    sn_of[j] = int(sns.size()) - 1;
  }
  auto width = [&](const Sn& s) {
    int64_t w = 0;
    for (int b = s.first; b <= s.last; ++b) w += ndim[b];
    return w;
  };
  auto height = [&](const std::vector<int32_t>& rows) {
    int64_t h = 0;
    for (int b : rows) h += ndim[b];
    return h;
  };
  for (auto& s : sns) s.parent = s.rows.empty() ? -1 : sn_of[s.rows.front()];
  // relaxed amalgamation: merge a child into its parent when the child's columns immediately
  // precede the parent's and the merged front stays small or the growth in front area is modest
  {
    const int64_t kSmall = 48;
    std::vector<std::vector<int>> skids(sns.size());
    for (int s = 0; s < int(sns.size()); ++s)
      if (sns[s].parent >= 0) skids[sns[s].parent].push_back(s);
    for (int p = 0; p < int(sns.size()); ++p) {
      bool merged = true;
      while (merged) {
        merged = false;
        for (int c : skids[p]) {
          if (!sns[c].alive || sns[c].last + 1 != sns[p].first) continue;
          // merged structure: rows = (rows_c U rows_p) minus cols of p
          std::vector<int32_t> rows;
          for (int r : sns[c].rows)
            if (r > sns[p].last) rows.push_back(r);
          rows.insert(rows.end(), sns[p].rows.begin(), sns[p].rows.end());
          std::sort(rows.begin(), rows.end());
          rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
          const int64_t wc = width(sns[c]), wp = width(sns[p]);
          const int64_t mc = wc + height(sns[c].rows), mp = wp + height(sns[p].rows);
          const int64_t mm = wc + wp + height(rows);
          const bool ok = mm <= kSmall || double(mm) * mm <= 1.3 * double(mc * mc + mp * mp);
          if (!ok) continue;
          sns[p].first = sns[c].first;
          sns[p].rows.swap(rows);
          sns[c].alive = false;
          for (int g : skids[c]) {
            sns[g].parent = p;
            skids[p].push_back(g);
          }
          merged = true;
          break;
        }
      }
    }
  }
  // compact, in order of first block (a postorder of the supernodal tree)
  std::vector<int> alive_ids;
  for (int s = 0; s < int(sns.size()); ++s)
    if (sns[s].alive) alive_ids.push_back(s);
  std::sort(alive_ids.begin(), alive_ids.end(),
            [&](int a, int b) { return sns[a].first < sns[b].first; });
  const int ns = int(alive_ids.size());
  S.ns = ns;
  std::fill(sn_of.begin(), sn_of.end(), -1);
  for (int q = 0; q < ns; ++q)
    for (int b = sns[alive_ids[q]].first; b <= sns[alive_ids[q]].last; ++b) sn_of[b] = q;
  S.sn_first.resize(ns);
  S.sn_last.resize(ns);
  S.sn_parent.resize(ns);
  S.sn_w.resize(ns);
  S.sn_h.resize(ns);
  S.sn_m.resize(ns);
  S.sn_rows.resize(ns);
  S.sn_children.assign(ns, {});
  S.sn_foff.resize(ns + 1);
  S.idx_off.assign(ns + 1, 0);
  int64_t pool = 0;
  for (int q = 0; q < ns; ++q) {
    const Sn& s = sns[alive_ids[q]];
    S.sn_first[q] = s.first;
    S.sn_last[q] = s.last;
    S.sn_rows[q] = s.rows;
    S.sn_parent[q] = s.rows.empty() ? -1 : sn_of[s.rows.front()];
    S.sn_w[q] = int32_t(width(s));
    S.sn_h[q] = int32_t(height(s.rows));
    S.sn_m[q] = S.sn_w[q] + S.sn_h[q];
    S.sn_foff[q] = pool;
    pool += int64_t(S.sn_m[q]) * S.sn_m[q];
    S.idx_off[q + 1] = S.idx_off[q] + S.sn_m[q];
  }
  S.sn_foff[ns] = pool;
  S.front_pool = pool;
  for (int q = 0; q < ns; ++q) {
    if (S.sn_parent[q] >= 0) {
      if (S.sn_parent[q] <= q) throw Error(SFG_ERR_STRUCTURE, "supernode tree is not postordered");
      S.sn_children[S.sn_parent[q]].push_back(q);
    }
  }
  // scalar index lists
  S.idx.resize(S.idx_off[ns]);
  for (int q = 0; q < ns; ++q) {
    int64_t o = S.idx_off[q];
    for (int b = S.sn_first[q]; b <= S.sn_last[q]; ++b)
      for (int t = 0; t < ndim[b]; ++t) S.idx[o++] = int32_t(S.pstart[b] + t);
    for (int b : S.sn_rows[q])
      for (int t = 0; t < ndim[b]; ++t) S.idx[o++] = int32_t(S.pstart[b] + t);
  }
  auto pos_in_front = [&](int q, int64_t scalar) -> int32_t {
    auto b = S.idx.begin() + S.idx_off[q], e = S.idx.begin() + S.idx_off[q + 1];
    auto it = std::lower_bound(b, e, int32_t(scalar));
    if (it == e || *it != scalar) throw Error(SFG_ERR_STRUCTURE, "index not in front");
    return int32_t(it - b);
  };
  // extend-add maps
  S.rel_off.assign(ns + 1, 0);
  for (int q = 0; q < ns; ++q) S.rel_off[q + 1] = S.rel_off[q] + S.sn_h[q];
  S.rel.resize(S.rel_off[ns]);
  for (int q = 0; q < ns; ++q) {
    const int p = S.sn_parent[q];
    if (p < 0) continue;
    for (int r = 0; r < S.sn_h[q]; ++r)
      S.rel[S.rel_off[q] + r] = pos_in_front(p, S.idx[S.idx_off[q] + S.sn_w[q] + r]);
  }
  // assembly lists
  std::vector<std::vector<Symbolic::Asm>> asml(ns);
  for (int oj = 0; oj < nb; ++oj)
    for (int64_t qb = A.colptr[oj]; qb < A.colptr[oj + 1]; ++qb) {
      const int oi = A.rows[qb];
      const int ni = S.bperm[oi], nj = S.bperm[oj];
      const int lo = std::min(ni, nj), hi = std::max(ni, nj);
      const int q = sn_of[lo];
      Symbolic::Asm a;
      a.src = A.boff[qb];
      a.col0 = int32_t(S.pstart[lo] - S.pstart[S.sn_first[q]]);
      a.row0 = pos_in_front(q, S.pstart[hi]);
      a.di = int16_t(A.dim[oi]);
      a.dj = int16_t(A.dim[oj]);
      a.transpose = int16_t(ni < nj ? 1 : 0);
      a.diag = int16_t(oi == oj ? 1 : 0);
      a.oi = oi;
      a.oj = oj;
      asml[q].push_back(a);
    }
  S.asm_off.assign(ns + 1, 0);
  for (int q = 0; q < ns; ++q) S.asm_off[q + 1] = S.asm_off[q] + int64_t(asml[q].size());
  S.asms.reserve(S.asm_off[ns]);
  for (int q = 0; q < ns; ++q) S.asms.insert(S.asms.end(), asml[q].begin(), asml[q].end());
  // counts
  for (int q = 0; q < ns; ++q) {
    const int64_t m = S.sn_m[q];
    for (int k = 0; k < S.sn_w[q]; ++k) {
      S.nnz_L += m - k - 1;
      S.flops += double(m - k - 1) * double(m - k) / 2.0 + double(m - k - 1);
    }
  }
  return S;
}

TaskPlan PlanTasks(const Symbolic& sym, int tile, bool separate_inverse, bool tc_updates) {
  TaskPlan T;
  T.tile = tile;
  T.tile_base.assign(sym.ns + 1, 0);
  T.ntiles.resize(sym.ns);
  T.npiv.resize(sym.ns);
  for (int s = 0; s < sym.ns; ++s) {
    const int np = (sym.sn_w[s] + tile - 1) / tile;
    const int nn = (sym.sn_h[s] + tile - 1) / tile;
    T.npiv[s] = np;
    T.ntiles[s] = np + nn;
    const int nt = np + nn;
    T.tile_base[s + 1] = T.tile_base[s] + nt * (nt + 1) / 2;
  }
  T.nstates = T.tile_base[sym.ns];
  // assembly entries per (front, tile column)
  T.asm_col_base.assign(sym.ns + 1, 0);
  for (int s = 0; s < sym.ns; ++s) T.asm_col_base[s + 1] = T.asm_col_base[s] + T.ntiles[s];
  std::vector<std::vector<int32_t>> percol(T.asm_col_base[sym.ns]);
  for (int s = 0; s < sym.ns; ++s) {
    const int np = T.npiv[s], w = sym.sn_w[s], m = sym.sn_m[s];
    auto col_tile = [&](int c) { return c < w ? c / tile : np + (c - w) / tile; };
    (void)m;
    for (int64_t a = sym.asm_off[s]; a < sym.asm_off[s + 1]; ++a) {
      const auto& as = sym.asms[a];
      const int ncols = as.transpose ? as.di : as.dj;
      int last = -1;
      for (int c = as.col0; c < as.col0 + ncols; ++c) {
        const int t = col_tile(c);
        if (t != last) percol[T.asm_col_base[s] + t].push_back(int32_t(a));
        last = t;
      }
    }
  }
  T.asm_col_off.assign(percol.size() + 1, 0);
  for (size_t q = 0; q < percol.size(); ++q) {
    T.asm_col_off[q + 1] = T.asm_col_off[q] + int64_t(percol[q].size());
    T.asm_col_list.insert(T.asm_col_list.end(), percol[q].begin(), percol[q].end());
  }
  // Tasks are generated front by front in postorder, each front panel by panel; every task comes
  // after the tasks it waits on.  The critical chain of a front (the LDL^T of tile (0, 0), then for
  // every panel k < np - 1 the panel solve of tile (k+1, k), the update of (k+1, k+1) by it and
  // the LDL^T of (k+1, k+1)) is one chain task, which stays in its CTA for the front's whole
  // factorization; the other panel solves and trailing updates follow in panel order.  A
  // single-panel front has a plain diagonal task.
  //
  // The list is then ordered by each task's start time in an as-soon-as-possible schedule with
  // unbounded CTAs and nominal durations (a topological order, since every task starts after the
  // tasks it waits on end): the kernel's CTAs claim tasks in list order, and in front order they
  // would claim thousands of one front's updates that wait on its chain while the independent
  // fronts beside it wait to be claimed.
  //
  // Deadlock freedom: a task only waits on tasks that start earlier, so on tasks earlier in the
  // list, claimed by running CTAs; chain step k waits only on tasks that end before the step
  // starts, and every task that waits on step k starts after the step starts, so those tasks are
  // claimed before any CTA can be held by a task waiting on step k: the chain always advances.
  struct Timed {
    double key;
    int4 task;
  };
  std::vector<Timed> timed;
  // nominal durations (microseconds; only the order matters)
  constexpr double kAsm = 5, kDiag = 5, kStep = 10, kTrsm = 4, kUpd = 5, kInv = 3, kUpdTc = 6;
  std::vector<double> front_done(sym.ns, 0.0);
  for (int s = 0; s < sym.ns; ++s) {
    const int nt = T.ntiles[s], np = T.npiv[s];
    // ver: time tile (i, j) reached its latest version so far; fin: time it became final
    std::vector<double> ver(size_t(nt) * nt, 0.0), fin(size_t(nt) * nt, 0.0);
    auto V = [&](int i, int j) -> double& { return ver[size_t(i) * nt + j]; };
    auto Fn = [&](int i, int j) -> double& { return fin[size_t(i) * nt + j]; };
    double t0 = 0.0, done = 0.0;
    for (int c : sym.sn_children[s]) t0 = std::max(t0, front_done[c]);
    auto add = [&](double start, double dur, int4 task) {
      timed.push_back({start, task});
      done = std::max(done, start + dur);
      return start + dur;
    };
    for (int j = 0; j < nt; ++j) {
      const double e = add(t0, kAsm, make_int4(kTaskAssemble, s, j, 0));
      for (int i = j; i < nt; ++i) V(i, j) = e;
    }
    if (np == 1) {
      Fn(0, 0) = add(V(0, 0), kDiag, make_int4(kTaskDiag, s, 0, 0));
    } else {
      // the chain task sits at its first step; its later steps are timed here, not listed
      Fn(0, 0) = add(V(0, 0), kDiag, make_int4(kTaskChain, s, 0, 0));
    }
    for (int k = 0; k < np; ++k) {
      const bool ahead = k + 1 < np;
      if (ahead) {
        const double st = std::max({Fn(k, k), V(k + 1, k), V(k + 1, k + 1)});
        Fn(k + 1, k) = st + kStep / 2;  // the panel tile is published halfway through the step
        Fn(k + 1, k + 1) = st + kStep;
        done = std::max(done, st + kStep);
      }
      for (int i = k + (ahead ? 2 : 1); i < nt; ++i)
        Fn(i, k) = add(std::max(Fn(k, k), V(i, k)), kTrsm, make_int4(kTaskTrsm, s, i * 65536 + k, k));
      for (int j = k + 1; j < nt; ++j) {
        // rows of tile column j that take panel k's update here (tile (k+1, k+1) is the chain's)
        std::vector<int> rows;
        for (int i = j; i < nt; ++i)
          if (!(ahead && i == k + 1 && j == k + 1)) rows.push_back(i);
        auto single = [&](int i) {
          V(i, j) = add(std::max({Fn(i, k), Fn(j, k), V(i, j)}), kUpd, make_int4(kTaskUpdate, s, i * 65536 + j, k));
        };
        if (!tc_updates) {
          for (int i : rows) single(i);
          continue;
        }
        // Tensor-core tasks take runs of up to four consecutive rows.  The tiles chain step k + 1
        // waits on, (k+2, k+1) and (k+2, k+2), stay single tasks that wait for nothing else.
        const bool chain_next = k + 2 < np;
        size_t q = 0;
        while (q < rows.size()) {
          const int i0 = rows[q];
          if (chain_next && i0 == k + 2 && (j == k + 1 || j == k + 2)) {
            single(i0);
            ++q;
            continue;
          }
          int cnt = 1;
          while (cnt < 4 && q + cnt < rows.size() && rows[q + cnt] == i0 + cnt) ++cnt;
          if (cnt == 1) {
            single(i0);
            ++q;
            continue;
          }
          double st = std::max(Fn(j, k), 0.0);
          for (int r = 0; r < cnt; ++r) st = std::max({st, Fn(i0 + r, k), V(i0 + r, j)});
          const double e = add(st, kUpdTc, make_int4(kTaskUpdateTc, s, i0 * 65536 + j, k | (cnt << 20)));
          for (int r = 0; r < cnt; ++r) V(i0 + r, j) = e;
          q += size_t(cnt);
        }
      }
    }
    // the inverses of the chain's diagonal factors, for the triangular solves only
    if (separate_inverse && np > 1)
      for (int k = 0; k < np; ++k) add(Fn(k, k), kInv, make_int4(kTaskInverse, s, k * 65536 + k, k));
    front_done[s] = done;
  }
  std::stable_sort(timed.begin(), timed.end(), [](const Timed& a, const Timed& b) { return a.key < b.key; });
  T.tasks.reserve(timed.size());
  for (const Timed& x : timed) T.tasks.push_back(x.task);
  return T;
}

FactorMaps BuildFactorMaps(const Symbolic& S, const TaskPlan& T, const BlockPattern& pat) {
  FactorMaps M;
  const int tile = T.tile;
  const std::vector<int32_t>& col_base = T.asm_col_base;
  const int nslots = col_base[S.ns];
  std::vector<std::vector<int64_t>> asrc(nslots);
  std::vector<std::vector<int32_t>> adst(nslots), adamp(nslots);
  std::vector<std::vector<std::pair<int64_t, int32_t>>> ea(nslots);  // (src, dst) in child order
  for (int s = 0; s < S.ns; ++s) {
    const int w = S.sn_w[s], m = S.sn_m[s], np = T.npiv[s];
    auto col_tile = [&](int c) { return c < w ? c / tile : np + (c - w) / tile; };
    for (int64_t q = S.asm_off[s]; q < S.asm_off[s + 1]; ++q) {
      const auto& a = S.asms[q];
      for (int r = 0; r < a.di; ++r)
        for (int c = 0; c < a.dj; ++c) {
          if (a.diag && r < c) continue;
          const int fr = a.transpose ? a.row0 + c : a.row0 + r;
          const int fc = a.transpose ? a.col0 + r : a.col0 + c;
          const int slot = col_base[s] + col_tile(fc);
          asrc[slot].push_back(a.src + int64_t(r) * a.dj + c);
          adst[slot].push_back(int32_t(fr + int64_t(fc) * m));
          adamp[slot].push_back(a.diag && r == c ? int32_t(pat.off[a.oi] + r) : -1);
        }
    }
    for (int c : S.sn_children[s]) {
      const int hc = S.sn_h[c], wc = S.sn_w[c], mc = S.sn_m[c];
      const int32_t* rel = S.rel.data() + S.rel_off[c];
      for (int qc = 0; qc < hc; ++qc) {
        const int slot = col_base[s] + col_tile(rel[qc]);
        for (int r = qc; r < hc; ++r)
          ea[slot].push_back({S.sn_foff[c] + (wc + r) + int64_t(wc + qc) * mc,
                              int32_t(rel[r] + int64_t(rel[qc]) * m)});
      }
    }
  }
  M.a_ptr.assign(nslots + 1, 0);
  M.e_rptr.assign(nslots + 1, 0);
  for (int q = 0; q < nslots; ++q) {
    M.a_src.insert(M.a_src.end(), asrc[q].begin(), asrc[q].end());
    M.a_dst.insert(M.a_dst.end(), adst[q].begin(), adst[q].end());
    M.a_damp.insert(M.a_damp.end(), adamp[q].begin(), adamp[q].end());
    M.a_ptr[q + 1] = int64_t(M.a_src.size());
    // rounds: the k-th occurrence of a destination goes to round k (children keep their order)
    std::unordered_map<int32_t, int> seen;
    std::vector<int> round(ea[q].size());
    int nround = 0;
    for (size_t e = 0; e < ea[q].size(); ++e) {
      round[e] = seen[ea[q][e].second]++;
      nround = std::max(nround, round[e] + 1);
    }
    for (int rd = 0; rd < nround; ++rd) {
      M.e_round.push_back(int64_t(M.e_src.size()));
      for (size_t e = 0; e < ea[q].size(); ++e)
        if (round[e] == rd) {
          M.e_src.push_back(ea[q][e].first);
          M.e_dst.push_back(ea[q][e].second);
        }
    }
    M.e_rptr[q + 1] = int64_t(M.e_round.size());
  }
  M.e_round.push_back(int64_t(M.e_src.size()));
  M.linv_base.assign(S.ns + 1, 0);
  for (int s = 0; s < S.ns; ++s) M.linv_base[s + 1] = M.linv_base[s] + int64_t(T.npiv[s]) * tile * tile;
  M.child_ptr.assign(S.ns + 1, 0);
  for (int s = 0; s < S.ns; ++s) {
    for (int c : S.sn_children[s]) M.child_list.push_back(c);
    M.child_ptr[s + 1] = int32_t(M.child_list.size());
  }
  M.scalar_old.assign(S.n, 0);
  for (int q = 0; q < S.nb; ++q) {
    const int old = S.border[q];
    for (int t = 0; t < pat.dim[old]; ++t) M.scalar_old[S.pstart[q] + t] = int32_t(pat.off[old] + t);
  }
  return M;
}

SolveSplit PlanSolveSplit(const TaskPlan& plan, int ns, int warps, int block_tiles, bool split) {
  SolveSplit out;
  out.kp.assign(size_t(ns), 0);
  out.ku.assign(size_t(ns), 0);
  bool any = false;
  for (int s = 0; s < ns; ++s) {
    const int np = plan.npiv[size_t(s)], nu = plan.ntiles[size_t(s)] - np;
    if (split && np > 0 && np + nu > warps) {
      out.kp[size_t(s)] = (np + block_tiles - 1) / block_tiles;
      out.ku[size_t(s)] = (nu + block_tiles - 1) / block_tiles;
      any = true;
    }
  }
  if (!any) return out;
  for (int s = 0; s < ns; ++s) {
    const int k = out.kp[size_t(s)] > 0 ? out.kp[size_t(s)] + out.ku[size_t(s)] : 1;
    for (int c = 0; c < k; ++c) {
      out.task_front.push_back(s);
      out.task_sub.push_back(c);
    }
  }
  out.nf = int(out.task_front.size());
  for (int s = ns - 1; s >= 0; --s) {
    const int k = out.kp[size_t(s)] > 0 ? out.kp[size_t(s)] : 1;
    for (int c = 0; c < k; ++c) {
      out.task_front.push_back(s);
      out.task_sub.push_back(c);
    }
  }
  return out;
}

}  // namespace sfg
