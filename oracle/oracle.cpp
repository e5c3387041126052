// Test infrastructure, not product code.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load this library; the GPU library never links it and the product path never
// calls it.
//
// CPU restatement of the reference's sym::Optimizer Levenberg-Marquardt hot path, in plain C++17
// without Eigen (the reference's Eigen 3.4 / METIS 5.1 dependencies are not available here):
//   - Linearizer: CSC hessian_lower pattern (every entry of every co-occurring lower key block plus
//     the full diagonal) and per-factor scatter  (symforce/opt/linearizer.cc:54-120, 148-433,
//     symforce/opt/internal/linearizer_utils.h:28-143)
//   - SparseCholeskySolver: elimination tree, column counts, up-looking LDL^T, permuted solves
//     (symforce/opt/sparse_cholesky/sparse_cholesky_solver.tcc:12-259)
//   - SparseSchurSolver: block-diagonal C inverses, S = B - E C^-1 E^T, back-substitution
//     (symforce/opt/sparse_schur_solver.tcc:15-170)
//   - LevenbergMarquardtSolver::Iterate with its three-block state
//     (symforce/opt/levenberg_marquardt_solver.tcc:22-343,
//      symforce/opt/internal/levenberg_marquardt_state.h:33-270,
//      symforce/opt/internal/optimizer_utils.h:34-104)
// Factor residuals and retractions are in factors.h; Jacobians come from forward-mode jets.
//
// The ordering: the reference orders with Eigen::MetisOrdering (METIS 5.1.0), which is not present.
// The oracle uses either the natural order or its own block minimum-degree order; final costs do
// not depend on the ordering beyond rounding, and the ordering itself is not pinned.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <queue>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../include/sfgpu.h"
#include "./factors.h"

namespace oracle {

// ---------------------------------------------------------------------------------------------
// Problem description
// ---------------------------------------------------------------------------------------------
inline void KeyDims(int type, int* sdim, int* tdim) {
  switch (type) {
    case SFG_KEY_VEC1: *sdim = 1; *tdim = 1; return;
    case SFG_KEY_VEC2: *sdim = 2; *tdim = 2; return;
    case SFG_KEY_VEC3: *sdim = 3; *tdim = 3; return;
    case SFG_KEY_POSE2: *sdim = 4; *tdim = 3; return;
    case SFG_KEY_POSE3: *sdim = 7; *tdim = 6; return;
    case SFG_KEY_ROT3: *sdim = 4; *tdim = 3; return;
    case SFG_KEY_VEC4: *sdim = 4; *tdim = 4; return;
    case SFG_KEY_VEC5: *sdim = 5; *tdim = 5; return;
    case SFG_KEY_VEC6: *sdim = 6; *tdim = 6; return;
  }
  throw std::invalid_argument("unknown key type " + std::to_string(type));
}

struct FactorSpec {
  int nkeys, nconsts, rdim;
  int key_types[3];
};

inline FactorSpec Spec(int kind) {
  switch (kind) {
    case SFG_FACTOR_BEARING_POSE2: return {1, 5, 1, {SFG_KEY_POSE2, 0, 0}};
    case SFG_FACTOR_ODOMETRY_POSE2: return {2, 3, 1, {SFG_KEY_POSE2, SFG_KEY_POSE2, 0}};
    case SFG_FACTOR_SNAVELY_REPROJECTION: return {3, 4, 2, {SFG_KEY_POSE3, SFG_KEY_VEC3, SFG_KEY_VEC3}};
    case SFG_FACTOR_BETWEEN_POSE3: return {2, 14, 6, {SFG_KEY_POSE3, SFG_KEY_POSE3, 0}};
    case SFG_FACTOR_PRIOR_POSE3: return {1, 14, 6, {SFG_KEY_POSE3, 0, 0}};
    case SFG_FACTOR_RANGE_POSE3: return {1, 6, 1, {SFG_KEY_POSE3, 0, 0}};
    case SFG_FACTOR_PRIOR_ROT3: return {1, 8, 3, {SFG_KEY_ROT3, 0, 0}};
    case SFG_FACTOR_BETWEEN_ROT3: return {2, 8, 3, {SFG_KEY_ROT3, SFG_KEY_ROT3, 0}};
    case SFG_FACTOR_BARRON_VEC5: return {1, 7, 5, {SFG_KEY_VEC5, 0, 0}};
    case SFG_FACTOR_LINEAR_VEC5: return {1, 54, 9, {SFG_KEY_VEC5, 0, 0}};
    case SFG_FACTOR_LINEAR_SCALAR2: return {2, 6, 2, {SFG_KEY_VEC1, SFG_KEY_VEC1, 0}};
  }
  throw std::invalid_argument("unknown factor kind " + std::to_string(kind));
}

struct Key {
  int type, sdim, tdim;
  int64_t soff, toff;
};

struct Factor {
  int kind, nkeys, rdim, tdim;
  int keys[3];
  int koff[3];  // offset of each key inside the factor's tangent vector
  const double* c;
  int64_t roff;
};

struct Problem {
  std::vector<Key> keys;
  std::vector<Factor> factors;
  std::vector<double> consts;  // owned copy of all constants
  int64_t S = 0, N = 0, M = 0;
  int num_schur = 0;
};

Problem BuildProblem(const sfg_problem_t* p) {
  Problem P;
  P.keys.resize(p->num_keys);
  for (int i = 0; i < p->num_keys; ++i) {
    Key& k = P.keys[i];
    k.type = p->key_types[i];
    KeyDims(k.type, &k.sdim, &k.tdim);
    k.soff = P.S;
    k.toff = P.N;
    P.S += k.sdim;
    P.N += k.tdim;
  }
  size_t total_consts = 0;
  for (int b = 0; b < p->num_batches; ++b) {
    const FactorSpec s = Spec(p->batches[b].kind);
    total_consts += size_t(p->batches[b].count) * s.nconsts;
  }
  P.consts.resize(total_consts);
  size_t coff = 0;
  for (int b = 0; b < p->num_batches; ++b) {
    const sfg_factor_batch_t& B = p->batches[b];
    const FactorSpec s = Spec(B.kind);
    for (int f = 0; f < B.count; ++f) {
      Factor F;
      F.kind = B.kind;
      F.nkeys = s.nkeys;
      F.rdim = s.rdim;
      F.tdim = 0;
      for (int j = 0; j < s.nkeys; ++j) {
        const int key = B.keys[size_t(f) * s.nkeys + j];
        if (key < 0 || key >= p->num_keys) throw std::invalid_argument("factor key out of range");
        if (P.keys[key].type != s.key_types[j]) throw std::invalid_argument("factor key type mismatch");
        for (int q = 0; q < j; ++q)
          if (F.keys[q] == key) throw std::invalid_argument("duplicate key in factor");
        F.keys[j] = key;
        F.koff[j] = F.tdim;
        F.tdim += P.keys[key].tdim;
      }
      std::memcpy(&P.consts[coff], B.consts + size_t(f) * s.nconsts, sizeof(double) * s.nconsts);
      F.c = nullptr;
      F.roff = P.M;
      P.M += s.rdim;
      P.factors.push_back(F);
      coff += s.nconsts;
    }
  }
  coff = 0;
  for (auto& F : P.factors) {
    F.c = &P.consts[coff];
    coff += Spec(F.kind).nconsts;
  }
  P.num_schur = p->num_schur_keys;
  return P;
}

// ---------------------------------------------------------------------------------------------
// Factor linearization through jets: J = d r(retract(x, delta)) / d delta at delta = 0.
// ---------------------------------------------------------------------------------------------
template <int NT>
void RetractKeyJet(const Key& k, const double* x, int seed_off, Jet<NT>* out) {
  Jet<NT> d[6];
  for (int i = 0; i < k.tdim; ++i) d[i] = Jet<NT>::Seed(0.0, seed_off + i);
  switch (k.type) {
    case SFG_KEY_POSE2: RetractPose2(x, d, out); return;
    case SFG_KEY_POSE3: RetractPose3(x, d, /*eps=*/0.0, out); return;
    default:
      for (int i = 0; i < k.tdim; ++i) out[i] = x[i] + d[i];
      return;
  }
}

template <int NT>
void LinearizeFactorT(const Problem& P, const Factor& F, const double* values, double* res,
                      double* J, double retract_eps) {
  Jet<NT> xs[3][7];
  for (int j = 0; j < F.nkeys; ++j) {
    const Key& k = P.keys[F.keys[j]];
    if (k.type == SFG_KEY_POSE3) {
      Jet<NT> d[6];
      for (int i = 0; i < 6; ++i) d[i] = Jet<NT>::Seed(0.0, F.koff[j] + i);
      RetractPose3(values + k.soff, d, retract_eps, xs[j]);
    } else if (k.type == SFG_KEY_ROT3) {
      Jet<NT> d[3];
      for (int i = 0; i < 3; ++i) d[i] = Jet<NT>::Seed(0.0, F.koff[j] + i);
      RetractRot3(values + k.soff, d, retract_eps, xs[j]);
    } else {
      RetractKeyJet<NT>(k, values + k.soff, F.koff[j], xs[j]);
    }
  }
  Jet<NT> r[9];
  switch (F.kind) {
    case SFG_FACTOR_BEARING_POSE2: BearingResidual(xs[0], F.c, r); break;
    case SFG_FACTOR_ODOMETRY_POSE2: OdometryResidual(xs[0], xs[1], F.c, r); break;
    case SFG_FACTOR_SNAVELY_REPROJECTION: SnavelyResidual(xs[0], xs[1], xs[2], F.c, r); break;
    case SFG_FACTOR_BETWEEN_POSE3: BetweenPose3Residual(xs[0], xs[1], F.c, r); break;
    case SFG_FACTOR_PRIOR_POSE3: PriorPose3Residual(xs[0], F.c, r); break;
    case SFG_FACTOR_RANGE_POSE3: RangePose3Residual(xs[0], F.c, r); break;
    case SFG_FACTOR_PRIOR_ROT3: PriorRot3Residual(xs[0], F.c, r); break;
    case SFG_FACTOR_BETWEEN_ROT3: BetweenRot3Residual(xs[0], xs[1], F.c, r); break;
    case SFG_FACTOR_BARRON_VEC5: BarronVec5Residual(xs[0], F.c, r); break;
    case SFG_FACTOR_LINEAR_VEC5: LinearResidual(xs[0], F.c, 9, 5, r); break;
    case SFG_FACTOR_LINEAR_SCALAR2: {
      const Jet<NT> xy[2] = {xs[0][0], xs[1][0]};
      LinearResidual(xy, F.c, 2, 2, r);
      break;
    }
  }
  for (int i = 0; i < F.rdim; ++i) {
    res[i] = r[i].a;
    if (J) for (int t = 0; t < F.tdim; ++t) J[i * F.tdim + t] = r[i].v[t];
  }
}

void LinearizeFactor(const Problem& P, const Factor& F, const double* values, double* res,
                     double* J, double retract_eps) {
  switch (F.tdim) {
    case 2: LinearizeFactorT<2>(P, F, values, res, J, retract_eps); return;
    case 5: LinearizeFactorT<5>(P, F, values, res, J, retract_eps); return;
    case 3: LinearizeFactorT<3>(P, F, values, res, J, retract_eps); return;
    case 6: LinearizeFactorT<6>(P, F, values, res, J, retract_eps); return;
    case 12: LinearizeFactorT<12>(P, F, values, res, J, retract_eps); return;
  }
  throw std::logic_error("unsupported factor tangent dim");
}

// ---------------------------------------------------------------------------------------------
// CSC matrices (column-major, row indices sorted within each column)
// ---------------------------------------------------------------------------------------------
struct Csc {
  int64_t n = 0;
  std::vector<int64_t> colptr;
  std::vector<int32_t> rowidx;
  int64_t Find(int64_t r, int64_t c) const {
    auto b = rowidx.begin() + colptr[c], e = rowidx.begin() + colptr[c + 1];
    auto it = std::lower_bound(b, e, int32_t(r));
    if (it == e || *it != r) return -1;
    return it - rowidx.begin();
  }
};

// ---------------------------------------------------------------------------------------------
// Linearizer (CSC lower Hessian)
// ---------------------------------------------------------------------------------------------
struct Linearization {
  std::vector<double> residual, rhs, hvals;
  bool initialized = false;
  double Error() const {
    double s = 0;
    for (double r : residual) s += r * r;
    return 0.5 * s;
  }
  double LinearDeltaError(const std::vector<double>& u, const std::vector<double>& d) const {
    double s = 0;
    for (size_t i = 0; i < u.size(); ++i) s += u[i] * (rhs[i] - d[i] * u[i]);
    return 0.5 * s;
  }
};

struct Linearizer {
  const Problem* P;
  Csc H;                                // hessian_lower structure
  std::vector<int64_t> diag;            // storage index of each diagonal entry
  std::vector<std::vector<int64_t>> fmap;  // per factor: tdim*tdim storage index (-1: upper)
  double retract_eps = 0.0;

  explicit Linearizer(const Problem& prob) : P(&prob) {
    const int64_t N = P->N;
    std::vector<std::vector<int32_t>> cols(N);
    for (int64_t i = 0; i < N; ++i) cols[i].push_back(int32_t(i));
    std::vector<int64_t> gidx;
    for (const Factor& F : P->factors) {
      gidx.clear();
      for (int j = 0; j < F.nkeys; ++j) {
        const Key& k = P->keys[F.keys[j]];
        for (int t = 0; t < k.tdim; ++t) gidx.push_back(k.toff + t);
      }
      // key blocks: diagonal blocks lower triangle, off-diagonal blocks complete
      for (int a = 0; a < F.tdim; ++a)
        for (int b = 0; b < F.tdim; ++b)
          if (gidx[a] >= gidx[b]) cols[gidx[b]].push_back(int32_t(gidx[a]));
    }
    H.n = N;
    H.colptr.assign(N + 1, 0);
    for (int64_t c = 0; c < N; ++c) {
      auto& v = cols[c];
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
      H.colptr[c + 1] = H.colptr[c] + int64_t(v.size());
    }
    H.rowidx.resize(H.colptr[N]);
    for (int64_t c = 0; c < N; ++c)
      std::copy(cols[c].begin(), cols[c].end(), H.rowidx.begin() + H.colptr[c]);
    diag.resize(N);
    for (int64_t i = 0; i < N; ++i) diag[i] = H.Find(i, i);
    fmap.resize(P->factors.size());
    for (size_t f = 0; f < P->factors.size(); ++f) {
      const Factor& F = P->factors[f];
      gidx.clear();
      for (int j = 0; j < F.nkeys; ++j) {
        const Key& k = P->keys[F.keys[j]];
        for (int t = 0; t < k.tdim; ++t) gidx.push_back(k.toff + t);
      }
      fmap[f].assign(size_t(F.tdim) * F.tdim, -1);
      for (int a = 0; a < F.tdim; ++a)
        for (int b = 0; b < F.tdim; ++b)
          if (gidx[a] >= gidx[b]) fmap[f][a * F.tdim + b] = H.Find(gidx[a], gidx[b]);
    }
  }

  void Relinearize(const std::vector<double>& values, Linearization& lin) const {
    lin.residual.assign(P->M, 0.0);
    lin.rhs.assign(P->N, 0.0);
    lin.hvals.assign(H.rowidx.size(), 0.0);
    double res[9], J[9 * 12];  // residual rows <= 9, tangent columns <= 12
    for (size_t f = 0; f < P->factors.size(); ++f) {
      const Factor& F = P->factors[f];
      LinearizeFactor(*P, F, values.data(), res, J, retract_eps);
      for (int i = 0; i < F.rdim; ++i) lin.residual[F.roff + i] = res[i];
      int a_key = 0;
      for (int a = 0; a < F.tdim; ++a) {
        while (a_key + 1 < F.nkeys && a >= F.koff[a_key + 1]) ++a_key;
        const Key& ka = P->keys[F.keys[a_key]];
        double g = 0;
        for (int i = 0; i < F.rdim; ++i) g += J[i * F.tdim + a] * res[i];
        lin.rhs[ka.toff + (a - F.koff[a_key])] += g;
        for (int b = 0; b < F.tdim; ++b) {
          const int64_t s = fmap[f][a * F.tdim + b];
          if (s < 0) continue;
          double h = 0;
          for (int i = 0; i < F.rdim; ++i) h += J[i * F.tdim + a] * J[i * F.tdim + b];
          lin.hvals[s] += h;
        }
      }
    }
    lin.initialized = true;
  }
};

// ---------------------------------------------------------------------------------------------
// Orderings.  Natural, or block minimum degree on the key-block graph (the oracle's own choice;
// the reference's METIS ordering is unavailable).  Both return order[new] = old (scalar level).
// ---------------------------------------------------------------------------------------------
std::vector<int32_t> BlockMinDegreeOrder(const std::vector<int>& dims,
                                         const std::vector<std::pair<int, int>>& edges) {
  const int nb = int(dims.size());
  std::vector<std::set<int>> adj(nb);
  for (auto& e : edges) {
    if (e.first == e.second) continue;
    adj[e.first].insert(e.second);
    adj[e.second].insert(e.first);
  }
  auto degree = [&](int v) {
    int64_t d = 0;
    for (int u : adj[v]) d += dims[u];
    return d;
  };
  using Item = std::pair<int64_t, int>;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
  std::vector<int64_t> deg(nb);
  std::vector<char> done(nb, 0);
  for (int v = 0; v < nb; ++v) {
    deg[v] = degree(v);
    pq.push({deg[v], v});
  }
  std::vector<int> border;
  while (!pq.empty()) {
    auto [d, v] = pq.top();
    pq.pop();
    if (done[v] || d != deg[v]) continue;
    done[v] = 1;
    border.push_back(v);
    std::vector<int> nbrs(adj[v].begin(), adj[v].end());
    for (int u : nbrs) adj[u].erase(v);
    for (size_t i = 0; i < nbrs.size(); ++i)
      for (size_t j = i + 1; j < nbrs.size(); ++j) {
        adj[nbrs[i]].insert(nbrs[j]);
        adj[nbrs[j]].insert(nbrs[i]);
      }
    for (int u : nbrs) {
      deg[u] = degree(u);
      pq.push({deg[u], u});
    }
    adj[v].clear();
  }
  std::vector<int64_t> start(nb + 1, 0);
  for (int b = 0; b < nb; ++b) start[b + 1] = start[b] + dims[b];
  std::vector<int32_t> order;
  for (int b : border)
    for (int t = 0; t < dims[b]; ++t) order.push_back(int32_t(start[b] + t));
  return order;
}

// ---------------------------------------------------------------------------------------------
// SparseCholeskySolver restatement: up-looking LDL^T, unit L, no pivoting.
// ---------------------------------------------------------------------------------------------
struct SparseLdlt {
  int64_t N = 0;
  std::vector<int32_t> perm, inv_perm;  // perm[old] = new, inv_perm[new] = old
  Csc Au;                               // permuted upper triangle structure
  std::vector<int64_t> a_map;           // lower-CSC entry -> Au entry
  std::vector<int64_t> parent, nnz_per_col, visited, L_outer, L_k_pattern;
  std::vector<int32_t> L_inner;
  std::vector<double> L_value, D, D_agg, Au_vals;

  // ComputeSymbolicSparsity (sparse_cholesky_solver.tcc:26-106); `order` = inv permutation.
  void Analyze(const Csc& A, const std::vector<int32_t>& order) {
    N = A.n;
    inv_perm = order;
    perm.assign(N, 0);
    for (int64_t i = 0; i < N; ++i) perm[inv_perm[i]] = int32_t(i);
    // twist: entries (i, j) of lower A -> (min, max) of (perm[i], perm[j]) in the upper triangle
    std::vector<std::vector<std::pair<int32_t, int64_t>>> cols(N);
    for (int64_t c = 0; c < N; ++c)
      for (int64_t p = A.colptr[c]; p < A.colptr[c + 1]; ++p) {
        const int32_t r = A.rowidx[p];
        const int32_t nr = perm[r], nc = perm[c];
        const int32_t lo = std::min(nr, nc), hi = std::max(nr, nc);
        cols[hi].push_back({lo, p});
      }
    Au.n = N;
    Au.colptr.assign(N + 1, 0);
    for (int64_t c = 0; c < N; ++c) {
      std::sort(cols[c].begin(), cols[c].end());
      Au.colptr[c + 1] = Au.colptr[c] + int64_t(cols[c].size());
    }
    Au.rowidx.resize(Au.colptr[N]);
    a_map.resize(A.rowidx.size());
    for (int64_t c = 0; c < N; ++c)
      for (size_t q = 0; q < cols[c].size(); ++q) {
        Au.rowidx[Au.colptr[c] + q] = cols[c][q].first;
        a_map[cols[c][q].second] = Au.colptr[c] + int64_t(q);
      }
    Au_vals.assign(Au.rowidx.size(), 0.0);

    visited.assign(N, -1);
    parent.assign(N, -1);
    nnz_per_col.assign(N, 0);
    for (int64_t k = 0; k < N; ++k) {
      visited[k] = k;
      for (int64_t p = Au.colptr[k]; p < Au.colptr[k + 1]; ++p) {
        int64_t i = Au.rowidx[p];
        if (i >= k) continue;
        while (visited[i] != k) {
          if (parent[i] == -1) parent[i] = k;
          nnz_per_col[i]++;
          visited[i] = k;
          i = parent[i];
        }
      }
    }
    L_outer.assign(N + 1, 0);
    for (int64_t k = 0; k < N; ++k) L_outer[k + 1] = L_outer[k] + nnz_per_col[k];
    L_inner.assign(L_outer[N], 0);
    L_value.assign(L_outer[N], 0.0);
    D.assign(N, 0.0);
    L_k_pattern.assign(N, 0);
    D_agg.assign(N, 0.0);
  }

  // Factorize (sparse_cholesky_solver.tcc:108-219) on lower-CSC values of A.
  void Factorize(const std::vector<double>& a_vals) {
    std::fill(Au_vals.begin(), Au_vals.end(), 0.0);
    for (size_t p = 0; p < a_vals.size(); ++p) Au_vals[a_map[p]] += a_vals[p];
    std::fill(nnz_per_col.begin(), nnz_per_col.end(), 0);
    std::fill(D_agg.begin(), D_agg.end(), 0.0);
    for (int64_t k = 0; k < N; ++k) {
      visited[k] = k;
      int64_t top = N;
      for (int64_t p = Au.colptr[k]; p < Au.colptr[k + 1]; ++p) {
        int64_t i = Au.rowidx[p];
        if (i > k) continue;
        D_agg[i] += Au_vals[p];
        int64_t depth = 0;
        while (visited[i] != k) {
          L_k_pattern[depth] = i;
          visited[i] = k;
          i = parent[i];
          depth += 1;
        }
        while (depth > 0) {
          top -= 1;
          depth -= 1;
          L_k_pattern[top] = L_k_pattern[depth];
        }
      }
      double D_k = D_agg[k];
      D_agg[k] = 0.0;
      for (; top < N; ++top) {
        const int64_t i = L_k_pattern[top];
        const double D_agg_i = D_agg[i];
        const double L_ki = D_agg_i / D[i];
        const int64_t ps = L_outer[i];
        const int64_t pe = ps + nnz_per_col[i];
        D_agg[i] = 0.0;
        int64_t ptr;
        for (ptr = ps; ptr < pe; ++ptr) D_agg[L_inner[ptr]] -= L_value[ptr] * D_agg_i;
        L_inner[ptr] = int32_t(k);
        L_value[ptr] = L_ki;
        D_k -= L_ki * D_agg_i;
        nnz_per_col[i] += 1;
      }
      D[k] = D_k;
    }
  }

  // SolveInPlace (sparse_cholesky_solver.tcc:230-259)
  void Solve(const double* b, double* x) const {
    std::vector<double> y(N);
    for (int64_t i = 0; i < N; ++i) y[perm[i]] = b[i];
    for (int64_t c = 0; c < N; ++c)  // L y = b, unit lower, column oriented
      for (int64_t p = L_outer[c]; p < L_outer[c] + nnz_per_col[c]; ++p) y[L_inner[p]] -= L_value[p] * y[c];
    for (int64_t i = 0; i < N; ++i) y[i] /= D[i];
    for (int64_t c = N - 1; c >= 0; --c)  // L^T x = y
      for (int64_t p = L_outer[c]; p < L_outer[c] + nnz_per_col[c]; ++p) y[c] -= L_value[p] * y[L_inner[p]];
    for (int64_t i = 0; i < N; ++i) x[i] = y[perm[i]];
  }
};

// Scalar order for a lower-CSC pattern: natural, or block minimum degree with unit blocks.
std::vector<int32_t> ScalarOrder(const Csc& A, int ordering, const std::vector<int>* block_dims) {
  std::vector<int32_t> order(A.n);
  std::iota(order.begin(), order.end(), 0);
  if (ordering == SFG_ORDERING_NATURAL) return order;
  std::vector<int> dims;
  std::vector<int64_t> first;  // block of each scalar
  std::vector<int> blk(A.n);
  if (block_dims) {
    dims = *block_dims;
  } else {
    dims.assign(A.n, 1);
  }
  {
    int64_t s = 0;
    for (int b = 0; b < int(dims.size()); ++b)
      for (int t = 0; t < dims[b]; ++t) blk[s++] = b;
  }
  std::set<std::pair<int, int>> es;
  for (int64_t c = 0; c < A.n; ++c)
    for (int64_t p = A.colptr[c]; p < A.colptr[c + 1]; ++p) {
      const int a = blk[A.rowidx[p]], b = blk[c];
      if (a != b) es.insert({std::max(a, b), std::min(a, b)});
    }
  std::vector<std::pair<int, int>> edges(es.begin(), es.end());
  return BlockMinDegreeOrder(dims, edges);
}

// ---------------------------------------------------------------------------------------------
// SparseSchurSolver restatement (sparse_schur_solver.tcc:15-170), dense S for the reduced system.
// ---------------------------------------------------------------------------------------------
struct SchurSolver {
  int64_t N = 0, B = 0, C = 0;
  struct CBlock { int64_t start; int dim; };
  std::vector<CBlock> blocks;
  std::vector<double> Cinv;               // per block dim*dim dense inverse, packed
  std::vector<int64_t> cinv_off;
  std::vector<std::vector<std::pair<int32_t, double>>> Et;  // per C row: (B col, value)
  Csc S_pattern;
  std::vector<double> S_vals;
  SparseLdlt S_solver;
  bool s_analyzed = false;
  int ordering = SFG_ORDERING_MIN_DEGREE;

  // ComputeSymbolicSparsity: find the dense diagonal blocks of C.
  void Analyze(const Csc& A, int64_t c_dim) {
    N = A.n;
    C = c_dim;
    B = N - C;
    int64_t col = B;
    while (col < N) {
      const int64_t p0 = A.colptr[col], p1 = A.colptr[col + 1];
      int64_t nz_c = 0, first = -1, prev = -1;
      for (int64_t p = p0; p < p1; ++p) {
        if (A.rowidx[p] < B) continue;
        if (first < 0) first = A.rowidx[p];
        if (prev >= 0 && A.rowidx[p] != prev + 1)
          throw std::runtime_error("Submatrix C of A is not block diagonal");
        prev = A.rowidx[p];
        ++nz_c;
      }
      if (first != col) throw std::runtime_error("C column does not start on the diagonal");
      const int dim = int(nz_c);
      blocks.push_back({col, dim});
      col += dim;
    }
    cinv_off.resize(blocks.size() + 1, 0);
    for (size_t b = 0; b < blocks.size(); ++b)
      cinv_off[b + 1] = cinv_off[b] + int64_t(blocks[b].dim) * blocks[b].dim;
    Cinv.assign(cinv_off.back(), 0.0);
  }

  void Factorize(const Csc& A, const std::vector<double>& vals) {
    // C_inv via dense LL^T of each block
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const auto& blk = blocks[bi];
      const int d = blk.dim;
      std::vector<double> M(d * d, 0.0), L(d * d, 0.0);
      for (int c = 0; c < d; ++c)
        for (int64_t p = A.colptr[blk.start + c]; p < A.colptr[blk.start + c + 1]; ++p) {
          const int64_t r = A.rowidx[p];
          if (r >= blk.start && r < blk.start + d) {
            M[(r - blk.start) * d + c] = vals[p];
            M[c * d + (r - blk.start)] = vals[p];
          }
        }
      for (int j = 0; j < d; ++j) {
        double s = M[j * d + j];
        for (int k = 0; k < j; ++k) s -= L[j * d + k] * L[j * d + k];
        L[j * d + j] = std::sqrt(s);
        for (int i = j + 1; i < d; ++i) {
          double t = M[i * d + j];
          for (int k = 0; k < j; ++k) t -= L[i * d + k] * L[j * d + k];
          L[i * d + j] = t / L[j * d + j];
        }
      }
      // inverse = L^-T L^-1 via solving for identity columns
      double* out = &Cinv[cinv_off[bi]];
      for (int c = 0; c < d; ++c) {
        std::vector<double> y(d, 0.0);
        y[c] = 1.0;
        for (int i = 0; i < d; ++i) {
          for (int k = 0; k < i; ++k) y[i] -= L[i * d + k] * y[k];
          y[i] /= L[i * d + i];
        }
        for (int i = d - 1; i >= 0; --i) {
          for (int k = i + 1; k < d; ++k) y[i] -= L[k * d + i] * y[k];
          y[i] /= L[i * d + i];
        }
        for (int i = 0; i < d; ++i) out[i * d + c] = y[i];
      }
    }
    // E^T rows (C x B) and B block
    Et.assign(C, {});
    std::vector<double> Sd(size_t(B) * B, 0.0);
    for (int64_t c = 0; c < N; ++c)
      for (int64_t p = A.colptr[c]; p < A.colptr[c + 1]; ++p) {
        const int64_t r = A.rowidx[p];
        if (c < B && r < B) {
          Sd[r * B + c] += vals[p];
          if (r != c) Sd[c * B + r] += vals[p];
        } else if (c < B && r >= B) {
          Et[r - B].push_back({int32_t(c), vals[p]});
        }
      }
    // S = B - E C^-1 E^T, one C block at a time
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const auto& blk = blocks[bi];
      const int d = blk.dim;
      const double* ci = &Cinv[cinv_off[bi]];
      std::map<int32_t, std::vector<double>> rows;  // B col -> d-vector of E^T column
      for (int i = 0; i < d; ++i)
        for (auto& e : Et[blk.start - B + i]) {
          auto& v = rows[e.first];
          if (v.empty()) v.assign(d, 0.0);
          v[i] = e.second;
        }
      for (auto& ra : rows)
        for (auto& rb : rows) {
          double s = 0;
          for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) s += ra.second[i] * ci[i * d + j] * rb.second[j];
          Sd[size_t(ra.first) * B + rb.first] -= s;
        }
    }
    if (!s_analyzed) {
      S_pattern.n = B;
      S_pattern.colptr.assign(B + 1, 0);
      S_pattern.rowidx.clear();
      for (int64_t c = 0; c < B; ++c) {
        for (int64_t r = c; r < B; ++r)
          if (Sd[r * B + c] != 0.0 || r == c) S_pattern.rowidx.push_back(int32_t(r));
        S_pattern.colptr[c + 1] = int64_t(S_pattern.rowidx.size());
      }
      S_solver.Analyze(S_pattern, ScalarOrder(S_pattern, ordering, nullptr));
      s_analyzed = true;
    }
    S_vals.assign(S_pattern.rowidx.size(), 0.0);
    for (int64_t c = 0; c < B; ++c)
      for (int64_t p = S_pattern.colptr[c]; p < S_pattern.colptr[c + 1]; ++p)
        S_vals[p] = Sd[size_t(S_pattern.rowidx[p]) * B + c];
    S_solver.Factorize(S_vals);
  }

  void Solve(const double* rhs, double* x) const {
    // v - E C^-1 w
    std::vector<double> cw(C, 0.0), srhs(rhs, rhs + B);
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const auto& blk = blocks[bi];
      const int d = blk.dim;
      const double* ci = &Cinv[cinv_off[bi]];
      for (int i = 0; i < d; ++i) {
        double s = 0;
        for (int j = 0; j < d; ++j) s += ci[i * d + j] * rhs[blk.start + j];
        cw[blk.start - B + i] = s;
      }
    }
    for (int64_t r = 0; r < C; ++r)
      for (auto& e : Et[r]) srhs[e.first] -= e.second * cw[r];
    std::vector<double> y(B);
    S_solver.Solve(srhs.data(), y.data());
    std::vector<double> wr(rhs + B, rhs + N);
    for (int64_t r = 0; r < C; ++r)
      for (auto& e : Et[r]) wr[r] -= e.second * y[e.first];
    for (int64_t i = 0; i < B; ++i) x[i] = y[i];
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const auto& blk = blocks[bi];
      const int d = blk.dim;
      const double* ci = &Cinv[cinv_off[bi]];
      for (int i = 0; i < d; ++i) {
        double s = 0;
        for (int j = 0; j < d; ++j) s += ci[i * d + j] * wr[blk.start - B + j];
        x[blk.start + i] = s;
      }
    }
  }
};

// ---------------------------------------------------------------------------------------------
// Values::Retract (symforce/opt/values.cc:315-327)
// ---------------------------------------------------------------------------------------------
void RetractValues(const Problem& P, const std::vector<double>& in, const double* delta, double eps,
                   std::vector<double>& out) {
  out = in;
  for (const Key& k : P.keys) {
    const double* a = &in[k.soff];
    double* o = &out[k.soff];
    const double* d = delta + k.toff;
    switch (k.type) {
      case SFG_KEY_POSE2: RetractPose2(a, d, o); break;
      case SFG_KEY_POSE3: RetractPose3(a, d, eps, o); break;
      case SFG_KEY_ROT3: RetractRot3(a, d, eps, o); break;
      default:
        for (int i = 0; i < k.tdim; ++i) o[i] = a[i] + d[i];
    }
  }
}

// ---------------------------------------------------------------------------------------------
// LevenbergMarquardtSolver restatement
// ---------------------------------------------------------------------------------------------
struct StateBlock {
  std::vector<double> values;
  Linearization lin;
  mutable bool have_err = false;
  mutable double err = 0;
  double Error() const {
    if (!have_err) {
      err = lin.Error();
      have_err = true;
    }
    return err;
  }
};

struct LmResult {
  std::vector<sfg_iteration_t> iters;
  int best_index = 0, status = 0, failure_reason = 0;
  std::vector<double> best_values;
  double seconds = 0;
  double seconds_linearize = 0, seconds_solve = 0;
};

struct LinearSolverChoice {
  int kind = SFG_LINEAR_SOLVER_SPARSE_LDLT;
  int ordering = SFG_ORDERING_MIN_DEGREE;
};

// State that OptimizeContinue keeps across calls (symforce/opt/gnc_optimizer.h:113-121): lambda,
// nu and the iteration counter (ResetState, symforce/opt/levenberg_marquardt_solver.h:176-183).
struct LmCarry {
  double lambda = 0, nu = 0;
  int iteration = -1;
};

LmResult Optimize(const Problem& P, const std::vector<double>& values0,
                  const sfg_optimizer_params_t& p, int num_iterations, double epsilon,
                  LinearSolverChoice ls, LmCarry* carry = nullptr, bool continue_state = false) {
  using Clock = std::chrono::steady_clock;
  const auto t_start = Clock::now();
  double t_lin = 0, t_sol = 0;
  Linearizer linz(P);
  linz.retract_eps = epsilon;
  const int64_t N = P.N;
  if (num_iterations < 0) num_iterations = p.iterations;
  if (num_iterations <= 0) throw std::invalid_argument("num_iterations must be positive");

  // block dims of the key graph, for the block minimum-degree ordering
  std::vector<int> dims;
  for (auto& k : P.keys) dims.push_back(k.tdim);

  StateBlock blocks[3];
  int init_idx = 0, new_idx = 1, best_idx = 0, free_idx = 2;
  bool best_valid = false;
  (void)best_valid;
  // Reset(values), or ResetState(values) when continuing
  double lambda = p.initial_lambda;
  double nu = p.dynamic_lambda_update_beta;
  int iteration = -1;
  if (continue_state && carry) {
    lambda = carry->lambda;
    nu = carry->nu;
    iteration = carry->iteration;
  }
  bool have_max_diagonal = false, have_last_update = false;
  blocks[new_idx].values = values0;
  for (auto& b : blocks) {
    b.lin.initialized = false;
    b.have_err = false;
  }
  bool solver_analyzed = false;
  SparseLdlt ldlt;
  SchurSolver schur;
  schur.ordering = ls.ordering;
  std::vector<double> max_diagonal, damping(N), undamped(N), update(N), last_update;

  LmResult R;
  if (continue_state) R.best_index = -1;
  auto relinearize = [&](StateBlock& b) {
    const auto t0 = Clock::now();
    linz.Relinearize(b.values, b.lin);
    b.have_err = false;
    t_lin += std::chrono::duration<double>(Clock::now() - t0).count();
  };

  int i;
  for (i = 0; i < num_iterations; ++i) {
    // ---- Iterate()
    std::swap(init_idx, new_idx);  // state_.Step()
    iteration++;
    StateBlock& Init = blocks[init_idx];
    if (!Init.lin.initialized) {
      relinearize(Init);
      // SetBestToInit
      best_valid = true;
      if (best_idx != init_idx) {
        if (best_idx != new_idx) free_idx = best_idx;
        best_idx = init_idx;
      }
    }
    bool done = false;
    int status = 0, reason = 0;
    if (iteration == 0) {
      sfg_iteration_t rec{};
      rec.iteration = -1;
      rec.new_error = Init.Error();
      rec.current_lambda = lambda;
      rec.best_error = rec.new_error;
      R.iters.push_back(rec);
      if (!std::isfinite(Init.Error())) {
        status = SFG_STATUS_FAILED;
        reason = SFG_FAILURE_INITIAL_ERROR_NOT_FINITE;
        R.status = status;
        R.failure_reason = reason;
        break;
      }
    }
    const auto t0 = Clock::now();
    if (!solver_analyzed) {
      if (ls.kind == SFG_LINEAR_SOLVER_SCHUR) {
        int64_t cdim = 0;
        for (int k = int(P.keys.size()) - P.num_schur; k < int(P.keys.size()); ++k) cdim += P.keys[k].tdim;
        schur.Analyze(linz.H, cdim);
      } else {
        ldlt.Analyze(linz.H, ScalarOrder(linz.H, ls.ordering, &dims));
      }
      solver_analyzed = true;
    }
    // DampHessian
    std::vector<double>& hv = Init.lin.hvals;
    for (int64_t k = 0; k < N; ++k) undamped[k] = hv[linz.diag[k]];
    if (p.use_diagonal_damping) {
      if (p.keep_max_diagonal_damping) {
        if (!have_max_diagonal) {
          max_diagonal.resize(N);
          for (int64_t k = 0; k < N; ++k) max_diagonal[k] = std::max(undamped[k], p.diagonal_damping_min);
        } else {
          for (int64_t k = 0; k < N; ++k) max_diagonal[k] = std::max(max_diagonal[k], undamped[k]);
        }
        have_max_diagonal = true;
        for (int64_t k = 0; k < N; ++k) damping[k] = max_diagonal[k] * lambda;
      } else {
        for (int64_t k = 0; k < N; ++k) damping[k] = std::max(undamped[k], p.diagonal_damping_min) * lambda;
      }
    } else {
      std::fill(damping.begin(), damping.end(), 0.0);
    }
    if (p.use_unit_damping)
      for (int64_t k = 0; k < N; ++k) damping[k] += lambda;
    for (int64_t k = 0; k < N; ++k) hv[linz.diag[k]] += damping[k];
    // Factorize + Solve
    if (ls.kind == SFG_LINEAR_SOLVER_SCHUR) {
      schur.Factorize(linz.H, hv);
      schur.Solve(Init.lin.rhs.data(), update.data());
    } else {
      ldlt.Factorize(hv);
      ldlt.Solve(Init.lin.rhs.data(), update.data());
    }
    for (auto& u : update) u = -u;
    for (int64_t k = 0; k < N; ++k) hv[linz.diag[k]] = undamped[k];
    t_sol += std::chrono::duration<double>(Clock::now() - t0).count();
    // UpdateNewFromInit + Relinearize
    StateBlock& New = blocks[new_idx];
    RetractValues(P, Init.values, update.data(), epsilon, New.values);
    relinearize(New);
    const double new_error = New.Error();
    const double init_error = Init.Error();
    const double relative_reduction = (init_error - new_error) / (init_error + epsilon);
    const double new_error_linear = init_error + Init.lin.LinearDeltaError(update, damping);
    const double gain_ratio = (init_error - new_error) / (init_error - new_error_linear);
    sfg_iteration_t rec{};
    rec.iteration = iteration;
    rec.current_lambda = lambda;
    rec.new_error = new_error;
    rec.new_error_linear = new_error_linear;
    rec.relative_reduction = relative_reduction;
    if ((relative_reduction > -p.early_exit_min_reduction / 10 &&
         relative_reduction < p.early_exit_min_reduction) ||
        new_error < p.early_exit_min_absolute_error) {
      done = true;
      status = SFG_STATUS_SUCCESS;
      reason = 0;
    }
    bool accept = relative_reduction > 0;
    double angle = 0;
    if (p.enable_bold_updates && have_last_update && !accept) {
      double nl = 0, nu2 = 0, dot = 0;
      for (int64_t k = 0; k < N; ++k) {
        nl += last_update[k] * last_update[k];
        nu2 += update[k] * update[k];
        dot += last_update[k] * update[k];
      }
      angle = dot / (std::sqrt(nl) * std::sqrt(nu2));
      accept = ((1 - angle) * (1 - angle) * new_error) <= blocks[best_idx].Error();
    }
    if (!accept && lambda >= p.lambda_upper_bound) {
      done = true;
      status = SFG_STATUS_FAILED;
      reason = SFG_FAILURE_LAMBDA_OUT_OF_BOUNDS;
    }
    if (!accept) {
      if (p.lambda_update_type == SFG_LAMBDA_UPDATE_STATIC) {
        lambda *= p.lambda_up_factor;
      } else {
        lambda *= nu;
        nu *= 2;
      }
      std::swap(init_idx, new_idx);  // SwapNewAndInit
    } else {
      if (p.lambda_update_type == SFG_LAMBDA_UPDATE_STATIC) {
        lambda *= p.lambda_down_factor;
      } else {
        lambda *= std::max(1.0 / p.dynamic_lambda_update_gamma,
                           1.0 - (p.dynamic_lambda_update_beta - 1) *
                                     std::pow(2 * gain_ratio - 1, double(p.dynamic_lambda_update_p)));
        nu = 2;
      }
      have_last_update = true;
      last_update = update;
      if (blocks[new_idx].Error() <= blocks[best_idx].Error()) {
        // SetBestToNew
        if (best_idx != new_idx) {
          if (best_idx != init_idx) free_idx = best_idx;
          best_idx = new_idx;
        }
        R.best_index = int(R.iters.size());  // index of the record pushed below
      }
      // SetInitToNotBest
      if (best_idx == init_idx) {
        init_idx = free_idx;
        free_idx = best_idx;
      }
    }
    lambda = std::min(std::max(lambda, p.lambda_lower_bound), p.lambda_upper_bound);
    rec.update_angle_change = angle;
    rec.update_accepted = accept ? 1 : 0;
    rec.best_error = blocks[best_idx].Error();
    R.iters.push_back(rec);
    if (done) {
      R.status = status;
      R.failure_reason = reason;
      break;
    }
  }
  if (i == num_iterations) {
    R.status = SFG_STATUS_HIT_ITERATION_LIMIT;
    R.failure_reason = 0;
  }
  R.best_values = blocks[best_idx].values;
  if (carry) {
    carry->lambda = lambda;
    carry->nu = nu;
    carry->iteration = iteration;
  }
  R.seconds = std::chrono::duration<double>(Clock::now() - t_start).count();
  R.seconds_linearize = t_lin;
  R.seconds_solve = t_sol;
  return R;
}

}  // namespace oracle

// =============================================================================================
// C ABI for the tests (ctypes).  Every function returns 0 on success, nonzero with a message
// available from orc_last_error() on failure.
// =============================================================================================
namespace {
thread_local std::string g_err;
template <typename F>
int Guard(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}
}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

// Linearize one factor at the given key storages; J is rdim x tdim row-major.
int orc_factor_linearize(int32_t kind, const int32_t* key_types, const double* storage,
                         const double* consts, double epsilon, double* res, double* J) {
  return Guard([&] {
    using namespace oracle;
    const FactorSpec s = Spec(kind);
    Problem P;
    int64_t so = 0, to = 0;
    for (int j = 0; j < s.nkeys; ++j) {
      Key k;
      k.type = key_types[j];
      KeyDims(k.type, &k.sdim, &k.tdim);
      k.soff = so;
      k.toff = to;
      so += k.sdim;
      to += k.tdim;
      P.keys.push_back(k);
    }
    Factor F;
    F.kind = kind;
    F.nkeys = s.nkeys;
    F.rdim = s.rdim;
    F.tdim = 0;
    for (int j = 0; j < s.nkeys; ++j) {
      F.keys[j] = j;
      F.koff[j] = F.tdim;
      F.tdim += P.keys[j].tdim;
    }
    F.c = consts;
    F.roff = 0;
    LinearizeFactor(P, F, storage, res, J, epsilon);
  });
}

// Residual, rhs and CSC hessian_lower of a whole problem.  Call with null outputs to get sizes.
int orc_linearize(const sfg_problem_t* prob, const double* values, double epsilon, int64_t* M,
                  int64_t* N, int64_t* nnz, double* residual, double* rhs, int64_t* col_ptr,
                  int32_t* row_idx, double* hvals) {
  return Guard([&] {
    using namespace oracle;
    Problem P = BuildProblem(prob);
    Linearizer L(P);
    L.retract_eps = epsilon;
    *M = P.M;
    *N = P.N;
    *nnz = int64_t(L.H.rowidx.size());
    if (!residual) return;
    Linearization lin;
    std::vector<double> v(values, values + P.S);
    L.Relinearize(v, lin);
    std::copy(lin.residual.begin(), lin.residual.end(), residual);
    std::copy(lin.rhs.begin(), lin.rhs.end(), rhs);
    std::copy(L.H.colptr.begin(), L.H.colptr.end(), col_ptr);
    std::copy(L.H.rowidx.begin(), L.H.rowidx.end(), row_idx);
    std::copy(lin.hvals.begin(), lin.hvals.end(), hvals);
  });
}

// Full LM optimization.  iters must hold params->iterations + 1 records.
int orc_optimize(const sfg_problem_t* prob, const double* values_in,
                 const sfg_optimizer_params_t* params, int32_t num_iterations, double epsilon,
                 int32_t linear_solver, int32_t ordering, double* values_out,
                 sfg_iteration_t* iters, int32_t capacity, int32_t* num_iters, int32_t* best_index,
                 int32_t* status, int32_t* failure_reason, double* seconds) {
  return Guard([&] {
    using namespace oracle;
    Problem P = BuildProblem(prob);
    std::vector<double> v(values_in, values_in + P.S);
    LinearSolverChoice ls;
    ls.kind = linear_solver;
    ls.ordering = ordering;
    LmResult R = Optimize(P, v, *params, num_iterations, epsilon, ls);
    if (int(R.iters.size()) > capacity) throw std::runtime_error("iteration buffer too small");
    std::copy(R.iters.begin(), R.iters.end(), iters);
    *num_iters = int32_t(R.iters.size());
    *best_index = R.best_index;
    *status = R.status;
    *failure_reason = R.failure_reason;
    std::copy(R.best_values.begin(), R.best_values.end(), values_out);
    if (seconds) {
      seconds[0] = R.seconds;
      seconds[1] = R.seconds_linearize;
      seconds[2] = R.seconds_solve;
    }
  });
}

// orc_optimize with the state OptimizeContinue keeps: carry = {lambda, nu, iteration}.  mode 0 runs
// a fresh optimization and writes the carry out; mode 1 continues from the carry (no iteration -1
// record, best_index -1 unless a record improves) and writes it back.
int orc_optimize_carry(const sfg_problem_t* prob, const double* values_in,
                       const sfg_optimizer_params_t* params, int32_t num_iterations, double epsilon,
                       int32_t linear_solver, int32_t ordering, double* values_out,
                       sfg_iteration_t* iters, int32_t capacity, int32_t* num_iters,
                       int32_t* best_index, int32_t* status, int32_t* failure_reason, double* carry,
                       int32_t mode) {
  return Guard([&] {
    using namespace oracle;
    Problem P = BuildProblem(prob);
    std::vector<double> v(values_in, values_in + P.S);
    LinearSolverChoice ls;
    ls.kind = linear_solver;
    ls.ordering = ordering;
    LmCarry c;
    c.lambda = carry[0];
    c.nu = carry[1];
    c.iteration = int(carry[2]);
    LmResult R = Optimize(P, v, *params, num_iterations, epsilon, ls, &c, mode == 1);
    if (int(R.iters.size()) > capacity) throw std::runtime_error("iteration buffer too small");
    std::copy(R.iters.begin(), R.iters.end(), iters);
    *num_iters = int32_t(R.iters.size());
    *best_index = R.best_index;
    *status = R.status;
    *failure_reason = R.failure_reason;
    std::copy(R.best_values.begin(), R.best_values.end(), values_out);
    carry[0] = c.lambda;
    carry[1] = c.nu;
    carry[2] = double(c.iteration);
  });
}

// SparseCholeskySolver on a lower CSC matrix; ordering SFG_ORDERING_NATURAL / MIN_DEGREE, or an
// explicit `order` (order[new] = old) when non-null.  Returns x and D (in the permuted order).
int orc_ldlt_solve(int64_t n, const int64_t* col_ptr, const int32_t* row_idx, const double* vals,
                   int32_t ordering, const int32_t* order, const double* b, double* x, double* D,
                   int32_t* perm_out) {
  return Guard([&] {
    using namespace oracle;
    Csc A;
    A.n = n;
    A.colptr.assign(col_ptr, col_ptr + n + 1);
    A.rowidx.assign(row_idx, row_idx + col_ptr[n]);
    SparseLdlt S;
    std::vector<int32_t> ord = order ? std::vector<int32_t>(order, order + n) : ScalarOrder(A, ordering, nullptr);
    S.Analyze(A, ord);
    S.Factorize(std::vector<double>(vals, vals + col_ptr[n]));
    S.Solve(b, x);
    if (D) std::copy(S.D.begin(), S.D.end(), D);
    if (perm_out) std::copy(S.perm.begin(), S.perm.end(), perm_out);
  });
}

int orc_schur_solve(int64_t n, const int64_t* col_ptr, const int32_t* row_idx, const double* vals,
                    int64_t c_dim, const double* b, double* x) {
  return Guard([&] {
    using namespace oracle;
    Csc A;
    A.n = n;
    A.colptr.assign(col_ptr, col_ptr + n + 1);
    A.rowidx.assign(row_idx, row_idx + col_ptr[n]);
    SchurSolver S;
    S.Analyze(A, c_dim);
    S.Factorize(A, std::vector<double>(vals, vals + col_ptr[n]));
    S.Solve(b, x);
  });
}

int orc_retract(int32_t key_type, const double* storage, const double* delta, double epsilon,
                double* out) {
  return Guard([&] {
    using namespace oracle;
    switch (key_type) {
      case SFG_KEY_POSE2: RetractPose2(storage, delta, out); break;
      case SFG_KEY_POSE3: RetractPose3(storage, delta, epsilon, out); break;
      case SFG_KEY_ROT3: RetractRot3(storage, delta, epsilon, out); break;
      default: {
        int sd, td;
        KeyDims(key_type, &sd, &td);
        for (int i = 0; i < td; ++i) out[i] = storage[i] + delta[i];
      }
    }
  });
}

// Initial values of the reference's Pose3 smoothing test (test/symforce_optimizer_test.cc:80-133):
// prior_start.Retract(0.4 * sym::Random<Vector6d>(std::mt19937(42))) for 10 keys, where
// Random<Vector6d> draws six std::normal_distribution<double> samples in order
// (gen/cpp/sym/ops/matrix/storage_ops.h:212-218).  prior_start is the identity pose.
int orc_pose_smoothing_initial_values(int32_t num_keys, double epsilon, double* out) {
  return Guard([&] {
    std::mt19937 gen(42);
    const double identity[7] = {0, 0, 0, 1, 0, 0, 0};
    for (int i = 0; i < num_keys; ++i) {
      std::normal_distribution<double> dist{};
      double d[6];
      for (int k = 0; k < 6; ++k) d[k] = 0.4 * dist(gen);
      oracle::RetractPose3(identity, d, epsilon, out + 7 * i);
    }
  });
}

// sym::Random<Eigen::Matrix<double, dim, 1>>(gen) called num_vectors times in a row on
// std::mt19937(seed): each call draws `dim` std::normal_distribution<double> samples in order from a
// fresh distribution (gen/cpp/sym/ops/matrix/storage_ops.h:212-218; a matrix is filled in its
// column-major coefficient order).  out: num_vectors x dim.
int orc_mt19937_normal_vectors(uint32_t seed, int32_t num_vectors, int32_t dim, double* out) {
  return Guard([&] {
    std::mt19937 gen(seed);
    for (int i = 0; i < num_vectors; ++i) {
      std::normal_distribution<double> dist{};
      for (int k = 0; k < dim; ++k) out[int64_t(i) * dim + k] = dist(gen);
    }
  });
}

// Initial values of the reference's Rot3 smoothing test (test/symforce_optimizer_test.cc:232-236):
// identity.Retract(0.4 * sym::Random<Vector3d>(std::mt19937(42)), epsilon) for num_keys keys,
// storage [x, y, z, w] each.
int orc_rot3_smoothing_initial_values(int32_t num_keys, double epsilon, double* out) {
  return Guard([&] {
    std::mt19937 gen(42);
    const double identity[4] = {0, 0, 0, 1};
    for (int i = 0; i < num_keys; ++i) {
      std::normal_distribution<double> dist{};
      double d[3];
      for (int k = 0; k < 3; ++k) d[k] = 0.4 * dist(gen);
      oracle::RetractRot3(identity, d, epsilon, out + 4 * i);
    }
  });
}

}  // extern "C"
