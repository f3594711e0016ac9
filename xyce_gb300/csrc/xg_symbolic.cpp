// xg_symbolic.cpp — host analysis for the frozen-pattern GPU LU.
//
// Replaces the symbolic part of the KLU path Xyce takes through Amesos
// (src/LinearAlgebraServicesPKG/N_LAS_AmesosSolver.C:309-335: symbolic
// factorization once per pattern) with an analysis designed for a
// level-scheduled GPU refactorization:
//   1. row matching from the current values (a nonzero, large diagonal;
//      voltage-source branch rows swap with their node rows),
//   2. peeling of row singletons to the front and column singletons to the
//      back (the 1x1 blocks a block-triangular form would find: ideal
//      voltage sources to ground and their branch currents),
//   3. an ordering of the remaining core: nested dissection (BFS level-set
//      bisection, each connected component — e.g. each circuit of a batch —
//      apart) or approximate minimum degree, whichever has the smaller
//      estimated refactorization time (fill work and dependency depth),
//   4. Gilbert-Peierls symbolic factorization of the permuted matrix, and
//   5. level schedules for the left-looking factorization and for the
//      row-oriented L and U solves.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <map>
#include <numeric>
#include <atomic>
#include <deque>
#include <queue>
#include <thread>

#include "xg_internal.h"

namespace xg {
namespace {

// Diagonal preference of the row matching.  Weak diagonals (e.g. 1% of the
// column, as in the operating point of a ring oscillator, where gds << gm)
// are not kept: a static pivot that small compounds growth along a cycle.
constexpr double kDiagPref = 0.1;

struct Csc {
  std::vector<int> cp, ri, src;  // src = CSR index of the entry
};

Csc to_csc(int n, const std::vector<int> &rp, const std::vector<int> &ci) {
  Csc c;
  c.cp.assign(n + 1, 0);
  for (int e = 0; e < (int)ci.size(); ++e) c.cp[ci[e] + 1]++;
  for (int j = 0; j < n; ++j) c.cp[j + 1] += c.cp[j];
  c.ri.resize(ci.size());
  c.src.resize(ci.size());
  std::vector<int> nxt(c.cp.begin(), c.cp.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      int q = nxt[ci[e]]++;
      c.ri[q] = i;
      c.src[q] = e;
    }
  return c;
}

// Maximum transversal preferring large entries: diagonal when it is at least
// kDiagPref of its column's largest entry, then greedy by magnitude, then augmenting
// paths (MC21-style depth-first search) for what is left.
bool match_rows(int n, const Csc &A, const std::vector<double> &vals, std::vector<int> &row_of_col,
                std::string &err, const std::vector<int> *keep) {
  std::vector<int> col_of_row(n, -1);
  row_of_col.assign(n, -1);
  // kept columns (keep[j] >= 0) take their earlier row first; they are
  // whole independent blocks, so the search below never reaches them
  if (keep)
    for (int j = 0; j < n; ++j)
      if ((*keep)[j] >= 0) { row_of_col[j] = (*keep)[j]; col_of_row[(*keep)[j]] = j; }
  std::vector<double> colmax(n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int q = A.cp[j]; q < A.cp[j + 1]; ++q) colmax[j] = std::max(colmax[j], std::fabs(vals[A.src[q]]));
  for (int j = 0; j < n; ++j) {
    if (row_of_col[j] >= 0) continue;
    for (int q = A.cp[j]; q < A.cp[j + 1]; ++q)
      if (A.ri[q] == j) {
        double a = std::fabs(vals[A.src[q]]);
        if (a > 0 && a >= kDiagPref * colmax[j]) { row_of_col[j] = j; col_of_row[j] = j; }
      }
  }
  for (int j = 0; j < n; ++j) {
    if (row_of_col[j] >= 0) continue;
    int best = -1;
    double bv = 0.0;
    for (int q = A.cp[j]; q < A.cp[j + 1]; ++q) {
      int i = A.ri[q];
      double a = std::fabs(vals[A.src[q]]);
      if (col_of_row[i] < 0 && a > bv) { bv = a; best = i; }
    }
    if (best >= 0) { row_of_col[j] = best; col_of_row[best] = j; }
  }
  // Augmenting paths for the unmatched columns (MC21: depth-first search with
  // a look-ahead for a free row at every visited column).  A first pass uses
  // only numerically nonzero entries; structural zeros are a last resort.
  std::vector<int> visited(n, -1), cols, pos, via;
  std::vector<char> looked;
  int stamp = 0;
  for (int j0 = 0; j0 < n; ++j0) {
    if (row_of_col[j0] >= 0) continue;
    int found = -1;
    for (int pass = 0; pass < 2 && found < 0; ++pass) {
      const bool allow_zero = pass == 1;
      ++stamp;
      cols.assign(1, j0);
      pos.assign(1, A.cp[j0]);
      looked.assign(1, 0);
      via.clear();
      while (!cols.empty()) {
        const int L = (int)cols.size() - 1;
        const int j = cols[L];
        if (!looked[L]) {
          looked[L] = 1;
          for (int q = A.cp[j]; q < A.cp[j + 1]; ++q) {
            const int i = A.ri[q];
            if (col_of_row[i] < 0 && (allow_zero || vals[A.src[q]] != 0.0)) { found = i; break; }
          }
          if (found >= 0) break;
        }
        if (pos[L] >= A.cp[j + 1]) {
          cols.pop_back();
          pos.pop_back();
          looked.pop_back();
          if (!via.empty() && via.size() >= cols.size()) via.pop_back();
          continue;
        }
        const int q = pos[L]++;
        const int i = A.ri[q];
        if (visited[i] == stamp || col_of_row[i] < 0) continue;
        if (!allow_zero && vals[A.src[q]] == 0.0) continue;
        visited[i] = stamp;
        via.push_back(i);
        cols.push_back(col_of_row[i]);
        pos.push_back(A.cp[col_of_row[i]]);
        looked.push_back(0);
      }
    }
    if (found < 0) {
      char buf[128];
      snprintf(buf, sizeof buf, "structurally singular matrix: column %d has no matching row", j0);
      err = buf;
      return false;
    }
    const int L = (int)cols.size() - 1;
    row_of_col[cols[L]] = found;
    col_of_row[found] = cols[L];
    for (int k = L - 1; k >= 0; --k) {
      row_of_col[cols[k]] = via[k];
      col_of_row[via[k]] = cols[k];
    }
  }
  return true;
}

// Nested dissection by BFS level-set bisection on the graph adj restricted to
// the nodes with part[v] == id.  Appends an elimination order to out.
struct ND {
  const std::vector<std::vector<int>> &adj;
  std::vector<int> part, dist;
  int next_id = 1;
  std::vector<int> *out;
  static constexpr int kLeaf = 8;
  ND(const std::vector<std::vector<int>> &a, std::vector<int> &o) : adj(a), out(&o) {
    part.assign(a.size(), 0);
    dist.assign(a.size(), -1);
  }

  // BFS inside subset `id` from `src`; returns visit order and fills levels.
  void bfs(int src, int id, std::vector<int> &order, std::vector<int> &lvl_ptr) {
    order.clear();
    lvl_ptr.assign(1, 0);
    order.push_back(src);
    dist[src] = 0;
    size_t head = 0;
    int cur = 0;
    while (head < order.size()) {
      int v = order[head++];
      if (dist[v] != cur) { lvl_ptr.push_back((int)head - 1); cur = dist[v]; }
      for (int w : adj[v])
        if (part[w] == id && dist[w] < 0) { dist[w] = dist[v] + 1; order.push_back(w); }
    }
    lvl_ptr.push_back((int)order.size());
    for (int v : order) dist[v] = -1;
  }

  void run(std::vector<int> nodes, int id) {
    if ((int)nodes.size() <= kLeaf) {
      for (int v : nodes) { out->push_back(v); part[v] = -1; }
      return;
    }
    std::vector<int> order, lvl;
    bfs(nodes[0], id, order, lvl);
    if (order.size() < nodes.size()) {
      // disconnected: split off each component
      std::vector<std::vector<int>> comps;
      for (int v : nodes) {
        if (part[v] != id) continue;
        std::vector<int> o, l;
        bfs(v, id, o, l);
        int cid = next_id++;
        for (int w : o) part[w] = cid;
        comps.push_back(o);
      }
      for (auto &cmp : comps) run(cmp, part[cmp[0]]);
      return;
    }
    // pseudo-peripheral node: two sweeps
    int start = order.back();
    for (int sweep = 0; sweep < 2; ++sweep) {
      bfs(start, id, order, lvl);
      int lo = lvl[lvl.size() - 2];
      int best = order[lo];
      for (int k = lo; k < (int)order.size(); ++k)
        if (adj[order[k]].size() < adj[best].size()) best = order[k];
      start = best;
    }
    bfs(start, id, order, lvl);
    int nl = (int)lvl.size() - 1;
    if (nl < 3) {
      for (int v : nodes) { out->push_back(v); part[v] = -1; }
      return;
    }
    int half = (int)order.size() / 2, m = 1;
    for (int k = 1; k < nl - 1; ++k) {
      m = k;
      if (lvl[k + 1] >= half) break;
    }
    int ida = next_id++, idb = next_id++;
    std::vector<int> A(order.begin(), order.begin() + lvl[m]);
    std::vector<int> S(order.begin() + lvl[m], order.begin() + lvl[m + 1]);
    std::vector<int> B(order.begin() + lvl[m + 1], order.end());
    for (int v : A) part[v] = ida;
    for (int v : B) part[v] = idb;
    for (int v : S) part[v] = -1;
    run(A, ida);
    run(B, idb);
    for (int v : S) out->push_back(v);
  }
};

// Approximate minimum degree ordering of the graph adj restricted to
// `nodes` (the published algorithm of Amestoy, Davis & Duff, SIAM J. Matrix
// Anal. Appl. 17(4), 1996, on the quotient graph; without supervariable
// detection or aggressive absorption).  Appends the elimination order to out.
// loc: scratch of adj.size() entries, all -1 on entry and on return.
void min_degree(const std::vector<std::vector<int>> &adj, const std::vector<int> &nodes, std::vector<int> &out,
                std::vector<int> &loc) {
  const int m = (int)nodes.size();
  if (m == 0) return;
  for (int i = 0; i < m; ++i) loc[nodes[i]] = i;
  std::vector<std::vector<int>> A(m), E(m), Le(m);  // variable adjacency, element adjacency, element lists
  for (int i = 0; i < m; ++i)
    for (int w : adj[nodes[i]])
      if (loc[w] >= 0 && loc[w] != i) A[i].push_back(loc[w]);
  for (int i = 0; i < m; ++i) loc[nodes[i]] = -1;
  std::vector<char> elim(m, 0), dead(m, 0);
  std::vector<int> deg(m), head(m + 1, -1), nxt(m, -1), prv(m, -1);
  auto bucket_add = [&](int i) {
    const int d = deg[i];
    nxt[i] = head[d]; prv[i] = -1;
    if (head[d] >= 0) prv[head[d]] = i;
    head[d] = i;
  };
  auto bucket_del = [&](int i) {
    if (prv[i] >= 0) nxt[prv[i]] = nxt[i]; else head[deg[i]] = nxt[i];
    if (nxt[i] >= 0) prv[nxt[i]] = prv[i];
  };
  for (int i = 0; i < m; ++i) { deg[i] = (int)A[i].size(); bucket_add(i); }
  std::vector<int> mark(m, -1), wmark(m, -1), w(m, 0), Lp;
  int mindeg = 0;
  for (int k = 0; k < m; ++k) {
    while (head[mindeg] < 0) ++mindeg;
    const int p = head[mindeg];
    bucket_del(p);
    elim[p] = 1;
    out.push_back(nodes[p]);
    // new element Lp = (A_p u union of the elements of p) \ {p}; those
    // elements are absorbed into it
    Lp.clear();
    mark[p] = k;
    for (int v : A[p])
      if (!elim[v] && mark[v] != k) { mark[v] = k; Lp.push_back(v); }
    for (int e : E[p]) {
      if (dead[e]) continue;
      for (int v : Le[e])
        if (!elim[v] && mark[v] != k) { mark[v] = k; Lp.push_back(v); }
      dead[e] = 1;
      std::vector<int>().swap(Le[e]);
    }
    std::vector<int>().swap(A[p]);
    std::vector<int>().swap(E[p]);
    Le[p] = Lp;
    const int lp = (int)Lp.size();
    // w(e) = |Le \ Lp| for the live elements next to Lp
    for (int i : Lp)
      for (int e : E[i]) {
        if (dead[e]) continue;
        if (wmark[e] != k) { wmark[e] = k; w[e] = (int)Le[e].size(); }
        --w[e];
      }
    const int remaining = m - k - 1;
    for (int i : Lp) {
      // prune: absorbed elements out of E_i, element p in; variables
      // covered by Lp (and p) out of A_i
      int ne = 0;
      for (int e : E[i])
        if (!dead[e]) E[i][ne++] = e;
      E[i].resize(ne);
      E[i].push_back(p);
      int na = 0;
      for (int v : A[i])
        if (!elim[v] && mark[v] != k) A[i][na++] = v;
      A[i].resize(na);
      // approximate external degree
      long long d = (long long)na + lp - 1;
      for (int e : E[i])
        if (e != p) d += w[e] > 0 ? w[e] : 0;
      d = std::min<long long>(d, (long long)deg[i] + lp - 1);
      d = std::min<long long>(d, remaining > 0 ? remaining - 1 : 0);
      if (d < 0) d = 0;
      bucket_del(i);
      deg[i] = (int)d;
      bucket_add(i);
      if (deg[i] < mindeg) mindeg = deg[i];
    }
    // elements whose variables all lie in Lp are absorbed too
    for (int i : Lp)
      for (int e : E[i])
        if (e != p && !dead[e] && w[e] == 0 && wmark[e] == k) {
          dead[e] = 1;
          std::vector<int>().swap(Le[e]);
        }
  }
}

// Estimated cost of factoring the symmetrized core graph in `order` (core
// nodes only): FMA count sum_k (|col k| - 1)^2 of the symmetric factor and
// the height of its elimination tree (the length of the dependency chain).
struct OrderCost { double fma = 0; int height = 0; };
// pos: scratch of adj.size() entries, all -1 on entry and on return.
OrderCost order_cost(const std::vector<std::vector<int>> &adj, const std::vector<int> &order,
                     std::vector<int> &pos) {
  const int m = (int)order.size();
  for (int k = 0; k < m; ++k) pos[order[k]] = k;
  std::vector<int> parent(m, -1), anc(m, -1), cnt(m, 1), mark(m, -1), h(m, 0);
  for (int k = 0; k < m; ++k)
    for (int u : adj[order[k]]) {
      int r = pos[u];
      if (r < 0 || r >= k) continue;
      while (anc[r] != -1 && anc[r] != k) { const int t = anc[r]; anc[r] = k; r = t; }
      if (anc[r] == -1) { anc[r] = k; parent[r] = k; }
    }
  for (int k = 0; k < m; ++k) {
    mark[k] = k;
    for (int u : adj[order[k]]) {
      int r = pos[u];
      if (r < 0 || r >= k) continue;
      while (r != -1 && mark[r] != k) { cnt[r]++; mark[r] = k; r = parent[r]; }
    }
  }
  for (int k = 0; k < m; ++k) pos[order[k]] = -1;
  OrderCost c;
  for (int k = 0; k < m; ++k) {
    c.fma += (double)(cnt[k] - 1) * (double)(cnt[k] - 1);
    if (parent[k] >= 0) h[parent[k]] = std::max(h[parent[k]], h[k] + 1);
    c.height = std::max(c.height, h[k] + 1);
  }
  return c;
}

// Runs body(0 .. count-1) on up to hardware_concurrency() threads, items
// handed out in order; one thread when the work (`weight`) is small.  Each
// item writes only its own results, so the outcome does not depend on the
// thread count.
void parallel_for(size_t count, long long weight, const std::function<void(size_t)> &body) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min({nt, 32u, (unsigned)count}));
  if (nt == 1 || weight < 20000) {
    for (size_t i = 0; i < count; ++i) body(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (size_t i = next++; i < count; i = next++) body(i);
    });
  for (auto &th : pool) th.join();
}

// Pivot rows of a left-looking LU with threshold partial pivoting
// (Gilbert-Peierls: the numeric factorization KLU runs, with its diagonal
// preference) in the column order col_order, for the columns in scope (whole
// connected components).  preferred[j] is kept while it is within kDiagPref
// of column j's largest candidate.  False when a column has no candidate row.
bool partial_pivot_rows(int n, const Csc &A, const std::vector<double> &vals, const std::vector<int> &col_order,
                        const std::vector<char> &scope, const std::vector<int> &preferred, std::vector<int> &rows) {
  std::vector<int> pinv(n, -1), prow, lp(1, 0), li;
  std::vector<double> lx, x(n, 0.0);
  std::vector<int> rmark(n, -1), smark, touched, topo, stk, spos;
  rows.assign(n, -1);
  int s = 0;
  for (int j : col_order) {
    if (!scope[j]) continue;
    touched.clear();
    topo.clear();
    smark.resize(s + 1, -1);
    auto touch = [&](int r) { if (rmark[r] != s) { rmark[r] = s; touched.push_back(r); } };
    // reach of A(:, j) through the columns of L, in topological order
    for (int q = A.cp[j]; q < A.cp[j + 1]; ++q) {
      const int i = A.ri[q];
      touch(i);
      x[i] = vals[A.src[q]];
      const int k0 = pinv[i];
      if (k0 < 0 || smark[k0] == s) continue;
      smark[k0] = s;
      stk.assign(1, k0);
      spos.assign(1, lp[k0]);
      while (!stk.empty()) {
        const int k = stk.back();
        int &t = spos.back();
        bool pushed = false;
        for (; t < lp[k + 1]; ++t) {
          const int k2 = pinv[li[t]];
          if (k2 >= 0 && smark[k2] != s) {
            smark[k2] = s;
            ++t;
            stk.push_back(k2);
            spos.push_back(lp[k2]);
            pushed = true;
            break;
          }
        }
        if (!pushed) { topo.push_back(k); stk.pop_back(); spos.pop_back(); }
      }
    }
    for (auto it = topo.rbegin(); it != topo.rend(); ++it) {
      const int k = *it;
      const double xk = x[prow[k]];
      if (xk == 0.0) continue;
      for (int t = lp[k]; t < lp[k + 1]; ++t) {
        touch(li[t]);
        x[li[t]] -= lx[t] * xk;
      }
    }
    int best = -1;
    double amax = -1.0;
    for (int r : touched)
      if (pinv[r] < 0 && std::fabs(x[r]) > amax) { amax = std::fabs(x[r]); best = r; }
    if (best < 0) return false;
    const int pr = preferred[j];
    if (pr >= 0 && pinv[pr] < 0 && rmark[pr] == s && std::fabs(x[pr]) >= kDiagPref * amax) best = pr;
    const double piv = x[best];
    for (int r : touched)
      if (pinv[r] < 0 && r != best && x[r] != 0.0) { li.push_back(r); lx.push_back(piv != 0.0 ? x[r] / piv : 0.0); }
    lp.push_back((int)li.size());
    pinv[best] = s;
    prow.push_back(best);
    rows[j] = best;
    for (int r : touched) x[r] = 0.0;
    ++s;
  }
  return true;
}

// The smallest pivot ratio among the columns the trial factorization exempted
// (1 when none): the exemption scale stores it.
double worst_exempt_ratio(const LUHost &H) {
  double w = 1.0;
  for (int p = 0; p < H.n; ++p)
    if (H.exempt[p]) w = std::min(w, H.pscale[p] * kRuntimePivotTol / kExemptSlack);
  return w;
}

}  // namespace

static int analyze_once(int n, const std::vector<int> &rp, const std::vector<int> &ci,
                        const std::vector<double> &vals, LUHost &out, std::string &err, int force_ordering,
                        const std::vector<int> *keep_rows, const std::vector<int> *force_order = nullptr);

// The analysis, repaired where its static pivots fail.  The row matching
// and the symmetric ordering pivot on the (matched) diagonal; elimination
// can cancel such a diagonal (a MOSFET's drain' node: the series conductance
// on the diagonal, gds ~ 0 left after the drain' is eliminated, while the
// next stage's gm sits below it).  The reference's KLU pivots during the
// numeric factorization instead.  So when the trial factorization of the
// analysis finds columns below the pivot threshold, the connected
// components holding them are pivoted once by threshold partial pivoting in
// the analysed order, and analysed again with those rows and that order
// kept (the same elimination, so the same pivots); the repair is taken when
// its worst pivot is better.
int lu_analyze_host(int n, const std::vector<int> &rp, const std::vector<int> &ci,
                    const std::vector<double> &vals, LUHost &out, std::string &err, int force_ordering,
                    const std::vector<int> *keep_rows) {
  int rc = analyze_once(n, rp, ci, vals, out, err, force_ordering, keep_rows);
  if (rc != XG_OK) return rc;
  for (int round = 0; round < 2; ++round) {
    const double worst = worst_exempt_ratio(out);
    if (worst >= 1.0) return XG_OK;
    // connected components of the pattern
    std::vector<int> comp(n);
    std::iota(comp.begin(), comp.end(), 0);
    std::function<int(int)> root = [&](int v) {
      while (comp[v] != v) { comp[v] = comp[comp[v]]; v = comp[v]; }
      return v;
    };
    for (int i = 0; i < n; ++i)
      for (int e = rp[i]; e < rp[i + 1]; ++e) {
        const int a = root(i), b = root(ci[e]);
        if (a != b) comp[a] = b;
      }
    std::vector<char> bad_comp(n, 0), scope(n, 0);
    for (int p = 0; p < n; ++p)
      if (out.exempt[p]) bad_comp[root(out.col_of_step[p])] = 1;
    std::vector<int> cur_row(n), keep2(n);
    for (int p = 0; p < n; ++p) cur_row[out.col_of_step[p]] = out.row_of_step[p];
    for (int j = 0; j < n; ++j)
      scope[j] = bad_comp[root(j)] && !(keep_rows && (*keep_rows)[j] >= 0);
    Csc A = to_csc(n, rp, ci);
    std::vector<int> gp_rows;
    if (!partial_pivot_rows(n, A, vals, out.col_of_step, scope, cur_row, gp_rows)) return XG_OK;
    for (int j = 0; j < n; ++j) keep2[j] = scope[j] ? gp_rows[j] : cur_row[j];
    LUHost rep;
    std::string err2;
    if (analyze_once(n, rp, ci, vals, rep, err2, force_ordering, &keep2, &out.col_of_step) != XG_OK) return XG_OK;
    if (!(worst_exempt_ratio(rep) > worst)) return XG_OK;
    out = std::move(rep);
  }
  return XG_OK;
}

static int analyze_once(int n, const std::vector<int> &rp, const std::vector<int> &ci,
                        const std::vector<double> &vals, LUHost &out, std::string &err, int force_ordering,
                        const std::vector<int> *keep_rows, const std::vector<int> *force_order) {
  out = LUHost();
  out.n = n;
  Csc A = to_csc(n, rp, ci);
  std::vector<int> row_of_col;
  if (!match_rows(n, A, vals, row_of_col, err, keep_rows)) return XG_ERR_SINGULAR;
  std::vector<int> inv(n);  // A row -> M index
  for (int j = 0; j < n; ++j) inv[row_of_col[j]] = j;
  // M = rows permuted: M row j = A row row_of_col[j].  M's columns are A's
  // (A.cp) with rows renumbered; M's rows as CSR, columns ascending.
  const int annz = (int)A.ri.size();
  std::vector<int> mcol_idx(annz), mrow_ptr(n + 1, 0), mrow_idx(annz);
  for (int q = 0; q < annz; ++q) {
    mcol_idx[q] = inv[A.ri[q]];
    mrow_ptr[mcol_idx[q] + 1]++;
  }
  for (int r = 0; r < n; ++r) mrow_ptr[r + 1] += mrow_ptr[r];
  {
    std::vector<int> fill(mrow_ptr.begin(), mrow_ptr.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int q = A.cp[j]; q < A.cp[j + 1]; ++q) mrow_idx[fill[mcol_idx[q]]++] = j;
  }
  // singleton peeling
  std::vector<int> rowcnt(n), colcnt(n);
  std::vector<char> removed(n, 0);
  for (int j = 0; j < n; ++j) { rowcnt[j] = mrow_ptr[j + 1] - mrow_ptr[j]; colcnt[j] = A.cp[j + 1] - A.cp[j]; }
  std::vector<int> front, back;
  std::deque<std::pair<int, int>> q;
  for (int j = 0; j < n; ++j) {
    if (rowcnt[j] == 1) q.push_back({j, 0});
    if (colcnt[j] == 1) q.push_back({j, 1});
  }
  auto remove = [&](int j) {
    removed[j] = 1;
    for (int t = A.cp[j]; t < A.cp[j + 1]; ++t) {
      const int r = mcol_idx[t];
      if (r != j && !removed[r] && --rowcnt[r] == 1) q.push_back({r, 0});
    }
    for (int t = mrow_ptr[j]; t < mrow_ptr[j + 1]; ++t) {
      const int c = mrow_idx[t];
      if (c != j && !removed[c] && --colcnt[c] == 1) q.push_back({c, 1});
    }
  };
  while (!q.empty()) {
    auto [j, kind] = q.front();
    q.pop_front();
    if (removed[j]) continue;
    if (kind == 0 && rowcnt[j] == 1) { front.push_back(j); remove(j); }
    else if (kind == 1 && colcnt[j] == 1) { back.push_back(j); remove(j); }
  }
  // core graph (symmetrized, without the diagonal)
  std::vector<std::vector<int>> adj(n);
  for (int j = 0; j < n; ++j) {
    if (removed[j]) continue;
    for (int t = mrow_ptr[j]; t < mrow_ptr[j + 1]; ++t) {
      const int c = mrow_idx[t];
      if (c != j && !removed[c]) { adj[j].push_back(c); adj[c].push_back(j); }
    }
  }
  std::vector<int> core;
  for (int j = 0; j < n; ++j)
    if (!removed[j]) {
      auto &a = adj[j];
      std::sort(a.begin(), a.end());
      a.erase(std::unique(a.begin(), a.end()), a.end());
      core.push_back(j);
    }
  std::vector<int> order;
  order.reserve(n);
  for (int j : front) order.push_back(j);
  if (!core.empty()) {
    // Per connected component (each circuit of a batch orders exactly as it
    // would alone): nested dissection keeps the dependency chains short
    // (levels run in parallel), minimum degree keeps the fill low; take the
    // one with the smaller estimated refactorization time.  Components are
    // ordered on local graphs (node i = the i-th smallest unknown of the
    // component), in parallel, and concatenated in the order of their
    // smallest unknown.
    std::vector<int> comp_of(n, -1), loc_of(n, -1);
    std::vector<std::vector<int>> comps;
    for (int s0 : core) {
      if (comp_of[s0] >= 0) continue;
      const int c = (int)comps.size();
      comps.emplace_back(1, s0);
      std::vector<int> &comp = comps.back();
      comp_of[s0] = c;
      for (size_t h = 0; h < comp.size(); ++h)
        for (int w : adj[comp[h]])
          if (comp_of[w] < 0) { comp_of[w] = c; comp.push_back(w); }
      std::sort(comp.begin(), comp.end());
      for (size_t i = 0; i < comp.size(); ++i) loc_of[comp[i]] = (int)i;
    }
    struct CompOrder {
      std::vector<int> order;  // global unknowns
      OrderCost cnd, cmd;
      bool md = false;
    };
    std::vector<CompOrder> res(comps.size());
    auto order_one = [&](size_t c) {
      const std::vector<int> &comp = comps[c];
      const int m = (int)comp.size();
      std::vector<std::vector<int>> ladj(m);
      for (int i = 0; i < m; ++i) {
        ladj[i].reserve(adj[comp[i]].size());
        for (int w : adj[comp[i]]) ladj[i].push_back(loc_of[w]);  // stays sorted
      }
      std::vector<int> all(m), ond, omd, scratch(m, -1);
      std::iota(all.begin(), all.end(), 0);
      ND nd(ladj, ond);
      nd.run(all, 0);
      min_degree(ladj, all, omd, scratch);
      CompOrder &r = res[c];
      r.cnd = order_cost(ladj, ond, scratch);
      r.cmd = order_cost(ladj, omd, scratch);
      const double tnd = r.cnd.fma / kOrderFmaRate + r.cnd.height * kOrderLevelTime;
      const double tmd = r.cmd.fma / kOrderFmaRate + r.cmd.height * kOrderLevelTime;
      r.md = force_ordering >= 0 ? force_ordering == 1 : tmd < tnd;
      const std::vector<int> &oc = r.md ? omd : ond;
      r.order.resize(m);
      for (int i = 0; i < m; ++i) r.order[i] = comp[oc[i]];
    };
    parallel_for(comps.size(), (long long)core.size(), order_one);
    int n_md = 0;  // unknowns ordered by minimum degree
    for (size_t c = 0; c < comps.size(); ++c) {
      const CompOrder &r = res[c];
      out.order_fma[0] += r.cnd.fma; out.order_fma[1] += r.cmd.fma;
      out.order_height[0] = std::max(out.order_height[0], r.cnd.height);
      out.order_height[1] = std::max(out.order_height[1], r.cmd.height);
      if (r.md) n_md += (int)r.order.size();
      order.insert(order.end(), r.order.begin(), r.order.end());
    }
    out.ordering = (n_md * 2 > (int)core.size()) ? 1 : 0;  // the ordering of most of the core
  }
  for (auto it = back.rbegin(); it != back.rend(); ++it) order.push_back(*it);
  if (force_order) order = *force_order;  // a repair keeps the order its pivots were chosen in
  if ((int)order.size() != n) {
    err = "ordering lost unknowns";
    return XG_ERR_STATE;
  }
  std::vector<int> qinv(n);
  for (int p = 0; p < n; ++p) qinv[order[p]] = p;
  out.row_of_step.resize(n);
  out.col_of_step.resize(n);
  for (int p = 0; p < n; ++p) {
    out.col_of_step[p] = order[p];
    out.row_of_step[p] = row_of_col[order[p]];
  }
  // Gilbert-Peierls symbolic: pattern of column p = reach of A'(:,p) through
  // L, A' = Q^T M Q (column p of A' = column order[p] of A, rows in step
  // indices); the L part of a finished column k is out.ri[diag[k]+1 ..
  // cp[k+1]).
  out.cp.assign(n + 1, 0);
  out.diag.assign(n, -1);
  std::vector<int> mark(n, -1), stk, pos;
  std::vector<int> colrows;
  for (int p = 0; p < n; ++p) {
    colrows.clear();
    const int j = order[p];
    for (int q2 = A.cp[j]; q2 < A.cp[j + 1]; ++q2) {
      const int r0 = qinv[inv[A.ri[q2]]];
      if (mark[r0] == p) continue;
      stk.assign(1, r0);
      mark[r0] = p;
      while (!stk.empty()) {
        int r = stk.back();
        stk.pop_back();
        colrows.push_back(r);
        if (r < p)
          for (int t = out.diag[r] + 1; t < out.cp[r + 1]; ++t) {
            const int i = out.ri[t];
            if (mark[i] != p) { mark[i] = p; stk.push_back(i); }
          }
      }
    }
    std::sort(colrows.begin(), colrows.end());
    if (!std::binary_search(colrows.begin(), colrows.end(), p)) {
      err = "missing structural diagonal after matching";
      return XG_ERR_SINGULAR;
    }
    out.ri.insert(out.ri.end(), colrows.begin(), colrows.end());
    out.cp[p + 1] = (int)out.ri.size();
    out.diag[p] = out.cp[p] + (int)(std::lower_bound(colrows.begin(), colrows.end(), p) - colrows.begin());
    if ((long long)out.ri.size() > 1900000000LL) {
      err = "LU fill exceeds the int32 index range";
      return XG_ERR_UNSUPPORTED;
    }
  }
  const long long nnz = (long long)out.ri.size();
  // value sources
  out.src.assign(nnz, -1);
  for (int p = 0; p < n; ++p) {
    int j = order[p];
    for (int q2 = A.cp[j]; q2 < A.cp[j + 1]; ++q2) {
      int r = qinv[inv[A.ri[q2]]];
      auto b = out.ri.begin() + out.cp[p], e = out.ri.begin() + out.cp[p + 1];
      auto it = std::lower_bound(b, e, r);
      out.src[it - out.ri.begin()] = A.src[q2];
    }
  }
  // factor levels: column p after every k with U(k,p) != 0
  std::vector<int> flev(n, 0);
  int fmaxl = 0;
  for (int p = 0; p < n; ++p) {
    int l = 0;
    for (int t = out.cp[p]; t < out.diag[p]; ++t) l = std::max(l, flev[out.ri[t]] + 1);
    flev[p] = l;
    fmaxl = std::max(fmaxl, l);
  }
  // row structures for the solves
  std::vector<int> lcnt(n, 0), ucnt(n, 0);
  for (int p = 0; p < n; ++p) {
    for (int t = out.cp[p]; t < out.diag[p]; ++t) ucnt[out.ri[t]]++;      // U(k,p): row k
    for (int t = out.diag[p] + 1; t < out.cp[p + 1]; ++t) lcnt[out.ri[t]]++;  // L(i,p): row i
  }
  out.l_ptr.assign(n + 1, 0);
  out.u_ptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) { out.l_ptr[i + 1] = out.l_ptr[i] + lcnt[i]; out.u_ptr[i + 1] = out.u_ptr[i] + ucnt[i]; }
  out.l_pos.resize(out.l_ptr[n]); out.l_col.resize(out.l_ptr[n]);
  out.u_pos.resize(out.u_ptr[n]); out.u_col.resize(out.u_ptr[n]);
  std::vector<int> lf(out.l_ptr.begin(), out.l_ptr.end() - 1), uf(out.u_ptr.begin(), out.u_ptr.end() - 1);
  for (int p = 0; p < n; ++p) {
    for (int t = out.cp[p]; t < out.diag[p]; ++t) {
      int k = out.ri[t];
      out.u_pos[uf[k]] = t; out.u_col[uf[k]++] = p;
    }
    for (int t = out.diag[p] + 1; t < out.cp[p + 1]; ++t) {
      int i = out.ri[t];
      out.l_pos[lf[i]] = t; out.l_col[lf[i]++] = p;
    }
  }
  std::vector<int> llev(n, 0), ulev(n, 0);
  int lmax = 0, umax = 0;
  for (int i = 0; i < n; ++i) {
    int l = 0;
    for (int t = out.l_ptr[i]; t < out.l_ptr[i + 1]; ++t) l = std::max(l, llev[out.l_col[t]] + 1);
    llev[i] = l;
    lmax = std::max(lmax, l);
  }
  for (int k = n - 1; k >= 0; --k) {
    int l = 0;
    for (int t = out.u_ptr[k]; t < out.u_ptr[k + 1]; ++t) l = std::max(l, ulev[out.u_col[t]] + 1);
    ulev[k] = l;
    umax = std::max(umax, l);
  }
  auto buckets = [&](const std::vector<int> &lev, int maxl, std::vector<int> &ptr, std::vector<int> &items) {
    ptr.assign(maxl + 2, 0);
    for (int v : lev) ptr[v + 1]++;
    for (int l = 0; l <= maxl; ++l) ptr[l + 1] += ptr[l];
    items.resize(lev.size());
    std::vector<int> f(ptr.begin(), ptr.end() - 1);
    for (int v = 0; v < (int)lev.size(); ++v) items[f[lev[v]]++] = v;
  };
  // Update maps: for U entry p = (k, j), upd_off[p] .. upd_off[p+1] lists the
  // positions in column j of the rows of L(:,k), so the device factorization
  // scatters without searching.
  out.upd_off.assign(nnz + 1, 0);
  {
    long long total = 0;
    for (int j = 0; j < n; ++j)
      for (int t = out.cp[j]; t < out.diag[j]; ++t) {
        const int k = out.ri[t];
        total += out.cp[k + 1] - out.diag[k] - 1;
      }
    if (total > 1900000000LL) {
      err = "LU update map exceeds the int32 index range";
      return XG_ERR_UNSUPPORTED;
    }
    out.upd_pos.resize(total);
    long long w = 0;
    for (int j = 0; j < n; ++j) {
      const int p1 = out.cp[j + 1];
      for (int t = out.cp[j]; t < out.cp[j + 1]; ++t) {
        out.upd_off[t] = (int)w;
        if (t >= out.diag[j]) continue;
        const int k = out.ri[t];
        int pos = t + 1;
        for (int q2 = out.diag[k] + 1; q2 < out.cp[k + 1]; ++q2) {
          const int i = out.ri[q2];
          while (pos < p1 && out.ri[pos] < i) ++pos;  // both lists ascend
          if (pos >= p1 || out.ri[pos] != i) {
            err = "symbolic factorization lost a fill entry";
            return XG_ERR_STATE;
          }
          out.upd_pos[w++] = pos;
        }
      }
    }
    out.upd_off[nnz] = (int)w;
  }
  // Host trial factorization with the analysis values: a column whose
  // frozen pivot fails the threshold test even right after re-pivoting is
  // exempt from that test on the device (re-pivoting cannot improve it; a
  // typical case is a structurally present but zero U row, or a block tied
  // to ground only by gmin-sized conductances).  The exemption is bounded:
  // the column is still held to kExemptSlack times the pivot ratio it has
  // here, so that a pivot that collapses on later values (the frozen order
  // gone bad) still triggers re-pivoting.
  out.exempt.assign(n, 0);
  out.pscale.assign(n, 1.0);
  {
    std::vector<double> lu(nnz);
    for (int p = 0; p < n; ++p) {
      const int p0 = out.cp[p], p1 = out.cp[p + 1], pd = out.diag[p];
      for (int t = p0; t < p1; ++t) lu[t] = out.src[t] >= 0 ? vals[out.src[t]] : 0.0;
      for (int t = p0; t < pd; ++t) {
        const int k = out.ri[t];
        const double ukj = lu[t];
        if (ukj == 0.0) continue;
        const int *tgt = out.upd_pos.data() + out.upd_off[t];
        const int q0 = out.diag[k] + 1;
        for (int q2 = q0; q2 < out.cp[k + 1]; ++q2) lu[tgt[q2 - q0]] -= lu[q2] * ukj;
      }
      const double d = lu[pd];
      double amax = 0.0;
      for (int t = pd; t < p1; ++t) amax = std::max(amax, std::fabs(lu[t]));
      if (!(std::fabs(d) >= kRuntimePivotTol * amax)) {
        out.exempt[p] = 1;
        out.pscale[p] = amax > 0.0 ? kExemptSlack * (std::fabs(d) / amax) / kRuntimePivotTol : 0.0;
      }
      if (d != 0.0)
        for (int t = pd + 1; t < p1; ++t) lu[t] /= d;
    }
  }
  // within each solve level, long rows go last: they get a whole block each
  auto split_long = [&](const std::vector<int> &ptr, std::vector<int> &items, const std::vector<int> &rptr,
                        std::vector<int> &nlong) {
    nlong.assign(ptr.size() > 0 ? ptr.size() - 1 : 0, 0);
    for (size_t l = 0; l + 1 < ptr.size(); ++l) {
      auto b = items.begin() + ptr[l], e = items.begin() + ptr[l + 1];
      auto mid = std::stable_partition(b, e, [&](int r) { return rptr[r + 1] - rptr[r] <= kLongSolveRow; });
      nlong[l] = (int)(e - mid);
    }
  };
  if (n > 0) {
    buckets(flev, fmaxl, out.f_lvl_ptr, out.f_cols);
    buckets(llev, lmax, out.l_lvl_ptr, out.l_rows);
    buckets(ulev, umax, out.u_lvl_ptr, out.u_rows);
    split_long(out.l_lvl_ptr, out.l_rows, out.l_ptr, out.l_long);
    split_long(out.u_lvl_ptr, out.u_rows, out.u_ptr, out.u_long);
  }
  // Grouped schedules: factorization (deps = U-part rows of each column) and
  // L solve (deps = L-row columns); the U solve runs the factor schedule backwards.
  // (the two are independent: built on two threads)
  parallel_for(2, (long long)n, [&](size_t w) {
    if (w == 0)
      out.fsched = build_schedule(
          n, [&](int j, std::vector<int> &d) { for (int t = out.cp[j]; t < out.diag[j]; ++t) d.push_back(out.ri[t]); },
          [&](int j) { return (out.cp[j + 1] - out.diag[j] - 1) > kLongColumn || (out.diag[j] - out.cp[j]) > kLongColumn; },
          [&](int j) { return (out.u_ptr[j + 1] - out.u_ptr[j]) > kLongSolveRow; },
          [&](int j) { return out.cp[j + 1] - out.cp[j] + out.u_ptr[j + 1] - out.u_ptr[j]; });
    else
      out.lsched = build_schedule(
          n, [&](int i, std::vector<int> &d) { for (int t = out.l_ptr[i]; t < out.l_ptr[i + 1]; ++t) d.push_back(out.l_col[t]); },
          [&](int i) { return (out.l_ptr[i + 1] - out.l_ptr[i]) > kLongSolveRow; }, nullptr,
          [&](int i) { return out.l_ptr[i + 1] - out.l_ptr[i] + 1; });
  });
  // Single-thread items: short factor columns (entries and update products),
  // short U rows (backward sweep of the factor schedule), short L rows.
  // A thread walks its column's updates one after the other (a load latency
  // each), a warp takes them in one step: single-thread columns pay off when
  // enough groups run at once to hide that latency (a batch of circuits), not
  // for a few large groups (one big circuit).
  const bool thread_columns = out.fsched.n_groups >= 4 * (int)kNumSms;
  out.fsched.is_thread.assign(n, 0);
  out.fsched.is_thread_rev.assign(n, 0);
  out.lsched.is_thread.assign(n, 0);
  out.lsched.is_thread_rev.assign(n, 0);
  for (int j = 0; j < n; ++j) {
    long long work = 0;
    for (int t = out.cp[j]; t < out.diag[j]; ++t) {
      const int k = out.ri[t];
      work += out.cp[k + 1] - out.diag[k] - 1;
    }
    if (thread_columns && !out.fsched.is_long[j] && out.cp[j + 1] - out.cp[j] <= kThreadColumn &&
        work <= kThreadWork)
      out.fsched.is_thread[j] = 1;
    if (!out.fsched.is_long_rev[j] && out.u_ptr[j + 1] - out.u_ptr[j] <= kThreadRow) out.fsched.is_thread_rev[j] = 1;
    if (!out.lsched.is_long[j] && out.l_ptr[j + 1] - out.l_ptr[j] <= kThreadRow) out.lsched.is_thread[j] = 1;
  }
  // CTA size of each group sweep.  The groups are latency-bound chains of
  // levels.  Level l of group g needs need(l) threads (a thread per
  // single-thread item, `team` per other item); a CTA of B threads walks it
  // in ceil(need / B) passes, so group g takes P_g(B) = sum_l ceil(need / B)
  // passes, and 2048 / B CTAs share an SM.  The sweep takes about
  // max(max_g P_g(B), sum_g P_g(B) * B / (SMs * 2048)) pass times: few
  // groups favour wide CTAs, many groups narrow ones.
  auto cta_size = [&](const Schedule &S, const std::vector<char> &thr, int team) {
    double best_cost = -1;
    int best = 512;
    for (int B = 64; B <= 512; B *= 2) {
      double total = 0, longest = 0;
      for (int g = 0; g < S.n_groups; ++g) {
        double passes = 0;
        for (int lv = S.grp_lvl[g]; lv < S.grp_lvl[g + 1]; ++lv) {
          long long need = 0;
          for (int t = S.lvl_ptr[lv]; t < S.lvl_ptr[lv + 1]; ++t) need += thr[S.items[t]] ? 1 : team;
          passes += (double)((need + B - 1) / B);
        }
        total += passes;
        longest = std::max(longest, passes);
      }
      const double cost = std::max(longest, total * B / (kNumSms * 2048.0));
      if (best_cost < 0 || cost < best_cost) { best_cost = cost; best = B; }
    }
    return best;
  };
  out.fs_threads = cta_size(out.fsched, out.fsched.is_thread, 32);
  out.ls_threads = cta_size(out.lsched, out.lsched.is_thread, 8);
  out.us_threads = cta_size(out.fsched, out.fsched.is_thread_rev, 8);
  // Solve groups staged in shared memory: per schedule position the row's
  // entries with the buffer slot of each entry's column (the L solve reads
  // L(i, k) y(k) for k in row i's L part, the U solve U(k, j) y(j)).
  auto stage_solve = [&](const Schedule &S, const std::vector<int> &ptr, const std::vector<int> &epos_src,
                         const std::vector<int> &ecol_src, int extra_per_row, std::vector<int> &eptr,
                         std::vector<int> &epos, std::vector<int> &esrc, std::vector<int> &gbytes) {
    const int ni = (int)S.items.size();
    std::vector<int> slot(n, -1), owner(n, -1);
    gbytes.assign(S.n_groups, 0);
    eptr.assign(ni + 1, 0);
    epos.clear();
    esrc.clear();
    for (int g = 0; g < S.n_groups; ++g) {
      const int it0 = S.lvl_ptr[S.grp_lvl[g]], it1 = S.lvl_ptr[S.grp_lvl[g + 1]];
      for (int t = it0; t < it1; ++t) { slot[S.items[t]] = t - it0; owner[S.items[t]] = g; }
    }
    for (int t = 0; t < ni; ++t) {
      const int i = S.items[t];
      eptr[t] = (int)epos.size();
      for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
        const int k = ecol_src[q];
        epos.push_back(epos_src[q]);
        esrc.push_back(owner[k] >= 0 && owner[k] == owner[i] ? slot[k] : -(k + 1));
      }
    }
    eptr[ni] = (int)epos.size();
    for (int g = 0; g < S.n_groups; ++g) {
      const int it0 = S.lvl_ptr[S.grp_lvl[g]], it1 = S.lvl_ptr[S.grp_lvl[g + 1]];
      const long long rows = it1 - it0, ents = eptr[it1] - eptr[it0];
      bool ok = true;
      for (int t = it0; t < it1 && ok; ++t) ok = eptr[t + 1] - eptr[t] <= kStageRow;
      // doubles: y (+ the diagonal for the U solve), entry values and the
      // y of each entry's column outside the group; ints: entry slots, the
      // row entry offsets and the rows' activity flags
      const long long bytes = 8 * (rows * (1 + extra_per_row) + 2 * ents) + 4 * (ents + rows + 1) + 4 * rows;
      if (ok && bytes <= kSolveSmemBytes) gbytes[g] = (int)((bytes + 15) / 16 * 16);
    }
  };
  stage_solve(out.lsched, out.l_ptr, out.l_pos, out.l_col, 0, out.ls_eptr, out.ls_epos, out.ls_esrc,
              out.ls_gbytes);
  stage_solve(out.fsched, out.u_ptr, out.u_pos, out.u_col, 1, out.us_eptr, out.us_epos, out.us_esrc,
              out.us_gbytes);
  // Shared-memory buffers of the factor groups (not the hubs, not the top).
  {
    const Schedule &S = out.fsched;
    out.grp_soff.assign(n, -1);
    out.grp_snz.assign(S.n_groups, 0);
    for (int g = 0; g < S.n_groups; ++g) {
      int off = 0;
      for (int q = S.lvl_ptr[S.grp_lvl[g]]; q < S.lvl_ptr[S.grp_lvl[g + 1]]; ++q) {
        const int j = S.items[q];
        out.grp_soff[j] = off;
        off += out.cp[j + 1] - out.cp[j];
      }
      out.grp_snz[g] = off;
    }
  }
  // Per U entry metadata of the update it drives (after grp_soff).
  out.umeta.assign((size_t)4 * nnz, 0);
  for (int j = 0; j < n; ++j)
    for (int p = out.cp[j]; p < out.diag[j]; ++p) {
      const int k = out.ri[p];
      int *u = &out.umeta[(size_t)4 * p];
      u[0] = (out.grp_soff[j] >= 0 && out.grp_soff[k] >= 0) ? out.grp_soff[k] + (out.diag[k] + 1 - out.cp[k]) : -1;
      u[1] = out.cp[k + 1] - out.diag[k] - 1;
      u[2] = out.upd_off[p];
      u[3] = out.diag[k] + 1;
    }
  // Update metadata of the factor groups staged in shared memory.  Sizes
  // first (per group: column records, U entries, update targets); the
  // arrays are built only when some group stages them.
  {
    const Schedule &S = out.fsched;
    const int ni = (int)S.items.size();
    out.fm_gbytes.assign(S.n_groups, 0);
    std::vector<int> owner(n, -1);
    for (int g = 0; g < S.n_groups; ++g)
      for (int t = S.lvl_ptr[S.grp_lvl[g]]; t < S.lvl_ptr[S.grp_lvl[g + 1]]; ++t) owner[S.items[t]] = g;
    for (int g = 0; g < S.n_groups; ++g) {
      const int it0 = S.lvl_ptr[S.grp_lvl[g]], it1 = S.lvl_ptr[S.grp_lvl[g + 1]];
      bool ok = true;
      long long ents = 0, tg = 0;
      for (int t = it0; t < it1 && ok; ++t) {
        const int j = S.items[t];
        ok = !S.is_long[j];
        ents += out.diag[j] - out.cp[j];
        for (int p = out.cp[j]; p < out.diag[j]; ++p) {
          const int k = out.ri[p];
          tg += out.cp[k + 1] - out.diag[k] - 1;
        }
      }
      const long long rows = it1 - it0;
      const long long meta = 16 * rows + 4 * (rows + 1) + 16 * ents + 4 * tg;
      const long long vals = ((long long)out.grp_snz[g] * 8 + 15) / 16 * 16;
      if (ok && vals + meta <= kGroupSmemBytes) out.fm_gbytes[g] = (int)((meta + 15) / 16 * 16);
    }
    // The metadata shortens each level's latency chain, but a larger buffer
    // lets fewer CTAs share an SM: the closed-form choice stages it only when
    // the launch buffer with it allows as many resident CTAs as the values
    // alone (the launch-shape tuner may choose otherwise by timing).
    long long vmax = 0, mmax = 0;
    for (int g = 0; g < S.n_groups; ++g) {
      const long long vb = ((long long)out.grp_snz[g] * 8 + 15) / 16 * 16;
      if (vb <= kGroupSmemBytes) vmax = std::max(vmax, vb);
      mmax = std::max(mmax, out.fm_gbytes[g] ? vb + out.fm_gbytes[g] : vb);
    }
    auto resident = [&](long long bytes) {
      const long long by_threads = 2048 / std::max(1, out.fs_threads);
      return bytes > 0 ? std::min(by_threads, (long long)kSmemPerSm / bytes) : by_threads;
    };
    out.fm_model_on = resident(mmax) >= resident(vmax);
    bool any = false;
    for (int b2 : out.fm_gbytes) any = any || b2 > 0;
    out.fm_col.clear();
    out.fm_eptr.clear();
    out.fm_ent.clear();
    out.fm_tgt.clear();
    out.fm_tptr.clear();
    if (any) {
      out.fm_col.assign((size_t)4 * ni, 0);
      out.fm_eptr.assign(ni + 1, 0);
      out.fm_tptr.assign(S.n_groups + 1, 0);
      int t_group_lo = 0;
      for (int t = 0; t < ni; ++t) {
        const int j = S.items[t];
        const int g = owner[j];
        out.fm_eptr[t] = (int)out.fm_ent.size() / 4;
        if (g < 0) continue;
        if (t == S.lvl_ptr[S.grp_lvl[g]]) {
          out.fm_tptr[g] = (int)out.fm_tgt.size();
          t_group_lo = (int)out.fm_tgt.size();
        }
        int *c = &out.fm_col[(size_t)4 * t];
        c[0] = out.grp_soff[j];
        c[1] = out.cp[j + 1] - out.cp[j];
        c[2] = out.diag[j] - out.cp[j];
        c[3] = (out.u_ptr[j + 1] > out.u_ptr[j]) ? (out.exempt[j] ? 2 : 1) : 0;
        for (int p = out.cp[j]; p < out.diag[j]; ++p) {
          const int k = out.ri[p];
          const int nl = out.cp[k + 1] - out.diag[k] - 1;
          out.fm_ent.push_back(owner[k] == g ? out.grp_soff[k] + (out.diag[k] + 1 - out.cp[k])
                                             : -(out.diag[k] + 1) - 1);
          out.fm_ent.push_back(nl);
          out.fm_ent.push_back((int)out.fm_tgt.size() - t_group_lo);
          out.fm_ent.push_back(p - out.cp[j]);
          for (int q = 0; q < nl; ++q) out.fm_tgt.push_back(out.upd_pos[out.upd_off[p] + q] - out.cp[j]);
        }
      }
      out.fm_eptr[ni] = (int)out.fm_ent.size() / 4;
      out.fm_tptr[S.n_groups] = (int)out.fm_tgt.size();
    }
  }
  // Can the factor schedule's top run right-looking?  The sub-tree (non-top)
  // rows k of a top column j are pulled first, in step order; that is exact
  // when no top column m < k updates such a row, i.e. when every non-top L
  // row r of a top column has no U entry in a top column.  (Typical non-top
  // L rows of the top: the branch unknowns of voltage sources peeled to the
  // end of the order, whose U rows are empty.)
  {
    const Schedule &S = out.fsched;
    out.top_items.clear();
    if (S.n_top_items >= kTopRightLooking) {
      const int first = S.lvl_ptr[S.grp_lvl[S.n_groups]];
      std::vector<char> is_top(n, 0);
      for (int q = first; q < (int)S.items.size(); ++q) is_top[S.items[q]] = 1;
      bool ok = true;
      std::vector<char> checked(n, 0);
      for (int m = 0; m < n && ok; ++m) {
        if (!is_top[m]) continue;
        for (int p = out.diag[m] + 1; p < out.cp[m + 1] && ok; ++p) {
          const int r = out.ri[p];
          if (is_top[r] || checked[r]) continue;
          checked[r] = 1;
          for (int t = out.u_ptr[r]; t < out.u_ptr[r + 1]; ++t)
            if (is_top[out.u_col[t]]) { ok = false; break; }
        }
      }
      if (ok) {
        for (int m = 0; m < n; ++m)
          if (is_top[m]) out.top_items.push_back(m);
        // right-looking levels: column k pivots after every top k' with
        // U(k', k) != 0 (its updates) and every top k' with L(k, k') != 0 (an
        // update of k' writes row k, which k reads as U(k, j))
        std::vector<int> lev(n, 0);
        int nlev = 0;
        for (int k : out.top_items) {
          int l = 0;
          for (int p = out.cp[k]; p < out.diag[k]; ++p)
            if (is_top[out.ri[p]]) l = std::max(l, lev[out.ri[p]] + 1);
          for (int t = out.l_ptr[k]; t < out.l_ptr[k + 1]; ++t)
            if (is_top[out.l_col[t]]) l = std::max(l, lev[out.l_col[t]] + 1);
          lev[k] = l;
          nlev = std::max(nlev, l + 1);
        }
        std::vector<std::vector<int>> at(nlev);
        for (int k : out.top_items) at[lev[k]].push_back(k);
        out.tlv_items.clear();
        out.tlv_item_ptr.assign(1, 0);
        out.tlv_grp_ptr.assign(1, 0);
        out.tgrp_col.clear();
        out.tgrp_ptr.assign(1, 0);
        out.tgrp_pos.clear();
        out.tgrp_k.clear();
        std::map<int, std::vector<std::pair<int, int>>> by_col;  // j -> (k, position of U(k, j))
        for (int l = 0; l < nlev; ++l) {
          by_col.clear();
          for (int k : at[l]) {
            out.tlv_items.push_back(k);
            for (int t = out.u_ptr[k]; t < out.u_ptr[k + 1]; ++t) by_col[out.u_col[t]].push_back({k, out.u_pos[t]});
          }
          out.tlv_item_ptr.push_back((int)out.tlv_items.size());
          for (auto &kv : by_col) {
            out.tgrp_col.push_back(kv.first);
            for (auto &e : kv.second) { out.tgrp_k.push_back(e.first); out.tgrp_pos.push_back(e.second); }
            out.tgrp_ptr.push_back((int)out.tgrp_pos.size());
          }
          out.tlv_grp_ptr.push_back((int)out.tgrp_col.size());
        }
        // One launch pair per level on all SMs, or the whole top in one CTA
        // (a barrier pair per column)?  Long chains of thin levels (minimum
        // degree orderings) favour the single CTA.
        double t_multi = 0, t_single = 0;
        for (int l = 0; l < nlev; ++l) {
          double work = 0;
          for (int t = out.tlv_item_ptr[l]; t < out.tlv_item_ptr[l + 1]; ++t) {
            const int k = out.tlv_items[t];
            work += (double)(out.cp[k + 1] - out.diag[k] - 1) * (double)(out.u_ptr[k + 1] - out.u_ptr[k]);
          }
          const int items = out.tlv_item_ptr[l + 1] - out.tlv_item_ptr[l];
          t_multi += 2 * kLaunchTime + work / (kSmFmaRate * kNumSms);
          t_single += items * 2 * kBarrierTime + work / kSmFmaRate;
        }
        out.top_multi = t_multi < t_single;
      }
    }
  }
  // The same choice for the tops of the two solves (a launch per level, or
  // one CTA with a barrier per level).
  {
    auto solve_multi = [&](const Schedule &S, const std::vector<int> &ptr) {
      const int lo = S.grp_lvl[S.n_groups], hi = S.grp_lvl[S.n_groups + 1];
      double t_multi = 0, t_single = 0;
      for (int lv = lo; lv < hi; ++lv) {
        double work = 0;
        for (int t = S.lvl_ptr[lv]; t < S.lvl_ptr[lv + 1]; ++t) {
          const int i = S.items[t];
          work += ptr[i + 1] - ptr[i];
        }
        t_multi += kLaunchTime + work / (kSmFmaRate * kNumSms);
        t_single += kBarrierTime + work / kSmFmaRate;
      }
      return t_multi < t_single;
    };
    out.solve_top_multi = out.fsched.n_top_items >= kTopRightLooking &&
                          (solve_multi(out.lsched, out.l_ptr) || solve_multi(out.fsched, out.u_ptr));
  }
  return XG_OK;
}

// Dependency-closed groups for one CTA each, a prologue of "hub" items (no
// dependencies, many dependents) and a single-CTA top for the rest.
Schedule build_schedule(int n, const std::function<void(int, std::vector<int> &)> &deps_of,
                        const std::function<bool(int)> &is_long,
                        const std::function<bool(int)> &is_long_rev,
                        const std::function<int(int)> &weight) {
  Schedule S;
  if (n == 0) {
    S.grp_lvl.assign(2, 0);
    S.lvl_ptr.assign(1, 0);
    return S;
  }
  std::vector<int> dptr(n + 1, 0), didx;
  std::vector<int> tmp;
  for (int j = 0; j < n; ++j) {
    tmp.clear();
    deps_of(j, tmp);
    didx.insert(didx.end(), tmp.begin(), tmp.end());
    dptr[j + 1] = (int)didx.size();
  }
  std::vector<int> outdeg(n, 0);
  for (int k : didx) outdeg[k]++;
  std::vector<char> hub(n, 0), top(n, 0);
  for (int j = 0; j < n; ++j)
    if (dptr[j + 1] == dptr[j] && outdeg[j] > kHubFanout) hub[j] = 1;
  std::vector<int> parent(n), gsize(n, 1);
  std::iota(parent.begin(), parent.end(), 0);
  std::function<int(int)> find = [&](int v) {
    while (parent[v] != v) { parent[v] = parent[parent[v]]; v = parent[v]; }
    return v;
  };
  std::vector<int> roots;
  for (int j = 0; j < n; ++j) {
    if (hub[j]) continue;
    roots.clear();
    bool to_top = false;
    for (int t = dptr[j]; t < dptr[j + 1]; ++t) {
      const int k = didx[t];
      if (hub[k]) continue;
      if (top[k]) { to_top = true; break; }
      roots.push_back(find(k));
    }
    if (!to_top) {
      std::sort(roots.begin(), roots.end());
      roots.erase(std::unique(roots.begin(), roots.end()), roots.end());
      long long total = 1;
      for (int r : roots) total += gsize[r];
      if (total > kGroupCap) to_top = true;
      else
        for (int r : roots) { parent[r] = j; gsize[j] += gsize[r]; }
    }
    if (to_top) top[j] = 1;
  }
  // levels: group-local for grouped items, top-local for the top
  std::vector<int> lev(n, 0);
  for (int j = 0; j < n; ++j) {
    if (hub[j]) continue;
    int l = 0;
    for (int t = dptr[j]; t < dptr[j + 1]; ++t) {
      const int k = didx[t];
      if (hub[k]) continue;
      if (top[j] && !top[k]) continue;  // groups finish before the top starts
      l = std::max(l, lev[k] + 1);
    }
    lev[j] = l;
  }
  // group ids in order of first appearance; the top is the last group
  std::vector<int> gid(n, -1);
  int ng = 0;
  for (int j = 0; j < n; ++j) {
    if (hub[j] || top[j]) continue;
    const int r = find(j);
    if (gid[r] < 0) gid[r] = ng++;
    gid[j] = gid[r];
  }
  // Groups are independent of one another, so their order is free: the
  // larger groups first, by decreasing work (the longest CTAs start first,
  // the launch's tail is short), then the tiny groups (e.g. the isolated
  // supply-node and branch columns of every circuit of a batch), packed
  // into shared CTAs up to a size and work cap — their local levels merge.
  // Packed groups may mix circuits; the kernels test each item's circuit.
  {
    std::vector<int> gsz(ng, 0);
    std::vector<long long> gw(ng, 0);
    for (int j = 0; j < n; ++j)
      if (gid[j] >= 0) { gsz[gid[j]]++; gw[gid[j]] += weight(j); }
    std::vector<int> gorder(ng);
    std::iota(gorder.begin(), gorder.end(), 0);
    std::stable_sort(gorder.begin(), gorder.end(), [&](int a, int b) {
      const bool sa = gsz[a] <= kPackSmall, sb = gsz[b] <= kPackSmall;
      if (sa != sb) return sb;  // tiny groups last
      return !sa && gw[a] > gw[b];
    });
    std::vector<int> pack(ng);
    int np = 0, cur_size = 0;
    long long cur_w = 0;
    bool cur_small = false;
    for (int g : gorder) {
      const bool small = gsz[g] <= kPackSmall && gw[g] <= kPackCapWeight;
      if (small && cur_small && cur_size + gsz[g] <= kPackCap && cur_w + gw[g] <= kPackCapWeight) {
        pack[g] = np - 1;
        cur_size += gsz[g];
        cur_w += gw[g];
      } else {
        pack[g] = np++;
        cur_size = gsz[g];
        cur_w = gw[g];
        cur_small = small;
      }
    }
    for (int j = 0; j < n; ++j)
      if (gid[j] >= 0) gid[j] = pack[gid[j]];
    ng = np;
  }
  for (int j = 0; j < n; ++j)
    if (top[j]) gid[j] = ng;
  S.n_groups = ng;
  std::vector<int> order;
  for (int j = 0; j < n; ++j)
    if (hub[j]) S.items.push_back(j);
  S.n_hub = (int)S.items.size();
  for (int j = 0; j < n; ++j)
    if (!hub[j]) order.push_back(j);
  // stable sort by (group, level): counting sort by level, then by group
  {
    int maxlev = 0;
    for (int j : order) maxlev = std::max(maxlev, lev[j]);
    auto counting = [&](const std::vector<int> &key, int nkeys) {
      std::vector<int> start(nkeys + 1, 0), sorted(order.size());
      for (int j : order) start[key[j] + 1]++;
      for (int k = 0; k < nkeys; ++k) start[k + 1] += start[k];
      for (int j : order) sorted[start[key[j]]++] = j;
      order.swap(sorted);
    };
    counting(lev, maxlev + 1);
    counting(gid, ng + 1);  // the top carries gid ng
  }
  S.lvl_ptr.push_back(S.n_hub);
  S.grp_lvl.assign(ng + 2, 0);
  int cur_g = -1, cur_l = -1;
  int nlv = 0;
  for (size_t q = 0; q < order.size(); ++q) {
    const int j = order[q];
    if (gid[j] != cur_g || lev[j] != cur_l) {
      if (q > 0) { S.lvl_ptr.push_back(S.n_hub + (int)q); nlv++; }
      while (cur_g < gid[j]) { cur_g++; S.grp_lvl[cur_g] = nlv; }
      cur_l = lev[j];
    }
    S.items.push_back(j);
  }
  if (!order.empty()) { S.lvl_ptr.push_back(S.n_hub + (int)order.size()); nlv++; }
  while (cur_g < ng + 1) { cur_g++; S.grp_lvl[cur_g] = nlv; }
  // long items are processed by the whole block, the others by warps
  S.is_long.assign(n, 0);
  S.is_long_rev.assign(n, 0);
  for (int j = 0; j < n; ++j) {
    S.is_long[j] = is_long(j) ? 1 : 0;
    if (is_long_rev) S.is_long_rev[j] = is_long_rev(j) ? 1 : 0;
  }
  S.n_top_items = 0;
  for (int j = 0; j < n; ++j) S.n_top_items += top[j];
  return S;
}

}  // namespace xg
