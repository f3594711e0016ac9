// Host-only probe of the LU analysis (lu_analyze_host, xyce_gb300/csrc/xg_symbolic.cpp)
// for the CPU tests: no GPU, no CUDA runtime calls.
//
// Input (binary, little-endian): int32 n, int32 nnz, int32 row_ptr[n+1],
// int32 col_idx[nnz], float64 vals_a[nnz], float64 vals_b[nnz].
// The analysis runs on vals_a; both value sets are then factored in the
// analysed (frozen) order exactly as the device factorization does
// (left-looking, the analysis' update maps), and the probe prints one line:
//   rc exempt min_ratio_a min_ratio_b recon_err_a factor_sched_ok lsolve_sched_ok
//   factor_hubs factor_top_items
// min_ratio_x: the smallest |pivot| / max|updated column| over the columns
// whose U row has entries right of the diagonal (the device's threshold
// test); recon_err_a: max |(L U)(i,j) - A'(i,j)| / max|A| over the
// permuted matrix A'(i, j) = A(row_of_step[i], col_of_step[j]);
// *_sched_ok: every step appears once in the schedule, hubs have no
// dependencies, an item of a group depends only on hubs and on earlier
// levels of its own group, and an item of the top only on hubs, groups and
// earlier levels of the top (factor: U(:, p); L solve: L(p, :)).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../xyce_gb300/csrc/xg_internal.h"

using namespace xg;

static bool schedule_ok(const Schedule &S, int n, const std::vector<std::vector<int>> &deps) {
  std::vector<int> grp(n, -2), lvl(n, -1);
  for (int t = 0; t < S.n_hub; ++t) {
    const int j = S.items[t];
    if (j < 0 || j >= n || grp[j] != -2) return false;
    grp[j] = -1;
  }
  for (int g = 0; g <= S.n_groups; ++g)  // g == n_groups: the top
    for (int lv = S.grp_lvl[g]; lv < S.grp_lvl[g + 1]; ++lv)
      for (int t = S.lvl_ptr[lv]; t < S.lvl_ptr[lv + 1]; ++t) {
        const int j = S.items[t];
        if (j < 0 || j >= n || grp[j] != -2) return false;
        grp[j] = g;
        lvl[j] = lv;
      }
  for (int j = 0; j < n; ++j) {
    if (grp[j] == -2) return false;
    if (grp[j] == -1 && !deps[j].empty()) return false;
    for (int k : deps[j]) {
      if (grp[k] == -1) continue;
      if (grp[j] == S.n_groups) {
        if (grp[k] == S.n_groups && lvl[k] >= lvl[j]) return false;
      } else if (grp[k] != grp[j] || lvl[k] >= lvl[j]) {
        return false;
      }
    }
  }
  return true;
}

static void factor(const LUHost &H, const std::vector<double> &vals, std::vector<double> &lu, double &min_ratio) {
  const int n = H.n;
  lu.assign(H.ri.size(), 0.0);
  min_ratio = 1.0;
  for (int p = 0; p < n; ++p) {
    const int p0 = H.cp[p], p1 = H.cp[p + 1], pd = H.diag[p];
    for (int t = p0; t < p1; ++t) lu[t] = H.src[t] >= 0 ? vals[H.src[t]] : 0.0;
    for (int t = p0; t < pd; ++t) {
      const int k = H.ri[t];
      const double ukj = lu[t];
      if (ukj == 0.0) continue;
      const int *tgt = H.upd_pos.data() + H.upd_off[t];
      const int q0 = H.diag[k] + 1;
      for (int q2 = q0; q2 < H.cp[k + 1]; ++q2) lu[tgt[q2 - q0]] -= lu[q2] * ukj;
    }
    const double d = lu[pd];
    double amax = 0.0;
    for (int t = pd; t < p1; ++t) amax = std::max(amax, std::fabs(lu[t]));
    if (H.u_ptr[p + 1] > H.u_ptr[p]) min_ratio = std::min(min_ratio, amax > 0.0 ? std::fabs(d) / amax : 0.0);
    if (d != 0.0)
      for (int t = pd + 1; t < p1; ++t) lu[t] /= d;
  }
}

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int n = 0, nnz = 0;
  bool ok = std::fread(&n, 4, 1, f) == 1 && std::fread(&nnz, 4, 1, f) == 1 && n > 0 && nnz > 0;
  std::vector<int> rp(ok ? n + 1 : 0), ci(ok ? nnz : 0);
  std::vector<double> va(ok ? nnz : 0), vb(ok ? nnz : 0);
  ok = ok && std::fread(rp.data(), 4, n + 1, f) == (size_t)(n + 1) && std::fread(ci.data(), 4, nnz, f) == (size_t)nnz &&
       std::fread(va.data(), 8, nnz, f) == (size_t)nnz && std::fread(vb.data(), 8, nnz, f) == (size_t)nnz;
  std::fclose(f);
  if (!ok) return 2;
  LUHost H;
  std::string err;
  const int rc = lu_analyze_host(n, rp, ci, va, H, err);
  if (rc != XG_OK) {
    std::printf("%d 0 0 0 0 0 0 0 0\n", rc);
    return 0;
  }
  int exempt = 0;
  for (int p = 0; p < n; ++p) exempt += H.exempt[p] ? 1 : 0;
  std::vector<double> lu;
  double ra = 0.0, rb = 0.0;
  factor(H, vb, lu, rb);
  factor(H, va, lu, ra);
  // reconstruction of A' from the factors of vals_a (dense; the tests keep n small)
  std::vector<int> step_of_row(n), step_of_col(n);
  for (int p = 0; p < n; ++p) { step_of_row[H.row_of_step[p]] = p; step_of_col[H.col_of_step[p]] = p; }
  std::vector<double> A(size_t(n) * n, 0.0), LU(size_t(n) * n, 0.0), Ld(size_t(n) * n, 0.0), Ud(size_t(n) * n, 0.0);
  double amax = 0.0;
  for (int r = 0; r < n; ++r)
    for (int e = rp[r]; e < rp[r + 1]; ++e) {
      A[size_t(step_of_row[r]) * n + step_of_col[ci[e]]] += va[e];
      amax = std::max(amax, std::fabs(va[e]));
    }
  for (int p = 0; p < n; ++p) {
    Ld[size_t(p) * n + p] = 1.0;
    for (int t = H.cp[p]; t < H.cp[p + 1]; ++t) {
      const int i = H.ri[t];
      if (t <= H.diag[p]) Ud[size_t(i) * n + p] = lu[t];
      else Ld[size_t(i) * n + p] = lu[t];
    }
  }
  double rerr = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k <= std::min(i, j); ++k) s += Ld[size_t(i) * n + k] * Ud[size_t(k) * n + j];
      rerr = std::max(rerr, std::fabs(s - A[size_t(i) * n + j]));
    }
  std::vector<std::vector<int>> fdeps(n), ldeps(n);
  for (int p = 0; p < n; ++p) {
    for (int t = H.cp[p]; t < H.diag[p]; ++t) fdeps[p].push_back(H.ri[t]);
    for (int t = H.l_ptr[p]; t < H.l_ptr[p + 1]; ++t) ldeps[p].push_back(H.l_col[t]);
  }
  const bool fok = schedule_ok(H.fsched, n, fdeps), lok = schedule_ok(H.lsched, n, ldeps);
  const Schedule &F = H.fsched;
  const int top_items = F.lvl_ptr[F.grp_lvl[F.n_groups + 1]] - F.lvl_ptr[F.grp_lvl[F.n_groups]];
  std::printf("%d %d %.17g %.17g %.17g %d %d %d %d\n", rc, exempt, ra, rb, amax > 0.0 ? rerr / amax : 0.0,
              fok ? 1 : 0, lok ? 1 : 0, F.n_hub, top_items);
  return 0;
}
