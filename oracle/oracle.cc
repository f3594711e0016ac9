// oracle.cc — CPU FP64 restatement of Xyce's transient Newton hot path.
//
// TEST INFRASTRUCTURE ONLY: the checker and the timed CPU baseline for the
// GPU library in xyce_gb300/.  Nothing in the product links or calls this.
// Every function names the reference code it restates (paths within the
// Xyce tree).
#include "oracle.h"
#include "devices.h"
#include "bsim4.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <vector>

using namespace orc;

namespace {

struct Wave {
  int kind = ORC_WAVE_DC;
  std::vector<double> d;
};

// SinData::updateSource (N_DEV_SourceData.C:475-497), PulseData::updateSource
// (:1168-1256, bpTol = 0 here), PWLinData::updateSource (:1770-1895, no REPEAT).
double wave_value(const Wave &w, double t) {
  const std::vector<double> &d = w.d;
  switch (w.kind) {
    case ORC_WAVE_DC: return d[0];
    case ORC_WAVE_SIN: {
      double V0 = d[0], VA = d[1], FREQ = d[2], TD = d[3], THETA = d[4], PHASE = d[5];
      double time = t - TD;
      if (time <= 0) return V0 + VA * std::sin(2.0 * M_PI * (PHASE / 360));
      return V0 + VA * std::sin(2.0 * M_PI * (FREQ * time + PHASE / 360)) * std::exp(-(time * THETA));
    }
    case ORC_WAVE_PULSE: {
      double V1 = d[0], V2 = d[1], TD = d[2], TR = d[3], TF = d[4], PW = d[5], PER = d[6];
      double time = t - TD;
      if (time > PER && PER != 0.0) time -= PER * std::floor(time / PER);
      if (time <= 0 || time > TR + PW + TF) return V1;
      if (time > TR && time < TR + PW) return V2;
      if (time > 0 && time <= TR) return (TR != 0.0) ? V1 + (V2 - V1) * time / TR : V1;
      if (time >= TR + PW && time <= TR + PW + TF)
        return (TF != 0.0) ? V2 + (V1 - V2) * (time - (TR + PW)) / TF : V2;
      return V2;
    }
    case ORC_WAVE_PWL: {
      int npts = (int)d.size() / 2;
      double time = t;
      if (time < 0) return 0.0;
      double t1, t2, v1, v2;
      if (time <= d[2 * (npts - 1)]) {
        int loc = npts - 1;
        for (int i = 0; i < npts; ++i)
          if (time < d[2 * i]) { loc = i; break; }
        if (loc == 0) { t1 = 0.0; v1 = 0.0; }
        else { t1 = d[2 * (loc - 1)]; v1 = d[2 * (loc - 1) + 1]; }
        t2 = d[2 * loc]; v2 = d[2 * loc + 1];
      } else {
        t1 = 0.0; t2 = 1.0; v1 = v2 = d[2 * (npts - 1) + 1];
      }
      if (t1 == t2) return v2;
      double length = t2 - t1;
      return (t2 - time) * v1 / length + (-t1 + time) * v2 / length;
    }
  }
  return 0.0;
}

// Breakpoints: PulseData::getBreakPoints (N_DEV_SourceData.C:1442) and
// PWLinData::getBreakPoints (:2044); SIN contributes none.
void wave_breakpoints(const Wave &w, double tstop, std::vector<double> &bp) {
  const std::vector<double> &d = w.d;
  if (w.kind == ORC_WAVE_PWL) {
    for (size_t i = 0; i + 1 < d.size(); i += 2)
      if (d[i] > 0 && d[i] < tstop) bp.push_back(d[i]);
  } else if (w.kind == ORC_WAVE_PULSE) {
    double TD = d[2], TR = d[3], TF = d[4], PW = d[5], PER = d[6];
    double base = TD;
    for (int k = 0; k < 100000 && base < tstop; ++k) {
      double c[4] = {base, base + TR, base + TR + PW, base + TR + PW + TF};
      for (double x : c)
        if (x > 0 && x < tstop) bp.push_back(x);
      if (PER <= 0) break;
      base += PER;
    }
  }
}

// ---------------------------------------------------------------------------
// Sparse LU: Gilbert-Peierls left-looking factorization with threshold
// partial pivoting, diagonal preferred — KLU's algorithm as called by
// N_LAS_AmesosSolver.C:309-396 with re-pivoting on every factor.  The
// diagonal-preference threshold is 0.1, not KLU's default 0.001: at 0.001 the
// operating-point Jacobian of a ring oscillator (weak diagonals, a cyclic
// chain of transconductances) grows by ~100 per eliminated stage and the
// solve loses every digit.
static const double kPivotTol = 0.1;
struct SparseLU {
  int n = 0;
  std::vector<int> Lp, Li, Up, Ui;   // L by columns (unit diag implicit), U by columns (diag last)
  std::vector<double> Lx, Ux;
  std::vector<int> pinv, perm;        // pinv[row] = pivot step, perm[step] = row
  std::vector<double> x;
  std::vector<int> stack, flag, pstack, topo;

  // A in CSC (Ap, Ai, Ax). Returns 0 ok, -1 singular.
  int factor(int n_, const std::vector<int> &Ap, const std::vector<int> &Ai, const double *Ax) {
    n = n_;
    Lp.assign(n + 1, 0); Up.assign(n + 1, 0);
    Li.clear(); Lx.clear(); Ui.clear(); Ux.clear();
    pinv.assign(n, -1); perm.assign(n, -1);
    x.assign(n, 0.0); flag.assign(n, -1); stack.resize(n); pstack.resize(n); topo.resize(n);
    for (int k = 0; k < n; ++k) {
      Lp[k] = (int)Li.size(); Up[k] = (int)Ui.size();
      // reach of A(:,k) through the graph of L (DFS)
      int top = n;
      for (int p = Ap[k]; p < Ap[k + 1]; ++p) {
        int i = Ai[p];
        if (flag[i] == k) continue;
        // dfs from row i
        int head = 0;
        stack[0] = i;
        while (head >= 0) {
          int r = stack[head];
          int j = pinv[r];
          if (flag[r] != k) {
            flag[r] = k;
            pstack[head] = (j < 0) ? 0 : Lp[j];
          }
          bool done = true;
          if (j >= 0) {
            int end = Lp[j + 1];
            for (int q = pstack[head]; q < end; ++q) {
              int r2 = Li[q];
              if (flag[r2] == k) continue;
              pstack[head] = q + 1;
              stack[++head] = r2;
              done = false;
              break;
            }
          }
          if (done) { --head; topo[--top] = r; }
        }
      }
      for (int p = Ap[k]; p < Ap[k + 1]; ++p) x[Ai[p]] = Ax[p];
      // numeric: sparse triangular solve in topological order
      for (int t = top; t < n; ++t) {
        int r = topo[t];
        int j = pinv[r];
        if (j < 0) continue;
        double xj = x[r];
        for (int q = Lp[j]; q < Lp[j + 1]; ++q) x[Li[q]] -= Lx[q] * xj;
      }
      // choose pivot among non-pivoted rows
      int ipiv = -1; double amax = -1.0;
      for (int t = top; t < n; ++t) {
        int r = topo[t];
        if (pinv[r] < 0) {
          double a = std::fabs(x[r]);
          if (a > amax) { amax = a; ipiv = r; }
        }
      }
      if (ipiv < 0 || amax <= 0.0 || !std::isfinite(amax)) return -1;
      if (pinv[k] < 0 && flag[k] == k && std::fabs(x[k]) >= kPivotTol * amax) ipiv = k;
      double piv = x[ipiv];
      for (int t = top; t < n; ++t) {
        int r = topo[t];
        int j = pinv[r];
        if (j >= 0) { Ui.push_back(j); Ux.push_back(x[r]); }
        else if (r != ipiv) { Li.push_back(r); Lx.push_back(x[r] / piv); }
        x[r] = 0.0;
      }
      Ui.push_back(k); Ux.push_back(piv);
      pinv[ipiv] = k; perm[k] = ipiv;
    }
    Lp[n] = (int)Li.size(); Up[n] = (int)Ui.size();
    // L row indices -> pivot steps
    for (int &r : Li) r = pinv[r];
    return 0;
  }

  void solve(const double *b, double *out) {
    std::vector<double> y(n);
    for (int k = 0; k < n; ++k) y[k] = b[perm[k]];
    for (int j = 0; j < n; ++j) {
      double yj = y[j];
      if (yj != 0.0)
        for (int q = Lp[j]; q < Lp[j + 1]; ++q) y[Li[q]] -= Lx[q] * yj;
    }
    for (int j = n - 1; j >= 0; --j) {
      int dq = Up[j + 1] - 1;
      y[j] /= Ux[dq];
      double yj = y[j];
      if (yj != 0.0)
        for (int q = Up[j]; q < dq; ++q) y[Ui[q]] -= Ux[q] * yj;
    }
    for (int k = 0; k < n; ++k) out[k] = y[k];
  }
};

}  // namespace

struct orc_ctx {
  int n = 0, ncirc = 1;
  std::vector<int> coff;
  // devices
  std::vector<int> r_p, r_n; std::vector<double> r_g;
  std::vector<int> c_p, c_n; std::vector<double> c_c;
  std::vector<int> v_p, v_n, v_b; std::vector<Wave> v_w;
  std::vector<int> l_p, l_n, l_b; std::vector<double> l_l;  // inductors
  std::vector<int> i_p, i_n; std::vector<Wave> i_w;
  std::vector<int> d_p, d_n, d_pri; std::vector<DiodeT> d_t;
  std::vector<int> m_d, m_g, m_s, m_b, m_dp, m_sp; std::vector<Mos1T> m_t;
  std::vector<int> b_d, b_g, b_s, b_b; std::vector<b4::Inst> b_t;
  std::vector<double> b_von;  // BSIM4 instance member von (last evaluation's Vth)
  // pattern (CSR) and per-device stamp positions
  std::vector<int> rp, ci;
  std::vector<int> pos_r, pos_c, pos_v, pos_l, pos_d, pos_m, pos_b;
  // CSC view for the LU, of P A P^T when an elimination order q is set
  // (q[k] = the unknown eliminated k-th; empty = the natural order)
  std::vector<int> Ap, Ai, csr2csc;
  std::vector<double> Ax;
  std::vector<int> q, qinv;
  std::vector<double> pb, px;  // b and x in the elimination order
  SparseLU lu;
  int nsta = 0, nsto = 0;
  std::vector<char> is_branch;  // unknown is a voltage-source branch current
  int last_limited = 0;  // devices whose junction voltages were limited in the last load
  double *wall_log = nullptr;  // optional: wall-clock seconds at each accepted step
  int wall_cap = 0;
  bool finalized = false;
  // linear solver: 0 = refactor on every Newton iteration (KLU through
  // AmesosSolver), 1 = LINSOL TYPE=IR (IRSolver: reuse earlier factors)
  int lin_type = 0;
  double ir_tol = 1e-9, ir_min_tol = 1e-2;  // IRSolver defaults, N_LAS_IRSolver.C:74-75
  bool lu_valid = false;
  // what the linear solves did: factorizations, reused solves accepted as
  // they were, reused solves accepted after refinement, refinement steps,
  // reused solves that fell back to a refactorization, and factorizations
  // of a matrix equal bit for bit to the one factored before it
  long long n_factor = 0, n_reuse = 0, n_refined = 0, n_refine_steps = 0, n_fallback = 0;
  long long n_repeat = 0;
  std::vector<double> last_factored;  // CSC values of the last factorization
  // replay of a given accepted-step sequence (orc_set_replay): times[k] and
  // integration order[k] of accepted point k (point 0 = the operating point)
  std::vector<double> replay_t;
  std::vector<int> replay_o;
  std::vector<int> rec_o;  // integration order of each point the last transient recorded
  // state layout: store diode [vd,qd,cd] then mos1 [vbd,vbs,vgs,vds,von,gm]
  // then bsim4 [vbd,vbs,vgs,vds,von]; state mos1 [capgs,capgd,capgb,qgs,qgd,
  // qgb,qbd,qbs] then bsim4 [qg,qd,qb]  (field-major, SoA)
};

namespace {

int csr_find(const orc_ctx *c, int r, int col) {
  if (r < 0 || col < 0) return -1;
  const int *b = c->ci.data() + c->rp[r], *e = c->ci.data() + c->rp[r + 1];
  const int *it = std::lower_bound(b, e, col);
  return (it != e && *it == col) ? (int)(it - c->ci.data()) : -1;
}

// Per-type stamp pair lists, in the order of the reference's jacobianStamp.
// Resistor (N_DEV_Resistor.C): (p,p)(p,n)(n,p)(n,n).  Capacitor likewise.
// Vsrc (N_DEV_Vsrc.C:1430-1460): (p,b)(n,b)(b,p)(b,n).
// Diode (N_DEV_Diode.C:741-768): (P,P)(P,Pri)(N,N)(N,Pri)(Pri,P)(Pri,N)(Pri,Pri).
// MOSFET1 (N_DEV_MOSFET1.C:1640-1700): full 4x4 over (D',G,S',B), then
// (D,D)(D,D')(D',D) and (S,S)(S,S')(S',S) for the series resistances (these
// land on the core's (D',D') / (S',S') when there is none).
void stamp_pairs(orc_ctx *c, std::vector<std::pair<int, int>> &all) {
  for (size_t k = 0; k < c->r_p.size(); ++k) {
    int p = c->r_p[k], n = c->r_n[k];
    all.push_back({p, p}); all.push_back({p, n}); all.push_back({n, p}); all.push_back({n, n});
  }
  for (size_t k = 0; k < c->c_p.size(); ++k) {
    int p = c->c_p[k], n = c->c_n[k];
    all.push_back({p, p}); all.push_back({p, n}); all.push_back({n, p}); all.push_back({n, n});
  }
  for (size_t k = 0; k < c->v_p.size(); ++k) {
    int p = c->v_p[k], n = c->v_n[k], b = c->v_b[k];
    all.push_back({p, b}); all.push_back({n, b}); all.push_back({b, p}); all.push_back({b, n});
  }
  // Inductor (N_DEV_Inductor.C:606-650): (p,b)(n,b)(b,p)(b,n)(b,b)
  for (size_t k = 0; k < c->l_p.size(); ++k) {
    int p = c->l_p[k], n = c->l_n[k], b = c->l_b[k];
    all.push_back({p, b}); all.push_back({n, b}); all.push_back({b, p}); all.push_back({b, n});
    all.push_back({b, b});
  }
  for (size_t k = 0; k < c->d_p.size(); ++k) {
    int P = c->d_p[k], N = c->d_n[k], R = c->d_pri[k];
    all.push_back({P, P}); all.push_back({P, R}); all.push_back({N, N}); all.push_back({N, R});
    all.push_back({R, P}); all.push_back({R, N}); all.push_back({R, R});
  }
  for (size_t k = 0; k < c->m_d.size(); ++k) {
    int nd[4] = {c->m_dp[k], c->m_g[k], c->m_sp[k], c->m_b[k]};
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) all.push_back({nd[a], nd[b]});
    const int D = c->m_d[k], Dp = c->m_dp[k], S = c->m_s[k], Sp = c->m_sp[k];
    all.push_back({D, D}); all.push_back({D, Dp}); all.push_back({Dp, D});
    all.push_back({S, S}); all.push_back({S, Sp}); all.push_back({Sp, S});
  }
  // BSIM4 without internal nodes: full 4x4 over (D,G,S,B)
  for (size_t k = 0; k < c->b_d.size(); ++k) {
    int nd[4] = {c->b_d[k], c->b_g[k], c->b_s[k], c->b_b[k]};
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) all.push_back({nd[a], nd[b]});
  }
}

inline void addv(double *v, int i, double x) { if (i >= 0) v[i] += x; }
inline void addm(double *m, int p, double x) { if (p >= 0) m[p] += x; }

}  // namespace

extern "C" {

orc_ctx *orc_create(int n_unknowns, int n_circuits, const int *offs) {
  orc_ctx *c = new orc_ctx;
  c->n = n_unknowns;
  c->ncirc = n_circuits;
  c->coff.assign(offs, offs + n_circuits + 1);
  return c;
}

void orc_destroy(orc_ctx *c) { delete c; }

int orc_add_resistors(orc_ctx *c, int n, const int *p, const int *m, const double *r) {
  for (int k = 0; k < n; ++k) { c->r_p.push_back(p[k]); c->r_n.push_back(m[k]); c->r_g.push_back(1.0 / r[k]); }
  return 0;
}
int orc_add_capacitors(orc_ctx *c, int n, const int *p, const int *m, const double *v) {
  for (int k = 0; k < n; ++k) { c->c_p.push_back(p[k]); c->c_n.push_back(m[k]); c->c_c.push_back(v[k]); }
  return 0;
}
int orc_add_vsources(orc_ctx *c, int n, const int *p, const int *m, const int *b, const int *kind,
                     const int *off, const double *data) {
  for (int k = 0; k < n; ++k) {
    c->v_p.push_back(p[k]); c->v_n.push_back(m[k]); c->v_b.push_back(b[k]);
    Wave w; w.kind = kind[k]; w.d.assign(data + off[k], data + off[k + 1]);
    c->v_w.push_back(w);
  }
  return 0;
}
int orc_add_inductors(orc_ctx *c, int n, const int *p, const int *m, const int *b, const double *l) {
  for (int k = 0; k < n; ++k) {
    c->l_p.push_back(p[k]); c->l_n.push_back(m[k]); c->l_b.push_back(b[k]); c->l_l.push_back(l[k]);
  }
  return 0;
}
int orc_add_isources(orc_ctx *c, int n, const int *p, const int *m, const int *kind, const int *off,
                     const double *data) {
  for (int k = 0; k < n; ++k) {
    c->i_p.push_back(p[k]); c->i_n.push_back(m[k]);
    Wave w; w.kind = kind[k]; w.d.assign(data + off[k], data + off[k + 1]);
    c->i_w.push_back(w);
  }
  return 0;
}
int orc_add_diodes(orc_ctx *c, int n, const int *p, const int *m, const int *pri, const double *params) {
  for (int k = 0; k < n; ++k) {
    c->d_p.push_back(p[k]); c->d_n.push_back(m[k]); c->d_pri.push_back(pri[k]);
    c->d_t.push_back(diode_temperature(params + (size_t)k * DP_COUNT));
  }
  return 0;
}
int orc_add_mosfet1(orc_ctx *c, int n, const int *d, const int *g, const int *s, const int *b,
                    const int *dp, const int *sp, const double *params) {
  for (int k = 0; k < n; ++k) {
    const double *pp = params + (size_t)k * MP_COUNT;
    const Mos1T t = mos1_temperature(pp);
    // the internal nodes exist exactly when the conductances are nonzero
    // (N_DEV_MOSFET1.C:1437-1445)
    if ((t.drainConductance != 0.0) == (dp[k] == d[k])) return -2;
    if ((t.sourceConductance != 0.0) == (sp[k] == s[k])) return -2;
    c->m_d.push_back(d[k]); c->m_g.push_back(g[k]); c->m_s.push_back(s[k]); c->m_b.push_back(b[k]);
    c->m_dp.push_back(dp[k]); c->m_sp.push_back(sp[k]);
    c->m_t.push_back(t);
  }
  return 0;
}

int orc_add_bsim4(orc_ctx *c, int n, const int *d, const int *g, const int *s, const int *b,
                  const double *params) {
  for (int k = 0; k < n; ++k) {
    b4::Inst I;
    std::string why;
    if (b4::setup(params + (size_t)k * b4::P_COUNT, I, &why) != 0) return -4;
    c->b_d.push_back(d[k]); c->b_g.push_back(g[k]); c->b_s.push_back(s[k]); c->b_b.push_back(b[k]);
    c->b_t.push_back(I);
    c->b_von.push_back(0.0);  // Instance constructor: von(0.0), N_DEV_MOSFET_B4.C:4995
  }
  return 0;
}

// Builder::generateGraphs + setupPointers restated: the CSR pattern is the
// union of every device's jacobianStamp; each stamp caches its position.
namespace {
// CSC structure of the pattern, symmetrically permuted by the elimination
// order when one is set: column k of P A P^T is column q[k] of A with row i
// moved to qinv[i].
void build_csc(orc_ctx *c) {
  const int nnz = (int)c->ci.size();
  auto pos = [&](int i) { return c->qinv.empty() ? i : c->qinv[i]; };
  c->Ap.assign(c->n + 1, 0);
  for (int p = 0; p < nnz; ++p) c->Ap[pos(c->ci[p]) + 1]++;
  for (int j = 0; j < c->n; ++j) c->Ap[j + 1] += c->Ap[j];
  c->Ai.resize(nnz); c->csr2csc.resize(nnz);
  std::vector<int> next(c->Ap.begin(), c->Ap.end() - 1);
  for (int i = 0; i < c->n; ++i)
    for (int p = c->rp[i]; p < c->rp[i + 1]; ++p) {
      const int k = next[pos(c->ci[p])]++;
      c->Ai[k] = pos(i); c->csr2csc[p] = k;
    }
  c->Ax.resize(nnz);
}

// x = A^-1 b with the current factors of P A P^T.
void lu_apply(orc_ctx *c, const double *b, double *x) {
  if (c->q.empty()) { c->lu.solve(b, x); return; }
  for (int k = 0; k < c->n; ++k) c->pb[k] = b[c->q[k]];
  c->lu.solve(c->pb.data(), c->px.data());
  for (int k = 0; k < c->n; ++k) x[c->q[k]] = c->px[k];
}
}  // namespace

int orc_finalize(orc_ctx *c) {
  std::vector<std::pair<int, int>> all;
  stamp_pairs(c, all);
  std::vector<std::vector<int>> rows(c->n);
  for (auto &pr : all)
    if (pr.first >= 0 && pr.second >= 0) rows[pr.first].push_back(pr.second);
  // every node unknown keeps its diagonal (gmin stepping shunts it); the
  // branch unknowns of voltage sources have none, as in the device stamps
  c->is_branch.assign(c->n, 0);
  for (int b : c->v_b) c->is_branch[b] = 1;
  for (int b : c->l_b) c->is_branch[b] = 1;
  for (int i = 0; i < c->n; ++i)
    if (!c->is_branch[i]) rows[i].push_back(i);
  c->rp.assign(c->n + 1, 0);
  c->ci.clear();
  for (int i = 0; i < c->n; ++i) {
    std::sort(rows[i].begin(), rows[i].end());
    rows[i].erase(std::unique(rows[i].begin(), rows[i].end()), rows[i].end());
    c->ci.insert(c->ci.end(), rows[i].begin(), rows[i].end());
    c->rp[i + 1] = (int)c->ci.size();
  }
  auto fill = [&](std::vector<int> &pos, size_t start, size_t count) {
    pos.resize(count);
    for (size_t k = 0; k < count; ++k) pos[k] = csr_find(c, all[start + k].first, all[start + k].second);
  };
  size_t o = 0;
  fill(c->pos_r, o, 4 * c->r_p.size()); o += 4 * c->r_p.size();
  fill(c->pos_c, o, 4 * c->c_p.size()); o += 4 * c->c_p.size();
  fill(c->pos_v, o, 4 * c->v_p.size()); o += 4 * c->v_p.size();
  fill(c->pos_l, o, 5 * c->l_p.size()); o += 5 * c->l_p.size();
  fill(c->pos_d, o, 7 * c->d_p.size()); o += 7 * c->d_p.size();
  fill(c->pos_m, o, 22 * c->m_d.size()); o += 22 * c->m_d.size();
  fill(c->pos_b, o, 16 * c->b_d.size()); o += 16 * c->b_d.size();
  build_csc(c);
  c->nsto = 3 * (int)c->d_p.size() + 6 * (int)c->m_d.size() + 5 * (int)c->b_d.size();
  c->nsta = 8 * (int)c->m_d.size() + 3 * (int)c->b_d.size();
  c->finalized = true;
  return 0;
}

int orc_sizes(orc_ctx *c, int *n, int *nnz, int *nsta, int *nsto) {
  *n = c->n; *nnz = (int)c->ci.size(); *nsta = c->nsta; *nsto = c->nsto;
  return 0;
}

int orc_pattern(orc_ctx *c, int *rp, int *ci) {
  std::copy(c->rp.begin(), c->rp.end(), rp);
  std::copy(c->ci.begin(), c->ci.end(), ci);
  return 0;
}

// NonlinearEquationLoader::loadRHS + loadJacobian restated
// (N_LOA_NonlinearEquationLoader.C:374-560): zero the outputs, then
// updateState / loadDAEVectors / loadDAEMatrices for every device type.
int orc_load(orc_ctx *c, double time, const double *x, const double *sta_curr, const double *sto_curr,
             const double *sto_next_in, int newton_iter, int flags, double *sta_next, double *sto_next,
             double *F, double *Q, double *B, double *dFdxdVp, double *dQdxdVp, double *dFdx,
             double *dQdx) {
  const int n = c->n;
  const size_t nnz = c->ci.size();
  const bool dcop = flags & 1, initJct = flags & 2;
  std::fill(F, F + n, 0.0); std::fill(Q, Q + n, 0.0); std::fill(B, B + n, 0.0);
  std::fill(dFdxdVp, dFdxdVp + n, 0.0); std::fill(dQdxdVp, dQdxdVp + n, 0.0);
  std::fill(dFdx, dFdx + nnz, 0.0); std::fill(dQdx, dQdx + nnz, 0.0);
  c->last_limited = 0;
  auto X = [&](int i) { return i >= 0 ? x[i] : 0.0; };
  // Resistor loadDAEVectors/Matrices, N_DEV_Resistor.C:1211-1375
  for (size_t k = 0; k < c->r_p.size(); ++k) {
    int p = c->r_p[k], m = c->r_n[k];
    double G = c->r_g[k];
    double i0 = (X(p) - X(m)) * G;
    addv(F, p, i0); addv(F, m, -i0);
    const int *ps = &c->pos_r[4 * k];
    addm(dFdx, ps[0], G); addm(dFdx, ps[1], -G); addm(dFdx, ps[2], -G); addm(dFdx, ps[3], G);
  }
  // Capacitor, N_DEV_Capacitor.C:1931-2260
  for (size_t k = 0; k < c->c_p.size(); ++k) {
    int p = c->c_p[k], m = c->c_n[k];
    double C = c->c_c[k];
    double q0 = C * (X(p) - X(m));
    addv(Q, p, q0); addv(Q, m, -q0);
    const int *ps = &c->pos_c[4 * k];
    addm(dQdx, ps[0], C); addm(dQdx, ps[1], -C); addm(dQdx, ps[2], -C); addm(dQdx, ps[3], C);
  }
  // Vsrc, N_DEV_Vsrc.C:1323-1460
  for (size_t k = 0; k < c->v_p.size(); ++k) {
    int p = c->v_p[k], m = c->v_n[k], b = c->v_b[k];
    double ib = x[b];
    addv(F, p, ib); addv(F, m, -ib); addv(F, b, X(p) - X(m));
    addv(B, b, wave_value(c->v_w[k], time));
    const int *ps = &c->pos_v[4 * k];
    addm(dFdx, ps[0], 1.0); addm(dFdx, ps[1], -1.0); addm(dFdx, ps[2], 1.0); addm(dFdx, ps[3], -1.0);
  }
  // Inductor, N_DEV_Inductor.C:540-650 (no IC): F[p] += i, F[n] -= i,
  // F[b] -= v(p) - v(n), Q[b] = L i
  for (size_t k = 0; k < c->l_p.size(); ++k) {
    int p = c->l_p[k], m = c->l_n[k], b = c->l_b[k];
    double ib = x[b];
    addv(F, p, ib); addv(F, m, -ib); addv(F, b, -(X(p) - X(m)));
    addv(Q, b, c->l_l[k] * ib);
    const int *ps = &c->pos_l[5 * k];
    addm(dFdx, ps[0], 1.0); addm(dFdx, ps[1], -1.0); addm(dFdx, ps[2], -1.0); addm(dFdx, ps[3], 1.0);
    addm(dQdx, ps[4], c->l_l[k]);
  }
  // ISRC, N_DEV_ISRC.C:1108-1172
  for (size_t k = 0; k < c->i_p.size(); ++k) {
    double s = wave_value(c->i_w[k], time);
    addv(B, c->i_p[k], -s); addv(B, c->i_n[k], s);
  }
  // Diode: Master::updateState/loadDAEVectors/loadDAEMatrices, N_DEV_Diode.C:1830-1950
  const int nd = (int)c->d_p.size();
  for (int k = 0; k < nd; ++k) {
    const DiodeT &t = c->d_t[k];
    int P = c->d_p[k], N = c->d_n[k], R = c->d_pri[k];
    double hist = (newton_iter == 0) ? sto_curr[k] : sto_next_in[k];
    DiodeOut o = diode_eval(t, X(R), X(N), hist, newton_iter, dcop, initJct);
    if (o.Vd != o.Vd_orig) c->last_limited++;
    sto_next[k] = o.Vd; sto_next[nd + k] = o.Qd; sto_next[2 * nd + k] = o.Cd;
    double Ir = t.Gspr * (X(P) - X(R));
    if (P != R) { addv(F, P, Ir); }
    addv(F, N, -o.Id);
    addv(F, R, -(-o.Id + Ir));
    addv(Q, N, -o.Qd);
    addv(Q, R, o.Qd);
    double Vd_diff = o.Vd - o.Vd_orig;
    double Cd_Jdxp = -o.Cd * Vd_diff, Gd_Jdxp = -o.Gd * Vd_diff;
    addv(dFdxdVp, N, Gd_Jdxp); addv(dFdxdVp, R, -Gd_Jdxp);
    addv(dQdxdVp, N, Cd_Jdxp); addv(dQdxdVp, R, -Cd_Jdxp);
    const int *ps = &c->pos_d[7 * k];
    addm(dFdx, ps[0], t.Gspr); addm(dFdx, ps[1], -t.Gspr);
    addm(dFdx, ps[2], o.Gd); addm(dFdx, ps[3], -o.Gd);
    addm(dFdx, ps[4], -t.Gspr); addm(dFdx, ps[5], -o.Gd); addm(dFdx, ps[6], t.Gspr + o.Gd);
    addm(dQdx, ps[2], o.Cd); addm(dQdx, ps[3], -o.Cd); addm(dQdx, ps[5], -o.Cd); addm(dQdx, ps[6], o.Cd);
  }
  // MOSFET1: Master::updateState/loadDAEVectors/loadDAEMatrices, N_DEV_MOSFET1.C:4241-4876
  const int nm = (int)c->m_d.size();
  const int so = 3 * nd;  // store offset of the MOSFET block
  for (int k = 0; k < nm; ++k) {
    const Mos1T &t = c->m_t[k];
    // D and S are the drain' and source' nodes the device equations act on;
    // Dx and Sx the external ones, joined to them by the series conductances
    int D = c->m_dp[k], G = c->m_g[k], S = c->m_sp[k], Bn = c->m_b[k];
    const int Dx = c->m_d[k], Sx = c->m_s[k];
    const double *hs = (newton_iter == 0) ? sto_curr : sto_next_in;
    double hist[5] = {hs[so + 0 * nm + k], hs[so + 1 * nm + k], hs[so + 2 * nm + k], hs[so + 3 * nm + k],
                      hs[so + 4 * nm + k]};
    double csta[6] = {sta_curr[0 * nm + k], sta_curr[1 * nm + k], sta_curr[2 * nm + k],
                      sta_curr[3 * nm + k], sta_curr[4 * nm + k], sta_curr[5 * nm + k]};
    double csto[3] = {sto_curr[so + 2 * nm + k], sto_curr[so + 1 * nm + k], sto_curr[so + 3 * nm + k]};
    Mos1Out o = mos1_eval(t, X(D), X(G), X(S), X(Bn), hist, csta, csto, newton_iter, dcop, initJct);
    if (!o.origFlag) c->last_limited++;
    sto_next[so + 0 * nm + k] = o.vbd; sto_next[so + 1 * nm + k] = o.vbs;
    sto_next[so + 2 * nm + k] = o.vgs; sto_next[so + 3 * nm + k] = o.vds;
    sto_next[so + 4 * nm + k] = o.von; sto_next[so + 5 * nm + k] = o.Gm;
    sta_next[0 * nm + k] = o.capgs; sta_next[1 * nm + k] = o.capgd; sta_next[2 * nm + k] = o.capgb;
    sta_next[3 * nm + k] = o.qgs; sta_next[4 * nm + k] = o.qgd; sta_next[5 * nm + k] = o.qgb;
    sta_next[6 * nm + k] = o.qbd; sta_next[7 * nm + k] = o.qbs;
    const double dt = t.dtype, M = t.M;
    double ceqbs = dt * o.cbs, ceqbd = dt * o.cbd;
    // series resistances: Idrain = drainConductance * Vddp (N_DEV_MOSFET1.C:3386),
    // loadDAEFVector :2212-2240
    const double gdpr = t.drainConductance, gspr = t.sourceConductance;
    const double Idrain = gdpr * (X(Dx) - X(D)), Isource = gspr * (X(Sx) - X(S));
    if (gdpr != 0.0) addv(F, Dx, Idrain * M);
    if (gspr != 0.0) addv(F, Sx, Isource * M);
    addv(F, Bn, (ceqbs + ceqbd) * M);
    addv(F, D, (-Idrain - (ceqbd - o.cdreq)) * M);
    addv(F, S, (-Isource - (ceqbs + o.cdreq)) * M);
    double Qeqbs = dt * o.qbs, Qeqbd = dt * o.qbd, Qeqgb = dt * o.qgb, Qeqgs = dt * o.qgs, Qeqgd = dt * o.qgd;
    addv(Q, G, (Qeqgs + Qeqgd + Qeqgb) * M);
    addv(Q, Bn, (Qeqbs + Qeqbd - Qeqgb) * M);
    addv(Q, D, -(Qeqbd + Qeqgd) * M);
    addv(Q, S, -(Qeqbs + Qeqgs) * M);
    if (!o.origFlag) {
      double dvbd = o.vbd - o.vbd_orig, dvbs = o.vbs - o.vbs_orig, dvds = o.vds - o.vds_orig;
      double dvgs = o.vgs - o.vgs_orig, dvgd = o.vgd - o.vgd_orig;
      double j4 = dt * ((o.gbd - kGmin) * dvbd + (o.gbs - kGmin) * dvbs);
      double sw = o.Gm * ((o.mode > 0) ? dvgs : dvgd) + o.Gmbs * ((o.mode > 0) ? dvbs : dvbd);
      double j5 = dt * (-(o.gbd - kGmin) * dvbd + o.gds * dvds + sw);
      double j6 = dt * (-(o.gbs - kGmin) * dvbs - o.gds * dvds - sw);
      addv(dFdxdVp, Bn, j4 * M); addv(dFdxdVp, D, j5 * M); addv(dFdxdVp, S, j6 * M);
      // Meyer (old) gate-charge limiter terms, :4440-4475.  The operating
      // point here is always the transient's TRANOP, so the capacitances load.
      double gcgd = o.Capgd, gcgs = o.Capgs, gcgb = o.Capgb, gcbs = o.capbs, gcbd = o.capbd;
      double q2 = dt * (gcgd * dvgd + gcgs * dvgs + gcgb * (dvgs - dvbs));
      double q4 = dt * (-gcgb * (dvgs - dvbs) + gcgb * dvbd + gcbs * dvbs);
      double q5 = dt * (-gcgd * dvgd - gcbd * dvbd);
      double q6 = dt * (-gcgs * dvgs - gcbs * dvbs);
      addv(dQdxdVp, G, q2 * M); addv(dQdxdVp, Bn, q4 * M); addv(dQdxdVp, D, q5 * M); addv(dQdxdVp, S, q6 * M);
    }
    // Jacobian: positions pos_m[22k + 4a + b] for nodes (D',G,S',B) = (0,1,2,3),
    // then pos_m[22k + 16..21] for (D,D)(D,D')(D',D)(S,S)(S,S')(S',S)
    const int *ps = &c->pos_m[22 * k];
    auto J = [&](int a, int b) { return ps[4 * a + b]; };
    // dFdx (loadDAEdFdx, N_DEV_MOSFET1.C:2484-2660)
    if (gdpr != 0.0) {
      addm(dFdx, ps[16], gdpr * M); addm(dFdx, ps[17], -(gdpr * M)); addm(dFdx, ps[18], -(gdpr * M));
    }
    if (gspr != 0.0) {
      addm(dFdx, ps[19], gspr * M); addm(dFdx, ps[20], -(gspr * M)); addm(dFdx, ps[21], -(gspr * M));
    }
    addm(dFdx, J(3, 3), (o.gbs + o.gbd) * M);
    addm(dFdx, J(3, 0), -o.gbd * M);
    addm(dFdx, J(3, 2), -o.gbs * M);
    addm(dFdx, J(0, 1), o.Gm * M);
    addm(dFdx, J(0, 3), (-o.gbd + o.Gmbs) * M);
    addm(dFdx, J(0, 0), (gdpr + o.gds + o.gbd + o.revsum) * M);
    addm(dFdx, J(0, 2), (-o.gds - o.nrmsum) * M);
    addm(dFdx, J(2, 1), -o.Gm * M);
    addm(dFdx, J(2, 3), -(o.gbs + o.Gmbs) * M);
    addm(dFdx, J(2, 0), -(o.gds + o.revsum) * M);
    addm(dFdx, J(2, 2), (gspr + o.gds + o.gbs + o.nrmsum) * M);
    // dQdx (old Meyer; TRANOP and transient load the capacitances)
    double gcgd = o.Capgd, gcgs = o.Capgs, gcgb = o.Capgb, gcbs = o.capbs, gcbd = o.capbd;
    addm(dQdx, J(1, 1), (gcgd + gcgs + gcgb) * M);
    addm(dQdx, J(1, 3), -gcgb * M);
    addm(dQdx, J(1, 0), -gcgd * M);
    addm(dQdx, J(1, 2), -gcgs * M);
    addm(dQdx, J(3, 1), -gcgb * M);
    addm(dQdx, J(3, 3), (gcbs + gcbd + gcgb) * M);
    addm(dQdx, J(3, 0), -gcbd * M);
    addm(dQdx, J(3, 2), -gcbs * M);
    addm(dQdx, J(0, 1), -gcgd * M);
    addm(dQdx, J(0, 3), -gcbd * M);
    addm(dQdx, J(0, 0), (gcbd + gcgd) * M);
    addm(dQdx, J(2, 1), -gcgs * M);
    addm(dQdx, J(2, 3), -gcbs * M);
    addm(dQdx, J(2, 2), (gcbs + gcgs) * M);
  }

  // BSIM4: Master::updateState / loadDAEVectors / loadDAEMatrices
  // (N_DEV_MOSFET_B4.C:10540-11687), limiting per updateIntermediateVars4p82_
  // (N_DEV_MOSFET_B4p82.C:3016-3240)
  const int nb = (int)c->b_d.size();
  const int sob = 3 * nd + 6 * nm, stb = 8 * nm;
  for (int k = 0; k < nb; ++k) {
    const b4::Inst &I = c->b_t[k];
    const int D = c->b_d[k], G = c->b_g[k], S = c->b_s[k], Bn = c->b_b[k];
    const double dt = I.dtype, M = I.M;
    double vgs = dt * (X(G) - X(S)), vds = dt * (X(D) - X(S)), vbs = dt * (X(Bn) - X(S));
    double vbd = vbs - vds, vgd = vgs - vds;
    const double vgs_o = vgs, vds_o = vds, vbs_o = vbs;
    int origFlag = 1;
    if (initJct) {
      vds = 0.1; vgs = dt * I.vth0 + 0.1; vbs = 0.0;
      vbd = vbs - vds; vgd = vgs - vds;
      origFlag = 0;
    }
    double vbd_old, vbs_old, vgs_old, vds_old;
    if (newton_iter == 0 && dcop) {
      vbd_old = vbd; vbs_old = vbs; vgs_old = vgs; vds_old = vds;
    } else {
      const double *h = (newton_iter == 0) ? sto_curr : sto_next_in;
      vbd_old = h[sob + k]; vbs_old = h[sob + nb + k]; vgs_old = h[sob + 2 * nb + k]; vds_old = h[sob + 3 * nb + k];
    }
    const double von_prev = sto_next_in[sob + 4 * nb + k];  // instance member von: last evaluation
    const double vgd_old = vgs_old - vds_old;
    if (!initJct) {
      int Check = 0;
      if (vds_old >= 0.0) {
        vgs = fetlim(vgs, vgs_old, von_prev);
        vds = vgs - vgd;
        vds = limvds(vds, vds_old);
        vgd = vgs - vds;
      } else {
        vgd = fetlim(vgd, vgd_old, von_prev);
        vds = vgs - vgd;
        vds = -limvds(-vds, -vds_old);
        vgs = vgd + vds;
      }
      if (vds >= 0.0) {
        vbs = pnjlim(vbs, vbs_old, b4::kVt0, I.vcrit, &Check);
        vbd = vbs - vds;
      } else {
        vbd = pnjlim(vbd, vbd_old, b4::kVt0, I.vcrit, &Check);
        vbs = vbd + vds;
      }
    }
    vbd = vbs - vds;
    const double eps = 2.220446049250313e-16;
    if (std::fabs(vbs_o - vbs) > eps || std::fabs(vgs_o - vgs) > eps || std::fabs(vds_o - vds) > eps) origFlag = 0;
    if (!origFlag) c->last_limited++;
    // values, then complex-step partials along vgs, vds, vbs
    b4::Out<double> o;
    b4::core(I, vgs, vds, vbs, o, -1);
    double dF[3][3], dq[3][3];  // [output D/S/B or G/D/B][vgs, vds, vbs]
    const double hcs = 1e-30;
    for (int dir = 0; dir < 3; ++dir) {
      using Cx = std::complex<double>;
      Cx a(vgs, dir == 0 ? hcs : 0.0), bb(vds, dir == 1 ? hcs : 0.0), cc(vbs, dir == 2 ? hcs : 0.0);
      b4::Out<Cx> oc;
      b4::core(I, a, bb, cc, oc, dir);
      dF[0][dir] = oc.Fd.imag() / hcs; dF[1][dir] = oc.Fs.imag() / hcs; dF[2][dir] = oc.Fb.imag() / hcs;
      dq[0][dir] = oc.qg.imag() / hcs; dq[1][dir] = oc.qd.imag() / hcs; dq[2][dir] = oc.qb.imag() / hcs;
    }
    sto_next[sob + k] = vbd; sto_next[sob + nb + k] = vbs;
    sto_next[sob + 2 * nb + k] = vgs; sto_next[sob + 3 * nb + k] = vds;
    sto_next[sob + 4 * nb + k] = o.von;
    c->b_von[k] = o.von;
    sta_next[stb + k] = o.qg; sta_next[stb + nb + k] = o.qd; sta_next[stb + 2 * nb + k] = o.qb;
    addv(F, D, o.Fd * M); addv(F, S, o.Fs * M); addv(F, Bn, o.Fb * M);
    addv(Q, G, dt * o.qg * M); addv(Q, D, dt * o.qd * M); addv(Q, Bn, dt * o.qb * M);
    addv(Q, S, -dt * (o.qg + o.qd + o.qb) * M);
    if (!origFlag) {
      const double dv[3] = {vgs - vgs_o, vds - vds_o, vbs - vbs_o};
      double lf[3] = {0, 0, 0}, lq[3] = {0, 0, 0};
      for (int a = 0; a < 3; ++a)
        for (int j = 0; j < 3; ++j) { lf[a] += dF[a][j] * dv[j]; lq[a] += dq[a][j] * dv[j]; }
      addv(dFdxdVp, D, lf[0] * M); addv(dFdxdVp, S, lf[1] * M); addv(dFdxdVp, Bn, lf[2] * M);
      // the gate-charge limiter terms carry no dtype (N_DEV_MOSFET_B4.C:7215-7232)
      addv(dQdxdVp, G, lq[0] * M); addv(dQdxdVp, D, lq[1] * M); addv(dQdxdVp, Bn, lq[2] * M);
      addv(dQdxdVp, S, -(lq[0] + lq[1] + lq[2]) * M);
    }
    // node columns: G <- vgs, D <- vds, B <- vbs, S <- -(sum); rows D,G,S,B = 0,1,2,3
    const int *ps = &c->pos_b[16 * k];
    auto Jp = [&](int a, int b) { return ps[4 * a + b]; };
    const int rowF[3] = {0, 2, 3};   // D, S, B
    const int rowQ[3] = {1, 0, 3};   // G, D, B
    const int colv[3] = {1, 0, 3};   // vgs -> G, vds -> D, vbs -> B
    for (int a = 0; a < 3; ++a) {
      double sf = 0.0, sq = 0.0;
      for (int j = 0; j < 3; ++j) {
        addm(dFdx, Jp(rowF[a], colv[j]), dt * dF[a][j] * M);
        addm(dQdx, Jp(rowQ[a], colv[j]), dq[a][j] * M);
        sf += dF[a][j]; sq += dq[a][j];
      }
      addm(dFdx, Jp(rowF[a], 2), -dt * sf * M);
      addm(dQdx, Jp(rowQ[a], 2), -sq * M);
    }
    // source row of Q: -(qg + qd + qb)
    double ss = 0.0;
    for (int j = 0; j < 3; ++j) {
      const double v = -(dq[0][j] + dq[1][j] + dq[2][j]);
      addm(dQdx, Jp(2, colv[j]), v * M);
      ss += v;
    }
    addm(dQdx, Jp(2, 2), -ss * M);
  }
  return 0;
}

int orc_lu_solve(orc_ctx *c, const double *vals, const double *b, double *x) {
  size_t nnz = c->ci.size();
  for (size_t p = 0; p < nnz; ++p) c->Ax[c->csr2csc[p]] = vals[p];
  if (c->lu.factor(c->n, c->Ap, c->Ai, c->Ax.data()) != 0) return -9;
  lu_apply(c, b, x);
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Nonlinear solve and time integration.
namespace {

struct NLParams {
  double reltol, abstol, deltaxtol, rhstol, smallupdatetol;
  int maxstep;
  bool transient;
  bool enforce_device_conv;
};

struct Work {
  int n, nnz, nsta, nsto;
  std::vector<double> x, xcurr, sta_curr, sto_curr, sta_next, sto_next, sto_prev;
  std::vector<double> F, Q, B, dFv, dQv, dFdx, dQdx, J, rhs, dx, solwt;
  std::vector<double> ir_r, ir_x, ir_d;  // refinement residual, iterate, correction
  bool any_limited = false;
  double t_load = 0, t_solve = 0;
};

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Coefficients of the nonlinear system: RHS = -(qscale*(Q - qhist0) + fscale*(F - B) + hscale*qhist2)
// + qscale*dQdxdVp + fscale*dFdxdVp, J = qscale*dQdx + fscale*dFdx (+gshunt on node diagonals).
struct Coef {
  double qscale, fscale, hscale;
  const double *qhist0, *qhist2;
  double gshunt;
  int n_nodes_shunt;  // shunts apply to all unknowns < this bound (per circuit none: all)
  // Gear12::obtainResidual (N_TIA_Gear12.C:208-271): F - B + (a0 Q + a1 qH0 + a2 qH1) / h
  int gear = 0;
  double ga[3] = {0, 0, 0}, hinv = 0;
  const double *gqh1 = nullptr;  // qH1 (second order only)
};

// origFlag test: did any nonlinear device limit its junction voltages?
// (Instance::isConverged, N_DEV_DeviceInstance.h:528, via allDevicesConverged.)
bool device_limited(orc_ctx *c, Work &) { return c->last_limited > 0; }

void assemble(orc_ctx *c, Work &w, double time, int iter, int flags, const Coef &cf) {
  double t0 = now();
  // BSIM4 limiting reads von of the instance's last evaluation (an instance
  // member in the reference); orc_load takes it from the von plane of its
  // store input
  {
    const int nb = (int)c->b_d.size(), sob = 3 * (int)c->d_p.size() + 6 * (int)c->m_d.size();
    for (int k = 0; k < nb; ++k) w.sto_prev[sob + 4 * nb + k] = c->b_von[k];
  }
  orc_load(c, time, w.x.data(), w.sta_curr.data(), w.sto_curr.data(), w.sto_prev.data(), iter, flags,
           w.sta_next.data(), w.sto_next.data(), w.F.data(), w.Q.data(), w.B.data(), w.dFv.data(),
           w.dQv.data(), w.dFdx.data(), w.dQdx.data());
  w.any_limited = device_limited(c, w);
  for (int i = 0; i < w.n; ++i) {
    double r;
    if (cf.gear) {
      double q = cf.ga[0] * w.Q[i] + cf.ga[1] * cf.qhist0[i];
      if (cf.gqh1) q += cf.ga[2] * cf.gqh1[i];
      r = (w.F[i] - w.B[i]) + cf.hinv * q;  // hinv = 1 / h
    } else {
      r = cf.fscale * (w.F[i] - w.B[i]);
      if (cf.qscale != 0.0) r += cf.qscale * (w.Q[i] - cf.qhist0[i]);
      if (cf.hscale != 0.0) r += cf.hscale * cf.qhist2[i];
    }
    if (cf.gshunt != 0.0 && !c->is_branch[i]) r += cf.gshunt * w.x[i];
    w.rhs[i] = -r + cf.qscale * w.dQv[i] + cf.fscale * w.dFv[i];
  }
  for (int p = 0; p < w.nnz; ++p) w.J[p] = cf.qscale * w.dQdx[p] + cf.fscale * w.dFdx[p];
  if (cf.gshunt != 0.0)
    for (int i = 0; i < w.n; ++i)
      if (!c->is_branch[i]) w.J[csr_find(c, i, i)] += cf.gshunt;
  w.t_load += now() - t0;
}

// One linear solve J dx = rhs for Newton iteration nlStep (1-based).
// Default: factor J, then solve (AmesosSolver::doSolve with KLU).  With
// lin_type 1, IRSolver::doSolve (N_LAS_IRSolver.C:428-560): the first
// iteration of every Newton solve factors; later iterations solve with the
// factors they find and test the relative residual ||rhs - J dx||_2 /
// ||rhs||_2 (unscaled when ||rhs||_2 is below machine epsilon).  At most
// ir_tol the solve stands; below ir_min_tol up to 10 refinement steps
// x += (LU)^-1 (rhs - J x) run while the residual is above ir_tol and does
// not grow, and stand if they end below ir_tol; anything else refactors.
// As in the reference, a NaN residual passes the first test (the Newton
// loop then fails on the non-finite update).
int linear_solve(orc_ctx *c, Work &w, int nlStep) {
  auto standard = [&]() {
    for (int p = 0; p < w.nnz; ++p) c->Ax[c->csr2csc[p]] = w.J[p];
    c->n_factor++;
    if (c->lu_valid && c->last_factored == c->Ax) c->n_repeat++;
    c->last_factored = c->Ax;
    const int fs = c->lu.factor(w.n, c->Ap, c->Ai, c->Ax.data());
    c->lu_valid = fs == 0;
    if (fs != 0) return -9;
    lu_apply(c, w.rhs.data(), w.dx.data());
    return 0;
  };
  if (c->lin_type != 1 || nlStep == 1 || !c->lu_valid) return standard();
  const double eps = 2.220446049250313e-16;
  auto residual = [&](const std::vector<double> &v) {  // ir_r = rhs - J v; returns ||ir_r||_2
    double s = 0;
    for (int i = 0; i < w.n; ++i) {
      double a = 0;
      for (int p = c->rp[i]; p < c->rp[i + 1]; ++p) a += w.J[p] * v[c->ci[p]];
      w.ir_r[i] = w.rhs[i] - a;
      s += w.ir_r[i] * w.ir_r[i];
    }
    return std::sqrt(s);
  };
  double bn = 0;
  for (double b : w.rhs) bn += b * b;
  bn = std::sqrt(bn);
  auto rel = [&](double rn) { return bn > eps ? rn / bn : rn; };
  lu_apply(c, w.rhs.data(), w.dx.data());
  double res = rel(residual(w.dx));
  if (!(res > c->ir_tol)) { c->n_reuse++; return 0; }
  if (res < c->ir_min_tol) {
    w.ir_x = w.dx;
    int it = 0;
    bool diverging = false;
    while (res > c->ir_tol && it < 10 && !diverging) {
      lu_apply(c, w.ir_r.data(), w.ir_d.data());
      for (int i = 0; i < w.n; ++i) w.ir_x[i] += w.ir_d[i];
      const double nr = rel(residual(w.ir_x));
      if (nr > res) diverging = true;
      res = nr;
      ++it;
    }
    c->n_refine_steps += it;
    if (res < c->ir_tol) {
      w.dx = w.ir_x;
      c->n_refined++;
      return 0;
    }
  }
  c->n_fallback++;
  return standard();
}

// DampedNewton::solve + converged_ (N_NLS_DampedNewton.C:362-520, 1191-1396),
// full Newton steps.  Returns the DampedNewton status code; *iters = nlStep_.
int newton(orc_ctx *c, Work &w, double time, const NLParams &nl, const Coef &cf, int first_flags,
           int *iters) {
  const double eps = 2.220446049250313e-16;
  const double convRateMax = 0.5 * 1.7976931348623157e308;
  int nlStep = 0;
  assemble(c, w, time, 0, first_flags, cf);
  auto norm2 = [&](const std::vector<double> &v) {
    double s = 0; for (double a : v) s += a * a; return std::sqrt(s);
  };
  double normRHS = norm2(w.rhs);
  double normRHS_init = normRHS, normRHS_old = normRHS;
  bool nan = !std::isfinite(normRHS);
  // updateWeights_ (:297-340) — once in transient, every iteration otherwise
  auto update_weights = [&]() {
    for (int i = 0; i < w.n; ++i)
      w.solwt[i] = nl.reltol * std::max(std::fabs(w.x[i]), std::fabs(w.xcurr[i])) + nl.abstol;
  };
  if (nl.transient) update_weights();
  int count = 0;
  double tmpConvRate = 1.0;
  int status = 0;
  while (status == 0) {
    nlStep++;
    if (nan) { status = -6; break; }
    // direction_: solve J dx = rhs
    double t0 = now();
    const int ls = linear_solve(c, w, nlStep);
    w.t_solve += now() - t0;
    if (ls != 0) { status = -9; break; }
    bool dxnan = false;
    for (int i = 0; i < w.n; ++i) if (!std::isfinite(w.dx[i])) dxnan = true;
    if (dxnan) { status = -6; break; }
    // fullNewton_ (:1147-1160): x += dx, then a new residual
    for (int i = 0; i < w.n; ++i) w.x[i] += w.dx[i];
    if (!nl.transient) update_weights();
    std::swap(w.sto_prev, w.sto_next);
    assemble(c, w, time, nlStep, first_flags & 1, cf);
    normRHS = norm2(w.rhs);
    nan = !std::isfinite(normRHS);
    // converged_
    if (nan) { status = -6; break; }
    if (nl.enforce_device_conv && w.any_limited) {
      if (nlStep < nl.maxstep) continue;
      status = -1; break;
    }
    double maxNormRHS = 0, wtNormDX = 0;
    for (int i = 0; i < w.n; ++i) {
      maxNormRHS = std::max(maxNormRHS, std::fabs(w.rhs[i]));
      wtNormDX = std::max(wtNormDX, std::fabs(w.dx[i]) / w.solwt[i]);
    }
    if (normRHS < eps) { status = 1; break; }
    double normRHS_rel = normRHS / normRHS_init;
    double resConvRate = normRHS / normRHS_old;
    normRHS_old = normRHS;
    if (maxNormRHS <= nl.rhstol && wtNormDX <= nl.deltaxtol) { status = 2; break; }
    if (nlStep >= nl.maxstep && nl.transient) {
      if (normRHS_rel <= 0.9 && resConvRate <= 1.0) { status = -3; break; }
    }
    if (wtNormDX <= nl.smallupdatetol) { status = 4; break; }
    if (nlStep >= nl.maxstep) { status = -1; break; }
    else if (resConvRate > convRateMax) { status = -2; break; }
    if (nl.transient && std::fabs(resConvRate - 1.0) <= 1.0e-3) {
      if (count == 0 || resConvRate < tmpConvRate) tmpConvRate = resConvRate;
      count++;
    } else {
      count = 0;
    }
    if (nl.transient && count == 5) {
      count = 0;
      // nearConvergence and stalled both map to -3 in the default return codes
      // (N_NLS_ReturnCodes.h:76-85), so either outcome is a failed solve.
      status = -3;
      break;
    }
  }
  *iters = nlStep;
  return status;
}

void work_init(orc_ctx *c, Work &w) {
  w.n = c->n; w.nnz = (int)c->ci.size(); w.nsta = c->nsta; w.nsto = c->nsto;
  w.x.assign(w.n, 0.0); w.xcurr.assign(w.n, 0.0);
  w.sta_curr.assign(std::max(1, w.nsta), 0.0); w.sta_next = w.sta_curr;
  w.sto_curr.assign(std::max(1, w.nsto), 0.0); w.sto_next = w.sto_curr; w.sto_prev = w.sto_curr;
  for (auto *v : {&w.F, &w.Q, &w.B, &w.dFv, &w.dQv, &w.rhs, &w.dx, &w.solwt, &w.ir_r, &w.ir_x, &w.ir_d})
    v->assign(w.n, 0.0);
  for (auto *v : {&w.dFdx, &w.dQdx, &w.J}) v->assign(w.nnz, 0.0);
}

// Operating point: DampedNewton with the DC option defaults
// (N_NLS_Manager.C:1030-1052: RELTOL 1e-3, DELTAXTOL 1, RHSTOL 1e-6,
// MAXSTEP 200, ENFORCEDEVICECONV 1), initJct on the first iteration, then
// gmin stepping if the plain solve fails.
int dcop(orc_ctx *c, Work &w, double t0, int *total_iters) {
  NLParams nl{1e-3, 1e-12, 1.0, 1e-6, 1e-6, 200, false, true};
  Coef cf{0.0, 1.0, 0.0, nullptr, nullptr, 0.0, 0};
  int it = 0;
  std::fill(w.x.begin(), w.x.end(), 0.0);
  std::fill(w.xcurr.begin(), w.xcurr.end(), 0.0);
  int st = newton(c, w, t0, nl, cf, 1 | 2, &it);
  *total_iters = it;
  if (st > 0) return st;
  // gmin stepping: shunt conductance from every node unknown to ground,
  // stepped 1e-2 -> 1e-12 by decades, then removed.
  std::fill(w.x.begin(), w.x.end(), 0.0);
  bool first = true;
  for (double g = 1e-2; g >= 1e-12 * 0.999; g /= 10.0) {
    cf.gshunt = g;
    st = newton(c, w, t0, nl, cf, first ? (1 | 2) : 1, &it);
    first = false;
    *total_iters += it;
    if (st <= 0) return st;
    w.sto_curr = w.sto_next;
  }
  cf.gshunt = 0.0;
  st = newton(c, w, t0, nl, cf, 1, &it);
  *total_iters += it;
  return st;
}

}  // namespace

// One DampedNewton solve with caller-given coefficients and histories (the
// checker of the GPU's xg_newton_solve): RHS = -[qscale (Q - qhist0) +
// fscale (F - B) + hscale qhist2] + limiter terms, J = qscale dQdx + fscale
// dFdx; weights reltol * max(|x|, |x_curr|) + abstol.  flags bit0: operating-
// point rules, bit1: initJct on the first iteration.  x in/out.
extern "C" int orc_newton(orc_ctx *c, double time, double qscale, double fscale, double hscale,
                          const double *qhist0, const double *qhist2, double *x, const double *x_curr,
                          const double *sta_curr, const double *sto_curr, double *sta_next, double *sto_next,
                          double reltol, double abstol, double deltaxtol, double rhstol, double smallupdatetol,
                          int maxstep, int flags, int *iters) {
  Work w;
  work_init(c, w);
  const bool dcop = (flags & 1) != 0;
  std::copy(x, x + w.n, w.x.begin());
  if (x_curr) std::copy(x_curr, x_curr + w.n, w.xcurr.begin());
  if (c->nsta) std::copy(sta_curr, sta_curr + c->nsta, w.sta_curr.begin());
  if (c->nsto) std::copy(sto_curr, sto_curr + c->nsto, w.sto_curr.begin());
  std::vector<double> zeros(w.n, 0.0);
  Coef cf{qscale, fscale, hscale, qhist0 ? qhist0 : zeros.data(), qhist2 ? qhist2 : zeros.data(), 0.0, 0};
  NLParams nl{reltol, abstol, deltaxtol, rhstol, smallupdatetol, maxstep, !dcop, dcop};
  const int st = newton(c, w, time, nl, cf, flags & 3, iters);
  std::copy(w.x.begin(), w.x.end(), x);
  if (c->nsta) std::copy(w.sta_next.begin(), w.sta_next.begin() + c->nsta, sta_next);
  if (c->nsto) std::copy(w.sto_next.begin(), w.sto_next.begin() + c->nsto, sto_next);
  return st;
}

extern "C" int orc_dcop(orc_ctx *c, double *x, int *iters) {
  Work w;
  work_init(c, w);
  int st = dcop(c, w, 0.0, iters);
  std::copy(w.x.begin(), w.x.end(), x);
  return st;
}

// Transient driver: Transient::doLoopProcess / takeAnIntegrationStep_
// (N_ANP_Transient.C:1184-1410, 3262-3325) with OneStep (trapezoid after a
// backward-Euler start) and StepErrorControl, restated in one loop.
extern "C" int orc_transient(orc_ctx *c, const orc_tran_params *p, int n_probe, const int *probes, int cap,
                             double *times, double *values, int *n_out, orc_tran_stats *st) {
  double tstart_wall = now();
  std::memset(st, 0, sizeof(*st));
  Work w;
  work_init(c, w);
  const int n = w.n;
  int it = 0;
  int ds = dcop(c, w, p->tstart, &it);
  st->dcop_iters = it;
  if (ds <= 0) { st->status = -100 + ds; return st->status; }
  // accepted operating point
  w.xcurr = w.x; w.sta_curr = w.sta_next; w.sto_curr = w.sto_next;
  std::vector<double> Fc = w.F, Qc = w.Q, Bc = w.B;
  // breakpoints
  std::vector<double> bps;
  for (auto &wv : c->v_w) wave_breakpoints(wv, p->tstop, bps);
  for (auto &wv : c->i_w) wave_breakpoints(wv, p->tstop, bps);
  bps.push_back(p->tstop);
  std::sort(bps.begin(), bps.end());
  const double bptol = 1e-15 * (p->tstop - p->tstart);
  auto next_bp = [&](double t) {
    for (double b : bps) if (b > t + bptol) return b;
    return p->tstop;
  };
  NLParams nl{p->nl_reltol, p->nl_abstol, p->nl_deltaxtol, p->nl_rhstol, p->nl_smallupdatetol,
              p->nl_maxstep, true, false};
  const double hmax = p->hmax > 0 ? p->hmax : 0.1 * (p->tstop - p->tstart);
  const double hmin = p->hmin;
  const int max_order = p->max_order > 0 ? p->max_order : 2;
  const bool gear = p->method == 8;  // Gear12 (N_TIA_Gear12.C); else OneStep
  // integrator state (StepErrorControl / OneStep members)
  double t = p->tstart, h = 0.0, lastTimeStep = 0.0, tsum = 0.0, saved = hmax, estOverTol = 0.0;
  double psi[3] = {0, 0, 0}, beta[3] = {1, 0, 0}, alpha[3] = {0, 0, 0}, ck = 0.0;
  int order = 1, numberOfSteps = 0, nef = 0, stepNumber = 0;
  bool beginning = true, lastOk = true;
  double stopTime = next_bp(t);
  std::vector<double> xh0(n), xh1(n, 0.0), xh2(n, 0.0), qh0(n), qh1(n, 0.0), qh2(n, 0.0), xn0(n), errwt(n);
  int nout = 0;
  c->rec_o.clear();
  int step_order = 0;  // order of the step being recorded (0: the operating point)
  auto record = [&](double tt, const std::vector<double> &xx) {
    if (nout < cap) c->rec_o.push_back(step_order);
    if (nout < cap) {
      times[nout] = tt;
      for (int k = 0; k < n_probe; ++k) values[(size_t)nout * n_probe + k] = xx[probes[k]];
      nout++;
    }
  };
  record(t, w.xcurr);
  // Replay: step k goes exactly to replay_t[k] with order replay_o[k], and
  // the step stands whenever Newton converges (no error test, no
  // rejections).  Everything else — histories, coefficients, predictors,
  // breakpoints — follows the same code as a free run.
  const int n_replay = (int)c->replay_t.size();
  const bool replay = n_replay > 0;
  while (t < p->tstop - bptol) {
    if (p->max_steps > 0 && st->accepted >= p->max_steps) break;
    if (replay && st->accepted + 1 >= n_replay) break;
    const double h_replay = replay ? c->replay_t[st->accepted + 1] - t : 0.0;
    if (beginning && lastOk) {
      // OneStep::initialize (N_TIA_OneStep.C:1684-1800)
      double time_to_stop = stopTime - t;
      double hn = (t == p->tstart) ? 0.005 * time_to_stop : 0.1 * std::min(saved, time_to_stop);
      if (hn > hmax) hn = hmax;
      // (Gear12::initialize takes the restart step as is, N_TIA_Gear12.C:1225-1245)
      h = (t != p->tstart && !gear) ? std::min(h, hn) : hn;
      h = std::min(std::max(h, hmin), hmax);
      if (replay) h = h_replay;
      tsum = 2.0 * h; lastTimeStep = h;
      if (gear) {
        // Gear12::initialize history (N_TIA_Gear12.C:1280-1300)
        xh0 = w.xcurr; xh1 = w.xcurr;
        qh0 = Qc; qh1 = Qc;
      } else {
        xh0 = w.xcurr; std::fill(xh1.begin(), xh1.end(), 0.0);
        qh0 = Qc;
        for (int i = 0; i < n; ++i) qh1[i] = -(Fc[i] - Bc[i]) * h;
      }
      numberOfSteps = 0; order = 1; psi[0] = h;
    }
    if (replay) {
      h = h_replay;
      order = c->replay_o[st->accepted + 1];
      if (!(h > 0.0) || (order != 1 && order != 2)) { st->status = -50; break; }
    }
    if (order == 2) psi[2] = psi[1];
    psi[1] = psi[0]; psi[0] = h;
    if (gear) {
      // Gear12::updateCoeffs (N_TIA_Gear12.C:1050-1110)
      if (order == 2) {
        beta[2] = h / psi[2] * (h + psi[1]) / (psi[1] + psi[2]);
        beta[1] = -h / psi[1] - beta[2] * (psi[1] + psi[2]) / psi[1];
        beta[0] = 1.0 - beta[2] - beta[1];
        alpha[2] = -h / psi[1] * h / (2 * h + psi[1]);
        alpha[1] = 1 - alpha[2];
        alpha[0] = -alpha[1] - alpha[2] * (1 + psi[1] / h);
        alpha[2] = alpha[2] / alpha[0];
        alpha[1] = alpha[1] / alpha[0];
        alpha[0] = -1 / alpha[0];
        ck = h / (h + psi[1] + psi[2]);
      } else {
        beta[0] = 1.0 + h / psi[1];
        beta[1] = -h / psi[1];
        alpha[0] = 1.0;
        alpha[1] = -1.0;
        ck = h / (h + psi[1]);
      }
    } else if (order == 2) {
      // OneStep::updateCoeffs (:1584-1640)
      beta[1] = h / psi[1] + (h / psi[1]) * (h / psi[1]) / 2;
      beta[2] = -1.0 * h * h / psi[1] / psi[2] / 2;
      ck = (h / tsum) / 3.0;
    } else {
      beta[1] = h / psi[1];
      ck = h / tsum;
    }
    // DataStore::setErrorWtVector, NEWLTE = 1 (N_TIA_DataStore.C:1304-1450)
    double xmax = 0;
    for (int i = 0; i < n; ++i) xmax = std::max(xmax, std::fabs(w.xcurr[i]));
    for (int i = 0; i < n; ++i) errwt[i] = p->reltol * xmax + p->abstol;
    // predictor: OneStep::obtainPredictor (:135-175) / Gear12::obtainPredictor (N_TIA_Gear12.C:131-190)
    for (int i = 0; i < n; ++i) {
      double v;
      if (gear) {
        v = beta[0] * xh0[i];
        v += beta[1] * xh1[i];
        if (order == 2) v += beta[2] * xh2[i];
      } else {
        v = xh0[i] + beta[1] * xh1[i];
        if (order == 2) v += beta[2] * xh2[i];
      }
      xn0[i] = v;
    }
    w.x = xn0;
    double tn = t + h;
    if (std::fabs(tn - stopTime) <= bptol) tn = stopTime;
    if (replay) tn = c->replay_t[st->accepted + 1];
    Coef cf{1.0 / h, order == 2 ? 0.5 : 1.0, order == 2 ? 0.5 : 0.0, qh0.data(), qh2.data(), 0.0, 0};
    if (gear) {
      // Gear12::obtainJacobian (N_TIA_Gear12.C:477-500): (a0 / h) dQdx + dFdx
      cf.qscale = alpha[0] / h; cf.fscale = 1.0; cf.hscale = 0.0;
      cf.gear = 1;
      cf.ga[0] = alpha[0]; cf.ga[1] = alpha[1]; cf.ga[2] = alpha[2];
      cf.hinv = 1.0 / h;
      cf.gqh1 = order == 2 ? qh1.data() : nullptr;
    }
    int iters = 0;
    int ns = newton(c, w, tn, nl, cf, 0, &iters);
    st->newton_iters += iters;
    bool ok = ns > 0;
    if (!ok) st->newton_fail++;
    if (replay && !ok) { st->status = -51; break; }  // the replayed step did not converge
    if (ok && !replay) {
      // StepErrorControl::evaluateStepError (N_TIA_StepErrorControl.C:458-575)
      bool test = (t == p->tstart) ? (stepNumber >= 1 && !beginning) : (stepNumber >= 1);
      if (test) {
        double s = 0;
        for (int i = 0; i < n; ++i) {
          double e = (w.x[i] - xn0[i]) / errwt[i];
          s += e * e;
        }
        estOverTol = ck * std::sqrt(s / n);
        if (!(estOverTol <= 1.0)) { ok = false; st->lte_fail++; }
      }
    }
    if (ok) {
      // OneStep::completeStep (:2124-2240)
      step_order = order;
      numberOfSteps++; nef = 0;
      double tprev = t;
      t = tn;
      double hstep = h;
      lastTimeStep = h;
      double rr = std::pow(0.5 / (estOverTol + 0.0001), 1.0 / (order + 1.0));
      if (numberOfSteps >= 2 && max_order == 2 && order == 1) {
        order = 2;
        rr = std::pow(0.5 / (estOverTol + 0.0001), 1.0 / 3.0);
        if (rr <= 1.05) order = 1;
      }
      double hnew = h;
      if (rr >= 2.0) hnew = 2.0 * h;
      else if (rr <= 1) hnew = std::max(0.25, std::min(0.9, rr)) * h;
      if (gear) {
        // Gear12::updateHistory (N_TIA_Gear12.C:822-870)
        if (order == 2) xh2 = xh1;
        qh1 = qh0;
        xh1 = xh0;
      } else {
        // OneStep::updateHistory (:1390-1440)
        if (order == 2) {
          xh2 = xh1;
          for (int i = 0; i < n; ++i) qh2[i] = w.F[i] - w.B[i];
        }
        for (int i = 0; i < n; ++i) {
          xh1[i] = w.x[i] - xh0[i];
          qh1[i] = w.Q[i] - qh0[i];
        }
      }
      xh0 = w.x; qh0 = w.Q;
      hnew = std::min(std::max(hnew, hmin), hmax);
      // breakpoint handling (Transient::processSuccessfulStep, N_ANP_Transient.C:1860-1950)
      bool hit_bp = std::fabs(t - stopTime) <= bptol && std::fabs(t - p->tstop) > bptol;
      if (hit_bp) {
        saved = hnew;
        beginning = true;
        stopTime = next_bp(t);
      } else {
        beginning = false;
        if (t + hnew > stopTime) { saved = hnew; hnew = stopTime - t; }
        h = hnew;
        tsum = h + lastTimeStep;
      }
      (void)tprev; (void)hstep;
      stepNumber++;
      st->accepted++;
      lastOk = true;
      w.xcurr = w.x; w.sta_curr = w.sta_next; w.sto_curr = w.sto_next;
      Fc = w.F; Qc = w.Q; Bc = w.B;
      record(t, w.xcurr);
      if (c->wall_log && st->accepted <= c->wall_cap) c->wall_log[st->accepted - 1] = now() - tstart_wall;
    } else {
      // OneStep::rejectStep (:1946-2105) and restoreHistory (:1540)
      st->rejected++;
      lastOk = false;
      nef++;
      for (int i = 1; i <= order; ++i) psi[i - 1] = psi[i];
      if (nef >= 15) { st->status = -1; break; }
      double hnew;
      if (ns <= 0) { hnew = h / 8; order = 1; }
      else if (nef == 1) {
        // OneStep drops to first order first; Gear12::rejectStep keeps the
        // order (N_TIA_Gear12.C:1500-1515)
        if (!gear) order = 1;
        double rr = std::pow(0.5 / (estOverTol + 0.0001), 1.0 / (order + 1.0));
        rr = std::max(0.25, std::min(0.9, rr));
        hnew = rr * h;
      } else {
        hnew = 0.25 * h; order = 1;
      }
      hnew = std::min(std::max(hnew, hmin), hmax);
      if (t + hnew > stopTime) hnew = stopTime - t;
      h = hnew;
      tsum = h + lastTimeStep;
      if (h <= 0.0 || !std::isfinite(h)) { st->status = -2; break; }
    }
  }
  st->t_final = t;
  st->time_load = w.t_load;
  st->time_solve = w.t_solve;
  st->time_total = now() - tstart_wall;
  *n_out = nout;
  return st->status;
}

// Elimination order of the LU (the ordering KLU's symbolic analysis
// computes once, AMD on the pattern of A + A^T): perm[k] = the unknown
// eliminated k-th, a permutation of 0..n-1; n = 0 restores the natural order.
extern "C" int orc_set_order(orc_ctx *c, const int *perm, int n) {
  if (!c->finalized) return -1;
  if (n == 0) {
    c->q.clear(); c->qinv.clear();
  } else {
    if (n != c->n) return -1;
    std::vector<int> inv(n, -1);
    for (int k = 0; k < n; ++k) {
      if (perm[k] < 0 || perm[k] >= n || inv[perm[k]] >= 0) return -1;
      inv[perm[k]] = k;
    }
    c->q.assign(perm, perm + n);
    c->qinv = std::move(inv);
    c->pb.assign(n, 0.0); c->px.assign(n, 0.0);
  }
  build_csc(c);
  c->lu_valid = false;
  c->last_factored.clear();
  return 0;
}

// .OPTIONS LINSOL TYPE: 0 refactors every Newton iteration (KLU), 1 is
// IRSolver with its IR_SOLVER_TOL / IR_MIN_TOL (N_LAS_IRSolver.C:131-145).
extern "C" int orc_set_linear_solver(orc_ctx *c, int type, double ir_tol, double ir_min_tol) {
  if (type != 0 && type != 1) return -1;
  if (!(ir_tol > 0.0) || !(ir_min_tol > 0.0)) return -1;
  c->lin_type = type;
  c->ir_tol = ir_tol;
  c->ir_min_tol = ir_min_tol;
  return 0;
}

// Counters of the linear solves since the last reset: factorizations,
// reused solves, refined solves, refinement steps, fallbacks, repeated
// factorizations (the matrix equal bit for bit to the last one factored).
extern "C" int orc_lu_counts(orc_ctx *c, long long *out, int reset) {
  out[0] = c->n_factor; out[1] = c->n_reuse; out[2] = c->n_refined;
  out[3] = c->n_refine_steps; out[4] = c->n_fallback; out[5] = c->n_repeat;
  if (reset)
    c->n_factor = c->n_reuse = c->n_refined = c->n_refine_steps = c->n_fallback = c->n_repeat = 0;
  return 0;
}

// Replay of an accepted-step sequence (test support): times[k] and orders[k]
// of the accepted points, k = 0 the operating point (its order is ignored);
// n = 0 returns to free runs.
extern "C" int orc_set_replay(orc_ctx *c, const double *times, const int *orders, int n) {
  if (n < 0 || (n > 0 && (!times || !orders))) return -1;
  for (int k = 1; k < n; ++k)
    if (!(times[k] > times[k - 1]) || (orders[k] != 1 && orders[k] != 2)) return -1;
  c->replay_t.assign(times, times + n);
  c->replay_o.assign(orders, orders + n);
  return 0;
}

// Integration order of each point the last transient recorded (0 for the
// operating point); returns the count, at most cap.
extern "C" int orc_recorded_orders(orc_ctx *c, int *out, int cap) {
  const int k = std::min(cap, (int)c->rec_o.size());
  for (int i = 0; i < k; ++i) out[i] = c->rec_o[i];
  return k;
}

// Benchmark support: wall-clock time (seconds since the start of the
// transient call) at every accepted step, into buf[0 .. cap).
extern "C" int orc_set_wall_log(orc_ctx *c, double *buf, int cap) {
  c->wall_log = buf;
  c->wall_cap = cap;
  return 0;
}
