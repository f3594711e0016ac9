// xg_api.cpp — the C-ABI of libxyce_gb300.so: context, topology upload,
// stamp-map construction, loader entry points, LU entry points and the
// device-resident transient driver.
#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "xg_internal.h"
#include "xg_params.h"

using namespace xg;

struct Wave {
  int kind;
  std::vector<double> d;
};

struct TranRun;

struct xg_ctx {
  TranRun *run = nullptr;          // transient in progress (xg_tran_start .. xg_tran_end)
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err = "";
  int n = 0, ncirc = 0;
  std::vector<int> offsets;
  bool unknowns_set = false, finalized = false;
  // host copies of the devices
  std::vector<int> r_p, r_n, c_p, c_n, v_p, v_n, v_b, i_p, i_n;
  // MOSFET-1 series conductances (drainConductance * M between d and d',
  // sourceConductance * M between s and s'): constant, in the linear part
  std::vector<int> sg_p, sg_n;
  std::vector<double> sg_v;
  // inductors: pos, neg, branch current unknown, inductance (all constant)
  std::vector<int> ind_p, ind_n, ind_b;
  std::vector<double> ind_l;
  std::vector<double> r_v, c_v;
  std::vector<Wave> v_w, i_w;
  std::vector<int> d_p, d_n, d_r;
  std::vector<double> d_par;
  std::vector<int> m_d, m_g, m_s, m_b;
  std::vector<double> m_par;
  std::vector<int> b_d, b_g, b_s, b_b;
  std::vector<double> b_par;
  // finalized structure
  std::vector<int> rp, ci, circ_of_row;
  std::vector<long long> inst_of_circ;  // nonlinear device instances per circuit
  std::vector<long long> circ_m1, circ_b4, circ_d;  // MOSFET-1 / BSIM4 / diode instances per circuit
  int nnz = 0, nm = 0, nd = 0, nv = 0, ni = 0, nb = 0;
  int nsto = 0, nsta = 0, sto_base_m = 0, sto_base_b = 0, sta_base_b = 0;
  int sF_m = 0, sF_d = 0, sQ_m = 0, sQ_d = 0, sL_m = 0, sL_d = 0, sM_m = 0, sM_d = 0;
  int sF_b = 0, sQ_b = 0, sL_b = 0, sM_b = 0;
  int n_pairs = 0, n_rowblocks = 0, n_long_rows = 0, n_long_ents = 0;
  int n_long_row_blocks = 0, n_long_ent_blocks = 0;
  // circuit of every MOSFET-1, diode and source, and the long rows / long
  // Jacobian entries (kept for the circuit-resident tick's per-circuit lists)
  std::vector<int> m1_circ_h, d_circ_h, src_circ_h, long_rows_h, long_ents_h;
  int form = XG_FORM_AUTO;          // xg_tran_set_form
  double tail_fraction = 0.25;      // xg_tran_set_tail
  bool resident_ok = false;         // the current analysis admits the circuit-resident tick
  FusedDev F;                       // its device lists (allocated with the analysis)
  int resident_slots[8] = {0};
  DevArrays d;
  LUDev L;
  int sched_order = -1, sched_ftop = -1, sched_stop = -1;  // xg_lu_set_schedule (-1: automatic)
  bool lu_ready = false;
  int n_analyze = 0;
  int lu_prec = XG_PREC_FP64, lu_refine = 2;  // xg_lu_set_precision
  int tune_mode = XG_TUNE_TIMED;               // xg_lu_set_tuning
  int fixed_shapes[4] = {0, -1, 0, 0};         // xg_lu_set_shapes: factor threads, meta, L / U solve threads
  int lu_reuse = 1;                            // xg_lu_set_reuse
  double pivot_tol = kRuntimePivotTol;         // xg_lu_set_pivot_tolerance
  std::vector<int> row_of_col_h;               // pivot row of every column in the current analysis
  int lu_gen = 0;                              // analyses uploaded so far
  xg_lu_tuning tuning{};                       // what the tuner chose for the current analysis
  int predictor = XG_PRED_POLY;                // xg_set_predictor
  std::vector<int> h_tlv_item_ptr, h_tlv_grp_ptr;  // host copies for the per-level top launches
  std::vector<int> h_ls_lvl_ptr, h_fs_lvl_ptr;
  bool mlp_ready = false;                      // weights set (xg_mlp_set) or trained
  float *mlp_m1 = nullptr, *mlp_m2 = nullptr, *mlp_grad = nullptr, *mlp_loss = nullptr;
  int mlp_adam_t = 0;
  std::vector<void *> allocs;      // device allocations owned by the context
  std::vector<void *> lu_allocs;   // allocations of the current LU analysis
  int *status_host = nullptr;      // mapped [finished, breakdown, Newton iterations (64-bit)]
  int *status_dev = nullptr;
  int *breakdown_dev = nullptr;
};

void xg_free_run(xg_ctx *ctx);

namespace {

int fail(xg_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(ctx, XG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dev_alloc(xg_ctx *ctx, T **p, size_t count, std::vector<void *> &owner) {
  *p = nullptr;
  size_t bytes = std::max<size_t>(1, count) * sizeof(T);
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess) return fail(ctx, XG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  owner.push_back(*p);
  e = cudaMemsetAsync(*p, 0, bytes, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, XG_ERR_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
  return XG_OK;
}

template <class T>
int dev_upload(xg_ctx *ctx, T **p, const std::vector<T> &v, std::vector<void *> &owner) {
  int rc = dev_alloc(ctx, p, v.size(), owner);
  if (rc) return rc;
  if (!v.empty()) {
    cudaError_t e = cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return fail(ctx, XG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  }
  return XG_OK;
}

void free_list(std::vector<void *> &v) {
  for (void *p : v) cudaFree(p);
  v.clear();
}

bool valid_node(const xg_ctx *c, int i) { return i >= -1 && i < c->n; }

// First circuit among the given nodes (ground ignored).
int circuit_of_nodes(const xg_ctx *c, std::initializer_list<int> nodes) {
  for (int v : nodes)
    if (v >= 0) return c->circ_of_row[v];
  return -1;
}

}  // namespace

extern "C" {

int xg_version(void) { return 100; }

int xg_create(xg_ctx **out, int device) {
  if (!out) return XG_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) return XG_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return XG_ERR_CUDA;
  if (!(prop.major == 10 && prop.minor == 3)) {
    // the kernels are built for sm_103a only; there is no other path
    return XG_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return XG_ERR_CUDA;
  xg_ctx *c = new xg_ctx;
  c->device = device;
  // a blocking stream: ordered with work the caller issued on the legacy default stream
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault) != cudaSuccess) {
    delete c;
    return XG_ERR_CUDA;
  }
  if (cudaHostAlloc((void **)&c->status_host, 4 * sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void **)&c->status_dev, c->status_host, 0) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return XG_ERR_CUDA;
  }
  memset(c->status_host, 0, 4 * sizeof(int));
  *out = c;
  return XG_OK;
}

int xg_destroy(xg_ctx *ctx) {
  if (!ctx) return XG_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->run) xg_free_run(ctx);
  free_list(ctx->lu_allocs);
  free_list(ctx->allocs);
  if (ctx->status_host) cudaFreeHost(ctx->status_host);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return XG_OK;
}

const char *xg_error_string(const xg_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void *xg_get_stream(xg_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int xg_synchronize(xg_ctx *ctx) {
  if (!ctx) return XG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return XG_OK;
}

int xg_set_unknowns(xg_ctx *ctx, int n, int ncirc, const int *offsets) {
  if (!ctx || n <= 0 || ncirc <= 0 || !offsets) return fail(ctx, XG_ERR_ARG, "xg_set_unknowns: bad arguments");
  if (ctx->finalized) return fail(ctx, XG_ERR_STATE, "xg_set_unknowns after finalize");
  if (offsets[0] != 0 || offsets[ncirc] != n) return fail(ctx, XG_ERR_ARG, "offsets must span [0, n]");
  for (int c = 0; c < ncirc; ++c)
    if (offsets[c + 1] <= offsets[c]) return fail(ctx, XG_ERR_ARG, "empty or decreasing circuit range");
  ctx->n = n;
  ctx->ncirc = ncirc;
  ctx->offsets.assign(offsets, offsets + ncirc + 1);
  ctx->circ_of_row.assign(n, 0);
  for (int c = 0; c < ncirc; ++c)
    for (int i = offsets[c]; i < offsets[c + 1]; ++i) ctx->circ_of_row[i] = c;
  ctx->unknowns_set = true;
  return XG_OK;
}

// Common checks of the xg_add_* calls.  Each call validates all n items
// before it appends any, so a rejected call leaves the topology as it was.
#define SETUP_CHECK(...)                                                               \
  if (!ctx) return XG_ERR_ARG;                                                         \
  if (!ctx->unknowns_set) return fail(ctx, XG_ERR_STATE, "call xg_set_unknowns first"); \
  if (ctx->finalized) return fail(ctx, XG_ERR_STATE, "topology is already finalized"); \
  if (n < 0) return fail(ctx, XG_ERR_ARG, "negative count");                           \
  if (n > 0 && !all_set({__VA_ARGS__})) return fail(ctx, XG_ERR_ARG, "null array");

static bool all_set(std::initializer_list<const void *> ptrs) {
  for (const void *p : ptrs)
    if (!p) return false;
  return true;
}

int xg_add_resistors(xg_ctx *ctx, int n, const int *pos, const int *neg, const double *r) {
  SETUP_CHECK(pos, neg, r);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, pos[k]) || !valid_node(ctx, neg[k])) return fail(ctx, XG_ERR_ARG, "resistor node out of range");
    if (!(r[k] != 0.0) || !std::isfinite(r[k])) return fail(ctx, XG_ERR_ARG, "resistor value must be finite and nonzero");
  }
  ctx->r_p.insert(ctx->r_p.end(), pos, pos + n);
  ctx->r_n.insert(ctx->r_n.end(), neg, neg + n);
  ctx->r_v.insert(ctx->r_v.end(), r, r + n);
  return XG_OK;
}

int xg_add_inductors(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *branch, const double *l) {
  SETUP_CHECK(pos, neg, branch, l);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, pos[k]) || !valid_node(ctx, neg[k]) || branch[k] < 0 || branch[k] >= ctx->n)
      return fail(ctx, XG_ERR_ARG, "inductor node or branch out of range");
    if (!std::isfinite(l[k])) return fail(ctx, XG_ERR_ARG, "inductance must be finite");
  }
  ctx->ind_p.insert(ctx->ind_p.end(), pos, pos + n);
  ctx->ind_n.insert(ctx->ind_n.end(), neg, neg + n);
  ctx->ind_b.insert(ctx->ind_b.end(), branch, branch + n);
  ctx->ind_l.insert(ctx->ind_l.end(), l, l + n);
  return XG_OK;
}

int xg_add_capacitors(xg_ctx *ctx, int n, const int *pos, const int *neg, const double *cv) {
  SETUP_CHECK(pos, neg, cv);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, pos[k]) || !valid_node(ctx, neg[k])) return fail(ctx, XG_ERR_ARG, "capacitor node out of range");
    if (!std::isfinite(cv[k])) return fail(ctx, XG_ERR_ARG, "capacitor value must be finite");
  }
  ctx->c_p.insert(ctx->c_p.end(), pos, pos + n);
  ctx->c_n.insert(ctx->c_n.end(), neg, neg + n);
  ctx->c_v.insert(ctx->c_v.end(), cv, cv + n);
  return XG_OK;
}

// Waveform k of a source list: kind, and its values data[off[k] .. off[k+1]).
static int check_wave(xg_ctx *ctx, int kind, int first, int end) {
  static const int need[4] = {1, 6, 7, 2};
  const int len = end - first;
  if (first < 0) return fail(ctx, XG_ERR_ARG, "negative waveform offset");
  if (kind < 0 || kind > 3) return fail(ctx, XG_ERR_ARG, "unknown waveform kind");
  if (len < need[kind]) return fail(ctx, XG_ERR_ARG, "waveform has too few values");
  if (kind == XG_WAVE_PWL && (len % 2) != 0) return fail(ctx, XG_ERR_ARG, "PWL needs time/value pairs");
  return XG_OK;
}

int xg_add_vsources(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *branch, const int *kind,
                    const int *off, const double *data) {
  SETUP_CHECK(pos, neg, branch, kind, off, data);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, pos[k]) || !valid_node(ctx, neg[k]) || branch[k] < 0 || branch[k] >= ctx->n)
      return fail(ctx, XG_ERR_ARG, "voltage source node out of range");
    int rc = check_wave(ctx, kind[k], off[k], off[k + 1]);
    if (rc) return rc;
  }
  for (int k = 0; k < n; ++k) {
    ctx->v_p.push_back(pos[k]); ctx->v_n.push_back(neg[k]); ctx->v_b.push_back(branch[k]);
    ctx->v_w.push_back({kind[k], std::vector<double>(data + off[k], data + off[k + 1])});
  }
  return XG_OK;
}

int xg_add_isources(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *kind, const int *off,
                    const double *data) {
  SETUP_CHECK(pos, neg, kind, off, data);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, pos[k]) || !valid_node(ctx, neg[k])) return fail(ctx, XG_ERR_ARG, "current source node out of range");
    int rc = check_wave(ctx, kind[k], off[k], off[k + 1]);
    if (rc) return rc;
  }
  for (int k = 0; k < n; ++k) {
    ctx->i_p.push_back(pos[k]); ctx->i_n.push_back(neg[k]);
    ctx->i_w.push_back({kind[k], std::vector<double>(data + off[k], data + off[k + 1])});
  }
  return XG_OK;
}

int xg_add_diodes(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *pri, const double *params) {
  SETUP_CHECK(pos, neg, pri, params);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, pos[k]) || !valid_node(ctx, neg[k]) || !valid_node(ctx, pri[k]))
      return fail(ctx, XG_ERR_ARG, "diode node out of range");
    const double *p = params + (size_t)k * XG_DIODE_NPARAM;
    if ((p[XG_DIODE_RS] == 0.0) != (pri[k] == pos[k]))
      return fail(ctx, XG_ERR_ARG, "diode internal node must equal pos exactly when RS = 0");
    if (!(p[XG_DIODE_TEMP] > 0.0) || !(p[XG_DIODE_TNOM] > 0.0) || !std::isfinite(p[XG_DIODE_TEMP]) ||
        !std::isfinite(p[XG_DIODE_TNOM]))
      return fail(ctx, XG_ERR_ARG, "diode TEMP and TNOM are kelvin: positive and finite");
  }
  ctx->d_p.insert(ctx->d_p.end(), pos, pos + n);
  ctx->d_n.insert(ctx->d_n.end(), neg, neg + n);
  ctx->d_r.insert(ctx->d_r.end(), pri, pri + n);
  ctx->d_par.insert(ctx->d_par.end(), params, params + (size_t)n * XG_DIODE_NPARAM);
  return XG_OK;
}

// Series drain or source conductance (Instance::processParams,
// N_DEV_MOSFET1.C:410-450): 1/R when R is nonzero, else 1/(RSH * squares)
// when RSH is nonzero, else 0.
static double mos1_series_conductance(double r, double rsh, double squares) {
  if (r != 0.0) return 1.0 / r;
  if (rsh != 0.0) return 1.0 / (rsh * squares);
  return 0.0;
}

// dp / sp null: the row must have no series resistance (xg_add_mosfet1).
static int add_mosfet1(xg_ctx *ctx, int n, const int *dd, const int *g, const int *s, const int *b,
                       const int *dp, const int *sp, const double *params) {
  std::vector<double> gd(n), gs(n);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, dd[k]) || !valid_node(ctx, g[k]) || !valid_node(ctx, s[k]) || !valid_node(ctx, b[k]))
      return fail(ctx, XG_ERR_ARG, "MOSFET node out of range");
    const double *p = params + (size_t)k * XG_MOS1_NPARAM;
    if (p[XG_MOS1_TYPE] != 1.0 && p[XG_MOS1_TYPE] != -1.0) return fail(ctx, XG_ERR_ARG, "MOSFET TYPE must be +1 or -1");
    if (!(p[XG_MOS1_TEMP] > 0.0) || !(p[XG_MOS1_TNOM] > 0.0) || !std::isfinite(p[XG_MOS1_TEMP]) ||
        !std::isfinite(p[XG_MOS1_TNOM]))
      return fail(ctx, XG_ERR_ARG, "MOSFET TEMP and TNOM are kelvin: positive and finite");
    gd[k] = mos1_series_conductance(p[XG_MOS1_RD], p[XG_MOS1_RSH], p[XG_MOS1_NRD]);
    gs[k] = mos1_series_conductance(p[XG_MOS1_RS], p[XG_MOS1_RSH], p[XG_MOS1_NRS]);
    if (!std::isfinite(gd[k]) || !std::isfinite(gs[k]) || !std::isfinite(gd[k] * p[XG_MOS1_M]) ||
        !std::isfinite(gs[k] * p[XG_MOS1_M]))
      return fail(ctx, XG_ERR_ARG, "MOSFET series conductance (RD, RS, RSH * NRD / NRS) must be finite");
    if (!dp) {
      if (gd[k] != 0.0 || gs[k] != 0.0)
        return fail(ctx, XG_ERR_ARG, "MOSFET series resistance needs the internal nodes: use xg_add_mosfet1_rs");
      continue;
    }
    if (!valid_node(ctx, dp[k]) || !valid_node(ctx, sp[k])) return fail(ctx, XG_ERR_ARG, "MOSFET node out of range");
    if ((gd[k] != 0.0) == (dp[k] == dd[k]))
      return fail(ctx, XG_ERR_ARG, "MOSFET drain' must differ from drain exactly when the drain conductance is nonzero");
    if ((gs[k] != 0.0) == (sp[k] == s[k]))
      return fail(ctx, XG_ERR_ARG, "MOSFET source' must differ from source exactly when the source conductance is nonzero");
    if ((gd[k] != 0.0 && dp[k] < 0) || (gs[k] != 0.0 && sp[k] < 0))
      return fail(ctx, XG_ERR_ARG, "MOSFET drain'/source' internal node cannot be ground");
  }
  ctx->m_d.insert(ctx->m_d.end(), dp ? dp : dd, (dp ? dp : dd) + n);
  ctx->m_g.insert(ctx->m_g.end(), g, g + n);
  ctx->m_s.insert(ctx->m_s.end(), sp ? sp : s, (sp ? sp : s) + n);
  ctx->m_b.insert(ctx->m_b.end(), b, b + n);
  ctx->m_par.insert(ctx->m_par.end(), params, params + (size_t)n * XG_MOS1_NPARAM);
  for (int k = 0; dp && k < n; ++k) {
    const double M = params[(size_t)k * XG_MOS1_NPARAM + XG_MOS1_M];
    if (gd[k] != 0.0) { ctx->sg_p.push_back(dd[k]); ctx->sg_n.push_back(dp[k]); ctx->sg_v.push_back(gd[k] * M); }
    if (gs[k] != 0.0) { ctx->sg_p.push_back(s[k]); ctx->sg_n.push_back(sp[k]); ctx->sg_v.push_back(gs[k] * M); }
  }
  return XG_OK;
}

int xg_add_mosfet1(xg_ctx *ctx, int n, const int *dd, const int *g, const int *s, const int *b,
                   const double *params) {
  SETUP_CHECK(dd, g, s, b, params);
  return add_mosfet1(ctx, n, dd, g, s, b, nullptr, nullptr, params);
}

int xg_add_mosfet1_rs(xg_ctx *ctx, int n, const int *dd, const int *g, const int *s, const int *b,
                      const int *dp, const int *sp, const double *params) {
  SETUP_CHECK(dd, g, s, b, dp, sp, params);
  return add_mosfet1(ctx, n, dd, g, s, b, dp, sp, params);
}

int xg_add_bsim4(xg_ctx *ctx, int n, const int *dd, const int *g, const int *s, const int *b,
                 const double *params) {
  SETUP_CHECK(dd, g, s, b, params);
  for (int k = 0; k < n; ++k) {
    if (!valid_node(ctx, dd[k]) || !valid_node(ctx, g[k]) || !valid_node(ctx, s[k]) || !valid_node(ctx, b[k]))
      return fail(ctx, XG_ERR_ARG, "BSIM4 node out of range");
    const double *p = params + (size_t)k * XG_B4_NPARAM;
    b4::B4Model probe;
    std::string why;
    int rc = b4::setup(p, probe, &why);
    if (rc) return fail(ctx, rc, "BSIM4: " + why);
  }
  ctx->b_d.insert(ctx->b_d.end(), dd, dd + n);
  ctx->b_g.insert(ctx->b_g.end(), g, g + n);
  ctx->b_s.insert(ctx->b_s.end(), s, s + n);
  ctx->b_b.insert(ctx->b_b.end(), b, b + n);
  ctx->b_par.insert(ctx->b_par.end(), params, params + (size_t)n * XG_B4_NPARAM);
  return XG_OK;
}

// ---------------------------------------------------------------------------
// finalize: pattern, stamp map, SoA tables, device buffers.
int xg_finalize(xg_ctx *ctx) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->unknowns_set) return fail(ctx, XG_ERR_STATE, "call xg_set_unknowns first");
  if (ctx->finalized) return fail(ctx, XG_ERR_STATE, "already finalized");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->n;
  ctx->nm = (int)ctx->m_d.size();
  ctx->nb = (int)ctx->b_d.size();
  ctx->nd = (int)ctx->d_p.size();
  ctx->nv = (int)ctx->v_p.size();
  ctx->ni = (int)ctx->i_p.size();
  const int nm = ctx->nm, nd = ctx->nd, nv = ctx->nv, ni = ctx->ni, nb = ctx->nb;
  // device circuits must not straddle circuits
  auto same_circuit = [&](std::initializer_list<int> nodes) {
    int c = -2;
    for (int v : nodes) {
      if (v < 0) continue;
      int cc = ctx->circ_of_row[v];
      if (c == -2) c = cc;
      else if (c != cc) return false;
    }
    return true;
  };
  for (int k = 0; k < nm; ++k)
    if (!same_circuit({ctx->m_d[k], ctx->m_g[k], ctx->m_s[k], ctx->m_b[k]})) return fail(ctx, XG_ERR_ARG, "MOSFET spans two circuits");
  for (int k = 0; k < nd; ++k)
    if (!same_circuit({ctx->d_p[k], ctx->d_n[k], ctx->d_r[k]})) return fail(ctx, XG_ERR_ARG, "diode spans two circuits");
  for (int k = 0; k < nb; ++k)
    if (!same_circuit({ctx->b_d[k], ctx->b_g[k], ctx->b_s[k], ctx->b_b[k]})) return fail(ctx, XG_ERR_ARG, "BSIM4 spans two circuits");
  for (size_t k = 0; k < ctx->r_p.size(); ++k)
    if (!same_circuit({ctx->r_p[k], ctx->r_n[k]})) return fail(ctx, XG_ERR_ARG, "resistor spans two circuits");
  for (size_t k = 0; k < ctx->sg_p.size(); ++k)
    if (!same_circuit({ctx->sg_p[k], ctx->sg_n[k]})) return fail(ctx, XG_ERR_ARG, "MOSFET spans two circuits");
  for (size_t k = 0; k < ctx->ind_p.size(); ++k)
    if (!same_circuit({ctx->ind_p[k], ctx->ind_n[k], ctx->ind_b[k]})) return fail(ctx, XG_ERR_ARG, "inductor spans two circuits");
  for (size_t k = 0; k < ctx->c_p.size(); ++k)
    if (!same_circuit({ctx->c_p[k], ctx->c_n[k]})) return fail(ctx, XG_ERR_ARG, "capacitor spans two circuits");
  for (int k = 0; k < nv; ++k)
    if (!same_circuit({ctx->v_p[k], ctx->v_n[k], ctx->v_b[k]}))
      return fail(ctx, XG_ERR_ARG, "voltage source spans two circuits");
  for (int k = 0; k < ni; ++k)
    if (!same_circuit({ctx->i_p[k], ctx->i_n[k]})) return fail(ctx, XG_ERR_ARG, "current source spans two circuits");
  {
    // two voltage sources on one branch unknown would share its row
    std::vector<char> seen(n, 0);
    for (int k = 0; k < nv; ++k) {
      if (seen[ctx->v_b[k]]) return fail(ctx, XG_ERR_ARG, "two voltage sources share a branch unknown");
      seen[ctx->v_b[k]] = 1;
    }
    for (size_t k = 0; k < ctx->ind_b.size(); ++k) {
      if (seen[ctx->ind_b[k]]) return fail(ctx, XG_ERR_ARG, "an inductor's branch unknown is shared");
      seen[ctx->ind_b[k]] = 1;
    }
  }
  // matrix stamp positions (row, col); -1 for ground rows/cols.  Every
  // position is enumerated twice (count, then fill) into one flat array, and
  // each row is sorted and deduplicated in place.  Node unknowns keep a
  // diagonal entry (the operating-point gmin shunt lands there); voltage-source
  // branch rows have none, as in the device stamps.
  std::vector<char> is_branch(n, 0);
  for (int k = 0; k < nv; ++k) is_branch[ctx->v_b[k]] = 1;
  for (int b : ctx->ind_b) is_branch[b] = 1;
  const int dpair[7][2] = {{0, 0}, {0, 2}, {1, 1}, {1, 2}, {2, 0}, {2, 1}, {2, 2}};
  auto for_positions = [&](auto &&emit) {
    for (size_t k = 0; k < ctx->r_p.size(); ++k) {
      int p = ctx->r_p[k], m = ctx->r_n[k];
      emit(p, p); emit(p, m); emit(m, p); emit(m, m);
    }
    for (size_t k = 0; k < ctx->sg_p.size(); ++k) {
      int p = ctx->sg_p[k], m = ctx->sg_n[k];
      emit(p, p); emit(p, m); emit(m, p); emit(m, m);
    }
    for (size_t k = 0; k < ctx->c_p.size(); ++k) {
      int p = ctx->c_p[k], m = ctx->c_n[k];
      emit(p, p); emit(p, m); emit(m, p); emit(m, m);
    }
    for (int k = 0; k < nv; ++k) {
      int p = ctx->v_p[k], m = ctx->v_n[k], b = ctx->v_b[k];
      emit(p, b); emit(m, b); emit(b, p); emit(b, m);
    }
    for (size_t k = 0; k < ctx->ind_p.size(); ++k) {
      int p = ctx->ind_p[k], m = ctx->ind_n[k], b = ctx->ind_b[k];
      emit(p, b); emit(m, b); emit(b, p); emit(b, m); emit(b, b);
    }
    for (int k = 0; k < nd; ++k) {
      int nn[3] = {ctx->d_p[k], ctx->d_n[k], ctx->d_r[k]};
      for (auto &pr : dpair) emit(nn[pr[0]], nn[pr[1]]);
    }
    for (int k = 0; k < nm; ++k) {
      int nn[4] = {ctx->m_d[k], ctx->m_g[k], ctx->m_s[k], ctx->m_b[k]};
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) emit(nn[a], nn[b]);
    }
    for (int k = 0; k < nb; ++k) {
      int nn[4] = {ctx->b_d[k], ctx->b_g[k], ctx->b_s[k], ctx->b_b[k]};
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) emit(nn[a], nn[b]);
    }
    for (int i = 0; i < n; ++i)
      if (!is_branch[i]) emit(i, i);
  };
  {
    std::vector<long long> cnt(n + 1, 0);
    for_positions([&](int r, int c) { if (r >= 0 && c >= 0) cnt[r + 1]++; });
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> flat(cnt[n]);
    std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
    for_positions([&](int r, int c) { if (r >= 0 && c >= 0) flat[fill[r]++] = c; });
    ctx->rp.assign(n + 1, 0);
    ctx->ci.clear();
    ctx->ci.reserve(flat.size());
    for (int i = 0; i < n; ++i) {
      auto b = flat.begin() + cnt[i], e = flat.begin() + cnt[i + 1];
      std::sort(b, e);
      e = std::unique(b, e);
      ctx->ci.insert(ctx->ci.end(), b, e);
      ctx->rp[i + 1] = (int)ctx->ci.size();
    }
  }
  const int nnz = ctx->nnz = (int)ctx->ci.size();
  auto find = [&](int r, int c) -> int {
    if (r < 0 || c < 0) return -1;
    auto b = ctx->ci.begin() + ctx->rp[r], e = ctx->ci.begin() + ctx->rp[r + 1];
    auto it = std::lower_bound(b, e, c);
    return (int)(it - ctx->ci.begin());
  };
  std::vector<int> erow(nnz);
  for (int i = 0; i < n; ++i)
    for (int e = ctx->rp[i]; e < ctx->rp[i + 1]; ++e) erow[e] = i;
  // linear part: constant G (R, V incidence) and C values per CSR entry
  std::vector<double> Glin(nnz, 0.0), Clin(nnz, 0.0);
  auto addv = [&](std::vector<double> &v, int r, int c, double x) { int e = find(r, c); if (e >= 0) v[e] += x; };
  for (size_t k = 0; k < ctx->r_p.size(); ++k) {
    int p = ctx->r_p[k], m = ctx->r_n[k];
    double G = 1.0 / ctx->r_v[k];
    addv(Glin, p, p, G); addv(Glin, p, m, -G); addv(Glin, m, p, -G); addv(Glin, m, m, G);
  }
  for (size_t k = 0; k < ctx->sg_p.size(); ++k) {
    int p = ctx->sg_p[k], m = ctx->sg_n[k];
    double G = ctx->sg_v[k];
    addv(Glin, p, p, G); addv(Glin, p, m, -G); addv(Glin, m, p, -G); addv(Glin, m, m, G);
  }
  for (size_t k = 0; k < ctx->c_p.size(); ++k) {
    int p = ctx->c_p[k], m = ctx->c_n[k];
    double C = ctx->c_v[k];
    addv(Clin, p, p, C); addv(Clin, p, m, -C); addv(Clin, m, p, -C); addv(Clin, m, m, C);
  }
  for (int k = 0; k < nv; ++k) {
    int p = ctx->v_p[k], m = ctx->v_n[k], b = ctx->v_b[k];
    addv(Glin, p, b, 1.0); addv(Glin, m, b, -1.0); addv(Glin, b, p, 1.0); addv(Glin, b, m, -1.0);
  }
  // inductors (N_DEV_Inductor.C:540-650): F[p] += i, F[n] -= i,
  // F[b] -= v(p) - v(n), Q[b] = L i
  for (size_t k = 0; k < ctx->ind_p.size(); ++k) {
    int p = ctx->ind_p[k], m = ctx->ind_n[k], b = ctx->ind_b[k];
    addv(Glin, p, b, 1.0); addv(Glin, m, b, -1.0); addv(Glin, b, p, -1.0); addv(Glin, b, m, 1.0);
    addv(Clin, b, b, ctx->ind_l[k]);
  }
  // slot layout: MOSFET level 1, then BSIM4 (same slot counts), then
  // diodes, plane-major within a type
  const int nmb = nm + nb;
  ctx->sF_m = 0; ctx->sF_b = kMosF * nm; ctx->sF_d = kMosF * nmb;
  ctx->sQ_m = 0; ctx->sQ_b = kMosQ * nm; ctx->sQ_d = kMosQ * nmb;
  ctx->sL_m = 0; ctx->sL_b = kMosL * nm; ctx->sL_d = kMosL * nmb;
  ctx->sM_m = 0; ctx->sM_b = kMosM * nm; ctx->sM_d = kMosM * nmb;
  const int nF = kMosF * nmb + kDioF * nd, nQ = kMosQ * nmb + kDioQ * nd, nL = kMosL * nmb + kDioL * nd;
  const int nMs = kMosM * nmb + kDioM * nd, nB = nv + 2 * ni;
  // contribution lists (row -> slots, CSR entry -> slots): every push is
  // recorded as (key, slot) in order, then a stable counting sort by key
  // gives each row's / entry's slots in push order (the gathers sum them in
  // that order)
  struct Contrib {
    std::vector<int> key, slot;
  };
  Contrib lF, lQ, lL, lB, lM;
  auto pushv = [&](Contrib &l, int r, int slot) { if (r >= 0) { l.key.push_back(r); l.slot.push_back(slot); } };
  for (int k = 0; k < nm; ++k) {
    int D = ctx->m_d[k], G = ctx->m_g[k], S = ctx->m_s[k], B = ctx->m_b[k];
    pushv(lF, D, ctx->sF_m + 0 * nm + k); pushv(lF, S, ctx->sF_m + 1 * nm + k); pushv(lF, B, ctx->sF_m + 2 * nm + k);
    int qn[4] = {G, B, D, S};
    for (int j = 0; j < 4; ++j) { pushv(lQ, qn[j], ctx->sQ_m + j * nm + k); pushv(lL, qn[j], ctx->sL_m + j * nm + k); }
    int nn[4] = {D, G, S, B};
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) pushv(lM, find(nn[a], nn[b]), ctx->sM_m + (4 * a + b) * nm + k);
  }
  for (int k = 0; k < nb; ++k) {
    int D = ctx->b_d[k], G = ctx->b_g[k], S = ctx->b_s[k], B = ctx->b_b[k];
    pushv(lF, D, ctx->sF_b + 0 * nb + k); pushv(lF, S, ctx->sF_b + 1 * nb + k); pushv(lF, B, ctx->sF_b + 2 * nb + k);
    int qn[4] = {G, B, D, S};
    for (int j = 0; j < 4; ++j) { pushv(lQ, qn[j], ctx->sQ_b + j * nb + k); pushv(lL, qn[j], ctx->sL_b + j * nb + k); }
    int nn[4] = {D, G, S, B};
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) pushv(lM, find(nn[a], nn[b]), ctx->sM_b + (4 * a + b) * nb + k);
  }
  for (int k = 0; k < nd; ++k) {
    int P = ctx->d_p[k], N = ctx->d_n[k], R = ctx->d_r[k];
    int fn[3] = {P, N, R};
    for (int j = 0; j < 3; ++j) pushv(lF, fn[j], ctx->sF_d + j * nd + k);
    int qn[2] = {N, R};
    for (int j = 0; j < 2; ++j) { pushv(lQ, qn[j], ctx->sQ_d + j * nd + k); pushv(lL, qn[j], ctx->sL_d + j * nd + k); }
    int nn[3] = {P, N, R};
    for (int s = 0; s < 7; ++s) pushv(lM, find(nn[dpair[s][0]], nn[dpair[s][1]]), ctx->sM_d + s * nd + k);
  }
  for (int k = 0; k < nv; ++k) pushv(lB, ctx->v_b[k], k);
  for (int k = 0; k < ni; ++k) { pushv(lB, ctx->i_p[k], nv + 2 * k); pushv(lB, ctx->i_n[k], nv + 2 * k + 1); }
  auto flatten = [&](Contrib &l, int nkeys, std::vector<int> &ptr, std::vector<int> &idx) {
    ptr.assign(nkeys + 1, 0);
    for (int k : l.key) ptr[k + 1]++;
    for (int i = 0; i < nkeys; ++i) ptr[i + 1] += ptr[i];
    idx.assign(l.key.size(), 0);
    std::vector<int> f(ptr.begin(), ptr.end() - 1);
    for (size_t t = 0; t < l.key.size(); ++t) idx[f[l.key[t]]++] = l.slot[t];
    std::vector<int>().swap(l.key);
    std::vector<int>().swap(l.slot);
  };
  std::vector<int> pF, iF, pQ, iQ, pL, iL, pB, iB, pM, iM;
  flatten(lF, n, pF, iF); flatten(lQ, n, pQ, iQ); flatten(lL, n, pL, iL); flatten(lB, n, pB, iB);
  flatten(lM, nnz, pM, iM);
  // Rows and entries with long gathers (a supply node touches every PMOS) are
  // reduced by a whole block in a pre-pass instead of one thread.
  std::vector<int> long_rows, row_long(n, -1), long_ents, ent_long(nnz, -1);
  for (int i = 0; i < n; ++i) {
    int work = (ctx->rp[i + 1] - ctx->rp[i]) + (pF[i + 1] - pF[i]) + (pQ[i + 1] - pQ[i]) +
               (pB[i + 1] - pB[i]) + (pL[i + 1] - pL[i]);
    if (work > kLongGather) { row_long[i] = (int)long_rows.size(); long_rows.push_back(i); }
  }
  for (int e = 0; e < nnz; ++e)
    if (pM[e + 1] - pM[e] > kLongGather) { ent_long[e] = (int)long_ents.size(); long_ents.push_back(e); }
  ctx->n_long_rows = (int)long_rows.size();
  ctx->n_long_ents = (int)long_ents.size();
  // blocks of the long gathers: ceil(items / kLongPart) each
  std::vector<int> lrow_ptr(1, 0), lrow_blk, lent_ptr(1, 0), lent_blk;
  for (int l = 0; l < (int)long_rows.size(); ++l) {
    const int i = long_rows[l];
    const int work = (ctx->rp[i + 1] - ctx->rp[i]) + (pF[i + 1] - pF[i]) + (pQ[i + 1] - pQ[i]) +
                     (pB[i + 1] - pB[i]) + (pL[i + 1] - pL[i]);
    const int parts = std::max(1, (work + kLongPart - 1) / kLongPart);
    for (int b = 0; b < parts; ++b) lrow_blk.push_back(l);
    lrow_ptr.push_back(lrow_ptr.back() + parts);
  }
  for (int l = 0; l < (int)long_ents.size(); ++l) {
    const int e = long_ents[l];
    const int parts = std::max(1, (pM[e + 1] - pM[e] + kLongPart - 1) / kLongPart);
    for (int b = 0; b < parts; ++b) lent_blk.push_back(l);
    lent_ptr.push_back(lent_ptr.back() + parts);
  }
  ctx->n_long_row_blocks = lrow_ptr.back();
  ctx->n_long_ent_blocks = lent_ptr.back();
  // sources (V first, then I)
  std::vector<int> skind, soff(1, 0), scirc;
  std::vector<double> sdata;
  for (int k = 0; k < nv; ++k) {
    skind.push_back(ctx->v_w[k].kind);
    sdata.insert(sdata.end(), ctx->v_w[k].d.begin(), ctx->v_w[k].d.end());
    soff.push_back((int)sdata.size());
    scirc.push_back(ctx->circ_of_row[ctx->v_b[k]]);
  }
  for (int k = 0; k < ni; ++k) {
    skind.push_back(ctx->i_w[k].kind);
    sdata.insert(sdata.end(), ctx->i_w[k].d.begin(), ctx->i_w[k].d.end());
    soff.push_back((int)sdata.size());
    int c = circuit_of_nodes(ctx, {ctx->i_p[k], ctx->i_n[k]});
    scirc.push_back(c < 0 ? 0 : c);
  }
  // MOSFET SoA with effective-model dedup
  std::vector<int> m1node(4 * (size_t)nm), m1model(nm), m1circ(nm);
  std::vector<double> m1beta(nm), m1vbi(nm);
  std::vector<Mos1Model> models;
  std::map<std::vector<double>, int> model_index;
  for (int k = 0; k < nm; ++k) {
    Mos1Instance mi = mos1_instance(&ctx->m_par[(size_t)k * XG_MOS1_NPARAM]);
    if (!mi.valid) return fail(ctx, XG_ERR_ARG, "MOSFET effective channel length or width is not positive");
    const double *mp = reinterpret_cast<const double *>(&mi.model);
    std::vector<double> key(mp, mp + offsetof(Mos1Model, has_gate_caps) / sizeof(double));
    auto it = model_index.find(key);
    int id;
    if (it == model_index.end()) {
      id = (int)models.size();
      model_index.emplace(key, id);
      models.push_back(mi.model);
    } else {
      id = it->second;
    }
    m1model[k] = id;
    m1beta[k] = mi.beta;
    m1vbi[k] = mi.tVbi;
    m1node[k] = ctx->m_d[k]; m1node[nm + k] = ctx->m_g[k];
    m1node[2 * (size_t)nm + k] = ctx->m_s[k]; m1node[3 * (size_t)nm + k] = ctx->m_b[k];
    int c = circuit_of_nodes(ctx, {ctx->m_d[k], ctx->m_g[k], ctx->m_s[k], ctx->m_b[k]});
    m1circ[k] = c < 0 ? 0 : c;
  }
  std::vector<int> dnode(3 * (size_t)nd), dmodel(nd), dcirc(nd);
  std::vector<DiodeModel> dmodels;
  std::map<std::vector<double>, int> dindex;
  for (int k = 0; k < nd; ++k) {
    std::vector<double> key(&ctx->d_par[(size_t)k * XG_DIODE_NPARAM], &ctx->d_par[(size_t)(k + 1) * XG_DIODE_NPARAM]);
    auto it = dindex.find(key);
    int id;
    if (it == dindex.end()) {
      id = (int)dmodels.size();
      dindex.emplace(key, id);
      dmodels.push_back(diode_model(key.data()));
    } else {
      id = it->second;
    }
    dmodel[k] = id;
    dnode[k] = ctx->d_p[k]; dnode[nd + k] = ctx->d_n[k]; dnode[2 * (size_t)nd + k] = ctx->d_r[k];
    int c = circuit_of_nodes(ctx, {ctx->d_p[k], ctx->d_n[k], ctx->d_r[k]});
    dcirc[k] = c < 0 ? 0 : c;
  }
  // BSIM4 SoA with a table of evaluated cards (one per distinct row)
  std::vector<int> b4node(4 * (size_t)nb), b4model(nb), b4circ(nb);
  std::vector<b4::B4Model> b4models;
  std::map<std::vector<double>, int> b4index;
  for (int k = 0; k < nb; ++k) {
    const double *row = &ctx->b_par[(size_t)k * XG_B4_NPARAM];
    std::vector<double> key(row, row + XG_B4_NPARAM);
    for (double &v : key)
      if (std::isnan(v)) v = -1.2345e-300;  // NaN never compares equal: give "not given" one key
    auto it = b4index.find(key);
    int id;
    if (it == b4index.end()) {
      b4::B4Model m;
      std::string why;
      int rc = b4::setup(row, m, &why);
      if (rc) return fail(ctx, rc, "BSIM4: " + why);
      id = (int)b4models.size();
      b4index.emplace(key, id);
      b4models.push_back(m);
    } else {
      id = it->second;
    }
    b4model[k] = id;
    b4node[k] = ctx->b_d[k]; b4node[nb + k] = ctx->b_g[k];
    b4node[2 * (size_t)nb + k] = ctx->b_s[k]; b4node[3 * (size_t)nb + k] = ctx->b_b[k];
    int c = circuit_of_nodes(ctx, {ctx->b_d[k], ctx->b_g[k], ctx->b_s[k], ctx->b_b[k]});
    b4circ[k] = c < 0 ? 0 : c;
  }
  ctx->m1_circ_h = m1circ;
  ctx->d_circ_h = dcirc;
  ctx->src_circ_h = scirc;
  ctx->long_rows_h = long_rows;
  ctx->long_ents_h = long_ents;
  ctx->inst_of_circ.assign(ctx->ncirc, 0);
  ctx->circ_m1.assign(ctx->ncirc, 0);
  ctx->circ_b4.assign(ctx->ncirc, 0);
  ctx->circ_d.assign(ctx->ncirc, 0);
  for (int k = 0; k < nm; ++k) ctx->circ_m1[m1circ[k]]++;
  for (int k = 0; k < nb; ++k) ctx->circ_b4[b4circ[k]]++;
  for (int k = 0; k < nd; ++k) ctx->circ_d[dcirc[k]]++;
  for (int c = 0; c < ctx->ncirc; ++c) ctx->inst_of_circ[c] = ctx->circ_m1[c] + ctx->circ_b4[c] + ctx->circ_d[c];
  // row blocks x circuits partial slots
  const int nblocks = (n + kRowBlock - 1) / kRowBlock;
  std::vector<int> pair_base(nblocks + 1), blk_cfirst(nblocks), pair_cstart(ctx->ncirc + 1, 0);
  int pairs = 0;
  std::vector<int> pair_circ;
  for (int b = 0; b < nblocks; ++b) {
    int r0 = b * kRowBlock, r1 = std::min(n, r0 + kRowBlock);
    int c0 = ctx->circ_of_row[r0], c1 = ctx->circ_of_row[r1 - 1];
    blk_cfirst[b] = c0;
    pair_base[b] = pairs;
    for (int c = c0; c <= c1; ++c) pair_circ.push_back(c);
    pairs += c1 - c0 + 1;
  }
  pair_base[nblocks] = pairs;
  // pairs are ordered by block then circuit, hence by circuit too
  for (int p = 0; p < pairs; ++p) pair_cstart[pair_circ[p] + 1]++;
  for (int c = 0; c < ctx->ncirc; ++c) pair_cstart[c + 1] += pair_cstart[c];
  ctx->n_pairs = pairs;
  ctx->n_rowblocks = nblocks;
  // state layout (SoA): store = diode [vd qd cd] then MOSFET [vbd vbs vgs vds von gm]; state = MOSFET 8 planes
  ctx->sto_base_m = 3 * nd;
  ctx->sto_base_b = 3 * nd + 6 * nm;   // BSIM4 store [vbd vbs vgs vds von]
  ctx->sta_base_b = 8 * nm;            // BSIM4 state [qg qd qb]
  ctx->nsto = 3 * nd + 6 * nm + 5 * nb;
  ctx->nsta = 8 * nm + 3 * nb;
  // upload
  DevArrays &d = ctx->d;
  auto &A = ctx->allocs;
  int rc = 0;
#define UP(ptr, vec) if ((rc = dev_upload(ctx, &ptr, vec, A))) return rc
#define AL(ptr, cnt) if ((rc = dev_alloc(ctx, &ptr, cnt, A))) return rc
  UP(d.circ_of_row, ctx->circ_of_row);
  UP(d.offsets, ctx->offsets);
  AL(d.cs, ctx->ncirc);
  AL(d.tp, 1);
  UP(d.rp, ctx->rp); UP(d.ci, ctx->ci); UP(d.erow, erow);
  UP(d.Glin, Glin); UP(d.Clin, Clin);
  UP(d.vF_ptr, pF); UP(d.vF_idx, iF); UP(d.vQ_ptr, pQ); UP(d.vQ_idx, iQ);
  UP(d.vL_ptr, pL); UP(d.vL_idx, iL); UP(d.vB_ptr, pB); UP(d.vB_idx, iB);
  UP(d.m_ptr, pM); UP(d.m_idx, iM);
  UP(d.is_branch, is_branch);
  UP(d.long_rows, long_rows); UP(d.row_long, row_long); UP(d.long_ents, long_ents); UP(d.ent_long, ent_long);
  UP(d.lrow_ptr, lrow_ptr); UP(d.lrow_blk, lrow_blk); UP(d.lent_ptr, lent_ptr); UP(d.lent_blk, lent_blk);
  AL(d.long_rsum, 4 * (size_t)ctx->n_long_row_blocks); AL(d.long_esum, (size_t)ctx->n_long_ent_blocks);
  AL(d.done_acc, 3);
  AL(d.sF, nF); AL(d.sQ, nQ); AL(d.sL, nL); AL(d.sL2, nL); AL(d.sB, nB); AL(d.sM, nMs); AL(d.sM2, nMs);
  UP(d.src_kind, skind); UP(d.src_off, soff); UP(d.src_circ, scirc); UP(d.src_data, sdata);
  UP(d.m1_node, m1node); UP(d.m1_model, m1model); UP(d.m1_circ, m1circ);
  UP(d.m1_beta, m1beta); UP(d.m1_vbi, m1vbi); UP(d.m1_models, models);
  UP(d.d_node, dnode); UP(d.d_model, dmodel); UP(d.d_circ, dcirc); UP(d.d_models, dmodels);
  UP(d.b4_node, b4node); UP(d.b4_model, b4model); UP(d.b4_circ, b4circ); UP(d.b4_models, b4models);
  AL(d.sta_curr, ctx->nsta); AL(d.sta_next, ctx->nsta); AL(d.sto_curr, ctx->nsto); AL(d.sto_next, ctx->nsto);
  for (double **v : {&d.x, &d.xcurr, &d.xn0, &d.dx, &d.rhs, &d.Qv, &d.FmB, &d.Fv, &d.Bv, &d.qh0, &d.qh1,
                     &d.qh2, &d.xh1, &d.xh2, &d.Qc, &d.FmBc, &d.solwt})
    AL(*v, n);
  AL(d.J, nnz);
  AL(d.mlh1, n); AL(d.mlh2, n); AL(d.mlh3, n);
  AL(d.mlp.theta, kMlpParams); AL(d.mlp.norm, kMlpNorm);
  AL(d.mlp.w1t, kMlpHid * kMlpInPad); AL(d.mlp.w2t, kMlpHid * kMlpHid); AL(d.mlp.w2, kMlpHid * kMlpHid);
  AL(ctx->mlp_m1, kMlpParams); AL(ctx->mlp_m2, kMlpParams); AL(ctx->mlp_grad, kMlpParams);
  AL(ctx->mlp_loss, 1);
  UP(d.pair_base, pair_base); UP(d.blk_cfirst, blk_cfirst); UP(d.pair_cstart, pair_cstart);
  AL(d.pmax, pairs); AL(d.psum, pairs);
  AL(d.probe_idx, n);
  AL(ctx->breakdown_dev, 1);
  AL(d.lu_gen, 1);
  {
    std::vector<char> lin(ctx->ncirc);
    for (int c = 0; c < ctx->ncirc; ++c) lin[c] = ctx->inst_of_circ[c] == 0 ? 1 : 0;
    UP(d.circ_linear, lin);
  }
  d.status = ctx->status_dev;
#undef UP
#undef AL
  CK(cudaMemsetAsync(d.probe_idx, 0xff, sizeof(int) * n, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->finalized = true;
  return XG_OK;
}

int xg_get_sizes(xg_ctx *ctx, int *n, int *nnz, int *nsta, int *nsto) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  if (n) *n = ctx->n;
  if (nnz) *nnz = ctx->nnz;
  if (nsta) *nsta = ctx->nsta;
  if (nsto) *nsto = ctx->nsto;
  return XG_OK;
}

int xg_get_pattern(xg_ctx *ctx, int *row_ptr, int *col_idx) {
  if (!ctx || !row_ptr || !col_idx) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  std::copy(ctx->rp.begin(), ctx->rp.end(), row_ptr);
  std::copy(ctx->ci.begin(), ctx->ci.end(), col_idx);
  return XG_OK;
}

// ---------------------------------------------------------------------------
// Loader entry points.
int xg_update_sources(xg_ctx *ctx, double time) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  launch_sources_k(ctx->stream, ctx->d, ctx->nv, ctx->nv + ctx->ni, 1, time);
  CK(cudaGetLastError());
  return XG_OK;
}

int xg_update_state(xg_ctx *ctx, const double *next_sol, const double *curr_sta, const double *curr_sto,
                    double *next_sta, double *next_sto, int newton_iter, int flags, int load_type) {
  if (!ctx || !next_sol) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  if (load_type < 0 || load_type > 2) return fail(ctx, XG_ERR_ARG, "bad load type");
  if (flags & ~(XG_FLAG_DCOP | XG_FLAG_INITJCT)) return fail(ctx, XG_ERR_ARG, "unknown solver-state flag");
  // DeviceMaster::updateState (N_DEV_DeviceMaster.h:688-700): a LINEAR load
  // updates the linear devices only, whose values here are the constant
  // linear part of the matrix — there is nothing to evaluate
  if (load_type == XG_LOAD_LINEAR) return XG_OK;
  if ((ctx->nsta > 0 && (!curr_sta || !next_sta)) || (ctx->nsto > 0 && (!curr_sto || !next_sto)))
    return fail(ctx, XG_ERR_ARG, "state/store vectors are required");
  DevArrays d = ctx->d;
  d.x = const_cast<double *>(next_sol);
  d.sta_curr = const_cast<double *>(curr_sta);
  d.sta_next = next_sta;
  d.sto_curr = const_cast<double *>(curr_sto);
  d.sto_next = next_sto;
  launch_bsim4_k(ctx->stream, d, ctx->nb, ctx->sto_base_b, ctx->sta_base_b, 0, 0, newton_iter, flags, ctx->sF_b,
                 ctx->sQ_b, ctx->sL_b, ctx->sM_b);
  launch_mos1_k(ctx->stream, d, ctx->nm, ctx->sto_base_m, 0, 0, newton_iter, flags, ctx->sF_m, ctx->sQ_m,
                ctx->sL_m, ctx->sM_m);
  launch_diode_k(ctx->stream, d, ctx->nd, 0, 0, newton_iter, flags, ctx->sF_d, ctx->sQ_d, ctx->sL_d, ctx->sM_d);
  CK(cudaGetLastError());
  return XG_OK;
}

int xg_load_dae_vectors(xg_ctx *ctx, const double *next_sol, double *Q, double *F, double *B, double *dFdxdVp,
                        double *dQdxdVp, int load_type) {
  if (!ctx || !next_sol || !Q || !F || !B || !dFdxdVp || !dQdxdVp) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  if (load_type < 0 || load_type > 2) return fail(ctx, XG_ERR_ARG, "bad load type");
  launch_load_vectors_k(ctx->stream, ctx->d, ctx->n, next_sol, Q, F, B, dFdxdVp, dQdxdVp, load_type);
  CK(cudaGetLastError());
  return XG_OK;
}

int xg_load_dae_matrices(xg_ctx *ctx, double *dQdx, double *dFdx, int load_type) {
  if (!ctx || !dQdx || !dFdx) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  if (load_type < 0 || load_type > 2) return fail(ctx, XG_ERR_ARG, "bad load type");
  launch_load_matrices_k(ctx->stream, ctx->d, ctx->nnz, dQdx, dFdx, load_type);
  CK(cudaGetLastError());
  return XG_OK;
}

// ---------------------------------------------------------------------------
// LU entry points.
// Per-circuit lists of the circuit-resident tick (FusedDev) for the
// analysis H, when the batch admits that form: many small circuits, MOSFET-1
// and diode devices only, FP64 factors, the polynomial predictor, and an LU
// without a top (every column in a hub or a dependency-closed group).
static int resident_build(xg_ctx *ctx, const LUHost &H) {
  ctx->resident_ok = false;
  ctx->F = FusedDev();
  const int n = H.n, ncirc = ctx->ncirc;
  int max_rows = 0;
  for (int c = 0; c < ncirc; ++c) max_rows = std::max(max_rows, ctx->offsets[c + 1] - ctx->offsets[c]);
  if (ncirc < kFusedMinCircuits || max_rows > kFusedMaxRows || ctx->nb > 0 || ctx->lu_prec != XG_PREC_FP64 ||
      ctx->predictor != XG_PRED_POLY || H.fsched.n_top_items > 0 || H.lsched.n_top_items > 0)
    return XG_OK;
  std::vector<int> circ_of_step(n);
  for (int j = 0; j < n; ++j) circ_of_step[j] = ctx->circ_of_row[H.col_of_step[j]];
  // levels per circuit: its hubs, then the local levels of its groups merged
  // (groups are independent of one another; a group depends only on hubs)
  auto levels = [&](const Schedule &S, std::vector<int> &cl, std::vector<int> &lptr, std::vector<int> &items) {
    std::vector<std::vector<std::vector<int>>> per(ncirc);
    for (int t = 0; t < S.n_hub; ++t) {
      auto &v = per[circ_of_step[S.items[t]]];
      if (v.empty()) v.resize(1);
      v[0].push_back(S.items[t]);
    }
    for (int g = 0; g < S.n_groups; ++g)
      for (int lv = S.grp_lvl[g]; lv < S.grp_lvl[g + 1]; ++lv)
        for (int t = S.lvl_ptr[lv]; t < S.lvl_ptr[lv + 1]; ++t) {
          auto &v = per[circ_of_step[S.items[t]]];
          const size_t li = 1 + (size_t)(lv - S.grp_lvl[g]);
          if (v.size() <= li) v.resize(li + 1);
          v[li].push_back(S.items[t]);
        }
    cl.assign(1, 0);
    lptr.assign(1, 0);
    items.clear();
    for (int c = 0; c < ncirc; ++c) {
      for (auto &lv : per[c]) {
        if (lv.empty()) continue;
        items.insert(items.end(), lv.begin(), lv.end());
        lptr.push_back((int)items.size());
      }
      cl.push_back((int)lptr.size() - 1);
    }
    return (int)items.size() == n;
  };
  std::vector<int> f_cl, f_lptr, f_items, l_cl, l_lptr, l_items;
  if (!levels(H.fsched, f_cl, f_lptr, f_items) || !levels(H.lsched, l_cl, l_lptr, l_items)) return XG_OK;
  // how the grouped kernels compute each column / row (see FusedDev)
  std::vector<signed char> f_kind(n, 1), l_meth(n, 2), u_meth(n, 2);
  for (int g = 0; g < H.fsched.n_groups; ++g)
    for (int t = H.fsched.lvl_ptr[H.fsched.grp_lvl[g]]; t < H.fsched.lvl_ptr[H.fsched.grp_lvl[g + 1]]; ++t) {
      const int j = H.fsched.items[t];
      f_kind[j] = H.fsched.is_thread[j] ? 0 : (H.fsched.is_long[j] ? 2 : 1);
      u_meth[j] = (H.us_gbytes[g] > 0 || H.fsched.is_thread_rev[j]) ? 1 : (H.fsched.is_long_rev[j] ? 3 : 2);
    }
  for (int t = 0; t < H.fsched.n_hub; ++t) {
    f_kind[H.fsched.items[t]] = 2;
    u_meth[H.fsched.items[t]] = 3;
  }
  for (int g = 0; g < H.lsched.n_groups; ++g)
    for (int t = H.lsched.lvl_ptr[H.lsched.grp_lvl[g]]; t < H.lsched.lvl_ptr[H.lsched.grp_lvl[g + 1]]; ++t) {
      const int i = H.lsched.items[t];
      l_meth[i] = (H.ls_gbytes[g] > 0 || H.lsched.is_thread[i]) ? 1 : (H.lsched.is_long[i] ? 3 : 2);
    }
  for (int t = 0; t < H.lsched.n_hub; ++t) l_meth[H.lsched.items[t]] = 0;
  // each level's items sorted by kind, with the start of the later kinds
  auto sort_levels = [](const std::vector<int> &lptr, std::vector<int> &items, std::vector<int2> &split,
                        auto &&kind) {
    split.assign(lptr.size() - 1, int2{0, 0});
    for (size_t lv = 0; lv + 1 < lptr.size(); ++lv) {
      auto b = items.begin() + lptr[lv], e = items.begin() + lptr[lv + 1];
      std::stable_sort(b, e, [&](int x, int y) { return kind(x) < kind(y); });
      int s1 = lptr[lv + 1], s2 = lptr[lv + 1];
      for (int t = lptr[lv + 1] - 1; t >= lptr[lv]; --t) {
        if (kind(items[t]) >= 1) s1 = t;
        if (kind(items[t]) >= 2) s2 = t;
      }
      split[lv] = int2{s1, s2};
    }
  };
  std::vector<int> u_items = f_items;
  std::vector<int2> f_split, u_split, l_split;
  sort_levels(f_lptr, f_items, f_split, [&](int j) { return (int)f_kind[j]; });
  sort_levels(f_lptr, u_items, u_split, [&](int k) { return (int)u_meth[k] - 1; });
  sort_levels(l_lptr, l_items, l_split, [&](int i) { return l_meth[i] <= 1 ? 0 : (int)l_meth[i] - 1; });
  // instances, sources, long rows and long entries of each circuit
  auto bucket = [&](const std::vector<int> &circ_of, std::vector<int> &ptr, std::vector<int> &list) {
    ptr.assign(ncirc + 1, 0);
    for (int c : circ_of) ptr[c + 1]++;
    for (int c = 0; c < ncirc; ++c) ptr[c + 1] += ptr[c];
    list.assign(circ_of.size(), 0);
    std::vector<int> f(ptr.begin(), ptr.end() - 1);
    for (size_t k = 0; k < circ_of.size(); ++k) list[f[circ_of[k]]++] = (int)k;
  };
  std::vector<int> m1_ptr, m1_list, d_ptr, d_list, src_ptr, src_list, lr_ptr, lr_list, le_ptr, le_list;
  bucket(ctx->m1_circ_h, m1_ptr, m1_list);
  bucket(ctx->d_circ_h, d_ptr, d_list);
  bucket(ctx->src_circ_h, src_ptr, src_list);
  std::vector<int> lr_circ, le_circ;
  for (int r : ctx->long_rows_h) lr_circ.push_back(ctx->circ_of_row[r]);
  for (int e : ctx->long_ents_h) {
    const int r = (int)(std::upper_bound(ctx->rp.begin(), ctx->rp.end(), e) - ctx->rp.begin()) - 1;
    le_circ.push_back(ctx->circ_of_row[r]);
  }
  bucket(lr_circ, lr_ptr, lr_list);
  bucket(le_circ, le_ptr, le_list);
  // largest circuits first: the queue then balances the CTAs
  std::vector<int> order(ncirc);
  for (int c = 0; c < ncirc; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const long long wa = ctx->offsets[a + 1] - ctx->offsets[a] + ctx->inst_of_circ[a];
    const long long wb = ctx->offsets[b + 1] - ctx->offsets[b] + ctx->inst_of_circ[b];
    return wa > wb;
  });
  // shared-memory buffers of the circuits' factor columns
  std::vector<int> c_soff(n, 0), c_fcnt(ncirc, 0), c_umeta((size_t)4 * H.ri.size(), 0);
  int max_fbuf = 0;
  for (int c = 0; c < ncirc; ++c) {
    int off = 0;
    for (int lv = f_cl[c]; lv < f_cl[c + 1]; ++lv)
      for (int t = f_lptr[lv]; t < f_lptr[lv + 1]; ++t) {
        const int j = f_items[t];
        c_soff[j] = off;
        off += H.cp[j + 1] - H.cp[j];
      }
    c_fcnt[c] = off;
    max_fbuf = std::max(max_fbuf, off);
  }
  for (int j = 0; j < n; ++j)
    for (int p = H.cp[j]; p < H.diag[j]; ++p) {
      const int k = H.ri[p];
      int *u = &c_umeta[(size_t)4 * p];
      u[0] = c_soff[k] + (H.diag[k] + 1 - H.cp[k]);
      u[1] = H.cp[k + 1] - H.diag[k] - 1;
      u[2] = H.upd_off[p];
      u[3] = H.diag[k] + 1;
    }
  const bool staged = (2 * (size_t)max_rows + (size_t)max_fbuf) * sizeof(double) <= (size_t)kFusedSmemBytes;
  FusedDev F;
  auto &A = ctx->lu_allocs;
  int rc = 0;
#define UP(ptr, vec) if ((rc = dev_upload(ctx, &ptr, vec, A))) return rc
  if (staged) {
    int *um = nullptr;
    UP(F.c_soff, c_soff);
    UP(F.c_fcnt, c_fcnt);
    UP(um, c_umeta);
    F.c_umeta = reinterpret_cast<const int4 *>(um);
    F.max_fbuf = max_fbuf;
  }
  UP(F.order, order);
  UP(F.m1_ptr, m1_ptr); UP(F.m1_list, m1_list); UP(F.d_ptr, d_ptr); UP(F.d_list, d_list);
  UP(F.src_ptr, src_ptr); UP(F.src_list, src_list);
  UP(F.lr_ptr, lr_ptr); UP(F.lr_list, lr_list); UP(F.le_ptr, le_ptr); UP(F.le_list, le_list);
  UP(F.f_cl, f_cl); UP(F.f_lptr, f_lptr); UP(F.f_items, f_items); UP(F.u_items, u_items);
  UP(F.l_cl, l_cl); UP(F.l_lptr, l_lptr); UP(F.l_items, l_items);
  UP(F.f_split, f_split); UP(F.u_split, u_split); UP(F.l_split, l_split);
  UP(F.f_kind, f_kind); UP(F.l_meth, l_meth); UP(F.u_meth, u_meth);
#undef UP
  if ((rc = dev_alloc(ctx, &F.queue, 1, A))) return rc;
  if ((rc = dev_alloc(ctx, &F.ticks, 2, A))) return rc;
  F.max_rows = max_rows;
  if (resident_prepare_k(max_rows, F.max_fbuf, ctx->device, F.grid) != XG_OK) return fail(ctx, XG_ERR_CUDA, "resident tick set-up");
  ctx->F = F;
  const int slots[8] = {ctx->sF_m, ctx->sQ_m, ctx->sL_m, ctx->sM_m, ctx->sF_d, ctx->sQ_d, ctx->sL_d, ctx->sM_d};
  std::copy(slots, slots + 8, ctx->resident_slots);
  ctx->resident_ok = true;
  return XG_OK;
}

static int lu_upload(xg_ctx *ctx, const LUHost &H) {
  CK(cudaStreamSynchronize(ctx->stream));
  free_list(ctx->lu_allocs);
  LUDev &L = ctx->L;
  L = LUDev();
  L.n = H.n;
  L.nnz = (long long)H.ri.size();
  auto &A = ctx->lu_allocs;
  int rc = 0;
#define UP(ptr, vec) if ((rc = dev_upload(ctx, &ptr, vec, A))) return rc
  UP(L.row_of_step, H.row_of_step); UP(L.col_of_step, H.col_of_step);
  std::vector<int> cstep(H.n);
  for (int p = 0; p < H.n; ++p) cstep[p] = ctx->circ_of_row[H.col_of_step[p]];
  UP(L.circ_of_step, cstep);
  UP(L.cp, H.cp); UP(L.ri, H.ri); UP(L.diag, H.diag); UP(L.src, H.src);
  UP(L.l_ptr, H.l_ptr); UP(L.l_pos, H.l_pos); UP(L.l_col, H.l_col);
  UP(L.u_ptr, H.u_ptr); UP(L.u_pos, H.u_pos); UP(L.u_col, H.u_col);
  UP(L.exempt, H.exempt); UP(L.pscale, H.pscale);
  UP(L.upd_off, H.upd_off); UP(L.upd_pos, H.upd_pos);
  {
    int *um = nullptr;
    UP(um, H.umeta);
    L.umeta = reinterpret_cast<const int4 *>(um);
  }
  for (int w = 0; w < 2; ++w) {
    const Schedule &S = w ? H.lsched : H.fsched;
    SchedDev &D = w ? L.ls : L.fs;
    UP(D.items, S.items); UP(D.lvl_ptr, S.lvl_ptr); UP(D.grp_lvl, S.grp_lvl);
    UP(D.is_long, S.is_long); UP(D.is_long_rev, S.is_long_rev);
    UP(D.is_thread, S.is_thread); UP(D.is_thread_rev, S.is_thread_rev);
    D.n_hub = S.n_hub;
    D.n_groups = S.n_groups;
    D.n_top_items = S.n_top_items;
  }
#undef UP
  if ((rc = dev_alloc(ctx, &L.lu, (size_t)L.nnz, A))) return rc;
  if ((rc = dev_alloc(ctx, &L.y, (size_t)H.n, A))) return rc;
  if (ctx->lu_prec == XG_PREC_FP32_IR) {
    if ((rc = dev_alloc(ctx, &L.lu32, (size_t)L.nnz, A))) return rc;
    if ((rc = dev_alloc(ctx, &L.ir_r, (size_t)H.n, A))) return rc;
    L.mixed = 1;
    L.n_refine = ctx->lu_refine;
    L.a_rp = ctx->d.rp;
    L.a_ci = ctx->d.ci;
    L.a_circ = ctx->d.circ_of_row;
    L.a_vals = ctx->d.J;  // the transient's Jacobian; xg_lu_factor points it at its values
  }
  L.breakdown = ctx->breakdown_dev;
  L.n_top_rl = (int)H.top_items.size();
  if (L.n_top_rl > 0) {
    if ((rc = dev_upload(ctx, &L.top_items, H.top_items, A))) return rc;
    std::vector<char> is_top(H.n, 0);
    for (int j : H.top_items) is_top[j] = 1;
    if ((rc = dev_upload(ctx, &L.is_top, is_top, A))) return rc;
    for (auto pr : {std::make_pair(&L.tlv_items, &H.tlv_items), std::make_pair(&L.tlv_item_ptr, &H.tlv_item_ptr),
                    std::make_pair(&L.tlv_grp_ptr, &H.tlv_grp_ptr), std::make_pair(&L.tgrp_col, &H.tgrp_col),
                    std::make_pair(&L.tgrp_ptr, &H.tgrp_ptr), std::make_pair(&L.tgrp_pos, &H.tgrp_pos),
                    std::make_pair(&L.tgrp_k, &H.tgrp_k)})
      if ((rc = dev_upload(ctx, pr.first, *pr.second, A))) return rc;
    if (H.top_multi) {
      ctx->h_tlv_item_ptr = H.tlv_item_ptr;
      ctx->h_tlv_grp_ptr = H.tlv_grp_ptr;
      L.n_top_lv = (int)H.tlv_item_ptr.size() - 1;
      L.h_tlv_item_ptr = ctx->h_tlv_item_ptr.data();
      L.h_tlv_grp_ptr = ctx->h_tlv_grp_ptr.data();
    }
  }
  L.ordering = H.ordering;
  for (int w = 0; w < 2; ++w) {
    const Schedule &S = w ? H.lsched : H.fsched;
    std::vector<int> gc(std::max(1, S.n_groups), -1);
    for (int g = 0; g < S.n_groups; ++g) {
      int c = -2;
      for (int t = S.lvl_ptr[S.grp_lvl[g]]; t < S.lvl_ptr[S.grp_lvl[g + 1]] && c != -1; ++t) {
        const int ct = cstep[S.items[t]];
        c = (c == -2 || c == ct) ? ct : -1;
      }
      gc[g] = c < 0 ? -1 : c;
    }
    if ((rc = dev_upload(ctx, w ? &L.ls_gcirc : &L.fs_gcirc, gc, A))) return rc;
  }
  for (int w = 0; w < 2; ++w) {
    const std::vector<int> &gb = w ? H.us_gbytes : H.ls_gbytes;
    int mx = 0;
    for (int b : gb) mx = std::max(mx, b);
    if (mx == 0) continue;
    if (w == 0) {
      if ((rc = dev_upload(ctx, &L.ls_eptr, H.ls_eptr, A))) return rc;
      if ((rc = dev_upload(ctx, &L.ls_epos, H.ls_epos, A))) return rc;
      if ((rc = dev_upload(ctx, &L.ls_esrc, H.ls_esrc, A))) return rc;
      if ((rc = dev_upload(ctx, &L.ls_gbytes, H.ls_gbytes, A))) return rc;
      L.ls_smem = mx;
    } else {
      if ((rc = dev_upload(ctx, &L.us_eptr, H.us_eptr, A))) return rc;
      if ((rc = dev_upload(ctx, &L.us_epos, H.us_epos, A))) return rc;
      if ((rc = dev_upload(ctx, &L.us_esrc, H.us_esrc, A))) return rc;
      if ((rc = dev_upload(ctx, &L.us_gbytes, H.us_gbytes, A))) return rc;
      L.us_smem = mx;
    }
  }
  L.fs_threads = H.fs_threads;
  L.ls_threads = H.ls_threads;
  L.us_threads = H.us_threads;
  if ((rc = lu_prepare_k())) return rc;  // shared-memory opt-ins of the staged kernels
  if (!H.grp_snz.empty()) {
    for (int w = 0; w < 2; ++w) {
      const int cap = kGroupSmemBytes / (w ? (int)sizeof(float) : (int)sizeof(double));
      for (int z : H.grp_snz)
        if (z <= cap) L.grp_fit[w] = std::max(L.grp_fit[w], z);
    }
    if (L.grp_fit[0] > 0 || L.grp_fit[1] > 0) {
      if ((rc = dev_upload(ctx, &L.grp_soff, H.grp_soff, A))) return rc;
      if ((rc = dev_upload(ctx, &L.grp_snz, H.grp_snz, A))) return rc;
      // groups staged with their update metadata: values (16-byte aligned),
      // then the metadata; the launch buffer covers the largest
      bool any_meta = false;
      for (size_t g = 0; g < H.fm_gbytes.size(); ++g) {
        if (H.fm_gbytes[g] == 0) continue;
        any_meta = true;
        for (int w = 0; w < 2; ++w) {
          const size_t vb = ((size_t)H.grp_snz[g] * (w ? sizeof(float) : sizeof(double)) + 15) / 16 * 16;
          L.fm_smem[w] = std::max(L.fm_smem[w], (int)(vb + H.fm_gbytes[g]));
        }
      }
      L.fm_on = any_meta && H.fm_model_on;
      if (any_meta) {
        int *c = nullptr, *e = nullptr;
        if ((rc = dev_upload(ctx, &c, H.fm_col, A))) return rc;
        if ((rc = dev_upload(ctx, &e, H.fm_ent, A))) return rc;
        L.fm_col = reinterpret_cast<const int4 *>(c);
        L.fm_ent = reinterpret_cast<const int4 *>(e);
        if ((rc = dev_upload(ctx, &L.fm_eptr, H.fm_eptr, A))) return rc;
        if ((rc = dev_upload(ctx, &L.fm_tptr, H.fm_tptr, A))) return rc;
        if ((rc = dev_upload(ctx, &L.fm_tgt, H.fm_tgt, A))) return rc;
        if ((rc = dev_upload(ctx, &L.fm_gbytes, H.fm_gbytes, A))) return rc;
      }
    }
  }
  if (H.solve_top_multi) {
    ctx->h_ls_lvl_ptr = H.lsched.lvl_ptr;
    ctx->h_fs_lvl_ptr = H.fsched.lvl_ptr;
    L.h_ls_lvl_ptr = ctx->h_ls_lvl_ptr.data();
    L.h_fs_lvl_ptr = ctx->h_fs_lvl_ptr.data();
    L.ls_top_lo = H.lsched.grp_lvl[H.lsched.n_groups];
    L.ls_top_hi = H.lsched.grp_lvl[H.lsched.n_groups + 1];
    L.fs_top_lo = H.fsched.grp_lvl[H.fsched.n_groups];
    L.fs_top_hi = H.fsched.grp_lvl[H.fsched.n_groups + 1];
  }
  L.f_levels = (int)H.f_lvl_ptr.size() - 1;
  L.l_levels = (int)H.l_lvl_ptr.size() - 1;
  L.u_levels = (int)H.u_lvl_ptr.size() - 1;
  if ((rc = resident_build(ctx, H))) return rc;
  ctx->row_of_col_h.assign(H.n, -1);
  for (int p = 0; p < H.n; ++p) ctx->row_of_col_h[H.col_of_step[p]] = H.row_of_step[p];
  // a new analysis: every circuit refactors before it may reuse factors again
  ctx->lu_gen++;
  CK(cudaMemcpyAsync(ctx->d.lu_gen, &ctx->lu_gen, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(ctx->breakdown_dev, 0, sizeof(int), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->lu_ready = true;
  ctx->n_analyze++;
  return XG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Launch-shape tuner of the LU sweeps.  Every candidate computes the same
// bits (the shapes change which threads do the work, not the order of any
// sum), so the choice is made by timing alone: the factorization with and
// without the staged update metadata at 64..512 threads per CTA, then the L
// and the U solve at 64..512 threads, each candidate launched on the
// matrix the analysis was computed from, L2 flushed before every timed
// launch (in a tick the device evaluation streams the state through L2
// between factorizations).  Choices are cached per analysis (a hash of the
// factor pattern, pivot order and schedules), so a re-analysis of the same
// pattern or a second context reuses them.
namespace {

struct TuneChoice {
  int fm_on, fs, ls, us;
  double factor_us, solve_us;
};
std::mutex g_tune_mu;
std::map<unsigned long long, TuneChoice> g_tune_cache;

unsigned long long fnv(unsigned long long h, const std::vector<int> &v) {
  for (int x : v) {
    h ^= (unsigned)x;
    h *= 1099511628211ULL;
  }
  h ^= v.size();
  return h * 1099511628211ULL;
}

unsigned long long analysis_hash(const LUHost &H, int prec, int sms) {
  unsigned long long h = 1469598103934665603ULL;
  h = fnv(h, {H.n, prec, sms});
  for (const std::vector<int> *v : {&H.cp, &H.ri, &H.row_of_step, &H.fsched.items, &H.fsched.grp_lvl,
                                    &H.lsched.items, &H.lsched.grp_lvl, &H.grp_snz, &H.fm_gbytes})
    h = fnv(h, *v);
  return h;
}

}  // namespace

// Median device time (us) of `timed` launches of fn after one warm-up, L2
// flushed before each.
template <class F>
static int time_launch(xg_ctx *ctx, void *flush, size_t flush_bytes, F &&fn, double *us) {
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return fail(ctx, XG_ERR_CUDA, "cudaEventCreate"); }
  fn();
  std::vector<double> t;
  int rc = XG_OK;
  for (int k = 0; k < 3 && rc == XG_OK; ++k) {
    if (cudaMemsetAsync(flush, k + 1, flush_bytes, ctx->stream) != cudaSuccess) { rc = XG_ERR_CUDA; break; }
    cudaEventRecord(e0, ctx->stream);
    fn();
    cudaEventRecord(e1, ctx->stream);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = XG_ERR_CUDA;
    t.push_back(ms * 1e3);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == XG_OK && cudaGetLastError() != cudaSuccess) rc = XG_ERR_CUDA;
  if (rc) return fail(ctx, rc, "LU tuner: CUDA failure");
  std::sort(t.begin(), t.end());
  *us = t[t.size() / 2];
  return XG_OK;
}

static int tune_lu(xg_ctx *ctx, const LUHost &H, const double *vals_dev) {
  LUDev &L = ctx->L;
  xg_lu_tuning &T = ctx->tuning;
  T = xg_lu_tuning{};
  T.mode = ctx->tune_mode;
  T.model_factor_threads = T.factor_threads = L.fs_threads;
  T.model_factor_meta = T.factor_meta = L.fm_on;
  T.model_lsolve_threads = T.lsolve_threads = L.ls_threads;
  T.model_usolve_threads = T.usolve_threads = L.us_threads;
  if (ctx->tune_mode == XG_TUNE_FIXED) {
    const int *f = ctx->fixed_shapes;
    if (f[0]) L.fs_threads = f[0];
    if (f[1] >= 0) L.fm_on = (f[1] && L.fm_gbytes) ? 1 : 0;
    if (f[2]) L.ls_threads = f[2];
    if (f[3]) L.us_threads = f[3];
    T.factor_threads = L.fs_threads; T.factor_meta = L.fm_on;
    T.lsolve_threads = L.ls_threads; T.usolve_threads = L.us_threads;
    return XG_OK;
  }
  if (ctx->tune_mode != XG_TUNE_TIMED || L.fs.n_groups + L.ls.n_groups == 0) return XG_OK;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const unsigned long long key = analysis_hash(H, ctx->lu_prec, sms);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      const TuneChoice &c = it->second;
      L.fm_on = c.fm_on; L.fs_threads = c.fs; L.ls_threads = c.ls; L.us_threads = c.us;
      T.factor_meta = c.fm_on; T.factor_threads = c.fs; T.lsolve_threads = c.ls; T.usolve_threads = c.us;
      T.factor_us = c.factor_us; T.solve_us = c.solve_us;
      T.from_cache = 1;
      return XG_OK;
    }
  }
  // scratch of the trials: an L2 flush buffer and solve vectors
  const size_t flush_bytes = 256u << 20;
  void *flush = nullptr;
  double *b = nullptr, *x = nullptr;
  CK(cudaMalloc(&flush, flush_bytes));
  int rc = XG_OK;
  if (cudaMalloc((void **)&b, sizeof(double) * L.n) != cudaSuccess ||
      cudaMalloc((void **)&x, sizeof(double) * L.n) != cudaSuccess) rc = fail(ctx, XG_ERR_CUDA, "cudaMalloc");
  if (rc == XG_OK) {
    std::vector<double> ones(L.n, 1.0);
    if (cudaMemcpyAsync(b, ones.data(), sizeof(double) * L.n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
      rc = fail(ctx, XG_ERR_CUDA, "cudaMemcpy");
    if (L.mixed) L.a_vals = vals_dev;
  }
  const int sizes[4] = {64, 128, 256, 512};
  auto factor = [&]() { launch_lu_factor_k(ctx->stream, L, vals_dev, ctx->d.cs, 0, kRuntimePivotTol); };
  auto solve = [&]() { launch_lu_solve_k(ctx->stream, L, b, x, ctx->d.cs, 0); };
  // the model's choice first (its time is reported beside the tuned one)
  if (rc == XG_OK) rc = time_launch(ctx, flush, flush_bytes, factor, &T.model_factor_us);
  if (rc == XG_OK) rc = time_launch(ctx, flush, flush_bytes, solve, &T.model_solve_us);
  double best = T.model_factor_us;
  const int fm_model = L.fm_on, fs_model = L.fs_threads;
  int best_fm = fm_model, best_fs = fs_model;
  const bool can_meta = L.fm_gbytes != nullptr;
  if (L.fs.n_groups > 0)
    for (int fm = 0; fm <= (can_meta ? 1 : 0) && rc == XG_OK; ++fm)
      for (int s : sizes) {
        if (fm == fm_model && s == fs_model) continue;
        L.fm_on = fm;
        L.fs_threads = s;
        double us = 0;
        if ((rc = time_launch(ctx, flush, flush_bytes, factor, &us))) break;
        if (us < best) { best = us; best_fm = fm; best_fs = s; }
      }
  L.fm_on = best_fm;
  L.fs_threads = best_fs;
  T.factor_us = best;
  double sbest = T.model_solve_us;
  for (int w = 0; w < 2 && rc == XG_OK; ++w) {  // L solve, then U solve
    int &thr = w ? L.us_threads : L.ls_threads;
    const int keep = thr;
    int pick = keep;
    if ((w ? L.fs.n_groups : L.ls.n_groups) == 0) continue;
    for (int s : sizes) {
      if (s == keep) continue;
      thr = s;
      double us = 0;
      if ((rc = time_launch(ctx, flush, flush_bytes, solve, &us))) break;
      if (us < sbest) { sbest = us; pick = s; }
    }
    thr = pick;
  }
  T.solve_us = sbest;
  cudaFree(flush);
  if (b) cudaFree(b);
  if (x) cudaFree(x);
  // the trials may have raised the breakdown flag: the analysis' values
  // are factored for real by the caller
  if (cudaMemsetAsync(L.breakdown, 0, sizeof(int), ctx->stream) != cudaSuccess && rc == XG_OK)
    rc = fail(ctx, XG_ERR_CUDA, "cudaMemset");
  if (rc) {
    L.fm_on = fm_model; L.fs_threads = fs_model;
    L.ls_threads = T.model_lsolve_threads; L.us_threads = T.model_usolve_threads;
    return rc;
  }
  T.factor_meta = L.fm_on; T.factor_threads = L.fs_threads;
  T.lsolve_threads = L.ls_threads; T.usolve_threads = L.us_threads;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[key] = TuneChoice{L.fm_on, L.fs_threads, L.ls_threads, L.us_threads, T.factor_us, T.solve_us};
  return XG_OK;
}

extern "C" {

// refresh (optional, per circuit): re-pivot only those circuits from the
// values; every other circuit keeps the pivot rows of the current analysis,
// so its factors, and its results, stay exactly what they were.
static int lu_analyze_from_device(xg_ctx *ctx, const double *vals_dev, const std::vector<char> *refresh = nullptr) {
  std::vector<double> v(ctx->nnz);
  CK(cudaMemcpyAsync(v.data(), vals_dev, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  LUHost H;
  std::string err;
  std::vector<int> keep;
  if (refresh && (int)ctx->row_of_col_h.size() == ctx->n) {
    keep.assign(ctx->n, -1);
    for (int j = 0; j < ctx->n; ++j)
      if (!(*refresh)[ctx->circ_of_row[j]]) keep[j] = ctx->row_of_col_h[j];
  }
  int rc = lu_analyze_host(ctx->n, ctx->rp, ctx->ci, v, H, err, ctx->sched_order, keep.empty() ? nullptr : &keep);
  if (rc == XG_OK) {
    if (ctx->sched_ftop >= 0) H.top_multi = (ctx->sched_ftop == XG_TOP_LEVELS);
    if (ctx->sched_stop >= 0) H.solve_top_multi = (ctx->sched_stop == XG_TOP_LEVELS);
  }
  if (rc) return fail(ctx, rc, "LU analysis: " + err);
  if ((rc = lu_upload(ctx, H))) return rc;
  return tune_lu(ctx, H, vals_dev);
}

int xg_lu_analyze(xg_ctx *ctx, const double *vals) {
  if (!ctx || !vals) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  return lu_analyze_from_device(ctx, vals);
}

int xg_lu_factor(xg_ctx *ctx, const double *vals) {
  if (!ctx || !vals) return XG_ERR_ARG;
  if (!ctx->lu_ready) return fail(ctx, XG_ERR_STATE, "call xg_lu_analyze first");
  CK(cudaMemsetAsync(ctx->breakdown_dev, 0, sizeof(int), ctx->stream));
  if (ctx->L.mixed) ctx->L.a_vals = vals;
  launch_lu_factor_k(ctx->stream, ctx->L, vals, ctx->d.cs, 0, ctx->pivot_tol);
  CK(cudaGetLastError());
  int bd = 0;
  CK(cudaMemcpyAsync(&bd, ctx->breakdown_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (bd) {
    char buf[96];
    snprintf(buf, sizeof buf, "pivot breakdown at step %d: re-run xg_lu_analyze", bd - 1);
    return fail(ctx, XG_ERR_SINGULAR, buf);
  }
  return XG_OK;
}

int xg_lu_solve(xg_ctx *ctx, const double *rhs, double *x) {
  if (!ctx || !rhs || !x) return XG_ERR_ARG;
  if (!ctx->lu_ready) return fail(ctx, XG_ERR_STATE, "call xg_lu_analyze first");
  launch_lu_solve_k(ctx->stream, ctx->L, rhs, x, ctx->d.cs, 0);
  CK(cudaGetLastError());
  return XG_OK;
}

// Allocation-free variant of xg_lu_solve: the solve's scratch vector lives in
// a static device array (see xg_lu.cu) instead of memory from cudaMalloc.
// For callers that must not call the CUDA allocator — code whose device memory
// is entirely owned by another allocator, or a loop that must not block on
// cudaMalloc/cudaFree.  The first call on a device looks up the scratch
// address (cudaGetSymbolAddress); make that first call before any stream
// capture.  All calls share the one scratch array: calls that overlap on the
// GPU (other streams, other host threads) race and must be serialized.
int xg_lu_solve_noalloc(xg_ctx *ctx, const double *rhs, double *x) {
  if (!ctx || !rhs || !x) return XG_ERR_ARG;
  if (ctx->n > kNoAllocMaxN) {
    char buf[160];
    snprintf(buf, sizeof buf, "xg_lu_solve_noalloc: %d unknowns exceed the scratch limit of %d", ctx->n,
             kNoAllocMaxN);
    return fail(ctx, XG_ERR_ARG, buf);
  }
  if (!ctx->lu_ready) return fail(ctx, XG_ERR_STATE, "call xg_lu_analyze first");
  CK(cudaSetDevice(ctx->device));
  double *scratch = nullptr;
  std::string err;
  int rc = noalloc_scratch(ctx->device, &scratch, err);
  if (rc) return fail(ctx, rc, err);
  launch_lu_solve_noalloc_k(ctx->stream, ctx->L, scratch, rhs, x, ctx->d.cs);
  CK(cudaGetLastError());
  return XG_OK;
}

int xg_lu_set_precision(xg_ctx *ctx, int precision, int n_refine) {
  if (!ctx) return XG_ERR_ARG;
  if (precision != XG_PREC_FP64 && precision != XG_PREC_FP32_IR)
    return fail(ctx, XG_ERR_ARG, "precision must be XG_PREC_FP64 or XG_PREC_FP32_IR");
  if (n_refine < 0 || n_refine > 16) return fail(ctx, XG_ERR_ARG, "n_refine must be in [0, 16]");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "precision cannot change during a transient");
  ctx->lu_prec = precision;
  ctx->lu_refine = n_refine;
  ctx->lu_ready = false;  // the next xg_lu_analyze (or transient) builds factors of this precision
  return XG_OK;
}

int xg_lu_set_pivot_tolerance(xg_ctx *ctx, double tol) {
  if (!ctx) return XG_ERR_ARG;
  if (!(tol > 0.0 && tol < 1.0)) return fail(ctx, XG_ERR_ARG, "pivot tolerance must lie in (0, 1)");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "the pivot tolerance cannot change during a transient");
  ctx->pivot_tol = tol;
  return XG_OK;
}

int xg_lu_set_reuse(xg_ctx *ctx, int on) {
  if (!ctx) return XG_ERR_ARG;
  if (on != 0 && on != 1) return fail(ctx, XG_ERR_ARG, "reuse must be 0 or 1");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "factor reuse cannot change during a transient");
  ctx->lu_reuse = on;
  return XG_OK;
}

int xg_lu_set_shapes(xg_ctx *ctx, int factor_threads, int factor_meta, int lsolve_threads, int usolve_threads) {
  if (!ctx) return XG_ERR_ARG;
  auto ok = [](int t) { return t == 0 || t == 64 || t == 128 || t == 256 || t == 512; };
  if (!ok(factor_threads) || !ok(lsolve_threads) || !ok(usolve_threads))
    return fail(ctx, XG_ERR_ARG, "threads must be 0, 64, 128, 256 or 512");
  if (factor_meta < -1 || factor_meta > 1) return fail(ctx, XG_ERR_ARG, "factor_meta must be -1, 0 or 1");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "launch shapes cannot change during a transient");
  ctx->fixed_shapes[0] = factor_threads;
  ctx->fixed_shapes[1] = factor_meta;
  ctx->fixed_shapes[2] = lsolve_threads;
  ctx->fixed_shapes[3] = usolve_threads;
  ctx->tune_mode = XG_TUNE_FIXED;
  ctx->lu_ready = false;  // applies from the next analysis
  return XG_OK;
}

int xg_lu_set_tuning(xg_ctx *ctx, int mode) {
  if (!ctx) return XG_ERR_ARG;
  if (mode != XG_TUNE_MODEL && mode != XG_TUNE_TIMED) return fail(ctx, XG_ERR_ARG, "mode must be XG_TUNE_MODEL or XG_TUNE_TIMED");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "tuning cannot change during a transient");
  ctx->tune_mode = mode;
  ctx->lu_ready = false;  // applies from the next analysis
  return XG_OK;
}

int xg_lu_tuning_info(xg_ctx *ctx, xg_lu_tuning *out) {
  if (!ctx || !out) return XG_ERR_ARG;
  if (!ctx->lu_ready) return fail(ctx, XG_ERR_STATE, "no LU analysis");
  *out = ctx->tuning;
  return XG_OK;
}

int xg_lu_set_schedule(xg_ctx *ctx, int ordering, int factor_top, int solve_top) {
  if (!ctx) return XG_ERR_ARG;
  if (ordering < -1 || ordering > XG_ORDER_MIN_DEGREE) return fail(ctx, XG_ERR_ARG, "unknown ordering");
  if ((factor_top != -1 && factor_top != XG_TOP_ONE_CTA && factor_top != XG_TOP_LEVELS) ||
      (solve_top != -1 && solve_top != XG_TOP_ONE_CTA && solve_top != XG_TOP_LEVELS))
    return fail(ctx, XG_ERR_ARG, "top schedule must be -1, XG_TOP_ONE_CTA or XG_TOP_LEVELS");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "the schedule cannot change during a transient");
  ctx->sched_order = ordering;
  ctx->sched_ftop = factor_top;
  ctx->sched_stop = solve_top;
  ctx->lu_ready = false;  // applies from the next analysis
  return XG_OK;
}

int xg_lu_analyze_pattern(int n, const int *row_ptr, const int *col_idx, const double *vals, int ordering,
                          long long *nnz_lu, int *ordering_out, int *n_groups, int *n_top) {
  if (n <= 0 || !row_ptr || !col_idx || !vals) return XG_ERR_ARG;
  if (ordering < -1 || ordering > XG_ORDER_MIN_DEGREE) return XG_ERR_ARG;
  const int nnz = row_ptr[n];
  if (row_ptr[0] != 0 || nnz < 0) return XG_ERR_ARG;
  for (int i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return XG_ERR_ARG;
  for (int p = 0; p < nnz; ++p)
    if (col_idx[p] < 0 || col_idx[p] >= n) return XG_ERR_ARG;
  std::vector<int> rp(row_ptr, row_ptr + n + 1), ci(col_idx, col_idx + nnz);
  std::vector<double> v(vals, vals + nnz);
  LUHost H;
  std::string err;
  const int rc = lu_analyze_host(n, rp, ci, v, H, err, ordering);
  if (rc != XG_OK) return rc;
  if (nnz_lu) *nnz_lu = (long long)H.ri.size();
  if (ordering_out) *ordering_out = H.ordering;
  if (n_groups) *n_groups = H.fsched.n_groups;
  if (n_top) *n_top = H.fsched.n_top_items;
  return XG_OK;
}

int xg_lu_info(xg_ctx *ctx, long long *nnz_lu, int *fl, int *ll, int *ul) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->lu_ready) return fail(ctx, XG_ERR_STATE, "no LU analysis");
  if (nnz_lu) *nnz_lu = ctx->L.nnz;
  if (fl) *fl = ctx->L.f_levels;
  if (ll) *ll = ctx->L.l_levels;
  if (ul) *ul = ctx->L.u_levels;
  return XG_OK;
}

int xg_lu_schedule_info(xg_ctx *ctx, int *ordering, int *factor_top, int *solve_top) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->lu_ready) return fail(ctx, XG_ERR_STATE, "no LU analysis");
  const LUDev &L = ctx->L;
  if (ordering) *ordering = L.ordering;
  if (factor_top)
    *factor_top = L.fs.n_top_items == 0 ? XG_TOP_NONE : (L.n_top_lv > 0 ? XG_TOP_LEVELS : XG_TOP_ONE_CTA);
  if (solve_top)
    *solve_top = L.fs.n_top_items == 0 ? XG_TOP_NONE : (L.h_ls_lvl_ptr ? XG_TOP_LEVELS : XG_TOP_ONE_CTA);
  return XG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Device-resident transient driver.
struct TranRun {
  xg_ctx *ctx = nullptr;
  int cap = 0, pmax = 1;
  double *bps = nullptr;
  int *bp_ptr = nullptr;
  cudaGraphExec_t exec = nullptr;
  double pivot_tol = kRuntimePivotTol;
  std::vector<void *> allocs;
  std::vector<int> pcount;
  long long ticks = 0;
  int kernels_per_tick = 0;  // kernel nodes of the captured tick graph
  int batch = 4;
  bool resident = false;          // advance with the circuit-resident tick (else the tick graph)
  long long circuit_ticks = 0;    // Newton iterations run by the resident tick, summed over circuits
  long long kernel_launches = 0;  // kernels launched while advancing
  unsigned long long tick_count[2] = {0, 0};
  // How the run advances.  Options 0..4: the resident kernel with CTAs of
  // kResidentThreads[k]; option 5: the tick graph.  Every option gives the
  // same bits, so the first advances of the transient (not the operating
  // point) time the admitted options and keep the one with the shortest
  // device time per circuit Newton iteration: the tick graph (under
  // XG_FORM_AUTO) over one advance, then resident CTA sizes one launch each,
  // from 128 threads up while larger sizes get faster, else down.
  static constexpr int kOptions = kResidentSizes + 1, kGraphOption = kResidentSizes;
  int option = -1;                        // chosen option (-1: trials not over)
  double opt_ms[kOptions] = {};
  double opt_iters[kOptions] = {};
  bool opt_done[kOptions] = {};
  int pending = -1;                       // option timed between res_ev[0] and res_ev[1]
  unsigned long long pending_iters0 = 0;  // Newton iterations before it
  cudaEvent_t res_ev[2] = {nullptr, nullptr};
  int res_threads = 0;                    // CTA size of the last resident launch
  long long graph_trial_ticks = 0;        // ticks of the tick-graph trial so far
  long long tail_launches = 0;            // resident launches that finished a tick-graph advance
  bool try_resident = false, try_graph = true;
  bool operating_point = false;           // xg_tran_start's run to the operating point: no trials
  std::chrono::steady_clock::time_point t0;
  ~TranRun() {
    if (exec) cudaGraphExecDestroy(exec);
    for (cudaEvent_t e : res_ev)
      if (e) cudaEventDestroy(e);
    free_list(allocs);
    if (ctx) { ctx->d.out_t = nullptr; ctx->d.out_v = nullptr; ctx->d.out_p = nullptr; ctx->d.out_o = nullptr; }
  }
};

void xg_free_run(xg_ctx *ctx) {
  delete ctx->run;
  ctx->run = nullptr;
}

namespace {

// The kernels of one tick before the LU (sources, device evaluation,
// assembly, Newton decision), on the arrays d (the context's, or a copy
// pointing at a caller's vectors).
void front_kernels(xg_ctx *c, const DevArrays &d) {
  launch_sources_k(c->stream, d, c->nv, c->nv + c->ni, 0, 0.0);
  launch_mos1_k(c->stream, d, c->nm, c->sto_base_m, 1, 1, 0, 0, c->sF_m, c->sQ_m, c->sL_m, c->sM_m);
  launch_bsim4_k(c->stream, d, c->nb, c->sto_base_b, c->sta_base_b, 1, 1, 0, 0, c->sF_b, c->sQ_b, c->sL_b,
                 c->sM_b);
  launch_diode_k(c->stream, d, c->nd, 1, 1, 0, 0, c->sF_d, c->sQ_d, c->sL_d, c->sM_d);
  launch_assemble_k(c->stream, d, c->n, c->nnz, c->n_long_row_blocks, c->n_long_ent_blocks);
  launch_newton_ctl_k(c->stream, d, c->ncirc);
}

// LU factor and solve, Newton update and the per-circuit step decision.
void back_kernels(xg_ctx *c, const DevArrays &d, double pivot_tol, const double *bps, const int *bp_ptr,
                  int cap) {
  launch_lu_factor_k(c->stream, c->L, d.J, d.cs, 1, pivot_tol);
  launch_lu_solve_k(c->stream, c->L, d.rhs, d.dx, d.cs, 1);
  launch_update_k(c->stream, d, c->n);
  launch_step_ctl_k(c->stream, d, c->ncirc, bps, bp_ptr, cap);
}

void launch_front(TranRun &R) { front_kernels(R.ctx, R.ctx->d); }

void launch_back(TranRun &R) {
  xg_ctx *c = R.ctx;
  DevArrays &d = c->d;
  back_kernels(c, d, R.pivot_tol, R.bps, R.bp_ptr, R.cap);
  launch_history_k(c->stream, d, c->n, R.cap, R.pmax);
  if (c->predictor == XG_PRED_LEARNED) launch_ml_predict_k(c->stream, d, c->n, c->ncirc, 1);
  launch_state_commit_k(c->stream, d, c->nm, c->nd, c->sto_base_m, c->nb, c->sto_base_b, c->sta_base_b);
}

int capture(TranRun &R) {
  xg_ctx *ctx = R.ctx;
  if (R.exec) { cudaGraphExecDestroy(R.exec); R.exec = nullptr; }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  launch_front(R);
  launch_back(R);
  CK(cudaStreamEndCapture(ctx->stream, &g));
  // kernels of one tick (every node of the captured tick is a kernel launch
  // unless the query says otherwise)
  {
    size_t nn = 0;
    R.kernels_per_tick = 0;
    if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn > 0) {
      std::vector<cudaGraphNode_t> nodes(nn);
      if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
        for (size_t k = 0; k < nn; ++k) {
          cudaGraphNodeType ty;
          if (cudaGraphNodeGetType(nodes[k], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
            R.kernels_per_tick++;
        }
    }
  }
  cudaError_t e = cudaGraphInstantiate(&R.exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(ctx, XG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return XG_OK;
}

// Source breakpoints of one circuit (PulseData/PWLinData::getBreakPoints,
// N_DEV_SourceData.C:1442, 2044) plus tstop.
void breakpoints(const Wave &w, double tstop, std::vector<double> &bp) {
  const auto &d = w.d;
  if (w.kind == XG_WAVE_PWL) {
    for (size_t i = 0; i + 1 < d.size(); i += 2)
      if (d[i] > 0 && d[i] < tstop) bp.push_back(d[i]);
  } else if (w.kind == XG_WAVE_PULSE) {
    double base = d[2];
    for (int k = 0; k < 100000 && base < tstop; ++k) {
      double cand[4] = {base, base + d[3], base + d[3] + d[5], base + d[3] + d[5] + d[4]};
      for (double x : cand)
        if (x > 0 && x < tstop) bp.push_back(x);
      if (d[6] <= 0) break;
      base += d[6];
    }
  }
}

// The circuits parked on a pivot breakdown (phase STALL): the ones a
// re-analysis re-pivots.  Empty vector: none parked (re-pivot all).
int stalled_circuits(xg_ctx *ctx, std::vector<char> &refresh) {
  std::vector<CircState> cs(ctx->ncirc);
  CK(cudaMemcpyAsync(cs.data(), ctx->d.cs, sizeof(CircState) * ctx->ncirc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  refresh.assign(ctx->ncirc, 0);
  bool any = false;
  for (int c = 0; c < ctx->ncirc; ++c)
    if (cs[c].phase == PH_STALL) { refresh[c] = 1; any = true; }
  if (!any) refresh.clear();
  return XG_OK;
}

// The next option to time (-1: none left).  The tick graph first; then the
// resident CTA sizes: 128 and 256 threads, then on in the direction that got
// faster (512, or 64 and then 32) until a size is slower than the last —
// unless both sizes took more than 1.15 times the tick graph's time.
int next_trial(const TranRun &R) {
  if (R.try_graph && !R.opt_done[TranRun::kGraphOption]) return TranRun::kGraphOption;
  if (!R.try_resident) return -1;
  auto per = [&](int k) { return R.opt_ms[k] / R.opt_iters[k]; };
  int k = 2;
  if (!R.opt_done[k]) return k;
  if (!R.opt_done[k + 1]) return k + 1;
  // both resident sizes well behind the tick graph: the others will not catch up
  if (R.try_graph && std::min(per(k), per(k + 1)) > 1.15 * per(TranRun::kGraphOption)) return -1;
  const int dir = per(k + 1) < per(k) ? 1 : -1;
  if (dir > 0) k = k + 1;
  while (k + dir >= 0 && k + dir < kResidentSizes) {
    if (!R.opt_done[k + dir]) return k + dir;
    if (!(per(k + dir) < per(k))) break;
    k += dir;
  }
  return -1;
}

// Runs tick batches until every circuit is done, failed or paused; re-pivots
// on LU breakdown.  One host synchronization per batch of ticks.
int run_until_idle(TranRun &R) {
  xg_ctx *ctx = R.ctx;
  DevArrays &d = ctx->d;
  const long long max_ticks = 400000000LL;
  int consecutive = 0;
  int rc = 0;
  while (true) {
    CK(cudaStreamSynchronize(ctx->stream));
    volatile int *st = ctx->status_host;
    const int finished = st[0], breakdown = st[1];
    if (breakdown) {
      // frozen pivots failed: re-pivot from the parked Jacobian and resume it
      consecutive++;
      if (consecutive > 4) return fail(ctx, XG_ERR_SINGULAR, "LU keeps breaking down after re-pivoting");
      std::vector<char> refresh;
      if ((rc = stalled_circuits(ctx, refresh))) return rc;
      if ((rc = lu_analyze_from_device(ctx, d.J, refresh.empty() ? nullptr : &refresh))) return rc;
      R.pivot_tol = (consecutive >= 2) ? 0.0 : ctx->pivot_tol;
      R.pending = -1;  // a timed launch that parked on a breakdown is not a trial
      if ((rc = capture(R))) return rc;
      launch_unstall_k(ctx->stream, d, ctx->ncirc);
      launch_back(R);
      launch_count_done_k(ctx->stream, d, ctx->ncirc, ctx->breakdown_dev, ctx->status_dev);
      CK(cudaGetLastError());
      R.kernel_launches += R.kernels_per_tick;
      continue;
    }
    if (consecutive && R.pivot_tol == 0.0) {
      R.pivot_tol = ctx->pivot_tol;
      if ((rc = capture(R))) return rc;
    }
    consecutive = 0;
    const unsigned long long iters_now = reinterpret_cast<volatile unsigned long long *>(st)[1];
    if (R.pending >= 0) {
      // one timed trial launch (or tick-graph batch) ended
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, R.res_ev[0], R.res_ev[1]) == cudaSuccess) {
        R.opt_ms[R.pending] += ms;
        R.opt_iters[R.pending] += (double)(iters_now - R.pending_iters0);
      }
      const bool idle = finished >= ctx->ncirc;
      if ((R.pending != TranRun::kGraphOption || idle || R.graph_trial_ticks >= kFusedMaxTicks) &&
          R.opt_iters[R.pending] > 0)
        R.opt_done[R.pending] = true;
      R.pending = -1;
      if (next_trial(R) < 0) {
        int best = -1;
        for (int k = 0; k < TranRun::kOptions; ++k)
          if (R.opt_done[k] && (best < 0 || R.opt_ms[k] / R.opt_iters[k] < R.opt_ms[best] / R.opt_iters[best]))
            best = k;
        if (best >= 0) R.option = best;
      }
    }
    if (R.tick_count[0]) {
      // the last resident launch: its longest circuit's ticks, and all of them
      R.ticks += (long long)R.tick_count[0];
      R.circuit_ticks += (long long)R.tick_count[1];
      R.tick_count[0] = R.tick_count[1] = 0;
    }
    if (finished >= ctx->ncirc) return XG_OK;
    if (R.ticks > max_ticks) return fail(ctx, XG_ERR_TIMEOUT, "transient exceeded the tick limit");
    int opt = R.option;
    bool trial = false;
    if (opt < 0 && R.operating_point) {
      // the operating point's Newton iterations are not the transient's:
      // the trials wait for the first advance
      opt = R.try_graph ? TranRun::kGraphOption : 2;
    } else if (opt < 0) {
      opt = next_trial(R);
      trial = opt >= 0;
      if (opt < 0) opt = TranRun::kGraphOption;
    }
    if (opt != TranRun::kGraphOption && !ctx->resident_ok) { opt = TranRun::kGraphOption; trial = false; }
    if (trial) {
      for (cudaEvent_t &e : R.res_ev)
        if (!e) CK(cudaEventCreate(&e));
      R.pending = opt;
      R.pending_iters0 = iters_now;
      CK(cudaEventRecord(R.res_ev[0], ctx->stream));
    }
    // the tail of an advance under the tick graph: once few circuits are
    // still active, the resident kernel finishes them (the same bits; a
    // handful of circuits no longer pays full-batch launches per tick)
    const int active = ctx->ncirc - finished;
    const bool tail = opt == TranRun::kGraphOption && ctx->form == XG_FORM_AUTO && ctx->resident_ok &&
                      ctx->tail_fraction > 0.0 && active <= ctx->tail_fraction * ctx->ncirc;
    R.resident = opt != TranRun::kGraphOption || tail;
    if (R.resident) {
      // every circuit runs its ticks in one CTA until it pauses, finishes,
      // fails or parks on a pivot breakdown
      R.res_threads = tail ? kResidentThreads[3] : kResidentThreads[opt];
      if (tail) R.tail_launches++;
      launch_resident_k(ctx->stream, d, ctx->L, ctx->F, R.res_threads, ctx->ncirc, ctx->nm, ctx->nd, ctx->nv,
                        ctx->sto_base_m, ctx->resident_slots, R.bps, R.bp_ptr, R.cap, R.pmax, R.pivot_tol);
      if (trial) CK(cudaEventRecord(R.res_ev[1], ctx->stream));
      launch_count_done_k(ctx->stream, d, ctx->ncirc, ctx->breakdown_dev, ctx->status_dev);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(R.tick_count, ctx->F.ticks, sizeof R.tick_count, cudaMemcpyDeviceToHost, ctx->stream));
      R.kernel_launches += 2;
      continue;
    }
    for (int k = 0; k < R.batch; ++k) CK(cudaGraphLaunch(R.exec, ctx->stream));
    // what the host reads between batches (the tick graph itself does not count)
    launch_count_done_k(ctx->stream, d, ctx->ncirc, ctx->breakdown_dev, ctx->status_dev);
    CK(cudaGetLastError());
    if (trial) {
      CK(cudaEventRecord(R.res_ev[1], ctx->stream));
      R.graph_trial_ticks += R.batch;
    }
    R.ticks += R.batch;
    R.kernel_launches += (long long)R.batch * R.kernels_per_tick + 1;
    if (R.batch < 64) R.batch *= 2;
    // near the tail threshold, short batches let the host see it promptly
    if (ctx->form == XG_FORM_AUTO && ctx->resident_ok && ctx->tail_fraction > 0.0 &&
        active <= 2.0 * ctx->tail_fraction * ctx->ncirc)
      R.batch = std::min(R.batch, 8);
  }
}

}  // namespace

static int tran_start_run(xg_ctx *ctx, const xg_tran_params *p, const std::vector<int> &probe_idx,
                          const std::vector<int> &pcount, int cap);

extern "C" int xg_tran_start(xg_ctx *ctx, const xg_tran_params *p, int n_probe, const int *probes, int cap) {
  if (!ctx || !p) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  if (!(p->tstop > p->tstart)) return fail(ctx, XG_ERR_ARG, "tstop must exceed tstart");
  if (!std::isfinite(p->tstart) || !std::isfinite(p->tstop)) return fail(ctx, XG_ERR_ARG, "tstart and tstop must be finite");
  if (cap < 0 || n_probe < 0) return fail(ctx, XG_ERR_ARG, "negative cap or probe count");
  if (n_probe > 0 && !probes) return fail(ctx, XG_ERR_ARG, "null probe list");
  if (p->method != 0 && p->method != XG_METHOD_ONESTEP && p->method != XG_METHOD_GEAR)
    return fail(ctx, XG_ERR_ARG, "method must be XG_METHOD_ONESTEP or XG_METHOD_GEAR");
  {
    // the error weights and the Newton tests divide by or compare against these
    auto positive = [](double v) { return v > 0.0 && std::isfinite(v); };
    auto nonnegative = [](double v) { return v >= 0.0 && std::isfinite(v); };
    if (!positive(p->reltol) || !positive(p->abstol) || !positive(p->nl_reltol) || !positive(p->nl_abstol) ||
        !positive(p->nl_deltaxtol) || !positive(p->nl_rhstol))
      return fail(ctx, XG_ERR_ARG, "tolerances must be positive and finite");
    if (!nonnegative(p->nl_smallupdatetol) || !nonnegative(p->hmin) || !nonnegative(p->hmax))
      return fail(ctx, XG_ERR_ARG, "nl_smallupdatetol, hmin and hmax must be non-negative and finite");
    if (p->nl_maxstep < 1) return fail(ctx, XG_ERR_ARG, "nl_maxstep must be at least 1");
    if (p->max_order < 0 || p->max_order > 2) return fail(ctx, XG_ERR_ARG, "max_order must be 1 or 2 (0 = 2)");
  }
  // Everything a call can be rejected for is checked before the previous
  // run is released: a rejected call leaves that run (and its results) as
  // they were.
  const int n = ctx->n, ncirc = ctx->ncirc;
  std::vector<int> probe_idx(n, -1), pcount(ncirc, 0);
  for (int k = 0; k < n_probe; ++k) {
    if (probes[k] < 0 || probes[k] >= n) return fail(ctx, XG_ERR_ARG, "probe out of range");
    if (probe_idx[probes[k]] != -1) return fail(ctx, XG_ERR_ARG, "probe listed twice");
    probe_idx[probes[k]] = pcount[ctx->circ_of_row[probes[k]]]++;
  }
  if (ctx->predictor == XG_PRED_LEARNED && !ctx->mlp_ready)
    return fail(ctx, XG_ERR_STATE, "learned predictor selected but no weights: call xg_mlp_set or xg_mlp_train");
  CK(cudaSetDevice(ctx->device));
  if (ctx->run) xg_free_run(ctx);
  ctx->run = new TranRun;
  const int rc = tran_start_run(ctx, p, probe_idx, pcount, cap);
  // a run that failed before its tick graph existed cannot advance: release it
  if (rc != XG_OK && ctx->run && !ctx->run->exec) {
    std::string keep = ctx->err;
    cudaStreamSynchronize(ctx->stream);
    xg_free_run(ctx);
    ctx->err = keep;
  }
  return rc;
}

static int tran_start_run(xg_ctx *ctx, const xg_tran_params *p, const std::vector<int> &probe_idx,
                          const std::vector<int> &pcount, int cap) {
  TranRun &R = *ctx->run;
  R.t0 = std::chrono::steady_clock::now();
  R.ctx = ctx;
  R.cap = cap;
  R.pivot_tol = ctx->pivot_tol;
  const int n = ctx->n, ncirc = ctx->ncirc;
  DevArrays &d = ctx->d;
  R.pcount = pcount;
  R.pmax = 1;
  for (int c = 0; c < ncirc; ++c) R.pmax = std::max(R.pmax, R.pcount[c]);
  CK(cudaMemcpyAsync(d.probe_idx, probe_idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = 0;
  if ((rc = dev_alloc(ctx, &d.out_t, (size_t)ncirc * std::max(cap, 1), R.allocs))) return rc;
  if ((rc = dev_alloc(ctx, &d.out_o, (size_t)ncirc * std::max(cap, 1), R.allocs))) return rc;
  if ((rc = dev_alloc(ctx, &d.out_v, (size_t)ncirc * std::max(cap, 1) * R.pmax, R.allocs))) return rc;
  if ((rc = dev_alloc(ctx, &d.out_p, (size_t)ncirc * std::max(cap, 1) * R.pmax, R.allocs))) return rc;
  std::vector<std::vector<double>> cb(ncirc);
  for (int k = 0; k < ctx->nv; ++k) breakpoints(ctx->v_w[k], p->tstop, cb[ctx->circ_of_row[ctx->v_b[k]]]);
  for (int k = 0; k < ctx->ni; ++k) {
    int c = circuit_of_nodes(ctx, {ctx->i_p[k], ctx->i_n[k]});
    breakpoints(ctx->i_w[k], p->tstop, cb[c < 0 ? 0 : c]);
  }
  std::vector<double> bps;
  std::vector<int> bp_ptr(1, 0);
  for (int c = 0; c < ncirc; ++c) {
    auto &v = cb[c];
    v.push_back(p->tstop);
    std::sort(v.begin(), v.end());
    bps.insert(bps.end(), v.begin(), v.end());
    bp_ptr.push_back((int)bps.size());
  }
  if ((rc = dev_upload(ctx, &R.bps, bps, R.allocs))) return rc;
  if ((rc = dev_upload(ctx, &R.bp_ptr, bp_ptr, R.allocs))) return rc;
  TranParams tp{};
  tp.tstart = p->tstart; tp.tstop = p->tstop;
  tp.hmax = p->hmax > 0 ? p->hmax : 0.1 * (p->tstop - p->tstart);
  tp.hmin = p->hmin;
  tp.reltol = p->reltol; tp.abstol = p->abstol;
  tp.nl_reltol = p->nl_reltol; tp.nl_abstol = p->nl_abstol; tp.nl_deltaxtol = p->nl_deltaxtol;
  tp.nl_rhstol = p->nl_rhstol; tp.nl_smallupdatetol = p->nl_smallupdatetol; tp.nl_maxstep = p->nl_maxstep;
  tp.max_steps = p->max_steps; tp.max_order = p->max_order > 0 ? p->max_order : 2;
  tp.gear = (p->method == XG_METHOD_GEAR) ? 1 : 0;
  tp.reuse_factors = ctx->lu_reuse;
  tp.bptol = 1e-15 * (p->tstop - p->tstart);
  tp.dc_reltol = 1e-3; tp.dc_abstol = 1e-12; tp.dc_deltaxtol = 1.0; tp.dc_rhstol = 1e-6; tp.dc_maxstep = 200;
  tp.dc_only = (p->max_steps < 0) ? 1 : 0;
  CK(cudaMemcpyAsync(d.tp, &tp, sizeof tp, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<CircState> cs(ncirc);
  for (auto &s : cs) {
    memset(&s, 0, sizeof s);
    s.phase = PH_DC;
    s.tn = p->tstart;
    s.t = p->tstart;
    s.qscale = 0.0; s.fscale = 1.0; s.hscale = 0.0;
    s.init_jct = 1;
    s.order = 1;
    s.refactor = 1;
    s.f_gen = -1;
    s.stop_at = 0;  // pause once the operating point is done
  }
  CK(cudaMemcpyAsync(d.cs, cs.data(), sizeof(CircState) * ncirc, cudaMemcpyHostToDevice, ctx->stream));
  for (double *v : {d.x, d.xcurr, d.xn0, d.dx, d.rhs, d.Qv, d.FmB, d.qh0, d.qh1, d.qh2, d.xh1, d.xh2, d.Qc, d.FmBc, d.solwt,
                    d.mlh1, d.mlh2, d.mlh3})
    CK(cudaMemsetAsync(v, 0, sizeof(double) * n, ctx->stream));
  for (double *v : {d.sta_curr, d.sta_next})
    CK(cudaMemsetAsync(v, 0, sizeof(double) * std::max(1, ctx->nsta), ctx->stream));
  for (double *v : {d.sto_curr, d.sto_next})
    CK(cudaMemsetAsync(v, 0, sizeof(double) * std::max(1, ctx->nsto), ctx->stream));
  CK(cudaMemsetAsync(ctx->breakdown_dev, 0, sizeof(int), ctx->stream));
  ctx->status_host[0] = ctx->status_host[1] = 0;
  // first tick: evaluate and assemble, analyze that Jacobian, finish the tick
  R.ticks = 1;
  launch_front(R);
  CK(cudaGetLastError());
  if ((rc = lu_analyze_from_device(ctx, d.J))) return rc;
  if (ctx->form == XG_FORM_RESIDENT && !ctx->resident_ok)
    return fail(ctx, XG_ERR_UNSUPPORTED,
                "circuit-resident tick: needs >= 64 circuits of <= 2048 unknowns, MOSFET-1 / diode devices, "
                "FP64 factors, the polynomial predictor and an LU without a top");
  R.try_resident = ctx->resident_ok && ctx->form != XG_FORM_TICK_GRAPH;
  R.try_graph = ctx->form != XG_FORM_RESIDENT;
  R.resident = R.try_resident;
  if ((rc = capture(R))) return rc;
  launch_back(R);
  launch_count_done_k(ctx->stream, d, ncirc, ctx->breakdown_dev, ctx->status_dev);
  CK(cudaGetLastError());
  R.operating_point = true;
  rc = run_until_idle(R);
  R.operating_point = false;
  return rc;
}

extern "C" int xg_tran_set_form(xg_ctx *ctx, int form) {
  if (!ctx) return XG_ERR_ARG;
  if (form != XG_FORM_AUTO && form != XG_FORM_TICK_GRAPH && form != XG_FORM_RESIDENT)
    return fail(ctx, XG_ERR_ARG, "form must be XG_FORM_AUTO, XG_FORM_TICK_GRAPH or XG_FORM_RESIDENT");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "the form cannot change during a transient");
  ctx->form = form;
  return XG_OK;
}

extern "C" int xg_tran_set_tail(xg_ctx *ctx, double active_fraction) {
  if (!ctx) return XG_ERR_ARG;
  if (!(active_fraction >= 0.0 && active_fraction <= 1.0))
    return fail(ctx, XG_ERR_ARG, "active_fraction must be in [0, 1]");
  ctx->tail_fraction = active_fraction;
  return XG_OK;
}

extern "C" int xg_tran_advance(xg_ctx *ctx, int n_steps) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->run || !ctx->run->exec) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  TranRun &R = *ctx->run;
  launch_set_target_k(ctx->stream, ctx->d, ctx->ncirc, n_steps);
  launch_count_done_k(ctx->stream, ctx->d, ctx->ncirc, ctx->breakdown_dev, ctx->status_dev);
  CK(cudaGetLastError());
  R.batch = 4;
  return run_until_idle(R);
}

extern "C" int xg_tran_results(xg_ctx *ctx, int *counts, double *times, double *values, xg_tran_stats *stats) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->run) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  TranRun &R = *ctx->run;
  const int ncirc = ctx->ncirc;
  DevArrays &d = ctx->d;
  std::vector<CircState> out(ncirc);
  CK(cudaMemcpyAsync(out.data(), d.cs, sizeof(CircState) * ncirc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const int cap = R.cap;
  if (cap > 0 && counts && times) {
    for (int c = 0; c < ncirc; ++c) counts[c] = std::min(out[c].n_out, cap);
    CK(cudaMemcpy(times, d.out_t, sizeof(double) * (size_t)ncirc * cap, cudaMemcpyDeviceToHost));
    if (values) CK(cudaMemcpy(values, d.out_v, sizeof(double) * (size_t)ncirc * cap * R.pmax, cudaMemcpyDeviceToHost));
  }
  int status = 0;
  for (auto &s : out)
    if (s.phase == PH_FAILED) { status = s.newton_status ? s.newton_status : -1; break; }
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->t_final_min = 1e300;
    stats->t_final_max = -1e300;
    long long evals = 0;
    for (int c = 0; c < ncirc; ++c) {
      const CircState &s = out[c];
      stats->accepted += s.accepted;
      stats->rejected += s.rejected;
      stats->newton_iters += s.newton_iters;
      stats->newton_fail += s.newton_fail;
      stats->lte_fail += s.lte_fail;
      stats->dcop_iters += s.dcop_iters;
      stats->factor_skips += s.factor_skips;
      stats->t_final_min = std::min(stats->t_final_min, s.t);
      stats->t_final_max = std::max(stats->t_final_max, s.t);
      // instance evaluations: one device pass per Newton solve, plus the
      // first pass of every step attempt and of the operating point
      const long long passes = s.newton_iters + s.accepted + s.rejected + s.dcop_iters + 1;
      evals += (long long)ctx->inst_of_circ[c] * passes;
    }
    stats->ticks = R.ticks;
    stats->kernels_per_tick = R.kernels_per_tick;
    // the form the run advances with (the option the trials kept, else the
    // last launch's; a resident tail does not change a tick-graph run's form)
    const bool res = R.option >= 0 ? R.option != TranRun::kGraphOption : (R.resident && R.tail_launches == 0);
    stats->form = res ? XG_FORM_RESIDENT : XG_FORM_TICK_GRAPH;
    stats->kernel_launches = R.kernel_launches;
    stats->circuit_ticks = R.circuit_ticks;
    stats->resident_threads = R.res_threads;
    stats->option = R.option;
    stats->tail_launches = R.tail_launches;
    for (int k = 0; k < TranRun::kOptions; ++k)
      stats->option_us_per_iter[k] = R.opt_iters[k] > 0 ? 1e3 * R.opt_ms[k] / R.opt_iters[k] : 0.0;
    stats->device_evals = evals;
    stats->n_analyze = ctx->n_analyze;
    stats->status = status;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - R.t0).count();
  }
  if (status) return fail(ctx, status, "a circuit failed to converge");
  return XG_OK;
}

extern "C" int xg_tran_predictors(xg_ctx *ctx, double *pred_values) {
  if (!ctx || !pred_values) return XG_ERR_ARG;
  if (!ctx->run) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  TranRun &R = *ctx->run;
  if (R.cap <= 0) return fail(ctx, XG_ERR_STATE, "nothing recorded (cap = 0)");
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(pred_values, ctx->d.out_p, sizeof(double) * (size_t)ctx->ncirc * R.cap * R.pmax,
                cudaMemcpyDeviceToHost));
  return XG_OK;
}

// Ticks of a transient in progress, each kernel stage launched on its own
// with CUDA events between the stages (the kernels and their order are those
// of the captured tick graph, so the run continues exactly as it would).
extern "C" int xg_tran_profile(xg_ctx *ctx, int n_steps, int n_ticks, double *stage_ms, long long *evals) {
  if (!ctx || !stage_ms || n_ticks < 0) return XG_ERR_ARG;
  if (!ctx->run || !ctx->run->exec) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  TranRun &R = *ctx->run;
  xg_ctx *c = ctx;
  DevArrays &d = c->d;
  const cudaStream_t st = c->stream;
  if (evals) for (int k = 0; k < 4; ++k) evals[k] = 0;
  if (n_steps > 0) {
    // a new window, as xg_tran_advance opens one
    launch_set_target_k(st, d, c->ncirc, n_steps);
    launch_count_done_k(st, d, c->ncirc, c->breakdown_dev, c->status_dev);
  }
  cudaEvent_t ev[XG_STAGE_COUNT + 1];
  int made = 0;
  for (auto &e : ev) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      for (int k = 0; k < made; ++k) cudaEventDestroy(ev[k]);
      return fail(ctx, XG_ERR_CUDA, "cudaEventCreate");
    }
    made++;
  }
  int rc = XG_OK;
  std::vector<CircState> cs(c->ncirc);
  for (int t = 0; t < n_ticks && rc == XG_OK; ++t) {
    if (evals) {
      // instances each model kernel evaluates this tick: those of active circuits
      if (cudaMemcpyAsync(cs.data(), d.cs, sizeof(CircState) * c->ncirc, cudaMemcpyDeviceToHost, st) !=
              cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) { rc = XG_ERR_CUDA; break; }
      for (int q = 0; q < c->ncirc; ++q)
        if (cs[q].phase == PH_DC || cs[q].phase == PH_TRAN) {
          evals[0] += c->circ_m1[q];
          evals[1] += c->circ_b4[q];
          evals[2] += c->circ_d[q];
          evals[3] += 1;
        }
    }
    int s = 0;
    cudaEventRecord(ev[s++], st);
    launch_sources_k(st, d, c->nv, c->nv + c->ni, 0, 0.0);
    cudaEventRecord(ev[s++], st);
    launch_mos1_k(st, d, c->nm, c->sto_base_m, 1, 1, 0, 0, c->sF_m, c->sQ_m, c->sL_m, c->sM_m);
    cudaEventRecord(ev[s++], st);
    launch_bsim4_k(st, d, c->nb, c->sto_base_b, c->sta_base_b, 1, 1, 0, 0, c->sF_b, c->sQ_b, c->sL_b, c->sM_b);
    cudaEventRecord(ev[s++], st);
    launch_diode_k(st, d, c->nd, 1, 1, 0, 0, c->sF_d, c->sQ_d, c->sL_d, c->sM_d);
    cudaEventRecord(ev[s++], st);
    launch_assemble_k(st, d, c->n, c->nnz, c->n_long_row_blocks, c->n_long_ent_blocks);
    cudaEventRecord(ev[s++], st);
    launch_newton_ctl_k(st, d, c->ncirc);
    cudaEventRecord(ev[s++], st);
    launch_lu_factor_k(st, c->L, d.J, d.cs, 1, R.pivot_tol);
    cudaEventRecord(ev[s++], st);
    launch_lu_solve_k(st, c->L, d.rhs, d.dx, d.cs, 1);
    cudaEventRecord(ev[s++], st);
    launch_update_k(st, d, c->n);
    cudaEventRecord(ev[s++], st);
    launch_step_ctl_k(st, d, c->ncirc, R.bps, R.bp_ptr, R.cap);
    cudaEventRecord(ev[s++], st);
    launch_history_k(st, d, c->n, R.cap, R.pmax);
    if (c->predictor == XG_PRED_LEARNED) launch_ml_predict_k(st, d, c->n, c->ncirc, 1);
    cudaEventRecord(ev[s++], st);
    launch_state_commit_k(st, d, c->nm, c->nd, c->sto_base_m, c->nb, c->sto_base_b, c->sta_base_b);
    cudaEventRecord(ev[s++], st);
    // the completion count runs once per batch of ticks, outside the tick
    launch_count_done_k(st, d, c->ncirc, c->breakdown_dev, c->status_dev);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) { rc = XG_ERR_CUDA; break; }
    for (int k = 0; k < XG_STAGE_COUNT; ++k) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      stage_ms[k] += ms;
    }
    R.ticks++;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (rc) return fail(ctx, rc, "tick profile: CUDA failure");
  return XG_OK;
}

extern "C" int xg_tran_profile_resident(xg_ctx *ctx, int n_steps, int threads, double *stage_cycles,
                                        long long *circuit_ticks) {
  if (!ctx || !stage_cycles) return XG_ERR_ARG;
  if (threads != 32 && threads != 64 && threads != 128)
    return fail(ctx, XG_ERR_ARG, "threads must be 32, 64 or 128");
  if (!ctx->run || !ctx->run->exec) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  if (!ctx->resident_ok) return fail(ctx, XG_ERR_UNSUPPORTED, "the run's analysis does not admit the resident tick");
  TranRun &R = *ctx->run;
  DevArrays &d = ctx->d;
  CK(cudaSetDevice(ctx->device));
  unsigned long long *clk = nullptr;
  CK(cudaMalloc(&clk, sizeof(unsigned long long) * XG_RSTAGE_COUNT));
  std::vector<unsigned long long> h(XG_RSTAGE_COUNT, 0);
  int rc = XG_OK;
  auto step = [&](cudaError_t e) {
    if (rc == XG_OK && e != cudaSuccess) rc = fail(ctx, XG_ERR_CUDA, std::string("resident profile: ") + cudaGetErrorString(e));
  };
  step(cudaMemsetAsync(clk, 0, sizeof(unsigned long long) * XG_RSTAGE_COUNT, ctx->stream));
  if (n_steps > 0) launch_set_target_k(ctx->stream, d, ctx->ncirc, n_steps);
  launch_resident_k(ctx->stream, d, ctx->L, ctx->F, threads, ctx->ncirc, ctx->nm, ctx->nd, ctx->nv, ctx->sto_base_m,
                    ctx->resident_slots, R.bps, R.bp_ptr, R.cap, R.pmax, R.pivot_tol, clk);
  launch_count_done_k(ctx->stream, d, ctx->ncirc, ctx->breakdown_dev, ctx->status_dev);
  step(cudaGetLastError());
  step(cudaMemcpyAsync(h.data(), clk, sizeof(unsigned long long) * XG_RSTAGE_COUNT, cudaMemcpyDeviceToHost,
                       ctx->stream));
  step(cudaMemcpyAsync(R.tick_count, ctx->F.ticks, sizeof R.tick_count, cudaMemcpyDeviceToHost, ctx->stream));
  step(cudaStreamSynchronize(ctx->stream));
  cudaFree(clk);
  if (rc) return rc;
  for (int k = 0; k < XG_RSTAGE_COUNT; ++k) stage_cycles[k] = (double)h[k];
  if (circuit_ticks) *circuit_ticks = (long long)R.tick_count[1];
  R.kernel_launches += 2;
  // circuits parked on a breakdown or stopped by the tick bound finish the window as an advance would
  return run_until_idle(R);
}

extern "C" int xg_tran_orders(xg_ctx *ctx, int *orders) {
  if (!ctx || !orders) return XG_ERR_ARG;
  if (!ctx->run) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  TranRun &R = *ctx->run;
  if (R.cap <= 0) return fail(ctx, XG_ERR_STATE, "nothing recorded (cap = 0)");
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<signed char> o((size_t)ctx->ncirc * R.cap);
  CK(cudaMemcpy(o.data(), ctx->d.out_o, o.size(), cudaMemcpyDeviceToHost));
  for (size_t k = 0; k < o.size(); ++k) orders[k] = o[k];
  return XG_OK;
}

extern "C" int xg_tran_predictor_stats(xg_ctx *ctx, long long *learned_steps, long long *learned_iters,
                                       long long *poly_steps, long long *poly_iters) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->run) return fail(ctx, XG_ERR_STATE, "call xg_tran_start first");
  std::vector<CircState> out(ctx->ncirc);
  CK(cudaMemcpyAsync(out.data(), ctx->d.cs, sizeof(CircState) * ctx->ncirc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  long long a = 0, b = 0, c = 0, e = 0;
  for (auto &s : out) { a += s.ml_steps; b += s.ml_iters; c += s.plain_steps; e += s.plain_iters; }
  if (learned_steps) *learned_steps = a;
  if (learned_iters) *learned_iters = b;
  if (poly_steps) *poly_steps = c;
  if (poly_iters) *poly_iters = e;
  return XG_OK;
}

extern "C" int xg_tran_end(xg_ctx *ctx) {
  if (!ctx) return XG_ERR_ARG;
  if (ctx->run) {
    cudaStreamSynchronize(ctx->stream);
    xg_free_run(ctx);
  }
  return XG_OK;
}

extern "C" int xg_transient(xg_ctx *ctx, const xg_tran_params *p, int n_probe, const int *probes, int cap,
                            int *counts, double *times, double *values, xg_tran_stats *stats) {
  if (!ctx || !p) return XG_ERR_ARG;
  if (cap > 0 && (!counts || !times || (n_probe > 0 && !values))) return fail(ctx, XG_ERR_ARG, "output buffers required");
  if (stats) memset(stats, 0, sizeof *stats);
  int rc = xg_tran_start(ctx, p, n_probe, probes, cap);
  if (rc == XG_OK && p->max_steps >= 0) rc = xg_tran_advance(ctx, p->max_steps > 0 ? p->max_steps : 0);
  int rr = XG_OK;
  if (ctx->run) rr = xg_tran_results(ctx, counts, times, values, stats);
  std::string keep = ctx->err;
  xg_tran_end(ctx);
  ctx->err = keep;
  return rc ? rc : rr;
}

extern "C" int xg_dcop(xg_ctx *ctx, double *x_host, int *iters) {
  if (!ctx || !x_host) return XG_ERR_ARG;
  xg_tran_params p{};
  p.tstart = 0.0; p.tstop = 1.0; p.hmax = 0.1;
  p.reltol = 1e-3; p.abstol = 1e-6;
  p.nl_reltol = 1e-2; p.nl_abstol = 1e-6; p.nl_deltaxtol = 0.33; p.nl_rhstol = 1e-2; p.nl_smallupdatetol = 1e-6;
  p.nl_maxstep = 20; p.max_steps = -1; p.max_order = 2;
  xg_tran_stats st;
  int rc = xg_transient(ctx, &p, 0, nullptr, 0, nullptr, nullptr, nullptr, &st);
  if (iters) *iters = (int)st.dcop_iters;
  if (rc) return rc;
  CK(cudaMemcpy(x_host, ctx->d.xcurr, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost));
  return XG_OK;
}

// ---------------------------------------------------------------------------
// One Newton solve per circuit on the device (DampedNewton::solve).
extern "C" int xg_newton_solve(xg_ctx *ctx, const xg_newton_params *p, double time, double qscale,
                               double fscale, double hscale, const double *qhist0, const double *qhist2,
                               double *x, const double *x_curr, const double *curr_sta, const double *curr_sto,
                               double *next_sta, double *next_sto, int flags, int *status, int *iters) {
  if (!ctx || !p || !x || !status) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "a transient is in progress: end it first");
  auto positive = [](double v) { return v > 0.0 && std::isfinite(v); };
  if (!positive(p->reltol) || !positive(p->abstol) || !positive(p->deltaxtol) || !positive(p->rhstol) ||
      !(p->smallupdatetol >= 0.0 && std::isfinite(p->smallupdatetol)))
    return fail(ctx, XG_ERR_ARG, "Newton tolerances must be positive and finite");
  if (p->maxstep < 1) return fail(ctx, XG_ERR_ARG, "maxstep must be at least 1");
  if (!std::isfinite(time) || !std::isfinite(qscale) || !std::isfinite(fscale) || !std::isfinite(hscale))
    return fail(ctx, XG_ERR_ARG, "time and coefficients must be finite");
  if ((qscale != 0.0 && !qhist0) || (hscale != 0.0 && !qhist2))
    return fail(ctx, XG_ERR_ARG, "a nonzero qscale / hscale needs its history vector");
  if ((ctx->nsta > 0 && (!curr_sta || !next_sta)) || (ctx->nsto > 0 && (!curr_sto || !next_sto)))
    return fail(ctx, XG_ERR_ARG, "state/store vectors are required");
  if (flags & ~(XG_FLAG_DCOP | XG_FLAG_INITJCT)) return fail(ctx, XG_ERR_ARG, "unknown solver-state flag");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->n, ncirc = ctx->ncirc;
  const bool dcop = (flags & XG_FLAG_DCOP) != 0;
  TranParams tp{};
  tp.tstart = time; tp.tstop = time + 1.0; tp.hmax = 1.0;
  tp.reltol = 1.0; tp.abstol = 1.0;
  tp.nl_reltol = p->reltol; tp.nl_abstol = p->abstol; tp.nl_deltaxtol = p->deltaxtol;
  tp.nl_rhstol = p->rhstol; tp.nl_smallupdatetol = p->smallupdatetol; tp.nl_maxstep = p->maxstep;
  tp.dc_reltol = p->reltol; tp.dc_abstol = p->abstol; tp.dc_deltaxtol = p->deltaxtol;
  tp.dc_rhstol = p->rhstol; tp.dc_maxstep = p->maxstep;
  tp.max_order = 1;
  tp.newton_only = 1;
  CK(cudaMemcpyAsync(ctx->d.tp, &tp, sizeof tp, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<CircState> cs(ncirc);
  for (auto &s : cs) {
    memset(&s, 0, sizeof s);
    s.phase = dcop ? PH_DC : PH_TRAN;
    s.t = s.tn = time;
    s.qscale = qscale; s.fscale = fscale; s.hscale = hscale;
    s.init_jct = (flags & XG_FLAG_INITJCT) ? 1 : 0;
    s.order = 1;
    s.refactor = 1;
    s.f_gen = -1;
    s.errwt = 1.0;
    s.stop_at = 0x7fffffffffffffffLL;
  }
  CK(cudaMemcpyAsync(ctx->d.cs, cs.data(), sizeof(CircState) * ncirc, cudaMemcpyHostToDevice, ctx->stream));
  // the caller's vectors stand in for the context's; absent histories are zeros
  DevArrays d = ctx->d;
  d.x = x;
  if (x_curr) d.xcurr = const_cast<double *>(x_curr);
  else CK(cudaMemsetAsync(d.xcurr, 0, sizeof(double) * n, ctx->stream));
  if (qhist0) d.qh0 = const_cast<double *>(qhist0);
  else CK(cudaMemsetAsync(d.qh0, 0, sizeof(double) * n, ctx->stream));
  if (qhist2) d.qh2 = const_cast<double *>(qhist2);
  else CK(cudaMemsetAsync(d.qh2, 0, sizeof(double) * n, ctx->stream));
  if (ctx->nsta > 0) { d.sta_curr = const_cast<double *>(curr_sta); d.sta_next = next_sta; }
  if (ctx->nsto > 0) { d.sto_curr = const_cast<double *>(curr_sto); d.sto_next = next_sto; }
  launch_newton_weights_k(ctx->stream, d, n);
  CK(cudaMemsetAsync(ctx->breakdown_dev, 0, sizeof(int), ctx->stream));
  ctx->status_host[0] = ctx->status_host[1] = 0;
  double pivot_tol = ctx->pivot_tol;
  int rc = 0;
  // one Newton iteration of every unfinished circuit per pass; DampedNewton
  // stops each circuit within maxstep iterations
  for (int pass = 0; pass <= p->maxstep + 1; ++pass) {
    front_kernels(ctx, d);
    CK(cudaGetLastError());
    if (!ctx->lu_ready && (rc = lu_analyze_from_device(ctx, d.J))) return rc;
    back_kernels(ctx, d, pivot_tol, nullptr, nullptr, 0);
    launch_count_done_k(ctx->stream, d, ncirc, ctx->breakdown_dev, ctx->status_dev);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    for (int consecutive = 1; ctx->status_host[1]; ++consecutive) {
      // a frozen pivot failed: re-pivot from the parked Jacobian and resume
      if (consecutive > 4) return fail(ctx, XG_ERR_SINGULAR, "LU keeps breaking down after re-pivoting");
      std::vector<char> refresh;
      if ((rc = stalled_circuits(ctx, refresh))) return rc;
      if ((rc = lu_analyze_from_device(ctx, d.J, refresh.empty() ? nullptr : &refresh))) return rc;
      pivot_tol = (consecutive >= 2) ? 0.0 : ctx->pivot_tol;
      launch_unstall_k(ctx->stream, d, ncirc);
      back_kernels(ctx, d, pivot_tol, nullptr, nullptr, 0);
      launch_count_done_k(ctx->stream, d, ncirc, ctx->breakdown_dev, ctx->status_dev);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(ctx->stream));
    }
    pivot_tol = ctx->pivot_tol;
    if (ctx->status_host[0] >= ncirc) break;
  }
  std::vector<CircState> out(ncirc);
  CK(cudaMemcpyAsync(out.data(), ctx->d.cs, sizeof(CircState) * ncirc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int c = 0; c < ncirc; ++c) {
    if (out[c].phase != PH_DONE && out[c].phase != PH_FAILED)
      return fail(ctx, XG_ERR_TIMEOUT, "a Newton solve did not stop within maxstep iterations");
    status[c] = out[c].newton_status;
    if (iters) iters[c] = out[c].iter;
  }
  return XG_OK;
}

// ---------------------------------------------------------------------------
// Learned predictor (xg_mlp.cu).
extern "C" int xg_set_predictor(xg_ctx *ctx, int mode) {
  if (!ctx) return XG_ERR_ARG;
  if (mode != XG_PRED_POLY && mode != XG_PRED_LEARNED) return fail(ctx, XG_ERR_ARG, "unknown predictor mode");
  if (ctx->run) return fail(ctx, XG_ERR_STATE, "predictor cannot change during a transient");
  ctx->predictor = mode;
  return XG_OK;
}

extern "C" int xg_mlp_set(xg_ctx *ctx, const float *theta, const float *norm) {
  if (!ctx || !theta || !norm) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  CK(cudaMemcpyAsync(ctx->d.mlp.theta, theta, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d.mlp.norm, norm, sizeof(float) * kMlpNorm, cudaMemcpyHostToDevice, ctx->stream));
  launch_mlp_refresh_k(ctx->stream, ctx->d.mlp);
  CK(cudaGetLastError());
  CK(cudaMemsetAsync(ctx->mlp_m1, 0, sizeof(float) * kMlpParams, ctx->stream));
  CK(cudaMemsetAsync(ctx->mlp_m2, 0, sizeof(float) * kMlpParams, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->mlp_adam_t = 0;
  ctx->mlp_ready = true;
  return XG_OK;
}

extern "C" int xg_mlp_get(xg_ctx *ctx, float *theta, float *norm) {
  if (!ctx) return XG_ERR_ARG;
  if (!ctx->finalized) return fail(ctx, XG_ERR_STATE, "not finalized");
  CK(cudaStreamSynchronize(ctx->stream));
  if (theta) CK(cudaMemcpy(theta, ctx->d.mlp.theta, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  if (norm) CK(cudaMemcpy(norm, ctx->d.mlp.norm, sizeof(float) * kMlpNorm, cudaMemcpyDeviceToHost));
  return XG_OK;
}

static int sm_count(xg_ctx *ctx) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || v <= 0) v = 132;
  return v;
}

extern "C" int xg_mlp_grad(xg_ctx *ctx, const float *X, const float *Y, int n, float *grad_host, float *loss_host) {
  if (!ctx || !X || !Y || n <= 0) return XG_ERR_ARG;
  if (!ctx->mlp_ready) return fail(ctx, XG_ERR_STATE, "call xg_mlp_set first");
  CK(cudaMemsetAsync(ctx->mlp_grad, 0, sizeof(float) * kMlpParams, ctx->stream));
  CK(cudaMemsetAsync(ctx->mlp_loss, 0, sizeof(float), ctx->stream));
  int rc = launch_mlp_grad_k(ctx->stream, ctx->d.mlp, X, Y, n, ctx->mlp_grad, ctx->mlp_loss, sm_count(ctx));
  if (rc) return fail(ctx, rc, "MLP gradient kernel launch");
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  if (grad_host) CK(cudaMemcpy(grad_host, ctx->mlp_grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  if (loss_host) CK(cudaMemcpy(loss_host, ctx->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost));
  return XG_OK;
}

extern "C" int xg_mlp_train(xg_ctx *ctx, const float *X, const float *Y, int n, int iters, float lr,
                            float *loss_hist) {
  if (!ctx || !X || !Y || n <= 0 || iters < 0) return XG_ERR_ARG;
  if (!ctx->mlp_ready) return fail(ctx, XG_ERR_STATE, "call xg_mlp_set first (initial weights)");
  const int sms = sm_count(ctx);
  std::vector<float> hist(iters > 0 ? iters : 1);
  for (int it = 0; it < iters; ++it) {
    CK(cudaMemsetAsync(ctx->mlp_grad, 0, sizeof(float) * kMlpParams, ctx->stream));
    CK(cudaMemsetAsync(ctx->mlp_loss, 0, sizeof(float), ctx->stream));
    int rc = launch_mlp_grad_k(ctx->stream, ctx->d.mlp, X, Y, n, ctx->mlp_grad, ctx->mlp_loss, sms);
    if (rc) return fail(ctx, rc, "MLP gradient kernel launch");
    ctx->mlp_adam_t++;
    const float b1c = 1.0f - std::pow(0.9f, (float)ctx->mlp_adam_t);
    const float b2c = 1.0f - std::pow(0.999f, (float)ctx->mlp_adam_t);
    launch_mlp_adam_k(ctx->stream, ctx->d.mlp, ctx->mlp_grad, ctx->mlp_m1, ctx->mlp_m2, lr, b1c, b2c);
    launch_mlp_refresh_k(ctx->stream, ctx->d.mlp);
    CK(cudaMemcpyAsync(&hist[it], ctx->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  if (loss_hist) std::copy(hist.begin(), hist.begin() + iters, loss_hist);
  return XG_OK;
}

extern "C" int xg_mlp_forward(xg_ctx *ctx, const float *X, int n, float *out) {
  if (!ctx || !X || !out || n <= 0) return XG_ERR_ARG;
  if (!ctx->mlp_ready) return fail(ctx, XG_ERR_STATE, "call xg_mlp_set first");
  launch_mlp_forward_k(ctx->stream, ctx->d.mlp, X, n, out);
  CK(cudaGetLastError());
  return XG_OK;
}
