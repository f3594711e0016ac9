// xg_kernels.cu — sm_103a kernels of the transient Newton hot path.
//
// Data flow of one Newton iteration ("tick"), every circuit of a batch at once:
//   k_sources        source values at each circuit's attempt time      (SourceData::updateSource)
//   k_mos1, k_diode  device evaluation, one thread per instance, SoA;   (Master::updateState +
//                    writes store/state and per-instance stamp slots     loadDAEVectors/Matrices)
//   k_assemble_rows  gather-sum of the vector slots per row (atomic-free), linear part as a
//                    CSR SpMV, residual of the integration method, per-circuit partial norms
//                                                                       (OneStep::obtainResidual)
//   k_assemble_J     gather-sum of the matrix slots per CSR entry       (OneStep::obtainJacobian)
//   k_newton_ctl     per-circuit DampedNewton::converged_ decision
//   LU factor/solve  level-scheduled, frozen pivots (xg_lu.cu)
//   k_update         x += dx, weighted update norm, LTE sums
//   k_step_ctl       per-circuit accept/reject and next step (StepErrorControl, OneStep)
//   k_history        OneStep::updateHistory, initialize, obtainPredictor
//   k_state_commit   accepted store/state become current
#include <cuda_runtime.h>

#include "xg_internal.h"
#include "xg_lu_dev.cuh"
#include "xg_models.cuh"

namespace xg {

__device__ __forceinline__ bool circ_active(const CircState &s) {
  return s.phase == PH_DC || s.phase == PH_TRAN;
}

// ---------------------------------------------------------------------------
// Sources: SinData/PulseData/PWLinData::updateSource (N_DEV_SourceData.C:475,1168,1770)
__device__ double wave_value_d(int kind, const double *d, int nd, double t) {
  switch (kind) {
    case XG_WAVE_DC: return d[0];
    case XG_WAVE_SIN: {
      double time = t - d[3];
      if (time <= 0) return d[0] + d[1] * sin(2.0 * M_PI * (d[5] / 360));
      return d[0] + d[1] * sin(2.0 * M_PI * (d[2] * time + d[5] / 360)) * exp(-(time * d[4]));
    }
    case XG_WAVE_PULSE: {
      double V1 = d[0], V2 = d[1], TR = d[3], TF = d[4], PW = d[5], PER = d[6];
      double time = t - d[2];
      if (time > PER && PER != 0.0) time -= PER * floor(time / PER);
      if (time <= 0 || time > TR + PW + TF) return V1;
      if (time > TR && time < TR + PW) return V2;
      if (time > 0 && time <= TR) return (TR != 0.0) ? V1 + (V2 - V1) * time / TR : V1;
      if (time >= TR + PW && time <= TR + PW + TF)
        return (TF != 0.0) ? V2 + (V1 - V2) * (time - (TR + PW)) / TF : V2;
      return V2;
    }
    case XG_WAVE_PWL: {
      int npts = nd / 2;
      if (t < 0) return 0.0;
      double t1, t2, v1, v2;
      if (t <= d[2 * (npts - 1)]) {
        int loc = npts - 1;
        for (int i = 0; i < npts && i < kMaxPwlScan; ++i)
          if (t < d[2 * i]) { loc = i; break; }
        if (loc == 0) { t1 = 0.0; v1 = 0.0; }
        else { t1 = d[2 * (loc - 1)]; v1 = d[2 * (loc - 1) + 1]; }
        t2 = d[2 * loc]; v2 = d[2 * loc + 1];
      } else {
        t1 = 0.0; t2 = 1.0; v1 = v2 = d[2 * (npts - 1) + 1];
      }
      if (t1 == t2) return v2;
      double length = t2 - t1;
      return (t2 - t) * v1 / length + (-t1 + t) * v2 / length;
    }
  }
  return 0.0;
}

// Source k's value into its B slots; V sources own one B slot, I sources
// two (pos, neg).
__device__ __forceinline__ void source_value(const DevArrays &d, int k, int n_v, int use_explicit,
                                             double t_explicit) {
  double t;
  if (use_explicit) {
    t = t_explicit;
  } else {
    const CircState &s = d.cs[d.src_circ[k]];
    if (!circ_active(s)) return;
    t = s.tn;
  }
  int o0 = d.src_off[k], o1 = d.src_off[k + 1];
  double v = wave_value_d(d.src_kind[k], d.src_data + o0, o1 - o0, t);
  if (k < n_v) {
    d.sB[k] = v;
  } else {
    int j = n_v + 2 * (k - n_v);
    d.sB[j] = -v;
    d.sB[j + 1] = v;
  }
}

// One thread per source.
__global__ void k_sources(DevArrays d, int n_v, int n_src, int use_explicit, double t_explicit) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_src) source_value(d, k, n_v, use_explicit, t_explicit);
}

// ---------------------------------------------------------------------------
// MOSFET level 1, drain/source primes merged (RD = RS = 0).
// Store planes (x nm): vbd vbs vgs vds von gm; state planes: capgs capgd capgb qgs qgd qgb qbd qbs.
// Slots: F[D,S,B]  Q[G,B,D,S]  L[G,B,D,S]  M[4x4 over D,G,S,B].
__device__ __forceinline__ void mos1_eval(const DevArrays &d, int i, int nm, int sto_base, int combined,
                                          int masked, int it_arg, int flags_arg, int slotF, int slotQ, int slotL,
                                          int slotM) {
  int c = __ldg(d.m1_circ + i);
  int iter = it_arg;
  bool dcop = flags_arg & XG_FLAG_DCOP, initJct = flags_arg & XG_FLAG_INITJCT;
  double qs = 1.0, fs = 1.0;
  if (masked) {
    const CircState &s = d.cs[c];
    if (!circ_active(s)) return;
    iter = s.iter;
    dcop = s.phase == PH_DC;
    initJct = dcop && s.init_jct && iter == 0;
    qs = s.qscale; fs = s.fscale;
  }
  const Mos1Model m = d.m1_models[__ldg(d.m1_model + i)];
  const int nD = __ldg(d.m1_node + i), nG = __ldg(d.m1_node + nm + i);
  const int nS = __ldg(d.m1_node + 2 * nm + i), nB = __ldg(d.m1_node + 3 * nm + i);
  const double *x = d.x;
  double Vd = nD >= 0 ? x[nD] : 0.0, Vg = nG >= 0 ? x[nG] : 0.0;
  double Vs = nS >= 0 ? x[nS] : 0.0, Vb = nB >= 0 ? x[nB] : 0.0;
  const double dt = m.dtype;
  // dt is +1 or -1: products with it are sign flips, done on the integer pipe
  // (exactly the IEEE product) — the FP64 pipe bounds this kernel on GB300
  const long long tsgn = f_lt0(dt) ? (long long)0x8000000000000000ULL : 0LL;
  auto T = [tsgn](double v) { return __longlong_as_double(__double_as_longlong(v) ^ tsgn); };
  const double Beta = __ldg(d.m1_beta + i), tVbi = __ldg(d.m1_vbi + i);
  const double tVto = tVbi + T(m.gammaSqrtPhi);
  double *sto_n = d.sto_next + sto_base;
  const double *sto_c = d.sto_curr + sto_base;

  double vbs = T(Vb - Vs), vgs = T(Vg - Vs), vds = T(Vd - Vs);
  double vbd = vbs - vds, vgd = vgs - vds;
  const double vgs_o = vgs, vds_o = vds, vbs_o = vbs, vbd_o = vbd, vgd_o = vgd;
  if (initJct) {
    vbs = -1; vgs = T(tVto); vds = 0; vbd = vbs - vds; vgd = vgs - vds;
  }
  double vbs_old, vbd_old, vgs_old, vds_old, Von;
  if (iter == 0 && dcop) {
    vbs_old = vbs; vbd_old = vbd; vgs_old = vgs; vds_old = vds; Von = 0.0;
  } else {
    const double *h = (iter == 0) ? sto_c : sto_n;
    vbd_old = h[i]; vbs_old = h[nm + i]; vgs_old = h[2 * nm + i]; vds_old = h[3 * nm + i];
    Von = T(h[4 * nm + i]);
  }
  double vgd_old = vgs_old - vds_old;
  int Check = 1;
  if (f_ge0(vds_old)) {
    vgs = fetlim_d(vgs, vgs_old, Von);
    vds = vgs - vgd;
    vds = limvds_d(vds, vds_old);
    vgd = vgs - vds;
  } else {
    vgd = fetlim_d(vgd, vgd_old, Von);
    vds = vgs - vgd;
    vds = -limvds_d(-vds, -vds_old);
    vgs = vgd + vds;
  }
  if (f_ge0(vds)) {
    vbs = pnjlim_d(vbs, vbs_old, m.vt, m.sourceVcrit, Check);
    vbd = vbs - vds;
  } else {
    vbd = pnjlim_d(vbd, vbd_old, m.vt, m.drainVcrit, Check);
    vbs = vbd + vds;
  }
  vbd = vbs - vds;
  vgd = vgs - vds;
  const double Vgb = vgs - vbs;
  // "no voltage was limited", compared on the bit patterns (integer pipe;
  // +0 and -0 compare equal as in FP64)
  auto same = [](double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return x == y || ((x | y) << 1) == 0;
  };
  const bool origFlag = same(vgs_o, vgs) && same(vds_o, vds) && same(vbs_o, vbs) && same(vbd_o, vbd) &&
                        same(vgd_o, vgd);
  double gbs, cbs, gbd, cbd;
  if (f_le0(vbs)) {
    gbs = m.gbsR;
    cbs = gbs * vbs;
  } else {
    double e = exp(f_min(kMaxExpArg, vbs / m.vt));
    gbs = m.SourceSatCur * e / m.vt + kGmin;
    cbs = m.SourceSatCur * (e - 1) + kGmin * vbs;
  }
  if (f_le0(vbd)) {
    gbd = m.gbdR;
    cbd = gbd * vbd;
  } else {
    double e = exp(f_min(kMaxExpArg, vbd / m.vt));
    gbd = m.DrainSatCur * e / m.vt + kGmin;
    cbd = m.DrainSatCur * (e - 1) + kGmin * vbd;
  }
  const int mode = f_ge0(vds) ? 1 : -1;
  double cdrain, gm, gds, gmbs, Vdsat;
  {
    double vbx = (mode == 1) ? vbs : vbd;
    // vbx = 0 (bulk tied to the source, the usual case) takes sqrt(phi) and
    // gamma / (2 sqrt(phi)) from the model: the same correctly rounded values
    const bool vbx0 = f_is0(vbx);
    double sarg;
    if (vbx0) {
      sarg = m.sqrtPhi;
    } else if (f_le0(vbx)) {
      sarg = sqrt(m.tPhi - vbx);
    } else {
      sarg = m.sqrtPhi;
      sarg = sarg - vbx / (sarg + sarg);
      sarg = f_max(0.0, sarg);
    }
    Von = T(tVbi) + m.gamma * sarg;
    double vgst = ((mode == 1) ? vgs : vgd) - Von;
    Vdsat = f_gt0(vgst) ? vgst : 0.0;
    if (f_le0(vgst)) {
      cdrain = 0; gm = 0; gds = 0; gmbs = 0;
    } else {
      const double arg = vbx0 ? m.argPhi : (f_le0(sarg) ? 0.0 : m.gamma / (sarg + sarg));
      double vdsm = (mode == 1) ? vds : -vds;
      double betap = Beta * (1 + m.lambda * vdsm);
      if (f_le(vgst, vdsm)) {
        cdrain = betap * vgst * vgst * .5;
        gm = betap * vgst;
        gds = m.lambda * Beta * vgst * vgst * .5;
      } else {
        cdrain = betap * vdsm * (vgst - .5 * vdsm);
        gm = betap * vdsm;
        gds = betap * (vgst - vdsm) + m.lambda * Beta * vdsm * (vgst - .5 * vdsm);
      }
      gmbs = gm * arg;
    }
  }
  double qbs = 0, capbs = 0, qbd = 0, capbd = 0;
  if (m.has_junc_caps) {
    mos1_junction(m, vbs, m.Cbs, m.Cbssw, m.f2s, m.f3s, m.f4s, qbs, capbs);
    mos1_junction(m, vbd, m.Cbd, m.Cbdsw, m.f2d, m.f3d, m.f4d, qbd, capbd);
  }
  double capgs = 0, capgd = 0, capgb = 0, Capgs = 0, Capgd = 0, Capgb = 0, qgs = 0, qgd = 0, qgb = 0;
  double *sta_n = d.sta_next;
  const double *sta_c = d.sta_curr;
  if (m.has_gate_caps) {
    if (mode > 0) qmeyer_d(vgs, vgd, Von, Vdsat, capgs, capgd, capgb, m.tPhi, m.OxideCap);
    else qmeyer_d(vgd, vgs, Von, Vdsat, capgd, capgs, capgb, m.tPhi, m.OxideCap);
    if (dcop) {
      Capgs = 2.0 * capgs + m.Cgso; Capgd = 2.0 * capgd + m.Cgdo; Capgb = 2.0 * capgb + m.Cgbo;
    } else {
      Capgs = capgs + sta_c[i] + m.Cgso;
      Capgd = capgd + sta_c[nm + i] + m.Cgdo;
      Capgb = capgb + sta_c[2 * nm + i] + m.Cgbo;
    }
    Capgs = fabs(Capgs); Capgd = fabs(Capgd); Capgb = fabs(Capgb);
    if (dcop) {
      qgs = Capgs * vgs; qgd = Capgd * vgd; qgb = Capgb * Vgb;
    } else {
      double vgs1 = sto_c[2 * nm + i], vbs1 = sto_c[nm + i], vds1 = sto_c[3 * nm + i];
      qgs = sta_c[3 * nm + i] + Capgs * (vgs - vgs1);
      qgd = sta_c[4 * nm + i] + Capgd * (vgd - (vgs1 - vds1));
      qgb = sta_c[5 * nm + i] + Capgb * ((vgs - vbs) - (vgs1 - vbs1));
    }
  }
  double Gm, Gmbs, nrmsum, revsum, cdreq;
  if (mode >= 0) {
    Gm = gm; Gmbs = gmbs; nrmsum = Gm + Gmbs; revsum = 0; cdreq = T(cdrain);
  } else {
    Gm = -gm; Gmbs = -gmbs; nrmsum = 0; revsum = -(Gm + Gmbs); cdreq = -T(cdrain);
  }
  // store / state (Master::updateState, N_DEV_MOSFET1.C:4241-4333)
  sto_n[i] = vbd; sto_n[nm + i] = vbs; sto_n[2 * nm + i] = vgs; sto_n[3 * nm + i] = vds;
  sto_n[4 * nm + i] = T(Von); sto_n[5 * nm + i] = Gm;
  sta_n[i] = capgs; sta_n[nm + i] = capgd; sta_n[2 * nm + i] = capgb;
  sta_n[3 * nm + i] = qgs; sta_n[4 * nm + i] = qgd; sta_n[5 * nm + i] = qgb;
  sta_n[6 * nm + i] = qbd; sta_n[7 * nm + i] = qbs;
  if (!origFlag && masked && dcop) {
    // "some device limited" flag for the operating-point device-convergence test
    atomicOr(&d.cs[c].limited, 1);
  }
  const double M = m.M;
  const bool unitM = f_is1(M);
  // A model without gate or junction capacitance has no charge: its Q
  // vector, charge limiter terms and dQdx stamps are zero and are stored
  // without FP64 arithmetic (as are products with a unit F scale)
  const bool noq = !m.has_gate_caps && !m.has_junc_caps;
  const bool fs1 = f_is1(fs);
  // loadDAEVectors (N_DEV_MOSFET1.C:4343-4576), old Meyer
  const double ceqbs = T(cbs), ceqbd = T(cbd);
  double fv[3] = {-(ceqbd - cdreq), -(ceqbs + cdreq), ceqbs + ceqbd};  // D S B
  double qv[4] = {0, 0, 0, 0};                                         // G B D S
  if (!noq) {
    const double Qbs = T(qbs), Qbd = T(qbd), Qgb = T(qgb), Qgs = T(qgs), Qgd = T(qgd);
    qv[0] = Qgs + Qgd + Qgb; qv[1] = Qbs + Qbd - Qgb; qv[2] = -(Qbd + Qgd); qv[3] = -(Qbs + Qgs);
  }
  double lf[4] = {0, 0, 0, 0}, lq[4] = {0, 0, 0, 0};
  if (!origFlag) {
    double dvbd = vbd - vbd_o, dvbs = vbs - vbs_o, dvds = vds - vds_o, dvgs = vgs - vgs_o,
           dvgd = vgd - vgd_o;
    double sw = Gm * ((mode > 0) ? dvgs : dvgd) + Gmbs * ((mode > 0) ? dvbs : dvbd);
    lf[1] = T((gbd - kGmin) * dvbd + (gbs - kGmin) * dvbs);
    lf[2] = T(-(gbd - kGmin) * dvbd + gds * dvds + sw);
    lf[3] = T(-(gbs - kGmin) * dvbs - gds * dvds - sw);
    if (!noq) {
      lq[0] = T(Capgd * dvgd + Capgs * dvgs + Capgb * (dvgs - dvbs));
      lq[1] = T(-Capgb * (dvgs - dvbs) + Capgb * dvbd + capbs * dvbs);
      lq[2] = T(-Capgd * dvgd - capbd * dvbd);
      lq[3] = T(-Capgs * dvgs - capbs * dvbs);
    }
  }
  // the multiplier is applied only when it is not 1 (a branch, not a select,
  // so that the FP64 products are skipped)
  if (!unitM) {
#pragma unroll
    for (int k = 0; k < 3; ++k) fv[k] *= M;
#pragma unroll
    for (int k = 0; k < 4; ++k) lf[k] *= M;
    if (!noq) {
#pragma unroll
      for (int k = 0; k < 4; ++k) { qv[k] *= M; lq[k] *= M; }
    }
  }
  double *sF = d.sF + slotF, *sQ = d.sQ + slotQ;
#pragma unroll
  for (int k = 0; k < 3; ++k) sF[k * nm + i] = fv[k];
#pragma unroll
  for (int k = 0; k < 4; ++k) sQ[k * nm + i] = qv[k];
  double *sL = d.sL + slotL;
  if (combined) {
    if (noq) {
#pragma unroll
      for (int k = 0; k < 4; ++k) sL[k * nm + i] = fs1 ? lf[k] : fs * lf[k];
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) sL[k * nm + i] = fs * lf[k] + qs * lq[k];
    }
  } else {
    double *sL2 = d.sL2 + slotL;
#pragma unroll
    for (int k = 0; k < 4; ++k) { sL[k * nm + i] = lf[k]; sL2[k * nm + i] = lq[k]; }
  }
  // loadDAEMatrices (N_DEV_MOSFET1.C:4587-4876), nodes (0=D,1=G,2=S,3=B)
  double f[16], q[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) { f[k] = 0.0; q[k] = 0.0; }
  f[15] = gbs + gbd; f[12] = -gbd; f[14] = -gbs;
  f[1] = Gm; f[3] = -gbd + Gmbs; f[9] = -Gm; f[11] = -(gbs + Gmbs);
  // one of revsum / nrmsum is zero (by the mode): its additions are skipped
  if (mode >= 0) {
    f[0] = gds + gbd; f[2] = -gds - nrmsum; f[8] = -gds; f[10] = gds + gbs + nrmsum;
  } else {
    f[0] = gds + gbd + revsum; f[2] = -gds; f[8] = -(gds + revsum); f[10] = gds + gbs;
  }
  if (!noq) {
    q[5] = Capgd + Capgs + Capgb; q[7] = -Capgb; q[4] = -Capgd; q[6] = -Capgs;
    q[13] = -Capgb; q[15] = capbs + capbd + Capgb; q[12] = -capbd; q[14] = -capbs;
    q[1] = -Capgd; q[3] = -capbd; q[0] = capbd + Capgd;
    q[9] = -Capgs; q[11] = -capbs; q[10] = capbs + Capgs;
  }
  // structural zeros of the two 4x4 blocks (the gate conducts no current;
  // no capacitance couples D-S) are stored without FP64 arithmetic
  constexpr bool kFnz[16] = {1, 1, 1, 1, 0, 0, 0, 0, 1, 1, 1, 1, 1, 0, 1, 1};
  constexpr bool kQnz[16] = {1, 1, 0, 1, 1, 1, 1, 1, 0, 1, 1, 1, 1, 1, 1, 1};
  if (!unitM) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (kFnz[k]) f[k] *= M;
      if (kQnz[k] && !noq) q[k] *= M;
    }
  }
  double *sM = d.sM + slotM;
  if (combined) {
    if (noq) {
#pragma unroll
      for (int k = 0; k < 16; ++k) sM[k * nm + i] = kFnz[k] ? (fs1 ? f[k] : fs * f[k]) : 0.0;
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        double v;
        if (kFnz[k] && kQnz[k]) v = fs * f[k] + qs * q[k];
        else if (kFnz[k]) v = fs * f[k];
        else if (kQnz[k]) v = qs * q[k];
        else v = 0.0;
        sM[k * nm + i] = v;
      }
    }
  } else {
    double *sM2 = d.sM2 + slotM;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      sM[k * nm + i] = kFnz[k] ? f[k] : 0.0;
      sM2[k * nm + i] = kQnz[k] ? q[k] : 0.0;
    }
  }
}

__global__ void __launch_bounds__(128) k_mos1(DevArrays d, int nm, int sto_base, int combined,
                                              int masked, int it_arg, int flags_arg,
                                              int slotF, int slotQ, int slotL, int slotM) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nm) mos1_eval(d, i, nm, sto_base, combined, masked, it_arg, flags_arg, slotF, slotQ, slotL, slotM);
}

// ---------------------------------------------------------------------------
// Diode level 1 (no sidewall).  Store planes: vd qd cd.
// Slots: F[P,N,R]  Q[N,R]  L[N,R]  M[(P,P)(P,R)(N,N)(N,R)(R,P)(R,N)(R,R)].
__device__ __forceinline__ void diode_eval(const DevArrays &d, int i, int nd, int combined, int masked,
                                           int it_arg, int flags_arg, int slotF, int slotQ, int slotL,
                                           int slotM) {
  int c = __ldg(d.d_circ + i);
  int iter = it_arg;
  bool dcop = flags_arg & XG_FLAG_DCOP, initJct = flags_arg & XG_FLAG_INITJCT;
  double qs = 1.0, fs = 1.0;
  if (masked) {
    const CircState &s = d.cs[c];
    if (!circ_active(s)) return;
    iter = s.iter;
    dcop = s.phase == PH_DC;
    initJct = dcop && s.init_jct && iter == 0;
    qs = s.qscale; fs = s.fscale;
  }
  const DiodeModel t = d.d_models[__ldg(d.d_model + i)];
  const int nP = __ldg(d.d_node + i), nN = __ldg(d.d_node + nd + i), nR = __ldg(d.d_node + 2 * nd + i);
  const double *x = d.x;
  const double VP = nP >= 0 ? x[nP] : 0.0, VN = nN >= 0 ? x[nN] : 0.0, VR = nR >= 0 ? x[nR] : 0.0;
  double Vd = VR - VN;
  const double Vd_orig = Vd;
  double Vd_old;
  if (iter == 0) {
    if (initJct) Vd = t.tVcrit;
    Vd_old = dcop ? Vd : d.sto_curr[i];
  } else {
    Vd_old = d.sto_next[i];
  }
  int ichk = 0;
  if (t.bvGiven && Vd < fmin(0.0, -t.tBrkdwnV + 10.0 * t.VteBRK)) {
    double Vdtmp = -(t.tBrkdwnV + Vd);
    Vdtmp = pnjlim_d(Vdtmp, -(Vd_old + t.tBrkdwnV), t.VteBRK, t.tVcrit, ichk);
    Vd = -(Vdtmp + t.tBrkdwnV);
  } else {
    Vd = pnjlim_d(Vd, Vd_old, t.Vte, t.tVcrit, ichk);
  }
  // sidewall current with its own characteristic (N_DEV_Diode.C:1226-1256)
  double IdSW = 0.0, GdSW = 0.0;
  if (t.sw == 1) {
    if (Vd >= -3.0 * t.VteSW) {
      const double evd = exp(fmin(kMaxExpArg, Vd / t.VteSW));
      IdSW = t.IsatSW * (evd - 1.0);
      GdSW = t.IsatSW * evd / t.VteSW;
    } else if (!t.tBrkdwnV || Vd >= -t.tBrkdwnV) {
      double argsw = 3.0 * t.VteSW / (Vd * kE);
      argsw = argsw * argsw * argsw;
      IdSW = -t.IsatSW * (1.0 + argsw);
      GdSW = t.IsatSW * 3.0 * argsw / Vd;
    } else {
      const double evrev = exp(fmin(kMaxExpArg, -(t.tBrkdwnV + Vd) / t.VteBRK));
      IdSW = -t.IsatSW * evrev;
      GdSW = t.IsatSW * evrev / t.VteBRK;
    }
  }
  double Id, Gd;
  if (Vd >= -3.0 * t.Vte) {
    double evd = exp(fmin(kMaxExpArg, Vd / t.Vte));
    double Inorm = t.Isat * (evd - 1.0) + kGmin * Vd;
    double Gd1 = t.Isat * evd / t.Vte + kGmin;
    evd = exp(fmin(kMaxExpArg, Vd / t.VteR));
    double Irec = t.IsatR * (evd - 1.0);
    double Gd2 = t.IsatR * evd / t.VteR;
    double Khi = 1, DKhi = 0;
    if (t.tIKF > 0) {
      Khi = sqrt(t.tIKF / (t.tIKF + Inorm));
      DKhi = -0.5 * Khi * Gd1 / (t.tIKF + Inorm);
    }
    double Kgen = 0, DKgen = 0;
    if (Irec != 0) {
      double a = 1 - Vd / t.tJctPot;
      Kgen = sqrt(pow(a * a + 0.005, t.M));
      DKgen = -t.M * a * Kgen / (t.tJctPot * (a * a + 0.005));
    }
    Id = Inorm * Khi + Irec * Kgen + IdSW;
    Gd = Gd1 * Khi + Inorm * DKhi + Gd2 * Kgen + Irec * DKgen + GdSW;
  } else if (!t.tBrkdwnV || Vd >= -t.tBrkdwnV) {
    double arg = 3.0 * t.Vte / (Vd * kE);
    arg = arg * arg * arg;
    Id = -t.Isat * (1.0 + arg) + IdSW + kGmin * Vd;
    Gd = t.Isat * 3.0 * arg / Vd + GdSW + kGmin;
  } else {
    double evrev = exp(fmin(kMaxExpArg, -(t.tBrkdwnV + Vd) / t.VteBRK));
    Id = -t.Isat * evrev + IdSW + kGmin * Vd;
    Gd = t.Isat * evrev / t.VteBRK + GdSW + kGmin;
  }
  double Qd = 0, Cd = 0;
  if (t.tJctCap != 0.0) {
    double Czero = t.tJctCap;
    if (Vd < t.tDepCap) {
      double arg = 1.0 - Vd / t.tJctPot;
      double sarg = exp(fmin(kMaxExpArg, -t.M * log(arg)));
      Qd = t.TT * Id + t.tJctPot * Czero * (1.0 - arg * sarg) / (1.0 - t.M);
      Cd = t.TT * Gd + Czero * sarg;
    } else {
      double Czof2 = Czero / t.F2;
      double MotJctPot = t.M / t.tJctPot;
      Qd = t.TT * Id + Czero * t.tF1 +
           Czof2 * (t.F3 * (Vd - t.tDepCap) + 0.5 * MotJctPot * (Vd * Vd - t.tDepCap * t.tDepCap));
      Cd = t.TT * Gd + Czof2 * (t.F3 + MotJctPot * Vd);
    }
    // sidewall depletion charge (N_DEV_Diode.C:1380-1400); it adds zeros when
    // the perimeter capacitance is zero, so that case skips it
    const double CzeroSW = t.CzeroSW;
    if (CzeroSW != 0.0) {
      if (Vd < t.tDepSWCap) {
        const double argSW = 1.0 - Vd / t.tJctSWPot;
        const double sargSW = exp(fmin(kMaxExpArg, -t.MJSW * log(argSW)));
        Qd += t.tJctSWPot * CzeroSW * (1.0 - argSW * sargSW) / (1.0 - t.MJSW);
        Cd += CzeroSW * sargSW;
      } else {
        const double Czof2SW = CzeroSW / t.F2SW;
        const double MotJctSWPot = t.MJSW / t.tJctSWPot;
        Qd += CzeroSW * t.tF1 + Czof2SW * (t.F3SW * (Vd - t.tDepSWCap) +
                                           0.5 * MotJctSWPot * (Vd * Vd - t.tDepSWCap * t.tDepSWCap));
        Cd += Czof2SW * (t.F3SW + MotJctSWPot * Vd);
      }
    }
  }
  d.sto_next[i] = Vd; d.sto_next[nd + i] = Qd; d.sto_next[2 * nd + i] = Cd;
  if (Vd != Vd_orig && masked && dcop) atomicOr(&d.cs[c].limited, 1);
  const double Ir = t.Gspr * (VP - VR);
  double *sF = d.sF + slotF, *sQ = d.sQ + slotQ;
  sF[i] = Ir; sF[nd + i] = -Id; sF[2 * nd + i] = Id - Ir;
  sQ[i] = -Qd; sQ[nd + i] = Qd;
  const double dv = Vd - Vd_orig;
  const double Gj = -Gd * dv, Cj = -Cd * dv;
  double *sL = d.sL + slotL;
  if (combined) {
    sL[i] = fs * Gj + qs * Cj; sL[nd + i] = -(fs * Gj + qs * Cj);
  } else {
    double *sL2 = d.sL2 + slotL;
    sL[i] = Gj; sL[nd + i] = -Gj; sL2[i] = Cj; sL2[nd + i] = -Cj;
  }
  const double G = t.Gspr;
  double f[7] = {G, -G, Gd, -Gd, -G, -Gd, G + Gd};
  double q[7] = {0, 0, Cd, -Cd, 0, -Cd, Cd};
  double *sM = d.sM + slotM;
  if (combined) {
#pragma unroll
    for (int k = 0; k < 7; ++k) sM[k * nd + i] = fs * f[k] + qs * q[k];
  } else {
    double *sM2 = d.sM2 + slotM;
#pragma unroll
    for (int k = 0; k < 7; ++k) { sM[k * nd + i] = f[k]; sM2[k * nd + i] = q[k]; }
  }
}

__global__ void __launch_bounds__(128) k_diode(DevArrays d, int nd, int combined, int masked,
                                               int it_arg, int flags_arg, int slotF, int slotQ,
                                               int slotL, int slotM) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nd) diode_eval(d, i, nd, combined, masked, it_arg, flags_arg, slotF, slotQ, slotL, slotM);
}

// ---------------------------------------------------------------------------
// Deterministic per-(block, circuit) partial reductions.  A row block covers
// rows [b*kRowBlock, (b+1)*kRowBlock); pair_base[b] is the first partial slot
// of the block, blk_cfirst[b] its first circuit.
__device__ void block_partials(const DevArrays &d, int n, double vmax, double vsum, int r) {
  __shared__ double smax[kRowBlock], ssum[kRowBlock];
  smax[threadIdx.x] = vmax;
  ssum[threadIdx.x] = vsum;
  __syncthreads();
  const int b = blockIdx.x;
  const int r0 = b * kRowBlock, r1 = min(n, r0 + kRowBlock);
  const int cfirst = d.blk_cfirst[b];
  const int nseg = d.circ_of_row[r1 - 1] - cfirst + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int seg = warp; seg < nseg; seg += kRowBlock / 32) {
    const int cc = cfirst + seg;
    const int lo = max(d.offsets[cc], r0) - r0, hi = min(d.offsets[cc + 1], r1) - r0;
    double m = 0.0, s = 0.0;
    for (int k = lo + lane; k < hi; k += 32) {
      m = fmax(m, smax[k]);
      s += ssum[k];
    }
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) {
      d.pmax[d.pair_base[b] + seg] = m;
      d.psum[d.pair_base[b] + seg] = s;
    }
  }
  (void)r;
}

// Long gathers: part p of a gather in P parts is summed by one warp — lane
// l adds the items p*32 + l + m*32*P of each list in order (four loads in
// flight), then a butterfly over the 32 lanes.  Every lane ends with the
// same total (the butterfly's additions commute); the parts of a gather are
// added in order by the row / entry that owns it.
__device__ __forceinline__ double gather_seq(double acc, const int *idx, const double *sv, int k, int k1,
                                             int stride) {
  for (; k + 3 * stride < k1; k += 4 * stride) {
    const int i0 = idx[k], i1 = idx[k + stride], i2 = idx[k + 2 * stride], i3 = idx[k + 3 * stride];
    const double a0 = sv[i0], a1 = sv[i1], a2 = sv[i2], a3 = sv[i3];
    acc += a0; acc += a1; acc += a2; acc += a3;
  }
  for (; k < k1; k += stride) acc += sv[idx[k]];
  return acc;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Part `part` of long row lr (e.g. a supply node touching every PMOS): the
// F, Q, B, L partial sums of its share of the row's lists, into
// long_rsum[4 * (lrow_ptr[lr] + part) ..].  One warp.
__device__ __forceinline__ void long_row_part(const DevArrays &d, int lr, int part) {
  const int lane = threadIdx.x & 31;
  const int nparts = d.lrow_ptr[lr + 1] - d.lrow_ptr[lr];
  const int r = d.long_rows[lr];
  const int stride = 32 * nparts, start = 32 * part + lane;
  double F = 0.0, Q = 0.0;
  {
    int e = d.rp[r] + start;
    const int e1 = d.rp[r + 1];
    for (; e + stride < e1; e += 2 * stride) {
      const double x0 = d.x[d.ci[e]], x1 = d.x[d.ci[e + stride]];
      F += d.Glin[e] * x0; Q += d.Clin[e] * x0;
      F += d.Glin[e + stride] * x1; Q += d.Clin[e + stride] * x1;
    }
    if (e < e1) {
      const double x0 = d.x[d.ci[e]];
      F += d.Glin[e] * x0; Q += d.Clin[e] * x0;
    }
  }
  F = gather_seq(F, d.vF_idx, d.sF, d.vF_ptr[r] + start, d.vF_ptr[r + 1], stride);
  Q = gather_seq(Q, d.vQ_idx, d.sQ, d.vQ_ptr[r] + start, d.vQ_ptr[r + 1], stride);
  const double B = gather_seq(0.0, d.vB_idx, d.sB, d.vB_ptr[r] + start, d.vB_ptr[r + 1], stride);
  const double L = gather_seq(0.0, d.vL_idx, d.sL, d.vL_ptr[r] + start, d.vL_ptr[r + 1], stride);
  const double tF = warp_sum(F), tQ = warp_sum(Q), tB = warp_sum(B), tL = warp_sum(L);
  if (lane == 0) {
    double *o = d.long_rsum + 4 * (size_t)(d.lrow_ptr[lr] + part);
    o[0] = tF; o[1] = tQ; o[2] = tB; o[3] = tL;
  }
}

// Part `part` of long Jacobian entry le (e.g. a supply node's diagonal).  One warp.
__device__ __forceinline__ void long_entry_part(const DevArrays &d, int le, int part) {
  const int lane = threadIdx.x & 31;
  const int nparts = d.lent_ptr[le + 1] - d.lent_ptr[le];
  const int e = d.long_ents[le];
  const double s = gather_seq(0.0, d.m_idx, d.sM, d.m_ptr[e] + 32 * part + lane, d.m_ptr[e + 1], 32 * nparts);
  const double t = warp_sum(s);
  if (lane == 0) d.long_esum[d.lent_ptr[le] + part] = t;
}

// Long rows: a warp per part (ceil(items / 256) parts per row).
__global__ void __launch_bounds__(256) k_long_rows(DevArrays d, int n_parts) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= n_parts) return;
  const int lr = d.lrow_blk[i];
  if (!circ_active(d.cs[d.circ_of_row[d.long_rows[lr]]])) return;
  long_row_part(d, lr, i - d.lrow_ptr[lr]);
}

// Long Jacobian entries: a warp per part.
__global__ void __launch_bounds__(256) k_long_entries(DevArrays d, int n_parts) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= n_parts) return;
  const int le = d.lent_blk[i];
  if (!circ_active(d.cs[d.circ_of_row[d.erow[d.long_ents[le]]]])) return;
  long_entry_part(d, le, i - d.lent_ptr[le]);
}

// Residual per row: RHS = -(qscale (Q - Q_hist0) + fscale (F - B) + hscale Q_hist2 + gshunt x)
//                        + limiter terms     (OneStep::obtainResidual, N_TIA_OneStep.C:219-290)
__device__ __forceinline__ void assemble_row(const DevArrays &d, int r, double &vmax, double &vsum) {
  vmax = 0.0;
  vsum = 0.0;
  {
    const int c = d.circ_of_row[r];
    const CircState &s = d.cs[c];
    if (circ_active(s)) {
      double F, Q, B, L;
      const int lr = d.row_long[r];
      if (lr >= 0) {
        F = 0.0; Q = 0.0; B = 0.0; L = 0.0;
        const double *o = d.long_rsum + 4 * (size_t)d.lrow_ptr[lr];
        for (int k = 0; k < d.lrow_ptr[lr + 1] - d.lrow_ptr[lr]; ++k) {
          F += o[4 * k]; Q += o[4 * k + 1]; B += o[4 * k + 2]; L += o[4 * k + 3];
        }
      } else {
        F = 0.0; Q = 0.0; B = 0.0; L = 0.0;
        for (int e = d.rp[r]; e < d.rp[r + 1]; ++e) {
          const double xv = d.x[d.ci[e]];
          F += d.Glin[e] * xv;
          Q += d.Clin[e] * xv;
        }
        for (int k = d.vF_ptr[r]; k < d.vF_ptr[r + 1]; ++k) F += d.sF[d.vF_idx[k]];
        for (int k = d.vQ_ptr[r]; k < d.vQ_ptr[r + 1]; ++k) Q += d.sQ[d.vQ_idx[k]];
        for (int k = d.vB_ptr[r]; k < d.vB_ptr[r + 1]; ++k) B += d.sB[d.vB_idx[k]];
        for (int k = d.vL_ptr[r]; k < d.vL_ptr[r + 1]; ++k) L += d.sL[d.vL_idx[k]];
      }
      double res;
      if (s.phase == PH_TRAN && d.tp->gear) {
        // Gear12::obtainResidual (N_TIA_Gear12.C:208-271)
        double q = s.alpha[0] * Q + s.alpha[1] * d.qh0[r];
        if (s.order == 2) q += s.alpha[2] * d.qh1[r];
        res = (F - B) + (1.0 / s.h) * q;
      } else {
        res = s.fscale * (F - B);
        if (s.qscale != 0.0) res += s.qscale * (Q - d.qh0[r]);
        if (s.hscale != 0.0) res += s.hscale * d.qh2[r];
      }
      if (s.gshunt != 0.0 && !d.is_branch[r]) res += s.gshunt * d.x[r];
      const double rhs = -res + L;
      d.rhs[r] = rhs;
      d.Qv[r] = Q;
      d.FmB[r] = F - B;
      vmax = fabs(rhs);
      vsum = rhs * rhs;
      if (!(vsum == vsum) || isinf(vsum)) vmax = vsum = __longlong_as_double(0x7ff8000000000000ULL);
    }
  }
}

__global__ void __launch_bounds__(kRowBlock) k_assemble_rows(DevArrays d, int n) {
  const int r = blockIdx.x * kRowBlock + threadIdx.x;
  double vmax = 0.0, vsum = 0.0;
  if (r < n) assemble_row(d, r, vmax, vsum);
  block_partials(d, n, vmax, vsum, r);
}

// Jacobian per CSR entry: J = qscale dQdx + fscale dFdx (+ gshunt on the diagonal)
// (OneStep::obtainJacobian, N_TIA_OneStep.C:469-500; EpetraMatrix::linearCombo)
__device__ __forceinline__ void assemble_entry(const DevArrays &d, int e) {
  const int r = d.erow[e];
  const CircState &s = d.cs[d.circ_of_row[r]];
  if (!circ_active(s)) return;
  double v = s.qscale * d.Clin[e] + s.fscale * d.Glin[e];
  const int le = d.ent_long[e];
  if (le >= 0) {
    const double *o = d.long_esum + (size_t)d.lent_ptr[le];
    for (int k = 0; k < d.lent_ptr[le + 1] - d.lent_ptr[le]; ++k) v += o[k];
  } else {
    for (int k = d.m_ptr[e]; k < d.m_ptr[e + 1]; ++k) v += d.sM[d.m_idx[k]];
  }
  if (s.gshunt != 0.0 && d.ci[e] == r) v += s.gshunt;  // branch rows have no diagonal entry
  d.J[e] = v;
}

__global__ void k_assemble_J(DevArrays d, int nnz) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nnz) assemble_entry(d, e);
}

// Loader-API assembly: ADD device contributions into caller vectors (loadDAEVectors).
__global__ void k_load_vectors(DevArrays d, int n, const double *x, double *Q, double *F, double *B,
                               double *dFv, double *dQv, int load_type) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  if (load_type != XG_LOAD_NONLINEAR) {
    double Fl = 0.0, Ql = 0.0;
    for (int e = d.rp[r]; e < d.rp[r + 1]; ++e) {
      const double xv = x[d.ci[e]];
      Fl += d.Glin[e] * xv;
      Ql += d.Clin[e] * xv;
    }
    double Bs = 0.0;
    for (int k = d.vB_ptr[r]; k < d.vB_ptr[r + 1]; ++k) Bs += d.sB[d.vB_idx[k]];
    F[r] += Fl; Q[r] += Ql; B[r] += Bs;
  }
  if (load_type != XG_LOAD_LINEAR) {
    double Fs = 0.0, Qs = 0.0, Lf = 0.0, Lq = 0.0;
    for (int k = d.vF_ptr[r]; k < d.vF_ptr[r + 1]; ++k) Fs += d.sF[d.vF_idx[k]];
    for (int k = d.vQ_ptr[r]; k < d.vQ_ptr[r + 1]; ++k) Qs += d.sQ[d.vQ_idx[k]];
    for (int k = d.vL_ptr[r]; k < d.vL_ptr[r + 1]; ++k) { Lf += d.sL[d.vL_idx[k]]; Lq += d.sL2[d.vL_idx[k]]; }
    F[r] += Fs; Q[r] += Qs; dFv[r] += Lf; dQv[r] += Lq;
  }
}

// Loader-API assembly: ADD into caller dQdx / dFdx CSR values (loadDAEMatrices).
__global__ void k_load_matrices(DevArrays d, int nnz, double *dQdx, double *dFdx, int load_type) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  double f = 0.0, q = 0.0;
  if (load_type != XG_LOAD_NONLINEAR) { f += d.Glin[e]; q += d.Clin[e]; }
  if (load_type != XG_LOAD_LINEAR)
    for (int k = d.m_ptr[e]; k < d.m_ptr[e + 1]; ++k) { f += d.sM[d.m_idx[k]]; q += d.sM2[d.m_idx[k]]; }
  dFdx[e] += f;
  dQdx[e] += q;
}

// ---------------------------------------------------------------------------
// Per-circuit Newton decision: DampedNewton::converged_ (N_NLS_DampedNewton.C:1191-1396).
// A warp reduces the row partials of a circuit's residual; one thread then
// takes the decision.
//
// The max and the sum of circuit c's per-(row block, circuit) partials, by
// one warp (lane-strided, then a butterfly: every lane gets the totals), and
// whether any partial is NaN.
__device__ __forceinline__ void circuit_norms(const DevArrays &d, int c, int lane, double &m, double &sum,
                                              bool *bad) {
  m = 0.0;
  sum = 0.0;
  bool b = false;
  for (int k = d.pair_cstart[c] + lane; k < d.pair_cstart[c + 1]; k += 32) {
    const double a = d.pmax[k], v = d.psum[k];
    if (!(a == a) || !(v == v)) b = true;
    m = fmax(m, a);
    sum += v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
  }
  if (bad) *bad = __any_sync(0xffffffffu, b);
}

// The Newton decision of an active circuit from its residual norms (one thread).
__device__ void newton_ctl_scalar(const DevArrays &d, int c, double m, double sum, bool bad);

// One warp per circuit (all 32 lanes call it).
__device__ __forceinline__ void newton_ctl_circuit(const DevArrays &d, int c, int lane) {
  CircState &s = d.cs[c];
  if (s.phase == PH_STALL) return;  // parked until the host re-pivots; flags kept
  if (!circ_active(s)) {
    if (lane == 0) { s.need_solve = 0; s.step_end = 0; s.accept = 0; s.start_step = 0; }
    return;
  }
  double m, sum;
  bool bad;
  circuit_norms(d, c, lane, m, sum, &bad);
  if (lane == 0) newton_ctl_scalar(d, c, m, sum, bad);
}

__device__ void newton_ctl_scalar(const DevArrays &d, int c, double m, double sum, bool bad) {
  CircState &s = d.cs[c];
  const TranParams &p = *d.tp;
  const bool tran = s.phase == PH_TRAN;
  const double normRHS = bad ? __longlong_as_double(0x7ff8000000000000ULL) : sqrt(sum);
  const bool nan = !(normRHS == normRHS) || isinf(normRHS);
  s.accept = 0; s.start_step = 0; s.step_end = 0; s.need_solve = 0;
  const int limited = s.limited;
  s.limited = 0;
  int status = 0;
  if (s.iter == 0) {
    s.normRHS = normRHS;
    s.normRHS_init = normRHS;
    s.normRHS_old = normRHS;
    s.count = 0;
    s.tmpConvRate = 1.0;
    if (nan) status = -6;
  } else {
    const double eps = 2.220446049250313e-16;
    const double convRateMax = 0.5 * 1.7976931348623157e308;
    const int maxstep = tran ? p.nl_maxstep : p.dc_maxstep;
    const int nlStep = s.iter;
    s.normRHS = normRHS;
    s.maxNormRHS = m;
    if (nan) {
      status = -6;
    } else if (!tran && limited) {
      status = (nlStep < maxstep) ? 0 : -1;
    } else if (normRHS < eps) {
      status = 1;
    } else {
      const double rel = normRHS / s.normRHS_init;
      const double rate = normRHS / s.normRHS_old;
      s.normRHS_old = normRHS;
      const double rhstol = tran ? p.nl_rhstol : p.dc_rhstol;
      const double dxtol = tran ? p.nl_deltaxtol : p.dc_deltaxtol;
      if (m <= rhstol && s.wtNormDX <= dxtol) status = 2;
      else if (nlStep >= maxstep && tran && rel <= 0.9 && rate <= 1.0) status = -3;
      else if (s.wtNormDX <= p.nl_smallupdatetol) status = 4;
      else if (nlStep >= maxstep) status = -1;
      else if (rate > convRateMax) status = -2;
      else {
        if (tran && fabs(rate - 1.0) <= 1.0e-3) {
          if (s.count == 0 || rate < s.tmpConvRate) s.tmpConvRate = rate;
          s.count++;
        } else {
          s.count = 0;
        }
        if (tran && s.count == 5) { s.count = 0; status = -3; }
      }
    }
  }
  s.newton_status = status;
  if (status != 0) {
    s.step_end = 1;
  } else {
    s.need_solve = 1;
    s.singular = 0;
    // the Jacobian of a circuit without nonlinear devices is qscale C +
    // fscale G (+ gshunt): the same coefficients under the same analysis
    // give the same matrix bit for bit, and its factors are still in place
    const int gen = *d.lu_gen;
    const bool same = p.reuse_factors && d.circ_linear[c] && s.f_gen == gen && s.f_qscale == s.qscale &&
                      s.f_fscale == s.fscale && s.f_gshunt == s.gshunt;
    s.refactor = same ? 0 : 1;
    if (same) {
      s.factor_skips++;
    } else {
      s.f_gen = gen;
      s.f_qscale = s.qscale;
      s.f_fscale = s.fscale;
      s.f_gshunt = s.gshunt;
    }
  }
}

// A warp per circuit.
__global__ void __launch_bounds__(128) k_newton_ctl(DevArrays d, int ncirc) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c < ncirc) newton_ctl_circuit(d, c, threadIdx.x & 31);
}

// x += dx with the update norm; at the end of a Newton solve, the LTE sum
// (DataStore::stepLinearCombo + WRMS_errorNorm, N_TIA_DataStore.C:1495,1737)
// and max|x| for the next error weights.
__device__ __forceinline__ void update_row(const DevArrays &d, int r, double &vmax, double &vsum) {
  vmax = 0.0;
  vsum = 0.0;
  {
    const int c = d.circ_of_row[r];
    const CircState &s = d.cs[c];
    if (circ_active(s)) {
      if (s.need_solve) {
        if (!s.singular) {
          const double dxr = d.dx[r];
          const double xnew = d.x[r] + dxr;
          d.x[r] = xnew;
          double w = d.solwt[r];
          if (s.phase == PH_DC) {
            const TranParams &p = *d.tp;
            w = p.dc_reltol * fmax(fabs(xnew), fabs(d.xcurr[r])) + p.dc_abstol;
            d.solwt[r] = w;
          }
          vmax = fabs(dxr) / w;
          if (!(dxr == dxr) || isinf(dxr)) vsum = 1.0;  // NaN / Inf marker
        }
      } else if (s.step_end) {
        const double xr = d.x[r];
        vmax = fabs(xr);
        if (s.phase == PH_TRAN && s.newton_status > 0) {
          const double e = (xr - d.xn0[r]) / s.errwt;
          vsum = e * e;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(kRowBlock) k_update(DevArrays d, int n) {
  const int r = blockIdx.x * kRowBlock + threadIdx.x;
  double vmax = 0.0, vsum = 0.0;
  if (r < n) update_row(d, r, vmax, vsum);
  block_partials(d, n, vmax, vsum, r);
}

// Next step of one circuit: OneStep::initialize (N_TIA_OneStep.C:1684-1800),
// updateCoeffs (:1584-1640) and the error weights of DataStore::setErrorWtVector.
__device__ void start_next_step(CircState &s, const TranParams &p, int &init_hist) {
  init_hist = 0;
  if (s.beginning && s.lastOk) {
    const double time_to_stop = s.stopTime - s.t;
    double hn = (s.t == p.tstart) ? 0.005 * time_to_stop : 0.1 * fmin(s.saved, time_to_stop);
    if (hn > p.hmax) hn = p.hmax;
    // (Gear12::initialize takes the restart step as is, N_TIA_Gear12.C:1225-1245)
    s.h = (s.t != p.tstart && !p.gear) ? fmin(s.h, hn) : hn;
    s.h = fmin(fmax(s.h, p.hmin), p.hmax);
    s.tsum = 2.0 * s.h;
    s.lastTimeStep = s.h;
    s.numberOfSteps = 0;
    s.order = 1;
    s.psi[0] = s.h;
    init_hist = 1;
  }
  const double h = s.h;
  if (s.order == 2) s.psi[2] = s.psi[1];
  s.psi[1] = s.psi[0];
  s.psi[0] = h;
  if (p.gear) {
    // Gear12::updateCoeffs (N_TIA_Gear12.C:1050-1110): variable-step BDF
    // predictor (beta) and corrector (alpha) coefficients
    if (s.order == 2) {
      s.beta[2] = h / s.psi[2] * (h + s.psi[1]) / (s.psi[1] + s.psi[2]);
      s.beta[1] = -h / s.psi[1] - s.beta[2] * (s.psi[1] + s.psi[2]) / s.psi[1];
      s.beta[0] = 1.0 - s.beta[2] - s.beta[1];
      double a2 = -h / s.psi[1] * h / (2 * h + s.psi[1]);
      double a1 = 1 - a2;
      const double a0 = -a1 - a2 * (1 + s.psi[1] / h);
      s.alpha[2] = a2 / a0;
      s.alpha[1] = a1 / a0;
      s.alpha[0] = -1 / a0;
      s.ck = h / (h + s.psi[1] + s.psi[2]);
    } else {
      s.beta[0] = 1.0 + h / s.psi[1];
      s.beta[1] = -h / s.psi[1];
      s.alpha[0] = 1.0;
      s.alpha[1] = -1.0;
      s.alpha[2] = 0.0;
      s.ck = h / (h + s.psi[1]);
    }
  } else if (s.order == 2) {
    s.beta[1] = h / s.psi[1] + (h / s.psi[1]) * (h / s.psi[1]) / 2;
    s.beta[2] = -1.0 * h * h / s.psi[1] / s.psi[2] / 2;
    s.ck = (h / s.tsum) / 3.0;
  } else {
    s.beta[1] = h / s.psi[1];
    s.ck = h / s.tsum;
  }
  s.errwt = p.reltol * s.xmax_curr + p.abstol;
  double tn = s.t + h;
  if (fabs(tn - s.stopTime) <= p.bptol) tn = s.stopTime;
  s.tn = tn;
  if (p.gear) {
    // Gear12::obtainJacobian (N_TIA_Gear12.C:477-500): (alpha0 / h) dQdx + dFdx
    s.qscale = s.alpha[0] / h;
    s.fscale = 1.0;
    s.hscale = 0.0;
  } else {
    s.qscale = 1.0 / h;
    s.fscale = (s.order == 2) ? 0.5 : 1.0;
    s.hscale = (s.order == 2) ? 0.5 : 0.0;
  }
  s.iter = 0;
  s.start_step = 1;
}

__device__ double next_bp(const double *bps, int lo, int hi, double t, double bptol, int &idx) {
  int k = idx;
  if (k < lo) k = lo;
  while (k < hi && !(bps[k] > t + bptol)) ++k;
  idx = k;
  return (k < hi) ? bps[k] : bps[hi - 1];
}

// Per-circuit step decision (StepErrorControl::evaluateStepError, OneStep::completeStep /
// rejectStep, Transient::processSuccessfulStep) and the operating-point stages:
// a warp reduces the norms of the circuit's update, one thread decides.
__device__ void step_ctl_scalar(const DevArrays &d, int c, double m, double sum, const double *bps,
                                const int *bp_ptr, int cap);

__device__ __forceinline__ void step_ctl_circuit(const DevArrays &d, int c, int lane, const double *bps,
                                                 const int *bp_ptr, int cap) {
  if (!circ_active(d.cs[c])) return;
  double m, sum;
  circuit_norms(d, c, lane, m, sum, nullptr);
  if (lane == 0) step_ctl_scalar(d, c, m, sum, bps, bp_ptr, cap);
}

// The step decision of an active circuit from the norms of its update (one thread).
__device__ void step_ctl_scalar(const DevArrays &d, int c, double m, double sum, const double *bps,
                                const int *bp_ptr, int cap) {
  CircState &s = d.cs[c];
  const TranParams &p = *d.tp;
  if (s.need_solve) {
    if (s.singular) {
      // frozen pivot failed the threshold test: park this Newton iteration
      // (J and RHS stay intact) until the host re-pivots and resumes it
      s.stall_prev = s.phase;
      s.phase = PH_STALL;
      return;
    } else if (sum != 0.0) {
      s.newton_status = -6;   // NaN or Inf in the Newton update
    } else {
      s.wtNormDX = m;
      s.iter++;
      return;
    }
    s.iter++;
    s.need_solve = 0;
    s.step_end = 1;
  }
  if (!s.step_end) return;
  const int n_c = d.offsets[c + 1] - d.offsets[c];
  const int status = s.newton_status;
  if (p.newton_only) {
    // a Newton solve on its own (xg_newton_solve): the circuit stops with
    // its DampedNewton status
    s.newton_iters += s.iter;
    s.phase = status > 0 ? PH_DONE : PH_FAILED;
    return;
  }
  const int b0 = bp_ptr[c], b1 = bp_ptr[c + 1];
  s.accept = 0;
  if (s.phase == PH_DC) {
    s.dcop_iters += s.iter;
    if (status > 0) {
      if (s.gshunt > 0.0) {
        s.gshunt = (s.gshunt / 10.0 >= 1e-12 * 0.999) ? s.gshunt / 10.0 : 0.0;
        s.iter = 0;
        s.init_jct = 0;
        return;
      }
      // operating point done: the DC solution is the accepted state at tstart
      s.accept = 2;  // "DC accepted" event for k_history / k_state_commit
      s.xmax_curr = m;
      s.phase = p.dc_only ? PH_DONE : PH_TRAN;
      s.t = p.tstart;
      s.beginning = 1;
      s.lastOk = 1;
      s.stepNumber = 0;
      s.estOverTol = 0.0;
      s.saved = p.hmax;
      s.nef = 0;
      s.order = 1;
      s.bp_index = b0;
      s.stopTime = next_bp(bps, b0, b1, s.t, p.bptol, s.bp_index);
      s.init_jct = 0;
      s.gshunt = 0.0;
      if (s.n_out < cap) {
        d.out_t[(size_t)c * cap + s.n_out] = s.t;
        d.out_o[(size_t)c * cap + s.n_out] = 0;
      }
      s.n_out++;
      if (p.dc_only) return;
    } else {
      if (s.dc_stage == 0) {
        s.dc_stage = 1;
        s.gshunt = 1e-2;
        s.init_jct = 1;
        s.iter = 0;
        s.accept = 3;  // restart from x = 0
        return;
      }
      s.phase = PH_FAILED;
      s.newton_status = status;
      return;
    }
  } else {
    // transient step end
    s.newton_iters += s.iter;
    s.last_iters = s.iter;
    bool ok = status > 0;
    if (!ok) s.newton_fail++;
    if (ok) {
      const bool test = (s.t == p.tstart) ? (s.stepNumber >= 1 && !s.beginning) : (s.stepNumber >= 1);
      if (test) {
        s.estOverTol = s.ck * sqrt(sum / n_c);
        if (!(s.estOverTol <= 1.0)) { ok = false; s.lte_fail++; }
      }
    }
    if (ok) {
      const int step_order = s.order;  // the order this step was integrated with
      s.numberOfSteps++;
      s.nef = 0;
      s.t = s.tn;
      s.lastTimeStep = s.h;
      double rr = pow(0.5 / (s.estOverTol + 0.0001), 1.0 / (s.order + 1.0));
      if (s.numberOfSteps >= 2 && p.max_order == 2 && s.order == 1) {
        s.order = 2;
        rr = pow(0.5 / (s.estOverTol + 0.0001), 1.0 / 3.0);
        if (rr <= 1.05) s.order = 1;
      }
      double hnew = s.h;
      if (rr >= 2.0) hnew = 2.0 * s.h;
      else if (rr <= 1) hnew = fmax(0.25, fmin(0.9, rr)) * s.h;
      hnew = fmin(fmax(hnew, p.hmin), p.hmax);
      const bool hit_bp = fabs(s.t - s.stopTime) <= p.bptol && fabs(s.t - p.tstop) > p.bptol;
      if (hit_bp) {
        s.saved = hnew;
        s.beginning = 1;
        s.stopTime = next_bp(bps, b0, b1, s.t, p.bptol, s.bp_index);
      } else {
        s.beginning = 0;
        if (s.t + hnew > s.stopTime) { s.saved = hnew; hnew = s.stopTime - s.t; }
        s.h = hnew;
        s.tsum = s.h + s.lastTimeStep;
      }
      s.stepNumber++;
      s.accepted++;
      s.lastOk = 1;
      s.accept = 1;
      s.xmax_curr = m;
      if (s.n_out < cap) {
        d.out_t[(size_t)c * cap + s.n_out] = s.t;
        d.out_o[(size_t)c * cap + s.n_out] = (signed char)step_order;
      }
      s.n_out++;
      if (s.t >= p.tstop - p.bptol || (p.max_steps > 0 && s.accepted >= p.max_steps)) {
        s.phase = PH_DONE;
        return;
      }
    } else {
      s.rejected++;
      s.lastOk = 0;
      s.nef++;
      for (int i = 1; i <= s.order; ++i) s.psi[i - 1] = s.psi[i];
      if (s.nef >= 15) { s.phase = PH_FAILED; s.newton_status = -1; return; }
      double hnew;
      if (status <= 0) {
        hnew = s.h / 8; s.order = 1;
      } else if (s.nef == 1) {
        // OneStep drops to first order first; Gear12::rejectStep keeps the
        // order (N_TIA_Gear12.C:1500-1515)
        if (!p.gear) s.order = 1;
        double rr = pow(0.5 / (s.estOverTol + 0.0001), 1.0 / (s.order + 1.0));
        rr = fmax(0.25, fmin(0.9, rr));
        hnew = rr * s.h;
      } else {
        hnew = 0.25 * s.h; s.order = 1;
      }
      hnew = fmin(fmax(hnew, p.hmin), p.hmax);
      if (s.t + hnew > s.stopTime) hnew = s.stopTime - s.t;
      s.h = hnew;
      s.tsum = s.h + s.lastTimeStep;
      if (!(s.h > 0.0)) { s.phase = PH_FAILED; s.newton_status = -2; return; }
    }
  }
  int init_hist = 0;
  start_next_step(s, p, init_hist);
  s.init_hist = init_hist;
  if (s.accepted >= s.stop_at) s.phase = PH_PAUSED;  // the predictor is applied, then the circuit waits
}

// A warp per circuit.
__global__ void __launch_bounds__(128) k_step_ctl(DevArrays d, int ncirc, const double *bps, const int *bp_ptr,
                                                  int cap) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c < ncirc) step_ctl_circuit(d, c, threadIdx.x & 31, bps, bp_ptr, cap);
}

// OneStep::updateHistory (N_TIA_OneStep.C:1390-1440), OneStep::initialize history
// (:1800-1830) and obtainPredictor (:135-175), per row.
__device__ __forceinline__ void history_row(const DevArrays &d, int r, int cap, int pmax) {
  const int c = d.circ_of_row[r];
  const CircState &s = d.cs[c];
  if (s.accept == 3) { d.x[r] = 0.0; return; }
  if (!s.step_end && !s.start_step) return;
  const bool accepted_tran = s.accept == 1;
  const bool accepted_dc = s.accept == 2;
  const bool gear = d.tp->gear;
  if (accepted_tran) {
    if (gear) {
      // Gear12::updateHistory (N_TIA_Gear12.C:822-870): absolute histories
      if (s.order == 2) d.xh2[r] = d.xh1[r];
      d.qh1[r] = d.qh0[r];
      d.xh1[r] = d.xcurr[r];
    } else {
      if (s.order == 2) { d.xh2[r] = d.xh1[r]; d.qh2[r] = d.FmB[r]; }
      d.xh1[r] = d.x[r] - d.xcurr[r];
      d.qh1[r] = d.Qv[r] - d.qh0[r];
    }
    // the learned predictor's history: differences of the last four solutions
    d.mlh3[r] = d.mlh2[r];
    d.mlh2[r] = d.mlh1[r];
    d.mlh1[r] = d.x[r] - d.xcurr[r];
  }
  if (accepted_tran || accepted_dc) {
    const double xr = d.x[r];
    d.xcurr[r] = xr;
    d.qh0[r] = d.Qv[r];
    d.Qc[r] = d.Qv[r];
    d.FmBc[r] = d.FmB[r];
    const int pj = d.probe_idx[r];
    if (pj >= 0 && s.n_out - 1 < cap) {
      const size_t o = ((size_t)c * cap + (s.n_out - 1)) * pmax + pj;
      d.out_v[o] = xr;
      d.out_p[o] = accepted_tran ? d.xn0[r] : xr;  // the predictor of the accepted step
    }
  }
  if (s.start_step && (s.phase == PH_TRAN || s.phase == PH_PAUSED)) {
    const TranParams &p = *d.tp;
    if (s.init_hist) {
      if (gear) {  // Gear12::initialize history (N_TIA_Gear12.C:1280-1300)
        d.xh1[r] = d.xcurr[r];
        d.qh1[r] = d.Qc[r];
      } else {     // OneStep::initialize history
        d.xh1[r] = 0.0;
        d.qh1[r] = -d.FmBc[r] * s.h;
      }
      d.qh0[r] = d.Qc[r];
    }
    const double xc = d.xcurr[r];
    double xn;
    if (gear) {  // Gear12::obtainPredictor (N_TIA_Gear12.C:131-145)
      xn = s.beta[0] * xc;
      xn += s.beta[1] * d.xh1[r];
    } else {
      xn = xc + s.beta[1] * d.xh1[r];
    }
    if (s.order == 2) xn += s.beta[2] * d.xh2[r];
    d.xn0[r] = xn;
    d.x[r] = xn;
    d.solwt[r] = p.nl_reltol * fmax(fabs(xn), fabs(xc)) + p.nl_abstol;
  }
}

__global__ void k_history(DevArrays d, int n, int cap, int pmax) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) history_row(d, r, cap, pmax);
}

// Accepted store/state become current (curr <- next) for accepted circuits;
// i indexes MOSFET-1 instances, then diodes, then BSIM4 instances.
__device__ __forceinline__ void commit_instance(const DevArrays &d, int i, int nm, int nd, int sto_base_m, int nb,
                                                int sto_base_b, int sta_base_b) {
  if (i >= nm + nd && i < nm + nd + nb) {
    const int j = i - nm - nd;
    const CircState &s = d.cs[d.b4_circ[j]];
    if (s.accept == 1 || s.accept == 2) {
#pragma unroll
      for (int k = 0; k < 5; ++k) d.sto_curr[sto_base_b + k * nb + j] = d.sto_next[sto_base_b + k * nb + j];
#pragma unroll
      for (int k = 0; k < 3; ++k) d.sta_curr[sta_base_b + k * nb + j] = d.sta_next[sta_base_b + k * nb + j];
    }
    return;
  }
  if (i < nm) {
    const CircState &s = d.cs[d.m1_circ[i]];
    if (s.accept == 1 || s.accept == 2) {
#pragma unroll
      for (int k = 0; k < 6; ++k) d.sto_curr[sto_base_m + k * nm + i] = d.sto_next[sto_base_m + k * nm + i];
#pragma unroll
      for (int k = 0; k < 8; ++k) d.sta_curr[k * nm + i] = d.sta_next[k * nm + i];
    }
  } else if (i < nm + nd) {
    const int j = i - nm;
    const CircState &s = d.cs[d.d_circ[j]];
    if (s.accept == 1 || s.accept == 2) {
#pragma unroll
      for (int k = 0; k < 3; ++k) d.sto_curr[k * nd + j] = d.sto_next[k * nd + j];
    }
  }
}

__global__ void k_state_commit(DevArrays d, int nm, int nd, int sto_base_m, int nb, int sto_base_b,
                               int sta_base_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  commit_instance(d, i, nm, nd, sto_base_m, nb, sto_base_b, sta_base_b);
}

// Number of finished circuits (done or failed) and the LU breakdown flag,
// into mapped host memory that the host loop reads between tick batches.
// status_out: [0] circuits done, failed or paused, [1] breakdown flag,
// [2..3] (one 64-bit word) Newton iterations run so far, summed over circuits.
// A thread per circuit; the blocks add into d.done_acc and the last block to
// finish writes the status and clears the accumulators for the next launch.
__global__ void __launch_bounds__(256) k_count_done(DevArrays d, int ncirc, const int *breakdown, int *status_out) {
  __shared__ unsigned long long s_cnt, s_it;
  __shared__ bool last;
  if (threadIdx.x == 0) { s_cnt = 0; s_it = 0; }
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long cnt = 0, it = 0;
  if (c < ncirc) {
    const CircState &s = d.cs[c];
    const int ph = s.phase;
    cnt = (ph == PH_DONE || ph == PH_FAILED || ph == PH_PAUSED) ? 1 : 0;
    it = (unsigned long long)(s.newton_iters + s.dcop_iters);
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    it += __shfl_xor_sync(0xffffffffu, it, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_cnt, cnt);
    atomicAdd(&s_it, it);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(d.done_acc, s_cnt);
    atomicAdd(d.done_acc + 1, s_it);
    __threadfence();
    last = atomicAdd(d.done_acc + 2, 1ULL) == (unsigned long long)gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const unsigned long long total = atomicAdd(d.done_acc, 0ULL), iters = atomicAdd(d.done_acc + 1, 0ULL);
    status_out[0] = (int)total;
    status_out[1] = *breakdown;
    reinterpret_cast<unsigned long long *>(status_out)[1] = iters;
    d.done_acc[0] = 0; d.done_acc[1] = 0; d.done_acc[2] = 0;
  }
}

// Circuits parked by an LU breakdown resume their phase after the host re-pivots.
__global__ void k_unstall(DevArrays d, int ncirc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncirc) return;
  CircState &s = d.cs[c];
  if (s.phase == PH_STALL) {
    s.phase = s.stall_prev;
    s.singular = 0;
  } else {
    // the other circuits already finished this tick: clear its events so the
    // resumed factor/solve/update/step/history launches leave them untouched
    s.need_solve = 0; s.step_end = 0; s.accept = 0; s.start_step = 0;
  }
}

// ---------------------------------------------------------------------------
// Circuit-resident tick (see FusedDev): one CTA per circuit runs every stage
// of a tick — the same per-item device functions as the kernels above, each
// item computed the way those kernels compute it — and loops over ticks
// until its circuit stops being active.  No stage waits on another CTA.

// The per-(row block, circuit) partial max / sum slots of circuit c, as
// block_partials computes them: a warp per slot, rows strided by 32 from the
// slot's first row, butterfly.
__device__ void circuit_partials(const DevArrays &d, int c, int o0, int o1, const double *vm, const double *vs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int b0 = o0 / kRowBlock, b1 = (o1 - 1) / kRowBlock;
  for (int b = b0 + warp; b <= b1; b += nwarps) {
    const int lo = max(o0, b * kRowBlock), hi = min(o1, (b + 1) * kRowBlock);
    double m = 0.0, s = 0.0;
    for (int r = lo + lane; r < hi; r += 32) {
      m = fmax(m, vm[r - o0]);
      s += vs[r - o0];
    }
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) {
      const int slot = d.pair_base[b] + (c - d.blk_cfirst[b]);
      d.pmax[slot] = m;
      d.psum[slot] = s;
    }
  }
}

// Arguments of the resident tick that the separate launches take one by one.
struct FusedArgs {
  int ncirc, nm, nd, nv, sto_base_m;
  int sF_m, sQ_m, sL_m, sM_m, sF_d, sQ_d, sL_d, sM_d;
  const double *bps;
  const int *bp_ptr;
  int cap, pmax;
  double pivot_tol;
  // per-stage clock: when not null, thread 0 of each CTA adds the cycles its
  // CTA spends in each stage of a tick (XG_RSTAGE_*) into clk[stage]
  unsigned long long *clk;
};

// Stage clock of the resident tick: cycles since the last mark, into stage k.
struct StageClock {
  unsigned long long *clk;
  long long t;
  __device__ explicit StageClock(unsigned long long *c) {
    clk = c;
    t = 0;
    if (c && threadIdx.x == 0) t = clock64();
  }
  __device__ void mark(int k) {
    if (clk && threadIdx.x == 0) {
      const long long now = clock64();
      atomicAdd(clk + k, (unsigned long long)(now - t));
      t = now;
    }
  }
};

// The factorization of circuit c (refactoring this tick: every column is
// factored), level by level: single-thread columns,
// warp columns, then the columns that take the whole CTA (each level's
// items are sorted by kind; F.f_split gives where the warp and CTA kinds
// start).  S (when the circuit's columns fit): the circuit's columns are
// loaded into shared memory once, factored there and written back once.
__device__ void resident_factor(const DevArrays &d, const LUDev &L, const FusedDev &F, int c, double pivot_tol,
                                double *sm, double *S) {
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31, nwarps = nth >> 5;
  const int lv0 = F.f_cl[c], lv1 = F.f_cl[c + 1];
  const int *soff = S ? F.c_soff : L.grp_soff;
  const int4 *umeta = S ? F.c_umeta : L.umeta;
  if (S) {
    for (int t = F.f_lptr[lv0] + warp; t < F.f_lptr[lv1]; t += nwarps) {
      const int j = F.f_items[t], p0 = L.cp[j], p1 = L.cp[j + 1], o = F.c_soff[j];
      for (int p = p0 + lane; p < p1; p += 32) {
        const int sp = L.src[p];
        S[o + (p - p0)] = (sp >= 0) ? d.J[sp] : 0.0;
      }
    }
    __syncthreads();
  }
  for (int lv = lv0; lv < lv1; ++lv) {
    const int a = F.f_lptr[lv], b = F.f_lptr[lv + 1];
    const int2 sp = F.f_split[lv];
    for (int t = a + tid; t < sp.x; t += nth) {
      const int j = F.f_items[t];
      factor_column_t<double>(L, d.J, j, d.cs, 1, pivot_tol, S, soff, umeta);
    }
    for (int t = sp.x + warp; t < sp.y; t += nwarps) {
      const int j = F.f_items[t];
      if (S) factor_column_s<false, double>(L, j, d.cs, 1, pivot_tol, sm, S, soff, umeta);
      else factor_column<false, double>(L, d.J, j, d.cs, 1, pivot_tol, sm);
    }
    // the thread and warp columns are done, and a breakdown they flagged is
    // visible to every thread: the tests below read the same values in all
    __syncthreads();
    for (int t = sp.y; t < b; ++t) {
      const int j = F.f_items[t];
      if (S) factor_column_s<true, double>(L, j, d.cs, 1, pivot_tol, sm, S, soff, umeta);
      else factor_column<true, double>(L, d.J, j, d.cs, 1, pivot_tol, sm);
      __syncthreads();
    }
  }
  if (S) {
    // the factored columns back to global memory (the solves read them there)
    for (int t = F.f_lptr[lv0] + warp; t < F.f_lptr[lv1]; t += nwarps) {
      const int j = F.f_items[t], p0 = L.cp[j], p1 = L.cp[j + 1], o = F.c_soff[j];
      for (int p = p0 + lane; p < p1; p += 32) L.lu[p] = S[o + (p - p0)];
    }
    __syncthreads();
  }
}

// The L solve (forward) and the U solve (backward) of circuit c; every row
// is summed the way the grouped kernels sum it (F.l_meth / F.u_meth), the
// level's rows sorted by method (F.l_split / F.u_split).
__device__ void resident_solve(const DevArrays &d, const LUDev &L, const FusedDev &F, int c, double *sm) {
  const int tid = threadIdx.x, nth = blockDim.x;
  const int team = tid >> 3, nteams = nth >> 3, sub = tid & 7;
  const double *lu = L.lu;
  const double *b = d.rhs;
  double *x = d.dx;
  for (int lv = F.l_cl[c]; lv < F.l_cl[c + 1]; ++lv) {
    const int a = F.l_lptr[lv], e = F.l_lptr[lv + 1];
    const int2 sp = F.l_split[lv];
    for (int t = a + tid; t < sp.x; t += nth) {
      const int i = F.l_items[t];
      if (F.l_meth[i] == 0) {
        L.y[i] = b[L.row_of_step[i]];
      } else {
        double sum = 0.0;
        for (int q = L.l_ptr[i]; q < L.l_ptr[i + 1]; ++q) sum += (double)lu[L.l_pos[q]] * L.y[L.l_col[q]];
        L.y[i] = b[L.row_of_step[i]] - sum;
      }
    }
    for (int t0 = sp.x; t0 < sp.y; t0 += nteams) {  // warp-uniform bound
      const int t = t0 + team;
      const bool act = t < sp.y;
      const int i = act ? F.l_items[t] : 0;
      double sum = 0.0;
      if (act)
        for (int q = L.l_ptr[i] + sub; q < L.l_ptr[i + 1]; q += 8) sum += (double)lu[L.l_pos[q]] * L.y[L.l_col[q]];
      for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
      if (act && sub == 0) L.y[i] = b[L.row_of_step[i]] - sum;
    }
    for (int t = sp.y; t < e; ++t) {
      const int i = F.l_items[t];
      const double sum = long_row_dot<double>(lu, L.l_pos, L.l_col, L.y, L.l_ptr[i], L.l_ptr[i + 1], sm);
      if (tid == 0) L.y[i] = b[L.row_of_step[i]] - sum;
    }
    __syncthreads();
  }
  for (int lv = F.f_cl[c + 1] - 1; lv >= F.f_cl[c]; --lv) {
    const int a = F.f_lptr[lv], e = F.f_lptr[lv + 1];
    const int2 sp = F.u_split[lv];
    for (int t = a + tid; t < sp.x; t += nth) {
      const int k = F.u_items[t];
      double sum = 0.0;
      for (int q = L.u_ptr[k]; q < L.u_ptr[k + 1]; ++q) sum += (double)lu[L.u_pos[q]] * L.y[L.u_col[q]];
      const double z = (L.y[k] - sum) / (double)lu[L.diag[k]];
      L.y[k] = z;
      x[L.col_of_step[k]] = z;
    }
    for (int t0 = sp.x; t0 < sp.y; t0 += nteams) {
      const int t = t0 + team;
      const bool act = t < sp.y;
      const int k = act ? F.u_items[t] : 0;
      double sum = 0.0;
      if (act)
        for (int q = L.u_ptr[k] + sub; q < L.u_ptr[k + 1]; q += 8) sum += (double)lu[L.u_pos[q]] * L.y[L.u_col[q]];
      for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
      if (act && sub == 0) {
        const double z = (L.y[k] - sum) / (double)lu[L.diag[k]];
        L.y[k] = z;
        x[L.col_of_step[k]] = z;
      }
    }
    for (int t = sp.y; t < e; ++t) {
      const int k = F.u_items[t];
      const double sum = long_row_dot<double>(lu, L.u_pos, L.u_col, L.y, L.u_ptr[k], L.u_ptr[k + 1], sm);
      if (tid == 0) {
        const double z = (L.y[k] - sum) / (double)lu[L.diag[k]];
        L.y[k] = z;
        x[L.col_of_step[k]] = z;
      }
    }
    __syncthreads();
  }
}

// Ticks of circuit c until it stops being active (paused, done, failed, or
// parked on a pivot breakdown for the host).
__device__ void resident_circuit(const DevArrays &d, const LUDev &L, const FusedDev &F, const FusedArgs &A, int c,
                                 double *vm, double *vs, double *ws, double *sm, double *S) {
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
  const int o0 = d.offsets[c], o1 = d.offsets[c + 1];
  const int e0 = d.rp[o0], e1 = d.rp[o1];
  const CircState &s = d.cs[c];
  StageClock clk(A.clk);
  int ticks = 0;
  for (; ticks < kFusedMaxTicks; ++ticks) {
    __syncthreads();
    const int ph = s.phase;
    if (!(ph == PH_DC || ph == PH_TRAN)) break;  // uniform: read after the barrier
    for (int k = F.src_ptr[c] + tid; k < F.src_ptr[c + 1]; k += nth) source_value(d, F.src_list[k], A.nv, 0, 0.0);
    __syncthreads();
    clk.mark(XG_RSTAGE_SOURCES);
    for (int k = F.m1_ptr[c] + tid; k < F.m1_ptr[c + 1]; k += nth)
      mos1_eval(d, F.m1_list[k], A.nm, A.sto_base_m, 1, 1, 0, 0, A.sF_m, A.sQ_m, A.sL_m, A.sM_m);
    for (int k = F.d_ptr[c] + tid; k < F.d_ptr[c + 1]; k += nth)
      diode_eval(d, F.d_list[k], A.nd, 1, 1, 0, 0, A.sF_d, A.sQ_d, A.sL_d, A.sM_d);
    __syncthreads();
    clk.mark(XG_RSTAGE_DEVICES);
    // a warp per part of the circuit's long rows, then of its long entries
    for (int q = F.lr_ptr[c]; q < F.lr_ptr[c + 1]; ++q) {
      const int lr = F.lr_list[q];
      for (int part = warp; part < d.lrow_ptr[lr + 1] - d.lrow_ptr[lr]; part += nth >> 5) long_row_part(d, lr, part);
    }
    for (int q = F.le_ptr[c]; q < F.le_ptr[c + 1]; ++q) {
      const int le = F.le_list[q];
      for (int part = warp; part < d.lent_ptr[le + 1] - d.lent_ptr[le]; part += nth >> 5) long_entry_part(d, le, part);
    }
    __syncthreads();
    clk.mark(XG_RSTAGE_LONG_GATHERS);
    for (int r = o0 + tid; r < o1; r += nth) {
      double a, b;
      assemble_row(d, r, a, b);
      vm[r - o0] = a;
      vs[r - o0] = b;
    }
    for (int e = e0 + tid; e < e1; e += nth) assemble_entry(d, e);
    __syncthreads();
    clk.mark(XG_RSTAGE_ASSEMBLE);
    circuit_partials(d, c, o0, o1, vm, vs);
    __syncthreads();
    if (warp == 0) newton_ctl_circuit(d, c, lane);
    __syncthreads();
    clk.mark(XG_RSTAGE_NEWTON);
    if (s.need_solve && !s.singular) {  // uniform
      if (s.refactor) resident_factor(d, L, F, c, A.pivot_tol, sm, S);
      clk.mark(XG_RSTAGE_FACTOR);
      if (!s.singular) resident_solve(d, L, F, c, sm);  // uniform: read after the factor's last barrier
    }
    __syncthreads();
    clk.mark(XG_RSTAGE_SOLVE);
    for (int r = o0 + tid; r < o1; r += nth) {
      double a, b;
      update_row(d, r, a, b);
      vm[r - o0] = a;
      vs[r - o0] = b;
    }
    __syncthreads();
    circuit_partials(d, c, o0, o1, vm, vs);
    __syncthreads();
    clk.mark(XG_RSTAGE_UPDATE);
    if (warp == 0) step_ctl_circuit(d, c, lane, A.bps, A.bp_ptr, A.cap);
    __syncthreads();
    clk.mark(XG_RSTAGE_STEP);
    for (int r = o0 + tid; r < o1; r += nth) history_row(d, r, A.cap, A.pmax);
    for (int k = F.m1_ptr[c] + tid; k < F.m1_ptr[c + 1]; k += nth)
      commit_instance(d, F.m1_list[k], A.nm, A.nd, A.sto_base_m, 0, 0, 0);
    for (int k = F.d_ptr[c] + tid; k < F.d_ptr[c + 1]; k += nth)
      commit_instance(d, A.nm + F.d_list[k], A.nm, A.nd, A.sto_base_m, 0, 0, 0);
    clk.mark(XG_RSTAGE_COMMIT);
  }
  if (tid == 0 && ticks > 0) {
    atomicMax(F.ticks, (unsigned long long)ticks);
    atomicAdd(F.ticks + 1, (unsigned long long)ticks);
  }
}

// CTAs take circuits from the queue (F.order: largest first) until it is
// empty.  THREADS per CTA, as many CTAs per SM as 128 registers a thread
// allow; every CTA size computes the same bits.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 512 / THREADS > 16 ? 16 : 512 / THREADS) k_resident(DevArrays d, LUDev L,
                                                                                          FusedDev F, FusedArgs A) {
  extern __shared__ __align__(16) double fz_rows[];
  __shared__ double ws[8 * 4], sm[32];
  __shared__ int next;
  double *vm = fz_rows, *vs = fz_rows + F.max_rows;
  double *S = F.max_fbuf > 0 ? fz_rows + 2 * F.max_rows : nullptr;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) next = atomicAdd(F.queue, 1);
    __syncthreads();
    const int q = next;
    if (q >= A.ncirc) return;
    resident_circuit(d, L, F, A, F.order[q], vm, vs, ws, sm, S);
  }
}

// ---------------------------------------------------------------------------
// Launchers.
static inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

template <int THREADS>
static int resident_grid(size_t smem, int sms, int *grid) {
  if (cudaFuncSetAttribute(k_resident<THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return XG_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resident<THREADS>, THREADS, smem) != cudaSuccess ||
      per_sm < 1)
    return XG_ERR_CUDA;
  *grid = per_sm * sms;
  return XG_OK;
}

// Persistent grids of the CTA sizes kResidentThreads (32 ... 512).
int resident_prepare_k(int max_rows, int max_fbuf, int device, int *grid) {
  const size_t smem = sizeof(double) * (2 * (size_t)max_rows + (size_t)max_fbuf);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return XG_ERR_CUDA;
  int rc = resident_grid<32>(smem, sms, &grid[0]);
  if (rc == XG_OK) rc = resident_grid<64>(smem, sms, &grid[1]);
  if (rc == XG_OK) rc = resident_grid<128>(smem, sms, &grid[2]);
  if (rc == XG_OK) rc = resident_grid<256>(smem, sms, &grid[3]);
  if (rc == XG_OK) rc = resident_grid<512>(smem, sms, &grid[4]);
  return rc;
}

void launch_resident_k(cudaStream_t st, const DevArrays &d, const LUDev &L, const FusedDev &F, int threads,
                       int ncirc, int nm, int nd, int nv, int sto_base_m, const int *slots, const double *bps,
                       const int *bp_ptr, int cap, int pmax, double pivot_tol, unsigned long long *clk) {
  FusedArgs A;
  A.clk = clk;
  A.ncirc = ncirc; A.nm = nm; A.nd = nd; A.nv = nv; A.sto_base_m = sto_base_m;
  A.sF_m = slots[0]; A.sQ_m = slots[1]; A.sL_m = slots[2]; A.sM_m = slots[3];
  A.sF_d = slots[4]; A.sQ_d = slots[5]; A.sL_d = slots[6]; A.sM_d = slots[7];
  A.bps = bps; A.bp_ptr = bp_ptr; A.cap = cap; A.pmax = pmax; A.pivot_tol = pivot_tol;
  cudaMemsetAsync(F.queue, 0, sizeof(int), st);
  cudaMemsetAsync(F.ticks, 0, 2 * sizeof(unsigned long long), st);
  const size_t smem = sizeof(double) * (2 * (size_t)F.max_rows + (size_t)F.max_fbuf);
  switch (threads) {
    case 32: k_resident<32><<<std::min(F.grid[0], ncirc), 32, smem, st>>>(d, L, F, A); break;
    case 64: k_resident<64><<<std::min(F.grid[1], ncirc), 64, smem, st>>>(d, L, F, A); break;
    case 128: k_resident<128><<<std::min(F.grid[2], ncirc), 128, smem, st>>>(d, L, F, A); break;
    case 256: k_resident<256><<<std::min(F.grid[3], ncirc), 256, smem, st>>>(d, L, F, A); break;
    default: k_resident<512><<<std::min(F.grid[4], ncirc), 512, smem, st>>>(d, L, F, A); break;
  }
}

void launch_sources_k(cudaStream_t st, const DevArrays &d, int n_v, int n_src, int use_explicit,
                      double t) {
  if (n_src > 0) k_sources<<<nblk(n_src, 128), 128, 0, st>>>(d, n_v, n_src, use_explicit, t);
}
void launch_mos1_k(cudaStream_t st, const DevArrays &d, int nm, int sto_base, int combined, int masked,
                   int it, int flags, int sF, int sQ, int sL, int sM) {
  if (nm > 0)
    k_mos1<<<nblk(nm, 128), 128, 0, st>>>(d, nm, sto_base, combined, masked, it, flags, sF, sQ, sL, sM);
}
void launch_diode_k(cudaStream_t st, const DevArrays &d, int nd, int combined, int masked, int it,
                    int flags, int sF, int sQ, int sL, int sM) {
  if (nd > 0)
    k_diode<<<nblk(nd, 128), 128, 0, st>>>(d, nd, combined, masked, it, flags, sF, sQ, sL, sM);
}
void launch_assemble_k(cudaStream_t st, const DevArrays &d, int n, int nnz, int n_long_row_blocks,
                       int n_long_ent_blocks) {
  if (n_long_row_blocks > 0) k_long_rows<<<nblk(n_long_row_blocks, 8), 256, 0, st>>>(d, n_long_row_blocks);
  if (n_long_ent_blocks > 0) k_long_entries<<<nblk(n_long_ent_blocks, 8), 256, 0, st>>>(d, n_long_ent_blocks);
  k_assemble_rows<<<nblk(n, kRowBlock), kRowBlock, 0, st>>>(d, n);
  k_assemble_J<<<nblk(nnz, 256), 256, 0, st>>>(d, nnz);
}
void launch_load_vectors_k(cudaStream_t st, const DevArrays &d, int n, const double *x, double *Q,
                           double *F, double *B, double *dFv, double *dQv, int lt) {
  k_load_vectors<<<nblk(n, 256), 256, 0, st>>>(d, n, x, Q, F, B, dFv, dQv, lt);
}
void launch_load_matrices_k(cudaStream_t st, const DevArrays &d, int nnz, double *dQdx, double *dFdx,
                            int lt) {
  k_load_matrices<<<nblk(nnz, 256), 256, 0, st>>>(d, nnz, dQdx, dFdx, lt);
}
void launch_newton_ctl_k(cudaStream_t st, const DevArrays &d, int ncirc) {
  k_newton_ctl<<<nblk(ncirc, 4), 128, 0, st>>>(d, ncirc);
}
void launch_update_k(cudaStream_t st, const DevArrays &d, int n) {
  k_update<<<nblk(n, kRowBlock), kRowBlock, 0, st>>>(d, n);
}
void launch_step_ctl_k(cudaStream_t st, const DevArrays &d, int ncirc, const double *bps,
                       const int *bp_ptr, int cap) {
  k_step_ctl<<<nblk(ncirc, 4), 128, 0, st>>>(d, ncirc, bps, bp_ptr, cap);
}
void launch_history_k(cudaStream_t st, const DevArrays &d, int n, int cap, int pmax) {
  k_history<<<nblk(n, 256), 256, 0, st>>>(d, n, cap, pmax);
}
void launch_state_commit_k(cudaStream_t st, const DevArrays &d, int nm, int nd, int sto_base_m, int nb,
                           int sto_base_b, int sta_base_b) {
  if (nm + nd + nb > 0)
    k_state_commit<<<nblk(nm + nd + nb, 256), 256, 0, st>>>(d, nm, nd, sto_base_m, nb, sto_base_b, sta_base_b);
}
void launch_count_done_k(cudaStream_t st, const DevArrays &d, int ncirc, const int *breakdown,
                         int *status_out) {
  k_count_done<<<nblk(ncirc, 256), 256, 0, st>>>(d, ncirc, breakdown, status_out);
}
// Next advance: pause again after n_steps more accepted steps (unbounded if <= 0).
__global__ void k_set_target(DevArrays d, int ncirc, int n_steps) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncirc) return;
  CircState &s = d.cs[c];
  s.stop_at = (n_steps > 0) ? s.accepted + n_steps : 0x7fffffffffffffffLL;
  if (s.phase == PH_PAUSED) s.phase = PH_TRAN;
}

void launch_set_target_k(cudaStream_t st, const DevArrays &d, int ncirc, int n_steps) {
  k_set_target<<<nblk(ncirc, 128), 128, 0, st>>>(d, ncirc, n_steps);
}

// Solution weights of a Newton solve (DampedNewton::updateWeights_,
// N_NLS_DampedNewton.C:297-340): reltol * max(|x|, |x_curr|) + abstol.
__global__ void k_newton_weights(DevArrays d, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const TranParams &p = *d.tp;
  d.solwt[r] = p.nl_reltol * fmax(fabs(d.x[r]), fabs(d.xcurr[r])) + p.nl_abstol;
}

void launch_newton_weights_k(cudaStream_t st, const DevArrays &d, int n) {
  k_newton_weights<<<nblk(n, 256), 256, 0, st>>>(d, n);
}

void launch_unstall_k(cudaStream_t st, const DevArrays &d, int ncirc) {
  k_unstall<<<nblk(ncirc, 128), 128, 0, st>>>(d, ncirc);
}

}  // namespace xg
