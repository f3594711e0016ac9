// xg_bsim4.cu — BSIM 4.8.2 (Xyce level 54) evaluation + stamp kernel (sm_103a).
//
// One thread per instance, SoA node planes, cards from a deduplicated table.
// Per instance: the SPICE limiters of updateIntermediateVars4p82_
// (src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4p82.C:3016-3240), one
// dual-number evaluation (xg_bsim4.cuh), then the stamps of
// Master::updateState / loadDAEVectors / loadDAEMatrices
// (src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4.C:10540-11687) written to
// plane-major slots that the row / entry gathers of xg_kernels.cu sum.
// Slots match the MOSFET level-1 layout: F[D,S,B]  Q[G,B,D,S]  L[G,B,D,S]
// M[4x4 over D,G,S,B].  Store planes: vbd vbs vgs vds von; state: qg qd qb.
#include <cuda_runtime.h>

#include "xg_bsim4.cuh"
#include "xg_internal.h"
#include "xg_models.cuh"

namespace xg {

__global__ void __launch_bounds__(128) k_bsim4(DevArrays d, int nb, int sto_base, int sta_base, int combined,
                                               int masked, int it_arg, int flags_arg, int slotF, int slotQ,
                                               int slotL, int slotM) {
  using b4::D3;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int c = __ldg(d.b4_circ + i);
  int iter = it_arg;
  bool dcop = flags_arg & XG_FLAG_DCOP, initJct = flags_arg & XG_FLAG_INITJCT;
  double qs = 1.0, fs = 1.0;
  if (masked) {
    const CircState &s = d.cs[c];
    if (!(s.phase == PH_DC || s.phase == PH_TRAN)) return;
    iter = s.iter;
    dcop = s.phase == PH_DC;
    initJct = dcop && s.init_jct && iter == 0;
    qs = s.qscale; fs = s.fscale;
  }
  const b4::B4Model &I = d.b4_models[__ldg(d.b4_model + i)];
  const int nD = __ldg(d.b4_node + i), nG = __ldg(d.b4_node + nb + i);
  const int nS = __ldg(d.b4_node + 2 * nb + i), nB = __ldg(d.b4_node + 3 * nb + i);
  const double *x = d.x;
  const double Vd = nD >= 0 ? x[nD] : 0.0, Vg = nG >= 0 ? x[nG] : 0.0;
  const double Vs = nS >= 0 ? x[nS] : 0.0, Vb = nB >= 0 ? x[nB] : 0.0;
  const double dt = I.dtype, M = I.M;
  double *sto_n = d.sto_next + sto_base;
  const double *sto_c = d.sto_curr + sto_base;
  // ---- limiting (updateIntermediateVars4p82_, :3016-3240) ----
  double vgs = dt * (Vg - Vs), vds = dt * (Vd - Vs), vbs = dt * (Vb - Vs);
  double vbd = vbs - vds, vgd = vgs - vds;
  const double vgs_o = vgs, vds_o = vds, vbs_o = vbs;
  int origFlag = 1;
  if (initJct) {
    vds = 0.1; vgs = dt * I.vth0 + 0.1; vbs = 0.0;
    vbd = vbs - vds; vgd = vgs - vds;
    origFlag = 0;
  }
  double vbd_old, vbs_old, vgs_old, vds_old;
  if (iter == 0 && dcop) {
    vbd_old = vbd; vbs_old = vbs; vgs_old = vgs; vds_old = vds;
  } else {
    const double *h = (iter == 0) ? sto_c : sto_n;
    vbd_old = h[i]; vbs_old = h[nb + i]; vgs_old = h[2 * nb + i]; vds_old = h[3 * nb + i];
  }
  // von: the instance's last evaluation (an instance member in the reference)
  const double von_prev = sto_n[4 * nb + i];
  const double vgd_old = vgs_old - vds_old;
  if (!initJct) {
    int Check = 0;
    if (vds_old >= 0.0) {
      vgs = fetlim_d(vgs, vgs_old, von_prev);
      vds = vgs - vgd;
      vds = limvds_d(vds, vds_old);
      vgd = vgs - vds;
    } else {
      vgd = fetlim_d(vgd, vgd_old, von_prev);
      vds = vgs - vgd;
      vds = -limvds_d(-vds, -vds_old);
      vgs = vgd + vds;
    }
    if (vds >= 0.0) {
      vbs = pnjlim_d(vbs, vbs_old, b4::kVt0, I.vcrit, Check);
      vbd = vbs - vds;
    } else {
      vbd = pnjlim_d(vbd, vbd_old, b4::kVt0, I.vcrit, Check);
      vbs = vbd + vds;
    }
  }
  vbd = vbs - vds;
  const double eps = 2.220446049250313e-16;
  if (fabs(vbs_o - vbs) > eps || fabs(vgs_o - vgs) > eps || fabs(vds_o - vds) > eps) origFlag = 0;
  if (!origFlag && masked && dcop) atomicOr(&d.cs[c].limited, 1);
  // ---- evaluation with partials along vgs, vds, vbs ----
  b4::Out<D3> o;
  b4::core(I, D3(vgs, 1.0, 0.0, 0.0), D3(vds, 0.0, 1.0, 0.0), D3(vbs, 0.0, 0.0, 1.0), o);
  // ---- store / state (Master::updateState, N_DEV_MOSFET_B4.C:10540-10600) ----
  sto_n[i] = vbd; sto_n[nb + i] = vbs; sto_n[2 * nb + i] = vgs; sto_n[3 * nb + i] = vds;
  sto_n[4 * nb + i] = o.von;
  double *sta_n = d.sta_next + sta_base;
  sta_n[i] = o.qg.v; sta_n[nb + i] = o.qd.v; sta_n[2 * nb + i] = o.qb.v;
  // ---- F, Q slots ----
  double *sF = d.sF + slotF, *sQ = d.sQ + slotQ;
  sF[i] = o.Fd.v * M; sF[nb + i] = o.Fs.v * M; sF[2 * nb + i] = o.Fb.v * M;
  const D3 qS = -(o.qg + o.qd + o.qb);
  sQ[i] = dt * o.qg.v * M; sQ[nb + i] = dt * o.qb.v * M; sQ[2 * nb + i] = dt * o.qd.v * M;
  sQ[3 * nb + i] = dt * qS.v * M;
  // ---- limiter vectors (dFdxdVp, dQdxdVp): J . (limited - original) ----
  double lf[4] = {0, 0, 0, 0}, lq[4] = {0, 0, 0, 0};  // over G, B, D, S
  if (!origFlag) {
    const double dg = vgs - vgs_o, dd = vds - vds_o, db = vbs - vbs_o;
    auto jd = [&](const D3 &y) { return y.g * dg + y.d * dd + y.b * db; };
    lf[1] = jd(o.Fb) * M; lf[2] = jd(o.Fd) * M; lf[3] = jd(o.Fs) * M;
    // the charge limiter terms carry no dtype (N_DEV_MOSFET_B4.C:7215-7232)
    lq[0] = jd(o.qg) * M; lq[1] = jd(o.qb) * M; lq[2] = jd(o.qd) * M; lq[3] = jd(qS) * M;
  }
  double *sL = d.sL + slotL;
  if (combined) {
#pragma unroll
    for (int k = 0; k < 4; ++k) sL[k * nb + i] = fs * lf[k] + qs * lq[k];
  } else {
    double *sL2 = d.sL2 + slotL;
#pragma unroll
    for (int k = 0; k < 4; ++k) { sL[k * nb + i] = lf[k]; sL2[k * nb + i] = lq[k]; }
  }
  // ---- Jacobian: rows/cols (D,G,S,B) = (0,1,2,3); columns G <- vgs, D <- vds,
  // B <- vbs, S <- -(sum); dFdx carries dtype, dQdx does not (dtype^2 = 1) ----
  double f[16], q[16];
  auto rowF = [&](int r, const D3 &y) {
    f[4 * r + 0] = dt * y.d * M; f[4 * r + 1] = dt * y.g * M; f[4 * r + 3] = dt * y.b * M;
    f[4 * r + 2] = -dt * (y.g + y.d + y.b) * M;
  };
  auto rowQ = [&](int r, const D3 &y) {
    q[4 * r + 0] = y.d * M; q[4 * r + 1] = y.g * M; q[4 * r + 3] = y.b * M;
    q[4 * r + 2] = -(y.g + y.d + y.b) * M;
  };
  rowF(0, o.Fd); rowF(2, o.Fs); rowF(3, o.Fb);
  f[4] = f[5] = f[6] = f[7] = 0.0;  // the gate carries no conduction current
  rowQ(0, o.qd); rowQ(1, o.qg); rowQ(2, qS); rowQ(3, o.qb);
  double *sM = d.sM + slotM;
  if (combined) {
#pragma unroll
    for (int k = 0; k < 16; ++k) sM[k * nb + i] = fs * f[k] + qs * q[k];
  } else {
    double *sM2 = d.sM2 + slotM;
#pragma unroll
    for (int k = 0; k < 16; ++k) { sM[k * nb + i] = f[k]; sM2[k * nb + i] = q[k]; }
  }
}

void launch_bsim4_k(cudaStream_t st, const DevArrays &d, int nb, int sto_base, int sta_base, int combined,
                    int masked, int it, int flags, int sF, int sQ, int sL, int sM) {
  if (nb > 0)
    k_bsim4<<<(nb + 127) / 128, 128, 0, st>>>(d, nb, sto_base, sta_base, combined, masked, it, flags, sF, sQ,
                                               sL, sM);
}

}  // namespace xg
