// xg_bsim4.cuh — BSIM 4.8.2 (Xyce level 54) evaluation on the device.
//
// The value path restates updateIntermediateVars4p82_
// (src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4p82.C:3316-7043),
// setupCapacitors_oldDAE and the F/Q assembly of loadDAEFVector,
// setupFVectorVars, loadDAEQVector and updatePrimaryState
// (src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4.C:6881-8431) for the scope
// of xg_bsim4.h.  Partial derivatives are carried forward with the value by
// the dual number D3 (value and d/dvgs, d/dvds, d/dvbs in the device's
// dtype frame): one pass gives the currents, charges and every conductance
// and capacitance the reference computes by hand (gm, gds, gmbs, cggb, ...).
// Where the reference changes a value and keeps its old partials (the
// Vdseff clamps), so does this code.
#pragma once
#include "xg_bsim4.h"

namespace xg {
namespace b4 {

struct D3 {
  double v, g, d, b;  // value; partials along vgs, vds, vbs
  __device__ __forceinline__ D3() : v(0.0), g(0.0), d(0.0), b(0.0) {}
  __device__ __forceinline__ D3(double x) : v(x), g(0.0), d(0.0), b(0.0) {}
  __device__ __forceinline__ D3(double x, double pg, double pd, double pb) : v(x), g(pg), d(pd), b(pb) {}
};
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.v + b.v, a.g + b.g, a.d + b.d, a.b + b.b}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.v - b.v, a.g - b.g, a.d - b.d, a.b - b.b}; }
__device__ __forceinline__ D3 operator-(D3 a) { return D3{-a.v, -a.g, -a.d, -a.b}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
  return D3{a.v * b.v, a.g * b.v + a.v * b.g, a.d * b.v + a.v * b.d, a.b * b.v + a.v * b.b};
}
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
  const double r = 1.0 / b.v, q = a.v * r;
  return D3{q, (a.g - q * b.g) * r, (a.d - q * b.d) * r, (a.b - q * b.b) * r};
}
__device__ __forceinline__ D3 operator+(D3 a, double c) { return D3{a.v + c, a.g, a.d, a.b}; }
__device__ __forceinline__ D3 operator+(double c, D3 a) { return D3{a.v + c, a.g, a.d, a.b}; }
__device__ __forceinline__ D3 operator-(D3 a, double c) { return D3{a.v - c, a.g, a.d, a.b}; }
__device__ __forceinline__ D3 operator-(double c, D3 a) { return D3{c - a.v, -a.g, -a.d, -a.b}; }
__device__ __forceinline__ D3 operator*(D3 a, double c) { return D3{a.v * c, a.g * c, a.d * c, a.b * c}; }
__device__ __forceinline__ D3 operator*(double c, D3 a) { return D3{a.v * c, a.g * c, a.d * c, a.b * c}; }
__device__ __forceinline__ D3 operator/(D3 a, double c) { return D3{a.v / c, a.g / c, a.d / c, a.b / c}; }
__device__ __forceinline__ D3 operator/(double c, D3 a) {
  const double q = c / a.v, s = -q / a.v;
  return D3{q, s * a.g, s * a.d, s * a.b};
}
__device__ __forceinline__ D3 sqrt(D3 a) {
  const double r = ::sqrt(a.v), s = 0.5 / r;
  return D3{r, s * a.g, s * a.d, s * a.b};
}
__device__ __forceinline__ D3 exp(D3 a) {
  const double e = ::exp(a.v);
  return D3{e, e * a.g, e * a.d, e * a.b};
}
__device__ __forceinline__ D3 log(D3 a) {
  const double r = 1.0 / a.v;
  return D3{::log(a.v), r * a.g, r * a.d, r * a.b};
}
__device__ __forceinline__ D3 &operator+=(D3 &a, D3 b) { a = a + b; return a; }
// the double overloads stay visible next to the D3 ones
using ::sqrt;
using ::exp;
using ::log;
__device__ __forceinline__ double rv(const D3 &x) { return x.v; }
__device__ __forceinline__ double rv(const double &x) { return x; }
// value-only assignment: keeps the partials (reference's value clamps)
__device__ __forceinline__ void set_value(D3 &x, double v) { x.v = v; }
// "if (Vds == 0.0)" blocks (N_DEV_MOSFET_B4p82.C:4500-4505, 6620-6625):
// value 0, the Vg and Vb partials 0, the Vd partial kept
__device__ __forceinline__ D3 vds_only(const D3 &x) { return D3{0.0, 0.0, x.d, 0.0}; }

template <class T>
struct Out {
  T Fd, Fs, Fb, qg, qd, qb;
  double von, vdsat;
  int mode;
};

// polyDepletion, N_DEV_MOSFET_B4.C:8819-8855
template <class T>
__device__ __forceinline__ T poly_depletion(double phi, double ngate, double epsgate, double coxe, const T &Vgs) {
  if (ngate > 1.0e18 && ngate < 1.0e25 && rv(Vgs) > phi && epsgate != 0) {
    double T1 = 1.0e6 * kQ * epsgate * ngate / (coxe * coxe);
    T T8 = Vgs - phi;
    T T4 = sqrt(1.0 + 2.0 * T8 / T1);
    T T2 = 2.0 * T8 / (T4 + 1.0);
    T T3 = 0.5 * T2 * T2 / T1;
    T T7 = 1.12 - T3 - 0.05;
    T T6 = sqrt(T7 * T7 + 0.224);
    T T5 = 1.12 - 0.5 * (T7 + T6);
    return Vgs - T5;
  }
  return Vgs;
}

// Junction charge of one bottom/sidewall/gate-sidewall trio
// (N_DEV_MOSFET_B4p82.C:6801-6860).
template <class T>
__device__ __forceinline__ T junction_charge(const T &v, double cz, double czsw, double czswg, double pb, double pbsw,
                         double pbswg, double mj, double mjsw, double mjswg) {
  T q = 0.0;
  // v == 0: zero charge, capacitance cz + czsw + czswg (value 0, slope kept)
  if (rv(v) == 0.0) return (cz + czsw + czswg) * v;
  if (rv(v) < 0.0) {
    if (cz > 0.0) {
      T arg = 1.0 - v / pb;
      T sarg = (mj == 0.5) ? 1.0 / sqrt(arg) : exp(-mj * log(arg));
      q = pb * cz * (1.0 - arg * sarg) / (1.0 - mj);
    }
    if (czsw > 0.0) {
      T arg = 1.0 - v / pbsw;
      T sarg = (mjsw == 0.5) ? 1.0 / sqrt(arg) : exp(-mjsw * log(arg));
      q += pbsw * czsw * (1.0 - arg * sarg) / (1.0 - mjsw);
    }
    if (czswg > 0.0) {
      T arg = 1.0 - v / pbswg;
      T sarg = (mjswg == 0.5) ? 1.0 / sqrt(arg) : exp(-mjswg * log(arg));
      q += pbswg * czswg * (1.0 - arg * sarg) / (1.0 - mjswg);
    }
  } else {
    double T0 = cz + czsw + czswg;
    T T1 = v * (cz * mj / pb + czsw * mjsw / pbsw + czswg * mjswg / pbswg);
    q = v * (T0 + 0.5 * T1);
  }
  return q;
}

// Junction diode current, dioMod 1 (N_DEV_MOSFET_B4p82.C:3362-3385 / 3474-3497).
template <class T>
__device__ __forceinline__ T junction_current(const T &v, double Isat, double Nvtm, double vjmFwd, double IVjmFwd) {
  if (Isat <= 0.0) return kGminB4 * v;
  T T2 = v / Nvtm;
  if (rv(T2) < -kExpThr) return Isat * (kMinExp - 1.0) + kGminB4 * v;
  if (rv(v) <= vjmFwd) return Isat * (exp(T2) - 1.0) + kGminB4 * v;
  double T0 = IVjmFwd / Nvtm;
  return IVjmFwd - Isat + T0 * (v - vjmFwd) + kGminB4 * v;
}

// updateIntermediateVars4p82_ value path (N_DEV_MOSFET_B4p82.C:3316-7043)
// plus setupCapacitors_oldDAE (N_DEV_MOSFET_B4.C:7671-7890) and the F/Q
// assembly of loadDAEFVector / setupFVectorVars / loadDAEQVector /
// updatePrimaryState (N_DEV_MOSFET_B4.C:7899-8431, 7125-7270, 6881-6960).
// dir: the voltage a complex-step evaluation perturbs (0 vgs, 1 vds, 2 vbs;
// -1 for a plain evaluation).
template <class T>
__device__ void core(const B4Model &I, const T &vgs, const T &vds, const T &vbs, Out<T> &o) {
  const T vbd = vbs - vds, vgd = vgs - vds, vgb = vgs - vbs;
  const T vbs_jct = vbs, vbd_jct = vbd;
  // junction diode DC currents (dioMod 1); trap-assisted tunnelling terms
  // vanish (JTSS = JTSD = JTSSWS = ... = 0 in the restated scope)
  const T cbs = junction_current(vbs_jct, I.SourceSatCurrent, I.vtm * I.NJS, I.vjsmFwd, I.IVjsmFwd);
  const T cbd = junction_current(vbd_jct, I.DrainSatCurrent, I.vtm * I.NJD, I.vjdmFwd, I.IVjdmFwd);

  int mode;
  T Vds, Vgs, Vbs;
  if (rv(vds) >= 0.0) { mode = 1; Vds = vds; Vgs = vgs; Vbs = vbs; }
  else { mode = -1; Vds = -vds; Vgs = vgd; Vbs = vbd; }
  o.mode = mode;
  const double epsrox = I.epsrox, toxe = I.toxe, epssub = kEpsSi;

  T T0, T1, T2, T3, T4, T5, T6, T7, T8, T9, T10, T11, T12;
  // Vbseff (:3757-3781)
  T0 = Vbs - I.vbsc - 0.001;
  T1 = sqrt(T0 * T0 - 0.004 * I.vbsc);
  T Vbseff;
  if (rv(T0) >= 0.0) Vbseff = I.vbsc + 0.5 * (T0 + T1);
  else { T2 = -0.002 / (T1 - T0); Vbseff = I.vbsc * (1.0 + T2); }
  {
    double T9b = 0.95 * I.phi;
    T0 = T9b - Vbseff - 0.001;
    T1 = sqrt(T0 * T0 + 0.004 * T9b);
    Vbseff = T9b - 0.5 * (T0 + T1);
  }
  const T Phis = I.phi - Vbseff;
  const T sqrtPhis = sqrt(Phis);
  const T Xdep = I.Xdep0 * sqrtPhis / I.sqrtPhi;
  const double Leff = I.leff, Vtm = I.vtm;
  // Vth (:3797-3960)
  T3 = sqrt(Xdep);
  const double V0 = I.vbi - I.phi;
  T0 = I.dvt2 * Vbseff;
  if (rv(T0) >= -0.5) T1 = 1.0 + T0;
  else { T4 = 1.0 / (3.0 + 8.0 * T0); T1 = (1.0 + 3.0 * T0) * T4; }
  const T lt1 = I.factor1 * T3 * T1;
  T0 = I.dvt2w * Vbseff;
  if (rv(T0) >= -0.5) T1 = 1.0 + T0;
  else { T4 = 1.0 / (3.0 + 8.0 * T0); T1 = (1.0 + 3.0 * T0) * T4; }
  const T ltw = I.factor1 * T3 * T1;
  T Theta0;
  T0 = I.dvt1 * Leff / lt1;
  if (rv(T0) < kExpThr) {
    T1 = exp(T0); T2 = T1 - 1.0; T3 = T2 * T2; T4 = T3 + 2.0 * T1 * kMinExp;
    Theta0 = T1 / T4;
  } else {
    Theta0 = 1.0 / (kMaxExp - 2.0);
  }
  const T Delt_vth = I.dvt0 * Theta0 * V0;
  T0 = I.dvt1w * I.weff * Leff / ltw;
  if (rv(T0) < kExpThr) {
    T1 = exp(T0); T2 = T1 - 1.0; T3 = T2 * T2; T4 = T3 + 2.0 * T1 * kMinExp;
    T5 = T1 / T4;
  } else {
    T5 = 1.0 / (kMaxExp - 2.0);
  }
  T0 = I.dvt0w * T5;
  T2 = T0 * V0;
  // TempRatio = temp / tnom - 1 = 0 at the restated temperature
  T0 = sqrt(1.0 + I.lpe0 / Leff);
  T1 = I.k1ox * (T0 - 1.0) * I.sqrtPhi;
  const double Vth_NarrowW = toxe * I.phi / (I.weff + I.w0);
  T3 = I.eta0 + I.etab * Vbseff;
  if (rv(T3) < 1.0e-4) {
    T9 = 1.0 / (3.0 - 2.0e4 * T3);
    T3 = (2.0e-4 - T3) * T9;
  }
  const T dDIBL_Sft_dVd = T3 * I.theta0vb0;
  const T DIBL_Sft = dDIBL_Sft_dVd * Vds;
  const double Lpe_Vb = sqrt(1.0 + I.lpeb / Leff);
  T Vth = I.dtype * I.vth0 + (I.k1ox * sqrtPhis - I.k1 * I.sqrtPhi) * Lpe_Vb - I.k2ox * Vbseff -
          Delt_vth - T2 + (I.k3 + I.k3b * Vbseff) * Vth_NarrowW + T1 - DIBL_Sft;
  // n (:3891-3915)
  T tmp1 = epssub / Xdep;
  T tmp2 = I.nfactor * tmp1;
  T tmp3 = I.cdsc + I.cdscb * Vbseff + I.cdscd * Vds;
  T tmp4 = (tmp2 + tmp3 * Theta0 + I.cit) / I.coxe;
  T n;
  if (rv(tmp4) >= -0.5) n = 1.0 + tmp4;
  else { T0 = 1.0 / (3.0 + 8.0 * tmp4); n = (1.0 + 3.0 * tmp4) * T0; }
  // pocket implant (:3917-3944), tempMod < 2
  if (I.dvtp0 > 0.0) {
    T0 = -I.dvtp1 * Vds;
    if (rv(T0) < -kExpThr) T2 = kMinExp;
    else T2 = exp(T0);
    T3 = Leff + I.dvtp0 * (1.0 + T2);
    T4 = Vtm * log(Leff / T3);
    Vth = Vth - n * T4;
  }
  // DITS_Sft2 vanishes (DVTP4 = 0)
  o.von = rv(Vth);
  // poly depletion (:3962-3985)
  const double T0pd = I.vfb + I.phi;
  const T vgs_eff = poly_depletion(T0pd, I.ngate, kEpsSi, I.coxe, vgs);
  const T vgd_eff = poly_depletion(T0pd, I.ngate, kEpsSi, I.coxe, vgd);
  const T Vgs_eff = (mode > 0) ? vgs_eff : vgd_eff;
  const T Vgst = Vgs_eff - Vth;
  // Vgsteff (:4008-4070)
  T0 = n * Vtm;
  T1 = I.mstar * Vgst;
  T2 = T1 / T0;
  if (rv(T2) > kExpThr) T10 = T1;
  else if (rv(T2) < -kExpThr) T10 = Vtm * log(1.0 + kMinExp) * n;
  else { T T3e = exp(T2); T10 = n * (Vtm * log(1.0 + T3e)); }
  T1 = I.voffcbn - (1.0 - I.mstar) * Vgst;
  T2 = T1 / T0;
  if (rv(T2) < -kExpThr) T9 = I.mstar + (I.coxe * kMinExp / I.cdep0) * n;
  else if (rv(T2) > kExpThr) T9 = I.mstar + (I.coxe * kMaxExp / I.cdep0) * n;
  else T9 = I.mstar + n * ((I.coxe / I.cdep0) * exp(T2));
  const T Vgsteff = T10 / T9;
  // Weff, Rds (:4072-4115)
  T9 = sqrtPhis - I.sqrtPhi;
  T Weff = I.weff - 2.0 * (I.dwg * Vgsteff + I.dwb * T9);
  if (rv(Weff) < 2.0e-8) {
    T0 = 1.0 / (6.0e-8 - 2.0 * Weff);
    Weff = 2.0e-8 * (4.0e-8 - Weff) * T0;
  }
  // rdsMod = 0: Rds from RDSW (:4095-4115)
  T0 = 1.0 + I.prwg * Vgsteff;
  T1 = I.prwb * T9;
  T2 = 1.0 / T0 + T1;
  T3 = T2 + sqrt(T2 * T2 + 0.01);
  const T Rds = I.rdswmin + T3 * (I.rds0 * 0.5);
  // Abulk (:4117-4186)
  T9 = 0.5 * I.k1ox * Lpe_Vb / sqrtPhis;
  T1 = T9 + I.k2ox - I.k3b * Vth_NarrowW;
  T9 = sqrt(I.xj * Xdep);
  tmp1 = Leff + 2.0 * T9;
  T5 = Leff / tmp1;
  tmp2 = I.a0 * T5;
  const double tmp3d = I.weff + I.b1;
  const double tmp4d = I.b0 / tmp3d;
  T2 = tmp2 + tmp4d;
  T6 = T5 * T5;
  T7 = T5 * T6;
  T Abulk0 = 1.0 + T1 * T2;
  T8 = I.ags * I.a0 * T7;
  T Abulk = Abulk0 + (-T1 * T8) * Vgsteff;
  if (rv(Abulk0) < 0.1) { T9 = 1.0 / (3.0 - 20.0 * Abulk0); Abulk0 = (0.2 - Abulk0) * T9; }
  if (rv(Abulk) < 0.1) { T9 = 1.0 / (3.0 - 20.0 * Abulk); Abulk = (0.2 - Abulk) * T9; }
  T2 = I.keta * Vbseff;
  if (rv(T2) >= -0.9) T0 = 1.0 / (1.0 + T2);
  else { T1 = 1.0 / (0.8 + T2); T0 = (17.0 + 20.0 * T2) * T1; }
  Abulk = Abulk * T0;
  Abulk0 = Abulk0 * T0;
  // mobility, mobMod 0 (:4190-4212)
  T0 = Vgsteff + Vth + Vth;
  T2 = I.ua + I.uc * Vbseff;
  T3 = T0 / toxe;
  T12 = sqrt(Vth * Vth + 0.0001);
  T9 = 1.0 / (Vgsteff + 2.0 * T12);
  T10 = T9 * toxe;
  T8 = I.ud * T10 * T10 * Vth;
  T6 = T8 * Vth;
  T5 = T3 * (T2 + I.ub * T3) + T6;
  T Denomi;
  if (rv(T5) >= -0.8) Denomi = 1.0 + T5;
  else { T9 = 1.0 / (7.0 + 10.0 * T5); Denomi = (0.6 + T5) * T9; }
  const T ueff = I.u0temp / Denomi;
  const T WVCox = Weff * I.vsattemp * I.coxe;
  const T WVCoxRds = WVCox * Rds;
  T Esat = 2.0 * I.vsattemp / ueff;
  T EsatL = Esat * Leff;
  // Lambda (:4338-4357)
  T Lambda;
  if (I.a1 == 0.0) Lambda = I.a2;
  else if (I.a1 > 0.0) {
    double T0d = 1.0 - I.a2;
    T1 = T0d - I.a1 * Vgsteff - 0.0001;
    T2 = sqrt(T1 * T1 + 0.0004 * T0d);
    Lambda = I.a2 + T0d - 0.5 * (T1 + T2);
  } else {
    T1 = I.a2 + I.a1 * Vgsteff - 0.0001;
    T2 = sqrt(T1 * T1 + 0.0004 * I.a2);
    Lambda = 0.5 * (T1 + T2);
  }
  const T Vgst2Vtm = Vgsteff + 2.0 * Vtm;
  // Vdsat (:4402-4465)
  T Vdsat;
  if (rv(Rds) == 0.0 && rv(Lambda) == 1.0) {
    T0 = 1.0 / (Abulk * EsatL + Vgst2Vtm);
    T3 = EsatL * Vgst2Vtm;
    Vdsat = T3 * T0;
  } else {
    T9 = Abulk * WVCoxRds;
    T7 = Vgst2Vtm * T9;
    T6 = Vgst2Vtm * WVCoxRds;
    T0 = 2.0 * Abulk * (T9 - 1.0 + 1.0 / Lambda);
    T1 = Vgst2Vtm * (2.0 / Lambda - 1.0) + Abulk * EsatL + 3.0 * T7;
    T2 = Vgst2Vtm * (EsatL + 2.0 * T6);
    T3 = sqrt(T1 * T1 - 2.0 * T0 * T2);
    Vdsat = (T1 - T3) / T0;
  }
  o.vdsat = rv(Vdsat);
  // Vdseff (:4467-4510)
  T1 = Vdsat - Vds - I.delta;
  T2 = sqrt(T1 * T1 + 4.0 * I.delta * Vdsat);
  T Vdseff;
  if (rv(T1) >= 0.0) Vdseff = Vdsat - 0.5 * (T1 + T2);
  else {
    T4 = (2.0 * I.delta) / (T2 - T1);
    T5 = 1.0 - T4;
    Vdseff = Vdsat * T5;
  }
  if (rv(Vds) == 0.0) Vdseff = vds_only(Vdseff);
  if (rv(Vdseff) > rv(Vds)) set_value(Vdseff, rv(Vds));
  const T diffVds = Vds - Vdseff;
  // (LAMBDA / VTL not given: no velocity-saturation corrections)
  // Vasat (:4561-4590)
  T tmp4v = 1.0 - 0.5 * Abulk * Vdsat / Vgst2Vtm;
  T9 = WVCoxRds * Vgsteff;
  T0 = EsatL + Vdsat + 2.0 * T9 * tmp4v;
  T9 = WVCoxRds * Abulk;
  T1 = 2.0 / Lambda - 1.0 + T9;
  const T Vasat = T0 / T1;
  // Coxeff for the drain current (:4592-4610)
  {
    double tmp1d = I.vtfbphi2, tmp2d = 2.0e8 * I.toxp;
    T0 = (Vgsteff + tmp1d) / tmp2d;
  }
  T tmp3c = exp(I.bdos * 0.7 * log(T0));
  T1 = 1.0 + tmp3c;
  T Tcen = I.ados * 1.9e-9 / T1;
  T Coxeff = epssub * I.coxp / (epssub + I.coxp * Tcen);
  const T CoxeffWovL = Coxeff * Weff / Leff;
  const T beta = ueff * CoxeffWovL;
  const T AbovVgst2Vtm = Abulk / Vgst2Vtm;
  T0 = 1.0 - 0.5 * Vdseff * AbovVgst2Vtm;
  const T fgche1 = Vgsteff * T0;
  T9 = Vdseff / EsatL;
  const T fgche2 = 1.0 + T9;
  const T gche = beta * fgche1 / fgche2;
  T0 = 1.0 + gche * Rds;
  const T Idl = gche / T0;
  // FP, PvagTerm (:4661-4695)
  T FP;
  if (I.fprout <= 0.0) FP = 1.0;
  else { T9 = I.fprout * sqrt(Leff) / Vgst2Vtm; FP = 1.0 / (1.0 + T9); }
  T8 = I.pvag / EsatL;
  T9 = T8 * Vgsteff;
  T PvagTerm;
  if (rv(T9) > -0.9) PvagTerm = 1.0 + T9;
  else { T4 = 1.0 / (17.0 + 20.0 * T9); PvagTerm = (0.8 + T9) * T4; }
  // VACLM (:4697-4730)
  T Cclm, VACLM;
  if (I.pclm > kMinExp && rv(diffVds) > 1.0e-10) {
    T0 = 1.0 + Rds * Idl;
    T2 = Vdsat / Esat;
    T1 = Leff + T2;
    Cclm = FP * PvagTerm * T0 * T1 / (I.pclm * I.litl);
    VACLM = Cclm * diffVds;
  } else {
    VACLM = kMaxExp;
    Cclm = kMaxExp;
  }
  // VADIBL (:4732-4780)
  T VADIBL;
  if (I.thetaRout > kMinExp) {
    T8 = Abulk * Vdsat;
    T0 = Vgst2Vtm * T8;
    T1 = Vgst2Vtm + T8;
    VADIBL = (Vgst2Vtm - T0 / T1) / I.thetaRout;
    T7 = I.pdiblb * Vbseff;
    if (rv(T7) >= -0.9) { T3 = 1.0 / (1.0 + T7); VADIBL = VADIBL * T3; }
    else { T4 = 1.0 / (0.8 + T7); T3 = (17.0 + 20.0 * T7) * T4; VADIBL = VADIBL * T3; }
    VADIBL = VADIBL * PvagTerm;
  } else {
    VADIBL = kMaxExp;
  }
  const T Va = Vasat + VACLM;
  // VADITS (:4786-4810)
  T0 = I.pditsd * Vds;
  if (rv(T0) > kExpThr) T1 = kMaxExp;
  else T1 = exp(T0);
  T VADITS;
  if (I.pdits > kMinExp) {
    double T2d = 1.0 + I.pditsl * Leff;
    VADITS = (1.0 + T2d * T1) / I.pdits;
    VADITS = VADITS * FP;
  } else {
    VADITS = kMaxExp;
  }
  // VASCBE (:4812-4835)
  T VASCBE;
  if (I.pscbe2 > 0.0 && I.pscbe1 >= 0.0) {
    if (rv(diffVds) > I.pscbe1 * I.litl / kExpThr) {
      T0 = I.pscbe1 * I.litl / diffVds;
      VASCBE = Leff * exp(T0) / I.pscbe2;
    } else {
      VASCBE = kMaxExp * Leff / I.pscbe2;
    }
  } else {
    VASCBE = kMaxExp;
  }
  // Ids (:4837-4880)
  T9 = diffVds / VADIBL;
  T0 = 1.0 + T9;
  T Idsa = Idl * T0;
  T9 = diffVds / VADITS;
  T0 = 1.0 + T9;
  Idsa = Idsa * T0;
  T0 = log(Va / Vasat);
  T1 = T0 / Cclm;
  T9 = 1.0 + T1;
  Idsa = Idsa * T9;
  // Isub (:4882-4925)
  T Isub = 0.0;
  {
    double tmp = I.alpha0 + I.alpha1 * Leff;
    if (!(tmp <= 0.0 || I.beta0 <= 0.0)) {
      double T2d = tmp / Leff;
      if (rv(diffVds) > I.beta0 / kExpThr) {
        T0 = -I.beta0 / diffVds;
        T1 = T2d * diffVds * exp(T0);
      } else {
        T1 = (T2d * kMinExp) * diffVds;
      }
      Isub = T1 * (Idsa * Vdseff);
    }
  }
  T9 = diffVds / VASCBE;
  T0 = 1.0 + T9;
  const T Ids = Idsa * T0;
  const T cdrain = Ids * Vdseff;
  // GIDL / GISL, gidlMod 0 (:5135-5250)
  T Igidl = 0.0, Igisl = 0.0;
  {
    const double T0g = 3.0 * toxe;
    T1 = (vds - vgs_eff - I.egidl) / T0g;
    if (!(I.agidl <= 0.0 || I.bgidl <= 0.0 || rv(T1) <= 0.0 || I.cgidl <= 0.0 || rv(vbd) > 0.0)) {
      T2 = I.bgidl / T1;
      if (rv(T2) < 100.0) Igidl = I.agidl * I.weffCJ * T1 * exp(-T2);
      else Igidl = (I.agidl * I.weffCJ * 3.720075976e-44) * T1;
      T4 = vbd * vbd;
      T5 = -vbd * T4;
      T6 = I.cgidl + T5;
      T7 = T5 / T6;
      Igidl = Igidl * T7;
    }
    T1 = (-vds - vgd_eff - I.egisl) / T0g;
    if (!(I.agisl <= 0.0 || I.bgisl <= 0.0 || rv(T1) <= 0.0 || I.cgisl <= 0.0 || rv(vbs) > 0.0)) {
      T2 = I.bgisl / T1;
      if (rv(T2) < 100.0) Igisl = I.agisl * I.weffCJ * T1 * exp(-T2);
      else Igisl = (I.agisl * I.weffCJ * 3.720075976e-44) * T1;
      T4 = vbs * vbs;
      T5 = -vbs * T4;
      T6 = I.cgisl + T5;
      T7 = T5 / T6;
      Igisl = Igisl * T7;
    }
  }
  // ---- charges, capMod 2 (:5844-5855, 6146-6170, 6458-6760) ----
  T VbseffCV;
  if (rv(Vbseff) < 0.0) VbseffCV = Vbseff;
  else VbseffCV = I.phi - Phis;
  const double CoxWL = I.coxe * I.weffCV * I.leffCV;  // nf = 1
  // Vgsteff for C-V, cvchargeMod 0 (:6171-6200)
  const T noff = n * I.noff;
  T0 = Vtm * noff;
  const T VgstNVt = (Vgst - I.voffcv) / T0;
  T VgsteffCV;
  if (rv(VgstNVt) > kExpThr) VgsteffCV = Vgst - I.voffcv;
  else if (rv(VgstNVt) < -kExpThr) VgsteffCV = T0 * log(1.0 + kMinExp);
  else VgsteffCV = T0 * log(1.0 + exp(VgstNVt));
  // capMod 2
  T qgate, qbulk, qsrc;
  {
    const T &Vg = VgsteffCV;
    T V3 = I.vfbzb - Vgs_eff + VbseffCV - kDelta3;
    if (I.vfbzb <= 0.0) T0 = sqrt(V3 * V3 - 4.0 * kDelta3 * I.vfbzb);
    else T0 = sqrt(V3 * V3 + 4.0 * kDelta3 * I.vfbzb);
    const T Vfbeff = I.vfbzb - 0.5 * (V3 + T0);
    const double Cox = I.coxp;
    double Tox = 1.0e8 * I.toxp;
    T0 = (Vgs_eff - VbseffCV - I.vfbzb) / Tox;
    T tmp = T0 * I.acde;
    T TcenC;
    if (-kExpThr < rv(tmp) && rv(tmp) < kExpThr) TcenC = I.ldeb * exp(tmp);
    else if (rv(tmp) <= -kExpThr) TcenC = I.ldeb * kMinExp;
    else TcenC = I.ldeb * kMaxExp;
    const double LINK = 1.0e-3 * I.toxp;
    V3 = I.ldeb - TcenC - LINK;
    T V4 = sqrt(V3 * V3 + 4.0 * LINK * I.ldeb);
    TcenC = I.ldeb - 0.5 * (V3 + V4);
    T Ccen = epssub / TcenC;
    T2 = Cox / (Cox + Ccen);
    T CoxeffC = T2 * Ccen;
    T CoxWLcen = CoxWL * CoxeffC / I.coxe;
    const T Qac0 = CoxWLcen * (Vfbeff - I.vfbzb);
    T0 = 0.5 * I.k1ox;
    T3 = Vgs_eff - Vfbeff - VbseffCV - Vg;
    if (I.k1ox == 0.0) T1 = 0.0;
    else if (rv(T3) < 0.0) T1 = T0 + T3 / I.k1ox;
    else T1 = sqrt(T0 * T0 + T3);
    const T Qsub0 = CoxWLcen * I.k1ox * (T1 - T0);
    double DenomiC, T0c;
    if (I.k1ox <= 0.0) { DenomiC = 0.25 * I.moin * Vtm; T0c = 0.5 * I.sqrtPhi; }
    else { DenomiC = I.moin * Vtm * I.k1ox * I.k1ox; T0c = I.k1ox * I.sqrtPhi; }
    T1 = 2.0 * T0c + Vg;
    const T DeltaPhi = Vtm * log(1.0 + T1 * Vg / DenomiC);
    T0 = Vg - DeltaPhi - 0.001;
    T1 = sqrt(T0 * T0 + Vg * 0.004);
    const T VgDP = 0.5 * (T0 + T1);
    Tox += Tox;
    T0 = (Vg + I.vtfbphi2) / Tox;
    tmp = exp(I.bdos * 0.7 * log(T0));
    T1 = 1.0 + tmp;
    TcenC = I.ados * 1.9e-9 / T1;
    Ccen = epssub / TcenC;
    T0 = Cox / (Cox + Ccen);
    CoxeffC = T0 * Ccen;
    CoxWLcen = CoxWL * CoxeffC / I.coxe;
    const T AbulkCV = Abulk0 * I.abulkCVfactor;
    const T VdsatCV = VgDP / AbulkCV;
    T0 = VdsatCV - Vds - kDelta4;
    T1 = sqrt(T0 * T0 + 4.0 * kDelta4 * VdsatCV);
    T VdseffCV;
    if (rv(T0) >= 0.0) VdseffCV = VdsatCV - 0.5 * (T0 + T1);
    else {
      T3 = (kDelta4 + kDelta4) / (T1 - T0);
      T4 = 1.0 - T3;
      VdseffCV = VdsatCV * T4;
    }
    if (rv(Vds) == 0.0) VdseffCV = vds_only(VdseffCV);
    T0 = AbulkCV * VdseffCV;
    T1 = VgDP;
    T2 = 12.0 * (T1 - 0.5 * T0 + 1.0e-20);
    T3 = T0 / T2;
    qgate = CoxWLcen * (T1 - T0 * (0.5 - T3));
    T7 = 1.0 - AbulkCV;
    qbulk = CoxWLcen * T7 * (0.5 * VdseffCV - T0 * VdseffCV / T2);
    if (I.xpart > 0.5) {
      qsrc = -CoxWLcen * (T1 / 2.0 + T0 / 4.0 - 0.5 * T0 * T0 / T2);
    } else if (I.xpart < 0.5) {
      T2 = T2 / 12.0;
      T3 = 0.5 * CoxWLcen / (T2 * T2);
      T4 = T1 * (2.0 * T0 * T0 / 3.0 + T1 * (T1 - 4.0 * T0 / 3.0)) - 2.0 * T0 * T0 * T0 / 15.0;
      qsrc = -T3 * T4;
    } else {
      qsrc = -0.5 * qgate;
    }
    qgate = qgate + Qac0 + Qsub0 - qbulk;
    qbulk = qbulk - (Qac0 + Qsub0);
  }
  T qdrn = -(qgate + qbulk + qsrc);
  // junction charges (:6784-6890)
  const T qbs = junction_charge(vbs_jct, I.czbs, I.czbssw, I.czbsswg, I.PhiBS, I.PhiBSWS, I.PhiBSWGS,
                                I.MJS, I.MJSWS, I.MJSWGS);
  const T qbd = junction_charge(vbd_jct, I.czbd, I.czbdsw, I.czbdswg, I.PhiBD, I.PhiBSWD, I.PhiBSWGD,
                                I.MJD, I.MJSWD, I.MJSWGD);
  // overlap charges, capMod 1/2 (:6975-6998)
  T qgdo, qgso;
  {
    T0 = vgd + kDelta1;
    T1 = sqrt(T0 * T0 + 4.0 * kDelta1);
    T2 = 0.5 * (T0 - T1);
    double T3d = I.weffCV * I.cgdl;
    T4 = sqrt(1.0 - 4.0 * T2 / I.ckappad);
    qgdo = (I.cgdo + T3d) * vgd - T3d * (T2 + 0.5 * I.ckappad * (T4 - 1.0));
    T0 = vgs + kDelta1;
    T1 = sqrt(T0 * T0 + 4.0 * kDelta1);
    T2 = 0.5 * (T0 - T1);
    T3d = I.weffCV * I.cgsl;
    T4 = sqrt(1.0 - 4.0 * T2 / I.ckappas);
    qgso = (I.cgso + T3d) * vgs - T3d * (T2 + 0.5 * I.ckappas * (T4 - 1.0));
  }
  // setupCapacitors_oldDAE, trnqsMod 0, rgateMod 0 (N_DEV_MOSFET_B4.C:7681-7700, 7790-7810)
  const T qgb = I.cgbo * vgb;
  if (mode > 0) {
    qdrn = qdrn - qgdo;
    qgate = qgate + qgdo + qgso + qgb;
    qbulk = qbulk - qgb;
    qsrc = -(qgate + qbulk + qdrn);
  } else {
    qsrc = qdrn - qgso;
    qgate = qgate + qgdo + qgso + qgb;
    qbulk = qbulk - qgb;
    qdrn = -(qgate + qbulk + qsrc);
  }
  // updatePrimaryState: qg, qd, qb (N_DEV_MOSFET_B4.C:6921-6930)
  o.qg = qgate;
  o.qd = qdrn - qbd;
  o.qb = qbulk + qbd + qbs;
  // setupFVectorVars + loadDAEFVector (N_DEV_MOSFET_B4.C:8101-8431, 7899-7940)
  const double dt = I.dtype;
  T ceqdrn, ceqbd, ceqbs;
  const T csub = Isub;
  if (mode >= 0) {
    ceqdrn = dt * cdrain;
    ceqbd = dt * (csub + Igidl);
    ceqbs = dt * Igisl;
  } else {
    ceqdrn = -dt * cdrain;
    ceqbs = dt * (csub + Igisl);
    ceqbd = dt * Igidl;
  }
  const T ceqjs = dt * cbs, ceqjd = dt * cbd;
  o.Fd = -(ceqjd - ceqbd - ceqdrn);
  o.Fb = -(ceqbd + ceqbs - ceqjd - ceqjs);
  o.Fs = -(ceqdrn - ceqbs + ceqjs);
}

}  // namespace b4
}  // namespace xg
