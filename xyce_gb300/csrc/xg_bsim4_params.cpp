// xg_bsim4_params.cpp — host set-up of BSIM 4.8.2 (Xyce level 54) instances.
//
// Restates, for the scope of xg_bsim4.h (temp = TNOM = 300.15 K):
//   Model::processParams4p82_        src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4p82.C:7769-8136
//   Instance::updateTemperature4p82_ src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4p82.C:346-2744
//   PAeffGeo / DioIjthVjmEval        src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4.C:8859-8960
// At temp = TNOM every temperature coefficient (KT1, UTE, AT, UA1, PRT, TCJ,
// TPB, ...) multiplies zero, so those parameters are not part of the row.
#include <algorithm>
#include <cmath>

#include "xg_bsim4.h"
#include "../../include/xyce_gb300.h"

namespace xg {
namespace b4 {

int setup(const double *r, B4Model &I, std::string *why) {
  auto given = [&](int p) { return !std::isnan(r[p]); };
  auto val = [&](int p, double d) { return given(p) ? r[p] : d; };
  auto bad = [&](const char *m) { if (why) *why = m; return XG_ERR_UNSUPPORTED; };
  I = B4Model();
  if (!given(XG_B4_TYPE) || (r[XG_B4_TYPE] != 1.0 && r[XG_B4_TYPE] != -1.0)) return bad("TYPE must be +1 or -1");
  const double dtype = r[XG_B4_TYPE];
  I.dtype = dtype;
  I.M = val(XG_B4_M, 1.0);
  const double L = r[XG_B4_L], W = r[XG_B4_W];
  if (!(L > 0.0) || !(W > 0.0)) return bad("L and W must be positive");
  const double nf = 1.0;
  const double Tnom = kTnom, temp = kTnom;

  // ---- Model::processParams4p82_ (defaults derived from other parameters) ----
  double toxe = val(XG_B4_TOXE, 30.0e-10);
  double toxp = val(XG_B4_TOXP, toxe), toxm = val(XG_B4_TOXM, toxe);
  const double dtox = val(XG_B4_DTOX, 0.0);
  const double drout = val(XG_B4_DROUT, 0.56);
  const double dsub = val(XG_B4_DSUB, drout);
  const double Lint = val(XG_B4_LINT, 0.0), Wint = val(XG_B4_WINT, 0.0);
  const double dlc = val(XG_B4_DLC, Lint), dwc = val(XG_B4_DWC, Wint), dwj = val(XG_B4_DWJ, dwc);
  const double u0_in = val(XG_B4_U0, dtype > 0 ? 0.067 : 0.025);
  const double ua = val(XG_B4_UA, 1.0e-9), uc = val(XG_B4_UC, -0.0465e-9);
  const double agidl = val(XG_B4_AGIDL, 0.0), bgidl = val(XG_B4_BGIDL, 2.3e9), cgidl = val(XG_B4_CGIDL, 0.5),
               egidl = val(XG_B4_EGIDL, 0.8);
  const double agisl = val(XG_B4_AGISL, agidl), bgisl = val(XG_B4_BGISL, bgidl), cgisl = val(XG_B4_CGISL, cgidl),
               egisl = val(XG_B4_EGISL, egidl);
  const double ckappas = val(XG_B4_CKAPPAS, 0.6), ckappad = val(XG_B4_CKAPPAD, ckappas);
  const double dmcg = val(XG_B4_DMCG, 0.0), dmci = val(XG_B4_DMCI, dmcg), dmdg = val(XG_B4_DMDG, 0.0),
               dmcgt = val(XG_B4_DMCGT, 0.0);
  // junction parameters: drain side defaults to the source side
  const double JSS = val(XG_B4_JSS, 1e-4), JSD = val(XG_B4_JSD, JSS);
  const double JSWS = val(XG_B4_JSWS, 0.0), JSWD = val(XG_B4_JSWD, JSWS);
  const double JSWGS = val(XG_B4_JSWGS, 0.0), JSWGD = val(XG_B4_JSWGD, JSWGS);
  double PBS = val(XG_B4_PBS, 1.0);
  double PBD = val(XG_B4_PBD, PBS);
  double PBSWS = val(XG_B4_PBSWS, 1.0);
  double PBSWD = val(XG_B4_PBSWD, PBSWS);
  double PBSWGS = val(XG_B4_PBSWGS, PBSWS);
  double PBSWGD = val(XG_B4_PBSWGD, PBSWD);
  const double NJS = val(XG_B4_NJS, 1.0), NJD = val(XG_B4_NJD, NJS);
  const double MJS = val(XG_B4_MJS, 0.5), MJD = val(XG_B4_MJD, MJS);
  const double MJSWS = val(XG_B4_MJSWS, 0.33), MJSWD = val(XG_B4_MJSWD, MJSWS);
  const double MJSWGS = val(XG_B4_MJSWGS, MJSWS), MJSWGD = val(XG_B4_MJSWGD, MJSWGS);
  const double CJS = val(XG_B4_CJS, 5e-4), CJD = val(XG_B4_CJD, CJS);
  const double CJSWS = val(XG_B4_CJSWS, 5e-10), CJSWD = val(XG_B4_CJSWD, CJSWS);
  const double CJSWGS = val(XG_B4_CJSWGS, CJSWS), CJSWGD = val(XG_B4_CJSWGD, CJSWGS);
  const double ijthsfwd = std::max(0.0, val(XG_B4_IJTHSFWD, 0.1));
  const double ijthdfwd = std::max(0.0, val(XG_B4_IJTHDFWD, ijthsfwd));
  // potentials below 0.1 V are raised to 0.1 V (processParams4p82_)
  for (double *pb : {&PBS, &PBD, &PBSWS, &PBSWD, &PBSWGS, &PBSWGD})
    if (*pb < 0.1) *pb = 0.1;

  // ---- updateTemperature4p82_: model part (:372-700) ----
  if (given(XG_B4_TOXE) && !given(XG_B4_TOXP)) {
    toxp = toxe - dtox;
  } else if (!given(XG_B4_TOXE) && given(XG_B4_TOXP)) {
    toxe = toxp + dtox;
    if (!given(XG_B4_TOXM)) toxm = toxe;
  }
  const double epsrox = val(XG_B4_EPSROX, 3.9);
  const double epssub = kEpsSi;
  const double cf = given(XG_B4_CF) ? r[XG_B4_CF] : 2.0 * epsrox * kEps0 / M_PI * std::log(1.0 + 0.4e-6 / toxe);
  const double coxe = epsrox * kEps0 / toxe;
  const double coxp = epsrox * kEps0 / toxp;
  const double xj = val(XG_B4_XJ, 0.15e-6);
  const double cgsl = val(XG_B4_CGSL, 0.0), cgdl = val(XG_B4_CGDL, 0.0);
  double cgdo, cgso, cgbo;
  if (given(XG_B4_CGDO)) cgdo = r[XG_B4_CGDO];
  else if (given(XG_B4_DLC) && dlc > 0.0) cgdo = dlc * coxe - cgdl;
  else cgdo = 0.6 * xj * coxe;
  if (given(XG_B4_CGSO)) cgso = r[XG_B4_CGSO];
  else if (given(XG_B4_DLC) && dlc > 0.0) cgso = dlc * coxe - cgsl;
  else cgso = 0.6 * xj * coxe;
  cgbo = given(XG_B4_CGBO) ? r[XG_B4_CGBO] : 2.0 * dwc * coxe;
  const double vcrit = kVt0 * std::log(kVt0 / (std::sqrt(2.0) * 1.0e-14));
  const double factor1 = std::sqrt(epssub / (epsrox * kEps0) * toxe);
  const double Vtm0 = kKboQ * Tnom;
  const double Eg0 = 1.16 - 7.02e-4 * Tnom * Tnom / (Tnom + 1108.0);
  const double ni = 1.45e10 * (Tnom / 300.15) * std::sqrt(Tnom / 300.15) * std::exp(21.5565981 - Eg0 / (2.0 * Vtm0));
  const double vtm = kKboQ * temp;
  // temp == Tnom: saturation current densities and junction capacitances unchanged
  I.PhiBS = std::max(PBS, 0.01);
  I.PhiBD = std::max(PBD, 0.01);
  I.PhiBSWS = PBSWS <= 0.01 ? 0.01 : PBSWS;
  I.PhiBSWD = PBSWD <= 0.01 ? 0.01 : PBSWD;
  I.PhiBSWGS = PBSWGS <= 0.01 ? 0.01 : PBSWGS;
  I.PhiBSWGD = PBSWGD <= 0.01 ? 0.01 : PBSWGD;
  I.MJS = MJS; I.MJD = MJD; I.MJSWS = MJSWS; I.MJSWD = MJSWD; I.MJSWGS = MJSWGS; I.MJSWGD = MJSWGD;
  I.NJS = NJS; I.NJD = NJD;

  // ---- size-dependent parameters (:740-1990), no binning ----
  const double Lnew = L + val(XG_B4_XL, 0.0), Wnew = W / nf + val(XG_B4_XW, 0.0);
  const double leff = Lnew - 2.0 * Lint, weff = Wnew - 2.0 * Wint;
  const double leffCV = Lnew - 2.0 * dlc, weffCV = Wnew - 2.0 * dwc, weffCJ = Wnew - 2.0 * dwj;
  if (leff <= 0.0) return bad("effective channel length <= 0");
  if (weff <= 0.0) return bad("effective channel width <= 0");
  if (leffCV <= 0.0 || weffCV <= 0.0 || weffCJ <= 0.0) return bad("effective C-V or junction size <= 0");
  I.leff = leff; I.weff = weff; I.leffCV = leffCV; I.weffCV = weffCV; I.weffCJ = weffCJ;
  I.cdsc = val(XG_B4_CDSC, 2.4e-4); I.cdscb = val(XG_B4_CDSCB, 0.0); I.cdscd = val(XG_B4_CDSCD, 0.0);
  I.cit = val(XG_B4_CIT, 0.0); I.nfactor = val(XG_B4_NFACTOR, 1.0); I.xj = xj;
  I.a0 = val(XG_B4_A0, 1.0); I.ags = val(XG_B4_AGS, 0.0); I.a1 = val(XG_B4_A1, 0.0); I.a2 = val(XG_B4_A2, 1.0);
  I.keta = val(XG_B4_KETA, -0.047); I.ngate = val(XG_B4_NGATE, 0.0);
  I.k3 = val(XG_B4_K3, 80.0); I.k3b = val(XG_B4_K3B, 0.0); I.w0 = val(XG_B4_W0, 2.5e-6);
  I.dvt0 = val(XG_B4_DVT0, 2.2); I.dvt1 = val(XG_B4_DVT1, 0.53); I.dvt2 = val(XG_B4_DVT2, -0.032);
  I.dvt0w = val(XG_B4_DVT0W, 0.0); I.dvt1w = val(XG_B4_DVT1W, 5.3e6); I.dvt2w = val(XG_B4_DVT2W, -0.032);
  I.lpe0 = val(XG_B4_LPE0, 1.74e-7); I.lpeb = val(XG_B4_LPEB, 0.0);
  I.dvtp0 = val(XG_B4_DVTP0, 0.0); I.dvtp1 = val(XG_B4_DVTP1, 0.0); I.etab = val(XG_B4_ETAB, -0.07);
  I.ua = ua; I.ub = val(XG_B4_UB, 1.0e-19); I.uc = uc; I.ud = val(XG_B4_UD, 0.0);
  I.b0 = val(XG_B4_B0, 0.0); I.b1 = val(XG_B4_B1, 0.0); I.dwg = val(XG_B4_DWG, 0.0); I.dwb = val(XG_B4_DWB, 0.0);
  I.prwg = val(XG_B4_PRWG, 1.0); I.prwb = val(XG_B4_PRWB, 0.0); I.pclm = val(XG_B4_PCLM, 1.3);
  I.pdiblb = val(XG_B4_PDIBLCB, 0.0); I.pvag = val(XG_B4_PVAG, 0.0); I.delta = val(XG_B4_DELTA, 0.01);
  I.fprout = val(XG_B4_FPROUT, 0.0); I.pdits = val(XG_B4_PDITS, 0.0); I.pditsd = val(XG_B4_PDITSD, 0.0);
  I.pditsl = val(XG_B4_PDITSL, 0.0); I.pscbe1 = val(XG_B4_PSCBE1, 4.24e8); I.pscbe2 = val(XG_B4_PSCBE2, 1.0e-5);
  I.alpha0 = val(XG_B4_ALPHA0, 0.0); I.alpha1 = val(XG_B4_ALPHA1, 0.0); I.beta0 = val(XG_B4_BETA0, 0.0);
  I.agidl = agidl; I.bgidl = bgidl; I.cgidl = cgidl; I.egidl = egidl;
  I.agisl = agisl; I.bgisl = bgisl; I.cgisl = cgisl; I.egisl = egisl;
  I.cgsl = cgsl; I.cgdl = cgdl; I.ckappas = ckappas; I.ckappad = ckappad;
  I.noff = val(XG_B4_NOFF, 1.0); I.voffcv = val(XG_B4_VOFFCV, 0.0); I.moin = val(XG_B4_MOIN, 15.0);
  I.ados = val(XG_B4_ADOS, 1.0); I.bdos = val(XG_B4_BDOS, 1.0); I.xpart = val(XG_B4_XPART, 0.0);
  I.abulkCVfactor = 1.0 + std::pow(val(XG_B4_CLC, 0.1e-6) / leffCV, val(XG_B4_CLE, 0.6));
  // TRatio = 1: UA..UD, VSAT, RDSW unchanged by temperature (tempMod 0)
  const double PowWeffWr = std::pow(weffCJ * 1.0e6, val(XG_B4_WR, 1.0)) * nf;
  I.vsattemp = val(XG_B4_VSAT, 8.0e4);
  I.rds0 = val(XG_B4_RDSW, 200.0) * nf / PowWeffWr;
  I.rdswmin = val(XG_B4_RDSWMIN, 0.0) * nf / PowWeffWr;
  double u0 = u0_in;
  if (u0 > 1.0) u0 = u0 / 1.0e4;
  const double T5u = 1.0 - val(XG_B4_UP, 0.0) * std::exp(-leff / val(XG_B4_LP, 1.0e-8));
  I.u0temp = u0 * T5u;  // * pow(TRatio, UTE) = 1
  const double voff = val(XG_B4_VOFF, -0.08);
  const double eta0 = val(XG_B4_ETA0, 0.08);
  I.cgdo = (cgdo + cf) * weffCV;
  I.cgso = (cgso + cf) * weffCV;
  I.cgbo = cgbo * leffCV * nf;
  double ndep = val(XG_B4_NDEP, 1.7e17);
  if (!given(XG_B4_NDEP) && given(XG_B4_GAMMA1)) {
    const double T0 = r[XG_B4_GAMMA1] * coxe;
    ndep = 3.01248e22 * T0 * T0;
  }
  const double phin = val(XG_B4_PHIN, 0.0), nsd = val(XG_B4_NSD, 1.0e20), nsub = val(XG_B4_NSUB, 6.0e16);
  const double phi = Vtm0 * std::log(ndep / ni) + phin + 0.4;
  const double sqrtPhi = std::sqrt(phi);
  I.phi = phi; I.sqrtPhi = sqrtPhi;
  I.Xdep0 = std::sqrt(2.0 * epssub / (kChargeQ * ndep * 1.0e6)) * sqrtPhi;
  I.litl = std::sqrt(3.0 * 3.9 / epsrox * xj * toxe);
  I.vbi = Vtm0 * std::log(nsd * ndep / (ni * ni));
  I.vfbsd = (I.ngate > 0.0) ? Vtm0 * std::log(I.ngate / nsd) : 0.0;
  I.cdep0 = std::sqrt(kChargeQ * epssub * ndep * 1.0e6 / 2.0 / phi);
  I.mstar = 0.5 + std::atan(val(XG_B4_MINV, 0.0)) / M_PI;
  I.mstarcv = 0.5 + std::atan(val(XG_B4_MINVCV, 0.0)) / M_PI;
  I.voffcbn = voff + val(XG_B4_VOFFL, 0.0) / leff;
  I.voffcbncv = I.voffcv + val(XG_B4_VOFFCVL, 0.0) / leff;
  I.ldeb = std::sqrt(epssub * Vtm0 / (kChargeQ * ndep * 1.0e6)) / 3.0;
  I.acde = val(XG_B4_ACDE, 1.0) * std::pow(ndep / 2.0e16, -0.25);
  double k1, k2, vbm = val(XG_B4_VBM, -3.0);
  if (given(XG_B4_K1) || given(XG_B4_K2)) {
    k1 = val(XG_B4_K1, 0.53);
    k2 = val(XG_B4_K2, -0.0186);
  } else {
    const double xt = val(XG_B4_XT, 1.55e-7);
    double vbx = given(XG_B4_VBX) ? r[XG_B4_VBX] : phi - 7.7348e-4 * ndep * xt * xt;
    if (vbx > 0.0) vbx = -vbx;
    if (vbm > 0.0) vbm = -vbm;
    const double gamma1 = given(XG_B4_GAMMA1) ? r[XG_B4_GAMMA1] : 5.753e-12 * std::sqrt(ndep) / coxe;
    const double gamma2 = given(XG_B4_GAMMA2) ? r[XG_B4_GAMMA2] : 5.753e-12 * std::sqrt(nsub) / coxe;
    const double T0 = gamma1 - gamma2;
    const double T1 = std::sqrt(phi - vbx) - sqrtPhi;
    const double T2 = std::sqrt(phi * (phi - vbm)) - phi;
    k2 = T0 * T1 / (2.0 * T2 + vbm);
    k1 = gamma2 - 2.0 * k2 * std::sqrt(phi - vbm);
  }
  double vfb;
  if (given(XG_B4_VFB)) vfb = r[XG_B4_VFB];
  else if (given(XG_B4_VTH0)) vfb = dtype * r[XG_B4_VTH0] - phi - k1 * sqrtPhi;
  else vfb = -1.0;
  const double vth0 = given(XG_B4_VTH0) ? r[XG_B4_VTH0] : dtype * (vfb + phi + k1 * sqrtPhi);
  I.k1 = k1; I.k2 = k2;
  I.k1ox = k1 * toxe / toxm;
  {
    const double tmp = std::sqrt(epssub / (epsrox * kEps0) * toxe * I.Xdep0);
    double T0 = dsub * leff / tmp;
    if (T0 < kExpThr) {
      const double T1 = std::exp(T0), T2 = T1 - 1.0, T3 = T2 * T2, T4 = T3 + 2.0 * T1 * kMinExp;
      I.theta0vb0 = T1 / T4;
    } else {
      I.theta0vb0 = 1.0 / (kMaxExp - 2.0);
    }
    T0 = drout * leff / tmp;
    double T5;
    if (T0 < kExpThr) {
      const double T1 = std::exp(T0), T2 = T1 - 1.0, T3 = T2 * T2, T4 = T3 + 2.0 * T1 * kMinExp;
      T5 = T1 / T4;
    } else {
      T5 = 1.0 / (kMaxExp - 2.0);
    }
    I.thetaRout = val(XG_B4_PDIBLC1, 0.39) * T5 + val(XG_B4_PDIBLC2, 0.0086);
  }
  {
    const double tmp = std::sqrt(I.Xdep0), tmp1 = I.vbi - phi, tmp2 = factor1 * tmp;
    double T0 = I.dvt1w * weff * leff / tmp2, T8, T9;
    if (T0 < kExpThr) {
      const double T1 = std::exp(T0), T2 = T1 - 1.0, T3 = T2 * T2, T4 = T3 + 2.0 * T1 * kMinExp;
      T8 = T1 / T4;
    } else {
      T8 = 1.0 / (kMaxExp - 2.0);
    }
    T8 = I.dvt0w * T8 * tmp1;
    T0 = I.dvt1 * leff / tmp2;
    if (T0 < kExpThr) {
      const double T1 = std::exp(T0), T2 = T1 - 1.0, T3 = T2 * T2, T4 = T3 + 2.0 * T1 * kMinExp;
      T9 = T1 / T4;
    } else {
      T9 = 1.0 / (kMaxExp - 2.0);
    }
    T9 = I.dvt0 * T9 * tmp1;
    const double T4 = toxe * phi / (weff + I.w0);
    const double T0b = std::sqrt(1.0 + I.lpe0 / leff);
    const double T5 = I.k1ox * (T0b - 1.0) * sqrtPhi;  // + (KT1 + KT1L/leff)(TRatio - 1) = 0
    I.vfbzbfactor = -T8 - T9 + I.k3 * T4 + T5 - phi - k1 * sqrtPhi;
  }

  // ---- instance part (:2060-2160), no stress, no WPE, DELVTO = 0 ----
  I.vth0 = vth0;
  I.eta0 = eta0;
  I.vfb = vfb;
  {
    const double T3 = dtype * vth0 - vfb - phi;
    I.vtfbphi1 = std::max(0.0, dtype > 0 ? T3 + T3 : 2.5 * T3);
    I.vtfbphi2 = std::max(0.0, 4.0 * T3);
  }
  if (k2 < 0.0) {
    const double T0 = 0.5 * k1 / k2;
    I.vbsc = 0.9 * (phi - T0 * T0);
    if (I.vbsc > -3.0) I.vbsc = -3.0;
    else if (I.vbsc < -30.0) I.vbsc = -30.0;
  } else {
    I.vbsc = -30.0;
  }
  if (I.vbsc > vbm) I.vbsc = vbm;
  I.k2ox = k2 * toxe / toxm;
  I.vfbzb = I.vfbzbfactor + dtype * vth0;
  I.toxe = toxe; I.toxp = toxp; I.coxe = coxe; I.coxp = coxp; I.epsrox = epsrox;
  I.vtm = vtm; I.vtm0 = Vtm0; I.factor1 = factor1; I.vcrit = vcrit;
  // areas and perimeters: PAeffGeo with geoMod 0, NF 1 (one end diffusion
  // each side): P = 2 (DMCG + DMCI) + Weffcj, A = (DMCG + DMCI) Weffcj
  const double DMCGeff = dmcg - dmcgt, DMCIeff = dmci;
  (void)dmdg;
  const double Tg = DMCGeff + DMCIeff;
  const double PSiso = Tg + Tg + weffCJ, ASiso = Tg * weffCJ;
  auto perim = [&](int p) {
    if (!given(p)) return std::max(0.0, PSiso);
    const double v = r[p];
    return (v <= 0.0) ? 0.0 : std::max(0.0, v - weffCJ * nf);  // perMod 1
  };
  I.Pseff = perim(XG_B4_PS);
  I.Pdeff = perim(XG_B4_PD);
  I.Aseff = std::max(0.0, given(XG_B4_AS) ? r[XG_B4_AS] : ASiso);
  I.Adeff = std::max(0.0, given(XG_B4_AD) ? r[XG_B4_AD] : ASiso);
  const double Nvtms = vtm * NJS, Nvtmd = vtm * NJD;
  I.SourceSatCurrent = (I.Aseff <= 0.0 && I.Pseff <= 0.0)
                           ? 0.0
                           : I.Aseff * JSS + I.Pseff * JSWS + weffCJ * nf * JSWGS;
  I.DrainSatCurrent = (I.Adeff <= 0.0 && I.Pdeff <= 0.0)
                          ? 0.0
                          : I.Adeff * JSD + I.Pdeff * JSWD + weffCJ * nf * JSWGD;
  // dioMod 1: DioIjthVjmEval with XExpBV = 0 gives Vjm = Nvtm log(1 + Ijth / Isb)
  if (I.SourceSatCurrent > 0.0) {
    const double Tb = 1.0 + ijthsfwd / I.SourceSatCurrent;
    I.vjsmFwd = Nvtms * std::log(0.5 * (Tb + std::sqrt(Tb * Tb)));
    I.IVjsmFwd = I.SourceSatCurrent * std::exp(I.vjsmFwd / Nvtms);
  }
  if (I.DrainSatCurrent > 0.0) {
    const double Tb = 1.0 + ijthdfwd / I.DrainSatCurrent;
    I.vjdmFwd = Nvtmd * std::log(0.5 * (Tb + std::sqrt(Tb * Tb)));
    I.IVjdmFwd = I.DrainSatCurrent * std::exp(I.vjdmFwd / Nvtmd);
  }
  I.czbs = CJS * I.Aseff;
  I.czbd = CJD * I.Adeff;
  I.czbssw = CJSWS * I.Pseff;
  I.czbdsw = CJSWD * I.Pdeff;
  I.czbsswg = CJSWGS * weffCJ * nf;
  I.czbdswg = CJSWGD * weffCJ * nf;
  return 0;
}

}  // namespace b4
}  // namespace xg
