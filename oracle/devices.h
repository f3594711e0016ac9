// devices.h — oracle restatement of the Xyce device models on the hot path.
// TEST INFRASTRUCTURE ONLY (the checker for xyce_gb300; never shipped).
#pragma once
#include <cmath>
#include <algorithm>

namespace orc {

// Physical constants, src/DeviceModelPKG/Core/N_DEV_Const.h:42-104.
static const double kQ = 1.6021918e-19;
static const double kBoltz = 1.3806226e-23;
static const double kRefTemp = 300.15;
static const double kKoverQ = kBoltz / kQ;
static const double kEg300 = 1.1150877;
static const double kEg0 = 1.16;
static const double kAlphaEg = 7.02e-4;
static const double kBetaEg = 1108.0;
static const double kMaxExpArg = 100.0;
static const double kGmin = 1.0e-12;  // N_DEV_DeviceOptions.C default gmin

// Parameter row layouts (identical numbering in include/xyce_gb300.h).
enum DiodeParam {
  DP_IS, DP_N, DP_RS, DP_CJO, DP_VJ, DP_M, DP_FC, DP_TT, DP_BV, DP_IBV, DP_NBV,
  DP_IKF, DP_ISR, DP_NR, DP_EG, DP_XTI, DP_AREA, DP_BVGIVEN,
  DP_JSW, DP_NS, DP_NSGIVEN, DP_CJSW, DP_VJSW, DP_MJSW, DP_FCS, DP_PJ,
  DP_TNOM, DP_TEMP, DP_TIKF, DP_TBV1, DP_TBV2, DP_TRS1, DP_TRS2, DP_COUNT
};
enum Mos1Param {
  MP_TYPE, MP_VTO, MP_KP, MP_GAMMA, MP_PHI, MP_LAMBDA, MP_RD, MP_RS, MP_CBD, MP_CBS,
  MP_IS, MP_PB, MP_CGSO, MP_CGDO, MP_CGBO, MP_CJ, MP_MJ, MP_CJSW, MP_MJSW, MP_JS,
  MP_TOX, MP_LD, MP_FC, MP_W, MP_L, MP_AD, MP_AS, MP_PD, MP_PS, MP_M, MP_RSH, MP_NRD, MP_NRS,
  MP_TNOM, MP_TEMP, MP_COUNT
};

// DeviceSupport::pnjlim, N_DEV_DeviceSupport.C:188-235.
inline double pnjlim(double vnew, double vold, double vt, double vcrit, int *icheck) {
  if (vnew > vcrit && std::fabs(vnew - vold) > (vt + vt)) {
    if (vold > 0) {
      double arg = 1 + (vnew - vold) / vt;
      vnew = (arg > 0) ? vold + vt * std::log(arg) : vcrit;
    } else {
      vnew = vt * std::log(vnew / vt);
    }
    *icheck = 1;
  } else {
    *icheck = 0;
  }
  return vnew;
}

// DeviceSupport::limvds, N_DEV_DeviceSupport.C:161-180.
inline double limvds(double vnew, double vold) {
  if (vold >= 3.5) {
    if (vnew > vold) vnew = std::min(vnew, 3.0 * vold + 2.0);
    else if (vnew < 3.5) vnew = std::max(vnew, 2.0);
  } else {
    if (vnew > vold) vnew = std::min(vnew, 4.0);
    else vnew = std::max(vnew, -0.5);
  }
  return vnew;
}

// DeviceSupport::fetlim, N_DEV_DeviceSupport.C:309-390.
inline double fetlim(double vnew, double vold, double vto) {
  double vtsthi = std::fabs(2 * (vold - vto)) + 2;
  double vtstlo = vtsthi / 2 + 2;
  double vtox = vto + 3.5;
  double delv = vnew - vold;
  if (vold >= vto) {
    if (vold >= vtox) {
      if (delv <= 0) {
        if (vnew >= vtox) {
          if (-delv > vtstlo) vnew = vold - vtstlo;
        } else {
          vnew = std::max(vnew, vto + 2.0);
        }
      } else if (delv >= vtsthi) {
        vnew = vold + vtsthi;
      }
    } else {
      if (delv <= 0) vnew = std::max(vnew, vto - 0.5);
      else vnew = std::min(vnew, vto + 4.0);
    }
  } else {
    if (delv <= 0) {
      if (-delv > vtsthi) vnew = vold - vtsthi;
    } else {
      double vtemp = vto + 0.5;
      if (vnew <= vtemp) {
        if (delv > vtstlo) vnew = vold + vtstlo;
      } else {
        vnew = vtemp;
      }
    }
  }
  return vnew;
}

// DeviceSupport::qmeyer, N_DEV_DeviceSupport.C:507-590.
inline void qmeyer(double vgs, double vgd, double von, double vdsat, double &capgs,
                   double &capgd, double &capgb, double phi, double cox) {
  double vgst = vgs - von;
  if (vgst <= -phi) {
    capgb = cox / 2; capgs = 0; capgd = 0;
  } else if (vgst <= -phi / 2) {
    capgb = -vgst * cox / (2 * phi); capgs = 0; capgd = 0;
  } else if (vgst <= 0) {
    capgb = -vgst * cox / (2 * phi);
    capgs = vgst * cox / (1.5 * phi) + cox / 3;
    capgd = 0;
  } else {
    double vds = vgs - vgd;
    if (vdsat <= vds) {
      capgs = cox / 3; capgd = 0; capgb = 0;
    } else {
      double vddif = 2.0 * vdsat - vds;
      double vddif1 = vdsat - vds;
      double vddif2 = vddif * vddif;
      capgd = cox * (1.0 - vdsat * vdsat / vddif2) / 3;
      capgs = cox * (1.0 - vddif1 * vddif1 / vddif2) / 3;
      capgb = 0;
    }
  }
}

// Temperature-adjusted diode parameters at TEMP = TNOM = 27 C
// (Diode updateTemperature, N_DEV_Diode.C:2040-2237; Model::processParams :1612).
struct DiodeT {
  double Isat, IsatR, Vte, VteR, VteBRK, Gspr, tVcrit, tIKF, tJctPot, tJctCap, tDepCap,
      tF1, F2, F3, M, TT, tBrkdwnV, area;
  bool bvGiven;
  // sidewall junction: sw 0 none, 1 own characteristic (NS given), 2 its
  // saturation current joined to the bottom one (JSW given, NS not)
  int sw;
  double IsatSW, VteSW, CzeroSW, tJctSWPot, tDepSWCap, F2SW, F3SW, MJSW;
};

inline DiodeT diode_temperature(const double *p) {
  DiodeT t{};
  double Temp = p[DP_TEMP], TNOM = p[DP_TNOM];
  double M = std::min(p[DP_M], 0.9);
  double FC = std::min(p[DP_FC], 0.95);
  double EG = std::max(p[DP_EG], 0.1);
  double N = p[DP_N], IS = p[DP_IS], VJ = p[DP_VJ], CJO = p[DP_CJO], XTI = p[DP_XTI];
  double vt = kKoverQ * Temp, vtnom = kKoverQ * TNOM;
  double fact2 = Temp / kRefTemp;
  double egfet = kEg0 - (kAlphaEg * Temp * Temp) / (Temp + kBetaEg);
  double arg = -egfet / (2.0 * kBoltz * Temp) + kEg300 / (kBoltz * (kRefTemp + kRefTemp));
  double pbfact = -2.0 * vt * (1.5 * std::log(fact2) + kQ * arg);
  double egfet1 = kEg0 - (kAlphaEg * TNOM * TNOM) / (TNOM + kBetaEg);
  double arg1 = -egfet1 / (2.0 * kBoltz * TNOM) + kEg300 / (2.0 * kBoltz * kRefTemp);
  double fact1 = TNOM / kRefTemp;
  double pbfact1 = -2.0 * vtnom * (1.5 * std::log(fact1) + kQ * arg1);
  double pbo = (VJ - pbfact1) / fact1;
  double gmaold = (VJ - pbo) / pbo;
  double tJctCap = CJO / (1.0 + M * (4.0e-4 * (TNOM - kRefTemp) - gmaold));
  double tJctPot = pbfact + fact2 * pbo;
  double gmanew = (tJctPot - pbo) / pbo;
  tJctCap *= 1.0 + M * (4.0e-4 * (Temp - kRefTemp) - gmanew);
  double tSatCur = IS * std::exp(((Temp / TNOM) - 1.0) * EG / (N * vt) + XTI / N * std::log(Temp / TNOM));
  double xfc = std::log(1.0 - FC);
  t.tF1 = tJctPot * (1.0 - std::exp((1.0 - M) * xfc)) / (1.0 - M);
  t.tDepCap = FC * tJctPot;
  double vte = N * vt;
  t.tVcrit = vte * std::log(vte / (std::sqrt(2.0) * (tSatCur == 0.0 ? 1e-14 : tSatCur)));
  double NR = p[DP_NR];
  double tSatCurR = p[DP_ISR] * std::exp((Temp / TNOM - 1.0) * EG / (NR * vt) + XTI / NR * std::log(Temp / TNOM));
  // N_DEV_Diode.C:1520-1529
  t.tIKF = p[DP_IKF] * (1 + p[DP_TIKF] * (Temp - TNOM));
  double tRS = p[DP_RS] * (1 + (Temp - TNOM) * (p[DP_TRS1] + p[DP_TRS2] * (Temp - TNOM)));
  double tCOND = (tRS != 0.0) ? 1.0 / tRS : 0.0;
  double NBV = p[DP_NBV];
  t.bvGiven = p[DP_BVGIVEN] != 0.0;
  t.tBrkdwnV = 0.0;
  if (t.bvGiven) {
    double tempBV = p[DP_BV] * (1 + (Temp - TNOM) * (p[DP_TBV1] + p[DP_TBV2] * (Temp - TNOM)));
    double cbv = p[DP_IBV], xbv;
    if (cbv < tSatCur * tempBV / vt) {
      xbv = tempBV;
    } else {
      double tol = 1.0e-3 * cbv;
      xbv = tempBV - NBV * vt * std::log(1.0 + cbv / tSatCur);
      for (int i = 0; i < 25; ++i) {
        xbv = tempBV - NBV * vt * std::log(cbv / tSatCur + 1.0 - xbv / vt);
        double xcbv = tSatCur * (std::exp((tempBV - xbv) / (NBV * vt)) - 1.0 + xbv / vt);
        if (std::fabs(xcbv - cbv) <= tol) break;
      }
    }
    t.tBrkdwnV = xbv;
  }
  // sidewall (updateTemperature N_DEV_Diode.C:1473-1494, Model::processParams
  // :1632-1636; PJ scales the sidewall as AREA scales the bottom)
  {
    const double VJSW = p[DP_VJSW], MJSW = p[DP_MJSW], FCS = p[DP_FCS], PJ = p[DP_PJ], NS = p[DP_NS];
    const double pboSW = (VJSW - pbfact1) / fact1;
    const double gmaSWold = (VJSW - pboSW) / pboSW;
    double tJctSWCap = p[DP_CJSW] / (1.0 + MJSW * (4.0e-4 * (TNOM - kRefTemp) - gmaSWold));
    const double tJctSWPot = pbfact + fact2 * pboSW;
    const double gmaSWnew = (tJctSWPot - pboSW) / pboSW;
    tJctSWCap *= 1.0 + MJSW * (4.0e-4 * (Temp - kRefTemp) - gmaSWnew);
    const double tSatSWCur =
        p[DP_JSW] * std::exp(((Temp / TNOM) - 1.0) * EG / (NS * vt) + XTI / NS * std::log(Temp / TNOM));
    const double xfcs = std::log(1.0 - FCS);
    t.tJctSWPot = tJctSWPot;
    t.tDepSWCap = FCS * tJctSWPot;
    t.F2SW = std::exp((1.0 + MJSW) * xfcs);
    t.F3SW = 1.0 - FCS * (1.0 + MJSW);
    t.MJSW = MJSW;
    t.IsatSW = tSatSWCur * PJ;
    t.VteSW = NS * vt;
    t.CzeroSW = tJctSWCap * PJ;
    t.sw = (p[DP_JSW] != 0.0) ? (p[DP_NSGIVEN] != 0.0 ? 1 : 2) : 0;
  }
  t.area = p[DP_AREA];
  t.Isat = tSatCur * t.area;
  if (t.sw == 2) t.Isat = t.Isat + t.IsatSW;  // the bottom characteristic carries both
  t.IsatR = tSatCurR * t.area;
  t.Vte = N * vt;
  t.VteR = NR * vt;
  t.VteBRK = NBV * vt;
  t.Gspr = tCOND * t.area;
  t.tJctPot = tJctPot;
  t.tJctCap = tJctCap;
  t.F2 = std::exp((1.0 + M) * xfc);
  t.F3 = 1.0 - FC * (1.0 + M);
  t.M = M;
  t.TT = p[DP_TT];
  return t;
}

struct DiodeOut {
  double Vd, Vd_orig, Id, Gd, Qd, Cd;
};

// Diode::Instance::updateIntermediateVars, N_DEV_Diode.C:1072-1420, with the
// sidewall current (:1226-1260) and charge (:1380-1400).
// vd_hist is the stored junction voltage: currSto at newton_iter 0, nextSto after.
inline DiodeOut diode_eval(const DiodeT &t, double Vpp, double Vn, double vd_hist, int newton_iter,
                           bool dcop, bool initJct) {
  DiodeOut o{};
  double Vd = Vpp - Vn;
  o.Vd_orig = Vd;
  double Vd_old;
  if (newton_iter == 0) {
    if (initJct) Vd = t.tVcrit;
    Vd_old = dcop ? Vd : vd_hist;  // the operating point has no history
  } else {
    Vd_old = vd_hist;
  }
  int ichk = 0;
  if (t.bvGiven && Vd < std::min(0.0, -t.tBrkdwnV + 10.0 * t.VteBRK)) {
    double Vdtmp = -(t.tBrkdwnV + Vd);
    Vdtmp = pnjlim(Vdtmp, -(Vd_old + t.tBrkdwnV), t.VteBRK, t.tVcrit, &ichk);
    Vd = -(Vdtmp + t.tBrkdwnV);
  } else {
    Vd = pnjlim(Vd, Vd_old, t.Vte, t.tVcrit, &ichk);
  }
  double IdSW = 0.0, GdSW = 0.0;
  if (t.sw == 1) {
    if (Vd >= -3.0 * t.VteSW) {  // sidewall forward
      double evd = std::exp(std::min(kMaxExpArg, Vd / t.VteSW));
      IdSW = t.IsatSW * (evd - 1.0);
      GdSW = t.IsatSW * evd / t.VteSW;
    } else if (!t.tBrkdwnV || Vd >= -t.tBrkdwnV) {  // sidewall reverse
      double argsw = 3.0 * t.VteSW / (Vd * std::exp(1.0));
      argsw = argsw * argsw * argsw;
      IdSW = -t.IsatSW * (1.0 + argsw);
      GdSW = t.IsatSW * 3.0 * argsw / Vd;
    } else {  // sidewall breakdown
      double evrev = std::exp(std::min(kMaxExpArg, -(t.tBrkdwnV + Vd) / t.VteBRK));
      IdSW = -t.IsatSW * evrev;
      GdSW = t.IsatSW * evrev / t.VteBRK;
    }
  }
  double Id, Gd;
  if (Vd >= -3.0 * t.Vte) {
    double evd = std::exp(std::min(kMaxExpArg, Vd / t.Vte));
    double Inorm = t.Isat * (evd - 1.0) + kGmin * Vd;
    double Gd1 = t.Isat * evd / t.Vte + kGmin;
    evd = std::exp(std::min(kMaxExpArg, Vd / t.VteR));
    double Irec = t.IsatR * (evd - 1.0);
    double Gd2 = t.IsatR * evd / t.VteR;
    double Khi = 1, DKhi = 0;
    if (t.tIKF > 0) {
      Khi = std::sqrt(t.tIKF / (t.tIKF + Inorm));
      DKhi = -0.5 * Khi * Gd1 / (t.tIKF + Inorm);
    }
    double Kgen = 0, DKgen = 0;
    if (Irec != 0) {
      double a = 1 - Vd / t.tJctPot;
      Kgen = std::sqrt(std::pow(a * a + 0.005, t.M));
      DKgen = -t.M * a * Kgen / (t.tJctPot * (a * a + 0.005));
    }
    Id = Inorm * Khi + Irec * Kgen + IdSW;
    Gd = Gd1 * Khi + Inorm * DKhi + Gd2 * Kgen + Irec * DKgen + GdSW;
  } else if (!t.tBrkdwnV || Vd >= -t.tBrkdwnV) {
    double arg = 3.0 * t.Vte / (Vd * std::exp(1.0));
    arg = arg * arg * arg;
    Id = -t.Isat * (1.0 + arg) + IdSW + kGmin * Vd;
    Gd = t.Isat * 3.0 * arg / Vd + GdSW + kGmin;
  } else {
    double evrev = std::exp(std::min(kMaxExpArg, -(t.tBrkdwnV + Vd) / t.VteBRK));
    Id = -t.Isat * evrev + IdSW + kGmin * Vd;
    Gd = t.Isat * evrev / t.VteBRK + GdSW + kGmin;
  }
  double Qd = 0, Cd = 0;
  if (t.tJctCap != 0.0) {
    double Czero = t.tJctCap * t.area;
    double Vc = Vd;
    if (Vc < t.tDepCap) {
      double arg = 1.0 - Vc / t.tJctPot;
      double sarg = std::exp(std::min(kMaxExpArg, -t.M * std::log(arg)));
      Qd = t.TT * Id + t.tJctPot * Czero * (1.0 - arg * sarg) / (1.0 - t.M);
      Cd = t.TT * Gd + Czero * sarg;
    } else {
      double Czof2 = Czero / t.F2;
      double MotJctPot = t.M / t.tJctPot;
      Qd = t.TT * Id + Czero * t.tF1 +
           Czof2 * (t.F3 * (Vc - t.tDepCap) + 0.5 * MotJctPot * (Vc * Vc - t.tDepCap * t.tDepCap));
      Cd = t.TT * Gd + Czof2 * (t.F3 + MotJctPot * Vc);
    }
    // sidewall depletion charge (computed where the bottom one is, as the
    // reference does)
    const double CzeroSW = t.CzeroSW;
    if (Vc < t.tDepSWCap) {
      double argSW = 1.0 - Vc / t.tJctSWPot;
      double sargSW = std::exp(std::min(kMaxExpArg, -t.MJSW * std::log(argSW)));
      Qd += t.tJctSWPot * CzeroSW * (1.0 - argSW * sargSW) / (1.0 - t.MJSW);
      Cd += CzeroSW * sargSW;
    } else {
      double Czof2SW = CzeroSW / t.F2SW;
      double MotJctSWPot = t.MJSW / t.tJctSWPot;
      Qd += CzeroSW * t.tF1 +
            Czof2SW * (t.F3SW * (Vc - t.tDepSWCap) + (0.5 * MotJctSWPot) * (Vc * Vc - t.tDepSWCap * t.tDepSWCap));
      Cd += Czof2SW * (t.F3SW + MotJctSWPot * Vc);
    }
  }
  o.Vd = Vd; o.Id = Id; o.Gd = Gd; o.Qd = Qd; o.Cd = Cd;
  return o;
}

// Temperature/geometry-processed MOSFET level-1 instance parameters
// (Instance::processParams N_DEV_MOSFET1.C:383-470, updateTemperature :3487-3730,
//  Model::processParams :3939-4020) at TEMP = TNOM = 27 C.
struct Mos1T {
  double dtype, Beta, tVbi, tVto, gamma, tPhi, lambda, vt, DrainSatCur, SourceSatCur,
      sourceVcrit, drainVcrit, OxideCap, Cgso, Cgdo, Cgbo, Cbd, Cbdsw, Cbs, Cbssw, tDepCap,
      tBulkPot, MJ, MJSW, f2d, f3d, f4d, f2s, f3s, f4s, M;
  double drainConductance, sourceConductance;  // series RD / RS (0 = none)
};

// Series drain/source conductance, Instance::processParams N_DEV_MOSFET1.C:410-450:
// RD (RS) when nonzero, else 1/(RSH * NRD (NRS)) when RSH is nonzero, else 0.
inline double mos1_series_conductance(double r, double rsh, double squares) {
  if (r != 0.0) return 1.0 / r;
  if (rsh != 0.0) return 1.0 / (rsh * squares);
  return 0.0;
}

inline Mos1T mos1_temperature(const double *p) {
  Mos1T t{};
  double temp = p[MP_TEMP], tnom = p[MP_TNOM];
  t.dtype = p[MP_TYPE];
  double fact1 = tnom / kRefTemp;
  double vtnom = tnom * kKoverQ;
  double kt1 = kBoltz * tnom;
  double egfet1 = 1.16 - (7.02e-4 * tnom * tnom) / (tnom + 1108);
  double arg1 = -egfet1 / (kt1 + kt1) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
  double pbfact1 = -2 * vtnom * (1.5 * std::log(fact1) + kQ * arg1);
  double oxideCapFactor = (p[MP_TOX] == 0.0) ? 0.0 : 3.9 * 8.854214871e-12 / p[MP_TOX];
  double vt = temp * kKoverQ;
  double ratio = temp / tnom;
  double fact2 = temp / kRefTemp;
  double kt = temp * kBoltz;
  double egfet = 1.16 - (7.02e-4 * temp * temp) / (temp + 1108);
  double arg = -egfet / (kt + kt) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
  double pbfact = -2 * vt * (1.5 * std::log(fact2) + kQ * arg);
  double ratio4 = ratio * std::sqrt(ratio);
  double tTrans = p[MP_KP] / ratio4;
  double phi = p[MP_PHI], gamma = p[MP_GAMMA];
  double phio = (phi - pbfact1) / fact1;
  double tPhi = fact2 * phio + pbfact;
  double tVbi = p[MP_VTO] - t.dtype * (gamma * std::sqrt(phi)) + .5 * (egfet1 - egfet) +
                t.dtype * .5 * (tPhi - phi);
  double tVto = tVbi + t.dtype * gamma * std::sqrt(tPhi);
  double tSatCur = p[MP_IS] * std::exp(-egfet / vt + egfet1 / vtnom);
  double tSatCurDens = p[MP_JS] * std::exp(-egfet / vt + egfet1 / vtnom);
  double pb = p[MP_PB], mj = p[MP_MJ], mjsw = p[MP_MJSW], fc = p[MP_FC];
  double pbo = (pb - pbfact1) / fact1;
  double gmaold = (pb - pbo) / pbo;
  double capfact = 1 / (1 + mj * (4e-4 * (tnom - kRefTemp) - gmaold));
  double tCbd = p[MP_CBD] * capfact, tCbs = p[MP_CBS] * capfact, tCj = p[MP_CJ] * capfact;
  capfact = 1 / (1 + mjsw * (4e-4 * (tnom - kRefTemp) - gmaold));
  double tCjsw = p[MP_CJSW] * capfact;
  double tBulkPot = fact2 * pbo + pbfact;
  double gmanew = (tBulkPot - pbo) / pbo;
  capfact = (1 + mj * (4e-4 * (temp - kRefTemp) - gmanew));
  tCbd *= capfact; tCbs *= capfact; tCj *= capfact;
  capfact = (1 + mjsw * (4e-4 * (temp - kRefTemp) - gmanew));
  tCjsw *= capfact;
  double tDepCap = fc * tBulkPot;
  double AD = p[MP_AD], AS = p[MP_AS], PD = p[MP_PD], PS = p[MP_PS];
  double js = p[MP_JS];
  if (js == 0 || AD == 0 || AS == 0) {
    t.sourceVcrit = t.drainVcrit = vt * std::log(vt / (std::sqrt(2.0) * p[MP_IS]));
  } else {
    t.drainVcrit = vt * std::log(vt / (std::sqrt(2.0) * js * AD));
    t.sourceVcrit = vt * std::log(vt / (std::sqrt(2.0) * js * AS));
  }
  double czbd = (p[MP_CBD] != 0) ? tCbd : ((p[MP_CJ] != 0) ? tCj * AD : 0);
  double czbdsw = (p[MP_CJSW] != 0) ? tCjsw * PD : 0;
  double czbs = (p[MP_CBS] != 0) ? tCbs : ((p[MP_CJ] != 0) ? tCj * AS : 0);
  double czbssw = (p[MP_CJSW] != 0) ? tCjsw * PS : 0;
  double a = 1 - fc;
  double sarg = std::exp(-mj * std::log(a));
  double sargsw = std::exp(-mjsw * std::log(a));
  t.Cbd = czbd; t.Cbdsw = czbdsw; t.Cbs = czbs; t.Cbssw = czbssw;
  t.f2d = czbd * (1 - fc * (1 + mj)) * sarg / a + czbdsw * (1 - fc * (1 + mjsw)) * sargsw / a;
  t.f3d = czbd * mj * sarg / a / tBulkPot + czbdsw * mjsw * sargsw / a / tBulkPot;
  t.f4d = czbd * tBulkPot * (1 - a * sarg) / (1 - mj) + czbdsw * tBulkPot * (1 - a * sargsw) / (1 - mjsw) -
          t.f3d / 2 * (tDepCap * tDepCap) - tDepCap * t.f2d;
  t.f2s = czbs * (1 - fc * (1 + mj)) * sarg / a + czbssw * (1 - fc * (1 + mjsw)) * sargsw / a;
  t.f3s = czbs * mj * sarg / a / tBulkPot + czbssw * mjsw * sargsw / a / tBulkPot;
  t.f4s = czbs * tBulkPot * (1 - a * sarg) / (1 - mj) + czbssw * tBulkPot * (1 - a * sargsw) / (1 - mjsw) -
          t.f3s / 2 * (tDepCap * tDepCap) - tDepCap * t.f2s;
  if (tSatCurDens == 0 || AD == 0 || AS == 0) {
    t.DrainSatCur = tSatCur; t.SourceSatCur = tSatCur;
  } else {
    t.DrainSatCur = tSatCurDens * AD; t.SourceSatCur = tSatCurDens * AS;
  }
  double W = p[MP_W], L = p[MP_L], LD = p[MP_LD];
  double Leff = L - 2 * LD;
  t.Beta = tTrans * W / Leff;
  t.tVbi = tVbi; t.tVto = tVto; t.gamma = gamma; t.tPhi = tPhi; t.lambda = p[MP_LAMBDA];
  t.vt = vt;
  t.OxideCap = oxideCapFactor * Leff * W;
  t.Cgso = p[MP_CGSO] * W; t.Cgdo = p[MP_CGDO] * W; t.Cgbo = p[MP_CGBO] * Leff;
  t.tDepCap = tDepCap; t.tBulkPot = tBulkPot; t.MJ = mj; t.MJSW = mjsw;
  t.M = p[MP_M];
  t.drainConductance = mos1_series_conductance(p[MP_RD], p[MP_RSH], p[MP_NRD]);
  t.sourceConductance = mos1_series_conductance(p[MP_RS], p[MP_RSH], p[MP_NRS]);
  return t;
}

// Results of one MOSFET-1 evaluation, at the drain' and source' nodes (the
// drain and source themselves when there is no series resistance).
struct Mos1Out {
  double vbs, vbd, vgs, vds, vgd, Vgb, von, vdsat;
  double vbs_orig, vbd_orig, vgs_orig, vds_orig, vgd_orig;
  bool origFlag;
  int mode;
  double gbs, gbd, cbs, cbd, gm, gds, gmbs, Gm, Gmbs, nrmsum, revsum, cdreq;
  double capbs, capbd, qbs, qbd, capgs, capgd, capgb, Capgs, Capgd, Capgb;
  double qgs, qgd, qgb;
};

// MOSFET1 Instance::updateIntermediateVars (N_DEV_MOSFET1.C:2689-3477) and
// the state part of Master::updateState (:4241-4333).
// hist: vbs, vbd, vgs, vds, von (store; from currSto at iteration 0, nextSto after)
// csta: capgs, capgd, capgb, qgs, qgd, qgb from currSta; csto: vgs, vbs, vds from currSto.
inline Mos1Out mos1_eval(const Mos1T &t, double Vd, double Vg, double Vs, double Vb,
                         const double *hist, const double *csta, const double *csto,
                         int newton_iter, bool dcop, bool initJct) {
  Mos1Out o{};
  const double dt = t.dtype;
  double vbs = dt * (Vb - Vs), vgs = dt * (Vg - Vs), vds = dt * (Vd - Vs);
  double vbd = vbs - vds, vgd = vgs - vds;
  o.vgs_orig = vgs; o.vds_orig = vds; o.vbs_orig = vbs; o.vbd_orig = vbd; o.vgd_orig = vgd;
  if (initJct) {
    vbs = -1; vgs = dt * t.tVto; vds = 0; vbd = vbs - vds; vgd = vgs - vds;
  }
  double vbs_old, vbd_old, vgs_old, vds_old, Von;
  if (newton_iter == 0 && dcop) {
    // operating point, first iteration: no history (N_DEV_MOSFET1.C:2864-2880).
    vbs_old = vbs; vbd_old = vbd; vgs_old = vgs; vds_old = vds; Von = 0.0;
  } else {
    vbs_old = hist[1]; vbd_old = hist[0]; vgs_old = hist[2]; vds_old = hist[3];
    Von = dt * hist[4];
  }
  double vgd_old = vgs_old - vds_old;
  int Check = 1;
  bool limited = false;
  if (vds_old >= 0) {
    vgs = fetlim(vgs, vgs_old, Von);
    vds = vgs - vgd;
    vds = limvds(vds, vds_old);
    vgd = vgs - vds;
  } else {
    vgd = fetlim(vgd, vgd_old, Von);
    vds = vgs - vgd;
    vds = -limvds(-vds, -vds_old);
    vgs = vgd + vds;
  }
  if (vds >= 0.0) {
    vbs = pnjlim(vbs, vbs_old, t.vt, t.sourceVcrit, &Check);
    vbd = vbs - vds;
  } else {
    vbd = pnjlim(vbd, vbd_old, t.vt, t.drainVcrit, &Check);
    vbs = vbd + vds;
  }
  if (Check == 1) limited = true;
  (void)limited;
  vbd = vbs - vds;
  vgd = vgs - vds;
  double Vgb = vgs - vbs;
  o.origFlag = !(o.vgs_orig != vgs || o.vds_orig != vds || o.vbs_orig != vbs ||
                 o.vbd_orig != vbd || o.vgd_orig != vgd);
  // bulk junction diodes
  if (vbs <= 0) {
    o.gbs = t.SourceSatCur / t.vt + kGmin;
    o.cbs = o.gbs * vbs;
  } else {
    double evbs = std::exp(std::min(kMaxExpArg, vbs / t.vt));
    o.gbs = t.SourceSatCur * evbs / t.vt + kGmin;
    o.cbs = t.SourceSatCur * (evbs - 1) + kGmin * vbs;
  }
  if (vbd <= 0) {
    o.gbd = t.DrainSatCur / t.vt + kGmin;
    o.cbd = o.gbd * vbd;
  } else {
    double evbd = std::exp(std::min(kMaxExpArg, vbd / t.vt));
    o.gbd = t.DrainSatCur * evbd / t.vt + kGmin;
    o.cbd = t.DrainSatCur * (evbd - 1) + kGmin * vbd;
  }
  int mode = (vds >= 0) ? 1 : -1;
  double cdrain, gm, gds, gmbs;
  {
    double vbx = (mode == 1) ? vbs : vbd;
    double sarg;
    if (vbx <= 0) {
      sarg = std::sqrt(t.tPhi - vbx);
    } else {
      sarg = std::sqrt(t.tPhi);
      sarg = sarg - vbx / (sarg + sarg);
      sarg = std::max(0.0, sarg);
    }
    Von = (t.tVbi * dt) + t.gamma * sarg;
    double vgst = ((mode == 1) ? vgs : vgd) - Von;
    double Vdsat = std::max(vgst, 0.0);
    double arg = (sarg <= 0) ? 0 : t.gamma / (sarg + sarg);
    if (vgst <= 0) {
      cdrain = 0; gm = 0; gds = 0; gmbs = 0;
    } else {
      double vdsm = vds * mode;
      double betap = t.Beta * (1 + t.lambda * vdsm);
      if (vgst <= vdsm) {
        cdrain = betap * vgst * vgst * .5;
        gm = betap * vgst;
        gds = t.lambda * t.Beta * vgst * vgst * .5;
        gmbs = gm * arg;
      } else {
        cdrain = betap * vdsm * (vgst - .5 * vdsm);
        gm = betap * vdsm;
        gds = betap * (vgst - vdsm) + t.lambda * t.Beta * vdsm * (vgst - .5 * vdsm);
        gmbs = gm * arg;
      }
    }
    o.von = dt * Von;
    o.vdsat = dt * Vdsat;
    // bulk junction charges (N_DEV_MOSFET1.C:3100-3210)
    if (t.Cbs != 0 || t.Cbssw != 0) {
      if (vbs < t.tDepCap) {
        double a = 1 - vbs / t.tBulkPot;
        double s1 = (t.MJ == .5) ? 1 / std::sqrt(a) : std::exp(-t.MJ * std::log(a));
        double s2 = (t.MJSW == .5) ? 1 / std::sqrt(a) : std::exp(-t.MJSW * std::log(a));
        o.qbs = t.tBulkPot * (t.Cbs * (1 - a * s1) / (1 - t.MJ) + t.Cbssw * (1 - a * s2) / (1 - t.MJSW));
        o.capbs = t.Cbs * s1 + t.Cbssw * s2;
      } else {
        o.qbs = t.f4s + vbs * (t.f2s + vbs * (t.f3s / 2));
        o.capbs = t.f2s + t.f3s * vbs;
      }
    }
    if (t.Cbd != 0 || t.Cbdsw != 0) {
      if (vbd < t.tDepCap) {
        double a = 1 - vbd / t.tBulkPot;
        double s1 = (t.MJ == .5) ? 1 / std::sqrt(a) : std::exp(-t.MJ * std::log(a));
        double s2 = (t.MJSW == .5) ? 1 / std::sqrt(a) : std::exp(-t.MJSW * std::log(a));
        o.qbd = t.tBulkPot * (t.Cbd * (1 - a * s1) / (1 - t.MJ) + t.Cbdsw * (1 - a * s2) / (1 - t.MJSW));
        o.capbd = t.Cbd * s1 + t.Cbdsw * s2;
      } else {
        o.qbd = t.f4d + vbd * (t.f2d + vbd * t.f3d / 2);
        o.capbd = t.f2d + vbd * t.f3d;
      }
    }
    // Meyer capacitances (old Meyer, back-averaged), :3225-3320
    if (mode > 0) qmeyer(vgs, vgd, Von, Vdsat, o.capgs, o.capgd, o.capgb, t.tPhi, t.OxideCap);
    else qmeyer(vgd, vgs, Von, Vdsat, o.capgd, o.capgs, o.capgb, t.tPhi, t.OxideCap);
    if (dcop) {
      o.Capgs = 2.0 * o.capgs + t.Cgso;
      o.Capgd = 2.0 * o.capgd + t.Cgdo;
      o.Capgb = 2.0 * o.capgb + t.Cgbo;
    } else {
      o.Capgs = o.capgs + csta[0] + t.Cgso;
      o.Capgd = o.capgd + csta[1] + t.Cgdo;
      o.Capgb = o.capgb + csta[2] + t.Cgbo;
    }
    o.Capgs *= (o.Capgs < 0.0) ? -1.0 : 1.0;
    o.Capgd *= (o.Capgd < 0.0) ? -1.0 : 1.0;
    o.Capgb *= (o.Capgb < 0.0) ? -1.0 : 1.0;
  }
  o.gm = gm; o.gds = gds; o.gmbs = gmbs;
  if (mode >= 0) {
    o.Gm = gm; o.Gmbs = gmbs; o.nrmsum = o.Gm + o.Gmbs; o.revsum = 0; o.cdreq = dt * cdrain;
  } else {
    o.Gm = -gm; o.Gmbs = -gmbs; o.nrmsum = 0; o.revsum = -(o.Gm + o.Gmbs); o.cdreq = -dt * cdrain;
  }
  o.mode = mode;
  o.vbs = vbs; o.vbd = vbd; o.vgs = vgs; o.vds = vds; o.vgd = vgd; o.Vgb = Vgb;
  // gate charges (Master::updateState, :4280-4320)
  if (dcop) {
    o.qgs = o.Capgs * vgs; o.qgd = o.Capgd * vgd; o.qgb = o.Capgb * Vgb;
  } else {
    double vgs1 = csto[0], vbs1 = csto[1], vds1 = csto[2];
    double vgb1 = vgs1 - vbs1, vgd1 = vgs1 - vds1;
    o.qgs = csta[3] + o.Capgs * (vgs - vgs1);
    o.qgd = csta[4] + o.Capgd * (vgd - vgd1);
    o.qgb = csta[5] + o.Capgb * ((vgs - vbs) - vgb1);
  }
  return o;
}

}  // namespace orc
