// xg_params.cpp — host processing of device parameters into the device-side
// model tables, at each device's temperature TEMP with its model's TNOM
// (kelvin, from the parameter row).
//
//   Diode: Model::processParams + updateTemperature
//          src/DeviceModelPKG/OpenModels/N_DEV_Diode.C:1612-1639, 2040-2237;
//          the sidewall junction :1473-1494, :1632-1636
//   MOSFET level 1: Model::processParams, Instance::processParams, updateTemperature
//          src/DeviceModelPKG/OpenModels/N_DEV_MOSFET1.C:3939-4020, 383-470, 3487-3730
#include <algorithm>
#include <cmath>

#include "xg_params.h"

namespace xg {
namespace {
const double Q = 1.6021918e-19, BOLTZ = 1.3806226e-23, REFTEMP = 300.15;
const double KOVERQ = BOLTZ / Q, EG300 = 1.1150877, EG0 = 1.16, ALPHAEG = 7.02e-4, BETAEG = 1108.0;

double egap(double T) { return EG0 - (ALPHAEG * T * T) / (T + BETAEG); }
// -2 vt (1.5 ln(T/Tref) + q * (-Eg(T)/(2kT) + Eg300/(2k Tref)))
double pb_factor(double T) {
  double vt = KOVERQ * T;
  double arg = -egap(T) / (2.0 * BOLTZ * T) + EG300 / (BOLTZ * (REFTEMP + REFTEMP));
  return -2.0 * vt * (1.5 * std::log(T / REFTEMP) + Q * arg);
}
}  // namespace

DiodeModel diode_model(const double *p) {
  DiodeModel m{};
  const double T = p[XG_DIODE_TEMP], TN = p[XG_DIODE_TNOM];
  const double M = std::min(p[XG_DIODE_M], 0.9);
  const double FC = std::min(p[XG_DIODE_FC], 0.95);
  const double EG = std::max(p[XG_DIODE_EG], 0.1);
  const double N = p[XG_DIODE_N], IS = p[XG_DIODE_IS], VJ = p[XG_DIODE_VJ], XTI = p[XG_DIODE_XTI];
  const double vt = KOVERQ * T;
  const double fact1 = TN / REFTEMP, fact2 = T / REFTEMP;
  const double pbfact = pb_factor(T), pbfact1 = pb_factor(TN);
  const double pbo = (VJ - pbfact1) / fact1;
  const double gmaold = (VJ - pbo) / pbo;
  double tJctCap = p[XG_DIODE_CJO] / (1.0 + M * (4.0e-4 * (TN - REFTEMP) - gmaold));
  const double tJctPot = pbfact + fact2 * pbo;
  const double gmanew = (tJctPot - pbo) / pbo;
  tJctCap *= 1.0 + M * (4.0e-4 * (T - REFTEMP) - gmanew);
  const double tSatCur = IS * std::exp(((T / TN) - 1.0) * EG / (N * vt) + XTI / N * std::log(T / TN));
  const double xfc = std::log(1.0 - FC);
  const double vte = N * vt;
  const double NR = p[XG_DIODE_NR], NBV = p[XG_DIODE_NBV];
  const double tSatCurR = p[XG_DIODE_ISR] * std::exp((T / TN - 1.0) * EG / (NR * vt) + XTI / NR * std::log(T / TN));
  const double area = p[XG_DIODE_AREA];
  // N_DEV_Diode.C:1520-1529: IKF, RS and BV at the device temperature
  const double RS = p[XG_DIODE_RS] * (1 + (T - TN) * (p[XG_DIODE_TRS1] + p[XG_DIODE_TRS2] * (T - TN)));
  m.tVcrit = vte * std::log(vte / (std::sqrt(2.0) * (tSatCur == 0.0 ? 1e-14 : tSatCur)));
  m.bvGiven = p[XG_DIODE_BVGIVEN] != 0.0;
  m.tBrkdwnV = 0.0;
  if (m.bvGiven) {
    const double BV = p[XG_DIODE_BV] * (1 + (T - TN) * (p[XG_DIODE_TBV1] + p[XG_DIODE_TBV2] * (T - TN)));
    const double cbv = p[XG_DIODE_IBV];
    double xbv;
    if (cbv < tSatCur * BV / vt) {
      xbv = BV;
    } else {
      const double tol = 1.0e-3 * cbv;
      xbv = BV - NBV * vt * std::log(1.0 + cbv / tSatCur);
      for (int i = 0; i < 25; ++i) {
        xbv = BV - NBV * vt * std::log(cbv / tSatCur + 1.0 - xbv / vt);
        const double xcbv = tSatCur * (std::exp((BV - xbv) / (NBV * vt)) - 1.0 + xbv / vt);
        if (std::fabs(xcbv - cbv) <= tol) break;
      }
    }
    m.tBrkdwnV = xbv;
  }
  // sidewall junction, scaled by the perimeter PJ as the bottom is by AREA
  const double VJSW = p[XG_DIODE_VJSW], MJSW = p[XG_DIODE_MJSW], FCS = p[XG_DIODE_FCS];
  const double NS = p[XG_DIODE_NS], PJ = p[XG_DIODE_PJ];
  const double pboSW = (VJSW - pbfact1) / fact1;
  const double gmaSWold = (VJSW - pboSW) / pboSW;
  double tJctSWCap = p[XG_DIODE_CJSW] / (1.0 + MJSW * (4.0e-4 * (TN - REFTEMP) - gmaSWold));
  const double tJctSWPot = pbfact + fact2 * pboSW;
  const double gmaSWnew = (tJctSWPot - pboSW) / pboSW;
  tJctSWCap *= 1.0 + MJSW * (4.0e-4 * (T - REFTEMP) - gmaSWnew);
  const double tSatSWCur =
      p[XG_DIODE_JSW] * std::exp(((T / TN) - 1.0) * EG / (NS * vt) + XTI / NS * std::log(T / TN));
  const double xfcs = std::log(1.0 - FCS);
  m.sw = p[XG_DIODE_JSW] != 0.0 ? (p[XG_DIODE_NSGIVEN] != 0.0 ? 1 : 2) : 0;
  m.IsatSW = tSatSWCur * PJ;
  m.VteSW = NS * vt;
  m.CzeroSW = tJctSWCap * PJ;
  m.tJctSWPot = tJctSWPot;
  m.tDepSWCap = FCS * tJctSWPot;
  m.F2SW = std::exp((1.0 + MJSW) * xfcs);
  m.F3SW = 1.0 - FCS * (1.0 + MJSW);
  m.MJSW = MJSW;
  m.Isat = tSatCur * area;
  if (m.sw == 2) m.Isat = m.Isat + m.IsatSW;  // one characteristic carries both
  m.IsatR = tSatCurR * area;
  m.Vte = vte;
  m.VteR = NR * vt;
  m.VteBRK = NBV * vt;
  m.Gspr = (RS != 0.0 ? 1.0 / RS : 0.0) * area;
  m.tIKF = p[XG_DIODE_IKF] * (1 + p[XG_DIODE_TIKF] * (T - TN));
  m.tJctPot = tJctPot;
  m.tJctCap = tJctCap * area;  // Czero = tJctCap * Area
  m.tDepCap = FC * tJctPot;
  m.tF1 = tJctPot * (1.0 - std::exp((1.0 - M) * xfc)) / (1.0 - M);
  m.F2 = std::exp((1.0 + M) * xfc);
  m.F3 = 1.0 - FC * (1.0 + M);
  m.M = M;
  m.TT = p[XG_DIODE_TT];
  return m;
}

Mos1Instance mos1_instance(const double *p) {
  Mos1Instance r{};
  Mos1Model &m = r.model;
  const double temp = p[XG_MOS1_TEMP], tnom = p[XG_MOS1_TNOM];
  const double dtype = p[XG_MOS1_TYPE];
  const double fact1 = tnom / REFTEMP, fact2 = temp / REFTEMP;
  const double vtnom = tnom * KOVERQ, vt = temp * KOVERQ;
  const double egfet1 = egap(tnom), egfet = egap(temp);
  const double pbfact1 = pb_factor(tnom), pbfact = pb_factor(temp);
  const double ratio = temp / tnom;
  const double ratio4 = ratio * std::sqrt(ratio);
  const double oxideCapFactor = (p[XG_MOS1_TOX] == 0.0) ? 0.0 : 3.9 * 8.854214871e-12 / p[XG_MOS1_TOX];
  const double tTrans = p[XG_MOS1_KP] / ratio4;
  const double phi = p[XG_MOS1_PHI], gamma = p[XG_MOS1_GAMMA];
  const double phio = (phi - pbfact1) / fact1;
  const double tPhi = fact2 * phio + pbfact;
  r.tVbi = p[XG_MOS1_VTO] - dtype * (gamma * std::sqrt(phi)) + .5 * (egfet1 - egfet) +
           dtype * .5 * (tPhi - phi);
  const double tSatCur = p[XG_MOS1_IS] * std::exp(-egfet / vt + egfet1 / vtnom);
  const double tSatCurDens = p[XG_MOS1_JS] * std::exp(-egfet / vt + egfet1 / vtnom);
  const double pb = p[XG_MOS1_PB], mj = p[XG_MOS1_MJ], mjsw = p[XG_MOS1_MJSW], fc = p[XG_MOS1_FC];
  const double pbo = (pb - pbfact1) / fact1;
  const double gmaold = (pb - pbo) / pbo;
  double capfact = 1 / (1 + mj * (4e-4 * (tnom - REFTEMP) - gmaold));
  double tCbd = p[XG_MOS1_CBD] * capfact, tCbs = p[XG_MOS1_CBS] * capfact, tCj = p[XG_MOS1_CJ] * capfact;
  capfact = 1 / (1 + mjsw * (4e-4 * (tnom - REFTEMP) - gmaold));
  double tCjsw = p[XG_MOS1_CJSW] * capfact;
  const double tBulkPot = fact2 * pbo + pbfact;
  const double gmanew = (tBulkPot - pbo) / pbo;
  capfact = 1 + mj * (4e-4 * (temp - REFTEMP) - gmanew);
  tCbd *= capfact; tCbs *= capfact; tCj *= capfact;
  tCjsw *= 1 + mjsw * (4e-4 * (temp - REFTEMP) - gmanew);
  const double tDepCap = fc * tBulkPot;
  const double AD = p[XG_MOS1_AD], AS = p[XG_MOS1_AS], PD = p[XG_MOS1_PD], PS = p[XG_MOS1_PS];
  const double js = p[XG_MOS1_JS];
  if (js == 0 || AD == 0 || AS == 0) {
    m.sourceVcrit = m.drainVcrit = vt * std::log(vt / (std::sqrt(2.0) * p[XG_MOS1_IS]));
  } else {
    m.drainVcrit = vt * std::log(vt / (std::sqrt(2.0) * js * AD));
    m.sourceVcrit = vt * std::log(vt / (std::sqrt(2.0) * js * AS));
  }
  const double czbd = (p[XG_MOS1_CBD] != 0) ? tCbd : ((p[XG_MOS1_CJ] != 0) ? tCj * AD : 0);
  const double czbdsw = (p[XG_MOS1_CJSW] != 0) ? tCjsw * PD : 0;
  const double czbs = (p[XG_MOS1_CBS] != 0) ? tCbs : ((p[XG_MOS1_CJ] != 0) ? tCj * AS : 0);
  const double czbssw = (p[XG_MOS1_CJSW] != 0) ? tCjsw * PS : 0;
  const double a = 1 - fc;
  const double sarg = std::exp(-mj * std::log(a)), sargsw = std::exp(-mjsw * std::log(a));
  m.Cbd = czbd; m.Cbdsw = czbdsw; m.Cbs = czbs; m.Cbssw = czbssw;
  m.f2d = czbd * (1 - fc * (1 + mj)) * sarg / a + czbdsw * (1 - fc * (1 + mjsw)) * sargsw / a;
  m.f3d = czbd * mj * sarg / a / tBulkPot + czbdsw * mjsw * sargsw / a / tBulkPot;
  m.f4d = czbd * tBulkPot * (1 - a * sarg) / (1 - mj) + czbdsw * tBulkPot * (1 - a * sargsw) / (1 - mjsw) -
          m.f3d / 2 * (tDepCap * tDepCap) - tDepCap * m.f2d;
  m.f2s = czbs * (1 - fc * (1 + mj)) * sarg / a + czbssw * (1 - fc * (1 + mjsw)) * sargsw / a;
  m.f3s = czbs * mj * sarg / a / tBulkPot + czbssw * mjsw * sargsw / a / tBulkPot;
  m.f4s = czbs * tBulkPot * (1 - a * sarg) / (1 - mj) + czbssw * tBulkPot * (1 - a * sargsw) / (1 - mjsw) -
          m.f3s / 2 * (tDepCap * tDepCap) - tDepCap * m.f2s;
  if (tSatCurDens == 0 || AD == 0 || AS == 0) {
    m.DrainSatCur = tSatCur; m.SourceSatCur = tSatCur;
  } else {
    m.DrainSatCur = tSatCurDens * AD; m.SourceSatCur = tSatCurDens * AS;
  }
  const double W = p[XG_MOS1_W], L = p[XG_MOS1_L], Leff = L - 2 * p[XG_MOS1_LD];
  r.beta = tTrans * W / Leff;
  m.dtype = dtype;
  m.gamma = gamma;
  m.tPhi = tPhi;
  m.gammaSqrtPhi = gamma * std::sqrt(tPhi);
  m.lambda = p[XG_MOS1_LAMBDA];
  m.vt = vt;
  m.gsatD = m.DrainSatCur / vt;
  m.gsatS = m.SourceSatCur / vt;
  // per-evaluation terms that depend on the model only (the device computes
  // the same IEEE operations on the same operands when it needs them)
  m.gbdR = m.gsatD + kGmin;
  m.gbsR = m.gsatS + kGmin;
  m.sqrtPhi = std::sqrt(tPhi);
  m.argPhi = (m.sqrtPhi <= 0) ? 0.0 : gamma / (m.sqrtPhi + m.sqrtPhi);
  m.OxideCap = oxideCapFactor * Leff * W;
  m.Cgso = p[XG_MOS1_CGSO] * W;
  m.Cgdo = p[XG_MOS1_CGDO] * W;
  m.Cgbo = p[XG_MOS1_CGBO] * Leff;
  m.tDepCap = tDepCap;
  m.tBulkPot = tBulkPot;
  m.MJ = mj;
  m.MJSW = mjsw;
  m.M = p[XG_MOS1_M];
  m.has_gate_caps = (m.OxideCap != 0.0 || m.Cgso != 0.0 || m.Cgdo != 0.0 || m.Cgbo != 0.0) ? 1 : 0;
  m.has_junc_caps = (czbd != 0 || czbdsw != 0 || czbs != 0 || czbssw != 0) ? 1 : 0;
  r.valid = (Leff > 0) && (W > 0);
  return r;
}

}  // namespace xg
