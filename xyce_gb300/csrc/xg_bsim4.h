// xg_bsim4.h — BSIM 4.8.2 (Xyce level 54) instance data shared by the host
// set-up (xg_bsim4_params.cpp) and the evaluation kernel (xg_bsim4.cuh).
//
// Scope of the restatement: the default model selection (capMod 2, mobMod 0,
// dioMod 1; rdsMod, rgateMod, rbodyMod, igcMod, igbMod, trnqsMod, acnqsMod,
// mtrlMod, tempMod, gidlMod, wpemod 0), no binning, no stress (SA/SB), NF 1,
// RSH 0 (no internal nodes), device temperature = TNOM.
#pragma once
#include <string>

namespace xg {
namespace b4 {

// Constants: src/DeviceModelPKG/Core/N_DEV_Const.h:42-104 and the BSIM4
// overrides at src/DeviceModelPKG/OpenModels/N_DEV_MOSFET_B4p82.C:65-96.
constexpr double kEps0 = 8.85418e-12;
constexpr double kEpsSi = 1.03594e-10;
constexpr double kQ = 1.6021918e-19;
constexpr double kChargeQ = 1.60219e-19;
constexpr double kBoltz = 1.3806226e-23;
constexpr double kKboQ = 8.617087e-5;
constexpr double kVt0 = kBoltz * (27.0 + 273.15) / kQ;
constexpr double kExpThr = 34.0;
constexpr double kMaxExp = 5.834617425e14;
constexpr double kMinExp = 1.713908431e-15;
constexpr double kDelta1 = 0.02, kDelta3 = 0.02, kDelta4 = 0.02;
constexpr double kTnom = 300.15;   // DeviceOptions tnom / temp default (27 C)
constexpr double kGminB4 = 1.0e-12;

// One evaluated card: Model::processParams4p82_ + updateTemperature4p82_
// (N_DEV_MOSFET_B4p82.C:346-2744, 7769-8136) for one (card, L, W) instance
// geometry.  Plain data, read by the kernel from a deduplicated table.
struct B4Model {
  double dtype, M;
  // model-level
  double toxe, toxp, coxe, coxp, epsrox, vtm, vtm0, factor1, vcrit;
  double PhiBS, PhiBD, PhiBSWS, PhiBSWD, PhiBSWGS, PhiBSWGD;
  double MJS, MJD, MJSWS, MJSWD, MJSWGS, MJSWGD, NJS, NJD, xpart;
  double ados, bdos;
  // size-dependent (paramPtr->*)
  double leff, weff, leffCV, weffCV, weffCJ;
  double cdsc, cdscb, cdscd, cit, nfactor, xj, a0, ags, a1, a2, keta, ngate, k1, k2, k3, k3b, w0;
  double dvt0, dvt1, dvt2, dvt0w, dvt1w, dvt2w, lpe0, lpeb, dvtp0, dvtp1, etab, ua, ub, uc, ud;
  double b0, b1, dwg, dwb, prwg, prwb, pclm, pdiblb, pvag, delta, fprout, pdits, pditsd, pditsl;
  double pscbe1, pscbe2, alpha0, alpha1, beta0, agidl, bgidl, cgidl, egidl, agisl, bgisl, cgisl, egisl;
  double cgsl, cgdl, ckappas, ckappad, noff, voffcv, acde, moin;
  double abulkCVfactor, rds0, rdswmin, u0temp, vsattemp, litl, vbi, phi, sqrtPhi, Xdep0, vfbsd;
  double cdep0, mstar, mstarcv, voffcbn, voffcbncv, ldeb, k1ox, theta0vb0, thetaRout, vfbzbfactor;
  double cgdo, cgso, cgbo;
  // instance-level
  double vth0, eta0, k2ox, vtfbphi1, vtfbphi2, vbsc, vfbzb, vfb;
  double Aseff, Adeff, Pseff, Pdeff;
  double SourceSatCurrent, DrainSatCurrent, vjsmFwd, IVjsmFwd, vjdmFwd, IVjdmFwd;
  double czbs, czbd, czbssw, czbdsw, czbsswg, czbdswg;
};

// Builds a B4Model from an XG_B4_* row (NaN = not given); returns XG_OK or
// XG_ERR_UNSUPPORTED / XG_ERR_ARG with *why.
int setup(const double *row, B4Model &I, std::string *why);

}  // namespace b4
}  // namespace xg
