// xg_models.cuh — device-side model evaluation for the nonlinear devices.
//
// One thread evaluates one instance; instances are stored structure-of-arrays
// so that each per-instance field is a coalesced load.  The arithmetic
// restates, in FP64:
//   Diode::Instance::updateIntermediateVars   src/DeviceModelPKG/OpenModels/N_DEV_Diode.C:1072-1420
//   MOSFET1::Instance::updateIntermediateVars src/DeviceModelPKG/OpenModels/N_DEV_MOSFET1.C:2689-3477
//   DeviceSupport pnjlim/fetlim/limvds/qmeyer src/DeviceModelPKG/Core/N_DEV_DeviceSupport.C:161-590
#pragma once
#include "xg_internal.h"

namespace xg {

constexpr double kGmin = 1.0e-12;      // DeviceOptions gmin default
constexpr double kMaxExpArg = 100.0;   // CONSTMAX_EXP_ARG
constexpr double kE = 2.718281828459045235360287471352662498;  // CONSTe

__device__ __forceinline__ double pnjlim_d(double vnew, double vold, double vt, double vcrit,
                                           int &icheck) {
  if (vnew > vcrit && fabs(vnew - vold) > (vt + vt)) {
    if (vold > 0) {
      double arg = 1 + (vnew - vold) / vt;
      vnew = (arg > 0) ? vold + vt * log(arg) : vcrit;
    } else {
      vnew = vt * log(vnew / vt);
    }
    icheck = 1;
  } else {
    icheck = 0;
  }
  return vnew;
}

__device__ __forceinline__ double limvds_d(double vnew, double vold) {
  if (vold >= 3.5) {
    if (vnew > vold) vnew = fmin(vnew, 3.0 * vold + 2.0);
    else if (vnew < 3.5) vnew = fmax(vnew, 2.0);
  } else {
    vnew = (vnew > vold) ? fmin(vnew, 4.0) : fmax(vnew, -0.5);
  }
  return vnew;
}

__device__ __forceinline__ double fetlim_d(double vnew, double vold, double vto) {
  double vtsthi = fabs(2 * (vold - vto)) + 2;
  double vtstlo = vtsthi / 2 + 2;
  double vtox = vto + 3.5;
  double delv = vnew - vold;
  if (vold >= vto) {
    if (vold >= vtox) {
      if (delv <= 0) {
        if (vnew >= vtox) {
          if (-delv > vtstlo) vnew = vold - vtstlo;
        } else {
          vnew = fmax(vnew, vto + 2.0);
        }
      } else if (delv >= vtsthi) {
        vnew = vold + vtsthi;
      }
    } else {
      vnew = (delv <= 0) ? fmax(vnew, vto - 0.5) : fmin(vnew, vto + 4.0);
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

__device__ __forceinline__ void qmeyer_d(double vgs, double vgd, double von, double vdsat,
                                         double &capgs, double &capgd, double &capgb, double phi,
                                         double cox) {
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

// Bulk junction charge/capacitance of one side (N_DEV_MOSFET1.C:3100-3210).
__device__ __forceinline__ void mos1_junction(const Mos1Model &m, double v, double C, double Csw,
                                              double f2, double f3, double f4, double &q,
                                              double &cap) {
  q = 0.0; cap = 0.0;
  if (C != 0 || Csw != 0) {
    if (v < m.tDepCap) {
      double a = 1 - v / m.tBulkPot;
      double s1 = (m.MJ == .5) ? 1 / sqrt(a) : exp(-m.MJ * log(a));
      double s2 = (m.MJSW == .5) ? 1 / sqrt(a) : exp(-m.MJSW * log(a));
      q = m.tBulkPot * (C * (1 - a * s1) / (1 - m.MJ) + Csw * (1 - a * s2) / (1 - m.MJSW));
      cap = C * s1 + Csw * s2;
    } else {
      q = f4 + v * (f2 + v * (f3 / 2));
      cap = f2 + f3 * v;
    }
  }
}

}  // namespace xg
