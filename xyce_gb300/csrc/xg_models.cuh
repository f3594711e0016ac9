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

constexpr double kMaxExpArg = 100.0;   // CONSTMAX_EXP_ARG
constexpr double kE = 2.718281828459045235360287471352662498;  // CONSTe

// Comparisons of doubles on the integer pipe.  GB300 issues FP64 at a small
// fraction of its integer rate and the device evaluations are bound by the
// FP64 pipe, so their sign tests, comparisons and clamps run on the bit
// patterns instead.  For operands that are not NaN each helper returns what
// the FP64 operation returns, with +0 and -0 equal.  fkey maps a double to an
// integer of the same order: sign-magnitude to two's complement.
__device__ __forceinline__ long long fkey(double a) {
  const long long b = __double_as_longlong(a);
  const long long mag = b & 0x7fffffffffffffffLL;
  return b < 0 ? -mag : mag;
}
__device__ __forceinline__ bool f_lt(double a, double b) { return fkey(a) < fkey(b); }
__device__ __forceinline__ bool f_le(double a, double b) { return fkey(a) <= fkey(b); }
__device__ __forceinline__ bool f_le0(double a) { return __double_as_longlong(a) <= 0; }
__device__ __forceinline__ bool f_gt0(double a) { return __double_as_longlong(a) > 0; }
__device__ __forceinline__ bool f_lt0(double a) { return fkey(a) < 0; }
__device__ __forceinline__ bool f_ge0(double a) { return fkey(a) >= 0; }
__device__ __forceinline__ bool f_is0(double a) { return (__double_as_longlong(a) << 1) == 0; }
__device__ __forceinline__ bool f_is1(double a) { return __double_as_longlong(a) == 0x3ff0000000000000LL; }
__device__ __forceinline__ double f_min(double a, double b) { return f_le(a, b) ? a : b; }
__device__ __forceinline__ double f_max(double a, double b) { return f_le(b, a) ? a : b; }

__device__ __forceinline__ double pnjlim_d(double vnew, double vold, double vt, double vcrit,
                                           int &icheck) {
  // |vnew - vold| > 2 vt, with the magnitude taken from the bit pattern
  if (f_lt(vcrit, vnew) &&
      fkey(vt + vt) < (__double_as_longlong(vnew - vold) & 0x7fffffffffffffffLL)) {
    if (f_gt0(vold)) {
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
  if (f_le(3.5, vold)) {
    if (f_lt(vold, vnew)) vnew = f_min(vnew, 3.0 * vold + 2.0);
    else if (f_lt(vnew, 3.5)) vnew = f_max(vnew, 2.0);
  } else {
    vnew = f_lt(vold, vnew) ? f_min(vnew, 4.0) : f_max(vnew, -0.5);
  }
  return vnew;
}

// The limits are formed only on the paths that read them.  -delv > x is
// tested as fkey(x) < -fkey(delv) (negation is exact).
__device__ __forceinline__ double fetlim_d(double vnew, double vold, double vto) {
  auto hi = [&] { return fabs(2 * (vold - vto)) + 2; };  // vtsthi
  const double delv = vnew - vold;
  if (f_le(vto, vold)) {
    const double vtox = vto + 3.5;
    if (f_le(vtox, vold)) {
      if (f_le0(delv)) {
        if (f_le(vtox, vnew)) {
          const double vtstlo = hi() / 2 + 2;
          if (fkey(vtstlo) < -fkey(delv)) vnew = vold - vtstlo;
        } else {
          vnew = f_max(vnew, vto + 2.0);
        }
      } else {
        const double vtsthi = hi();
        if (f_le(vtsthi, delv)) vnew = vold + vtsthi;
      }
    } else {
      vnew = f_le0(delv) ? f_max(vnew, vto - 0.5) : f_min(vnew, vto + 4.0);
    }
  } else {
    if (f_le0(delv)) {
      const double vtsthi = hi();
      if (fkey(vtsthi) < -fkey(delv)) vnew = vold - vtsthi;
    } else {
      double vtemp = vto + 0.5;
      if (f_le(vnew, vtemp)) {
        const double vtstlo = hi() / 2 + 2;
        if (f_lt(vtstlo, delv)) vnew = vold + vtstlo;
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
