// xg_lu_dev.cuh — device functions of the LU sweeps shared by the grouped
// kernels (xg_lu.cu) and the circuit-resident tick (xg_kernels.cu): the
// per-column factorization, the pivot test, and the row dot products of the
// triangular solves.  Each computes the same bits whatever team of threads
// runs it, so a column or row gives the same result in every kernel.
#pragma once
#include <cuda_runtime.h>

#include "xg_internal.h"

namespace xg {

__device__ __forceinline__ bool item_active(const LUDev &L, const CircState *cs, int masked, int j) {
  if (!masked) return true;
  const CircState &s = cs[L.circ_of_step[j]];
  return s.need_solve && !s.singular && (s.phase == PH_DC || s.phase == PH_TRAN);
}

// A column is refactored this tick when its circuit has LU work and its
// Jacobian changed since its last factorization (CircState::refactor).
__device__ __forceinline__ bool factor_active(const LUDev &L, const CircState *cs, int masked, int j) {
  if (!masked) return true;
  const CircState &s = cs[L.circ_of_step[j]];
  return s.need_solve && s.refactor && !s.singular && (s.phase == PH_DC || s.phase == PH_TRAN);
}

// A group of one circuit that has no LU work this tick returns at once
// (before staging anything); packed groups (gcirc < 0) test their items.
__device__ __forceinline__ bool group_idle(const LUDev &L, const CircState *cs, int masked, const int *gcirc,
                                          int g) {
  if (!masked || !gcirc) return false;
  const int c = gcirc[g];
  if (c < 0) return false;
  const CircState &s = cs[c];
  return !(s.need_solve && !s.singular && (s.phase == PH_DC || s.phase == PH_TRAN));
}

// The same for a factor group: also idle when its circuit reuses its factors.
__device__ __forceinline__ bool factor_group_idle(const LUDev &L, const CircState *cs, int masked, const int *gcirc,
                                                 int g) {
  if (!masked || !gcirc) return false;
  const int c = gcirc[g];
  if (c < 0) return false;
  const CircState &s = cs[c];
  return !(s.need_solve && s.refactor && !s.singular && (s.phase == PH_DC || s.phase == PH_TRAN));
}

template <bool BLOCK>
__device__ __forceinline__ void team_sync() {
  if (BLOCK) __syncthreads();
  else __syncwarp();
}

// max over the team (warp or whole CTA); every thread gets the result
template <bool BLOCK>
__device__ __forceinline__ double team_max(double v, double *sm) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (!BLOCK) return v;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sm[w]);
  return r;
}

// Zero tests and magnitude maxima of the factorization run on the integer
// pipe: GB300's FP64 pipe is narrow and a warp-wide FP64 instruction costs
// the same with one active lane as with 32.
__device__ __forceinline__ bool nz(double v) { return (__double_as_longlong(v) << 1) != 0; }
__device__ __forceinline__ bool nz(float v) { return (__float_as_uint(v) << 1) != 0u; }
// |v| as an integer key ordered like |v|; NaN maps to 0 (ignored, as by fmax)
__device__ __forceinline__ unsigned long long mag_key(double v) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
  return a > 0x7ff0000000000000ULL ? 0ULL : a;
}
__device__ __forceinline__ unsigned long long mag_key(float v) {
  const unsigned a = __float_as_uint(v) & 0x7fffffffu;
  return a > 0x7f800000u ? 0ULL : (unsigned long long)a;
}
template <typename T> __device__ __forceinline__ double key_value(unsigned long long k);
template <> __device__ __forceinline__ double key_value<double>(unsigned long long k) {
  return __longlong_as_double((long long)k);
}
template <> __device__ __forceinline__ double key_value<float>(unsigned long long k) {
  return (double)__uint_as_float((unsigned)k);
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}
// max of keys over the team (warp or whole CTA); every thread gets the result
template <bool BLOCK>
__device__ __forceinline__ unsigned long long team_max_key(unsigned long long v, double *sm) {
  for (int o = 16; o > 0; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (!BLOCK) return v;
  unsigned long long *su = reinterpret_cast<unsigned long long *>(sm);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) su[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long r = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = umax64(r, su[w]);
  return r;
}
template <bool BLOCK>
__device__ __forceinline__ bool team_any(bool v) {
  if (BLOCK) return __syncthreads_or(v) != 0;
  return __any_sync(0xffffffffu, v) != 0;
}


// Factor values of precision T: L.lu (FP64) or L.lu32 (FP32, refined solves).
template <typename T> __device__ __forceinline__ T *lu_of(const LUDev &L);
template <> __device__ __forceinline__ double *lu_of<double>(const LUDev &L) { return L.lu; }
template <> __device__ __forceinline__ float *lu_of<float>(const LUDev &L) { return L.lu32; }

// Pivot test and scaling of column j once its updates are in: d = U(j,j),
// amax = the largest |L(:,j)| entry (as a key), lost = an update that missed
// the pattern.  Returns false on breakdown (flag raised by `leader`).
__device__ __forceinline__ bool pivot_ok_u(const LUDev &L, int j, CircState *cs, int masked, double pivot_tol,
                                           double d, double amax, bool lost, bool leader, bool urow) {
  const bool bad = lost || (urow && !(fabs(d) >= pivot_tol * amax)) || !(fabs(d) > 0.0) || isinf(d);
  if (bad && leader) {
    atomicCAS(L.breakdown, 0, j + 1);
    if (masked) cs[L.circ_of_step[j]].singular = 1;
  }
  return !bad;
}

__device__ __forceinline__ bool pivot_ok(const LUDev &L, int j, CircState *cs, int masked, double pivot_tol,
                                         double d, double amax, bool lost, bool leader) {
  // The threshold only matters when row j of U has entries right of the
  // diagonal: otherwise the multipliers never reach the Schur complement
  // (e.g. the branch row of a grounded voltage source).  An exempt column's
  // threshold is scaled down (kExemptSlack).
  const bool urow = L.u_ptr[j + 1] > L.u_ptr[j];
  const double tol = L.exempt[j] ? pivot_tol * L.pscale[j] : pivot_tol;
  return pivot_ok_u(L, j, cs, masked, tol, d, amax, lost, leader, urow);
}

template <bool BLOCK, typename T>
__device__ void factor_column(const LUDev &L, const double *__restrict__ vals, int j, CircState *cs,
                              int masked, double pivot_tol, double *sm) {
  const int lane = BLOCK ? (int)threadIdx.x : (int)(threadIdx.x & 31);
  const int nl = BLOCK ? (int)blockDim.x : 32;
  const int p0 = L.cp[j], p1 = L.cp[j + 1], pd = L.diag[j];
  T *lu = lu_of<T>(L);
  for (int p = p0 + lane; p < p1; p += nl) {
    const int s = L.src[p];
    lu[p] = (s >= 0) ? (T)vals[s] : (T)0;
  }
  team_sync<BLOCK>();
  bool lost = false;
  for (int p = p0; p < pd; ++p) {
    const int4 um = L.umeta[p];
    const T ukj = lu[p];
    if (nz(ukj)) {
      // positions of L(:,k)'s rows in column j come from the analysis
      const int *tgt = L.upd_pos + um.z;
      const T *lk = lu + um.w;
      for (int q = lane; q < um.y; q += nl) {
        const int pos = tgt[q];
        if (pos > p && pos < p1) lu[pos] -= lk[q] * ukj;
        else lost = true;
      }
    }
    team_sync<BLOCK>();
  }
  unsigned long long ak = 0;
  for (int p = pd + lane; p < p1; p += nl) ak = umax64(ak, mag_key(lu[p]));
  ak = team_max_key<BLOCK>(ak, sm);
  lost = team_any<BLOCK>(lost);
  if (!pivot_ok(L, j, cs, masked, pivot_tol, (double)lu[pd], key_value<T>(ak), lost, lane == 0)) return;
  const T inv = (T)1 / lu[pd];
  for (int p = pd + 1 + lane; p < p1; p += nl) lu[p] *= inv;
}

// A short column on one thread.  S: a shared-memory buffer of staged
// columns (column k at S[soff[k]]; umeta[p].x the buffer offset of
// L(k+1.., k), as LUDev::umeta), or nullptr to factor in place in global
// memory.
template <typename T>
__device__ void factor_column_t(const LUDev &L, const double *__restrict__ vals, int j, CircState *cs,
                                int masked, double pivot_tol, T *S, const int *soff, const int4 *umeta) {
  const int p0 = L.cp[j], p1 = L.cp[j + 1], pd = L.diag[j];
  T *glu = lu_of<T>(L);
  T *cj = S ? S + soff[j] : glu + p0;  // cj[p - p0]
  if (!S)
    for (int p = p0; p < p1; ++p) {
      const int s = L.src[p];
      cj[p - p0] = (s >= 0) ? (T)vals[s] : (T)0;
    }
  bool lost = false;
  for (int p = p0; p < pd; ++p) {
    const int4 um = umeta[p];
    const T ukj = cj[p - p0];
    if (!nz(ukj)) continue;
    const T *lk = (S && um.x >= 0) ? S + um.x : glu + um.w;
    const int *tgt = L.upd_pos + um.z;
    // four targets and sources loaded before their updates: one latency per
    // four products
    for (int q = 0; q < um.y; q += 4) {
      int t[4];
      T l[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (q + u < um.y) { t[u] = tgt[q + u]; l[u] = lk[q + u]; }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (q + u < um.y) {
          const int pos = t[u];
          if (pos > p && pos < p1) cj[pos - p0] -= l[u] * ukj;
          else lost = true;
        }
    }
  }
  unsigned long long ak = 0;
  for (int p = pd; p < p1; ++p) ak = umax64(ak, mag_key(cj[p - p0]));
  if (!pivot_ok(L, j, cs, masked, pivot_tol, (double)cj[pd - p0], key_value<T>(ak), lost, true)) return;
  const T inv = (T)1 / cj[pd - p0];
  for (int p = pd + 1; p < p1; ++p) cj[p - p0] *= inv;
}

// A column in a shared-memory buffer of staged columns (see
// factor_column_t), by a warp (BLOCK false) or the whole CTA.  L columns of
// columns outside the buffer (umeta[p].x < 0) are read from global memory.
template <bool BLOCK, typename T>
__device__ void factor_column_s(const LUDev &L, int j, CircState *cs, int masked, double pivot_tol, double *sm,
                                T *S, const int *soff, const int4 *umeta) {
  const int lane = BLOCK ? (int)threadIdx.x : (int)(threadIdx.x & 31);
  const int nl = BLOCK ? (int)blockDim.x : 32;
  const int p0 = L.cp[j], p1 = L.cp[j + 1], pd = L.diag[j];
  T *cj = S + soff[j];  // cj[p - p0]
  const T *glu = lu_of<T>(L);
  bool lost = false;
  for (int p = p0; p < pd; ++p) {
    const int4 um = umeta[p];
    const T ukj = cj[p - p0];
    if (nz(ukj)) {
      const T *lk = (um.x >= 0) ? S + um.x : glu + um.w;
      const int *tgt = L.upd_pos + um.z;
      for (int q = lane; q < um.y; q += nl) {
        const int pos = tgt[q];
        if (pos > p && pos < p1) cj[pos - p0] -= lk[q] * ukj;
        else lost = true;
      }
    }
    team_sync<BLOCK>();
  }
  unsigned long long ak = 0;
  for (int p = pd + lane; p < p1; p += nl) ak = umax64(ak, mag_key(cj[p - p0]));
  ak = team_max_key<BLOCK>(ak, sm);
  lost = team_any<BLOCK>(lost);
  if (!pivot_ok(L, j, cs, masked, pivot_tol, (double)cj[pd - p0], key_value<T>(ak), lost, lane == 0)) return;
  const T inv = (T)1 / cj[pd - p0];
  for (int p = pd + 1 + lane; p < p1; p += nl) cj[p - p0] *= inv;
}

// Dot product of a long row (more than kLongSolveRow entries) by the whole
// CTA in a summation order that does not depend on the CTA size: 256
// virtual lanes each sum the entries lane, lane + 256, ...; each virtual
// warp of 32 reduces by a butterfly; the 8 warp sums add in order.  (Every
// launch shape of a sweep then computes the same bits, so launch shapes can
// be chosen by timing alone.)  sm: 8 doubles; the result is in every thread.
constexpr int kRowLanes = 256;
template <typename T>
__device__ double long_row_dot(const T *__restrict__ lu, const int *__restrict__ pos, const int *__restrict__ col,
                               const double *y, int q0, int q1, double *sm) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  __syncthreads();
  for (int vw = warp; vw < kRowLanes / 32; vw += nwarps) {
    double s = 0.0;
    for (int q = q0 + vw * 32 + lane; q < q1; q += kRowLanes) s += (double)lu[pos[q]] * y[col[q]];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sm[vw] = s;
  }
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < kRowLanes / 32; ++w) r += sm[w];
  return r;
}

// y[i] = b[row_of_step[i]] - sum_k L(i,k) y[k]          (LOWER)
// y[i] = (y[i] - sum_j U(i,j) y[j]) / U(i,i); x[col_of_step[i]] = y[i]   (upper;
//   ACC: x[col_of_step[i]] += y[i], the correction step of a refined solve)
// Team: 8 lanes (width 8) or the whole CTA (BLOCK).  Factors of precision T,
// accumulation in FP64.
template <bool LOWER, bool BLOCK, typename T, bool ACC>
__device__ void solve_row(const LUDev &L, const double *__restrict__ b, double *__restrict__ x, int i,
                          int sub, double *sm) {
  const int *ptr = LOWER ? L.l_ptr : L.u_ptr;
  const int *pos = LOWER ? L.l_pos : L.u_pos;
  const int *col = LOWER ? L.l_col : L.u_col;
  const T *lu = lu_of<T>(L);
  double sum = 0.0;
  if (BLOCK) {
    sum = long_row_dot<T>(lu, pos, col, L.y, ptr[i], ptr[i + 1], sm);
  } else {
    for (int t = ptr[i] + sub; t < ptr[i + 1]; t += 8) sum += (double)lu[pos[t]] * L.y[col[t]];
    for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
  }
  if (sub == 0) {
    if (LOWER) {
      L.y[i] = b[L.row_of_step[i]] - sum;
    } else {
      const double z = (L.y[i] - sum) / (double)lu[L.diag[i]];
      L.y[i] = z;
      if (ACC) x[L.col_of_step[i]] += z;
      else x[L.col_of_step[i]] = z;
    }
  }
}


// Dot product of a short row (at most kThreadRow entries) on one thread:
// all indices are loaded, then all values, then summed in entry order, so a
// row costs two load latencies whatever its length.
template <typename T>
__device__ __forceinline__ double row_dot_t(const T *__restrict__ lu, const int *__restrict__ pos,
                                            const int *__restrict__ col, const double *y, int q0, int n) {
  int ps[kThreadRow], cl[kThreadRow];
#pragma unroll
  for (int u = 0; u < kThreadRow; ++u)
    if (u < n) { ps[u] = pos[q0 + u]; cl[u] = col[q0 + u]; }
  double a[kThreadRow], b[kThreadRow];
#pragma unroll
  for (int u = 0; u < kThreadRow; ++u)
    if (u < n) { a[u] = (double)lu[ps[u]]; b[u] = y[cl[u]]; }
  double sum = 0.0;
#pragma unroll
  for (int u = 0; u < kThreadRow; ++u)
    if (u < n) sum += a[u] * b[u];
  return sum;
}

}  // namespace xg
