// xg_lu.cu — level-scheduled sparse LU refactorization and solves (sm_103a).
//
// Replaces the KLU numeric factorization + solve that Xyce runs on every
// Newton iteration (src/LinearAlgebraServicesPKG/N_LAS_AmesosSolver.C:358-396).
// Pivots are frozen by the host analysis (xg_symbolic.cpp); every column of
// a level is independent, one warp per column, left-looking:
//   load column j of A'  ->  for each U(k,j), k ascending: col_j -= L(:,k) * U(k,j)
//   ->  threshold test of the diagonal against the updated column
//       (kRuntimePivotTol); failing columns raise a breakdown flag so the
//       host re-pivots  ->  L(:,j) /= U(j,j).
// The triangular solves are row-oriented (gather, no atomics), 8 lanes per row.
#include <cuda_runtime.h>

#include "xg_internal.h"

namespace xg {

__device__ __forceinline__ int find_row(const int *ri, int lo, int hi, int key) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ri[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_lu_factor_level(LUDev L, const double *__restrict__ vals, const int *cols, int count,
                                  CircState *cs, int masked, double pivot_tol) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const int j = cols[w];
  if (masked) {
    const CircState &s = cs[L.circ_of_step[j]];
    if (!s.need_solve || (s.phase != PH_DC && s.phase != PH_TRAN)) return;
  }
  const int p0 = L.cp[j], p1 = L.cp[j + 1], pd = L.diag[j];
  double *lu = L.lu;
  for (int p = p0 + lane; p < p1; p += 32) {
    const int s = L.src[p];
    lu[p] = (s >= 0) ? vals[s] : 0.0;
  }
  __syncwarp();
  bool lost = false;
  for (int p = p0; p < pd; ++p) {
    const int k = L.ri[p];
    const double ukj = lu[p];
    if (ukj != 0.0) {
      const int q1 = L.cp[k + 1];
      for (int q = L.diag[k] + 1 + lane; q < q1; q += 32) {
        const int i = L.ri[q];
        const int pos = find_row(L.ri, p + 1, p1, i);
        if (pos < p1 && L.ri[pos] == i) lu[pos] -= lu[q] * ukj;
        else lost = true;
      }
    }
    __syncwarp();
  }
  const double d = lu[pd];
  double amax = 0.0;
  for (int p = pd + lane; p < p1; p += 32) amax = fmax(amax, fabs(lu[p]));
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  lost = __any_sync(0xffffffffu, lost);
  // The threshold only matters when row j of U has entries right of the
  // diagonal: otherwise the multipliers never reach the Schur complement
  // (e.g. the branch row of a grounded voltage source).
  const bool urow = L.u_ptr[j + 1] > L.u_ptr[j] && !L.exempt[j];
  const bool bad = lost || (urow && !(fabs(d) >= pivot_tol * amax)) || !(fabs(d) > 0.0) || isinf(d);
  if (bad) {
    if (lane == 0) {
      atomicCAS(L.breakdown, 0, j + 1);
      if (masked) cs[L.circ_of_step[j]].singular = 1;
    }
    return;
  }
  const double inv = 1.0 / d;
  for (int p = pd + 1 + lane; p < p1; p += 32) lu[p] *= inv;
}

// y[i] = b[row_of_step[i]] - sum_k L(i,k) y[k]
__global__ void k_lu_lsolve_level(LUDev L, const double *__restrict__ b, const int *rows, int count,
                                  const CircState *cs, int masked) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int sub = threadIdx.x & 7;
  if (g >= count) return;
  const int i = rows[g];
  if (masked) {
    const CircState &s = cs[L.circ_of_step[i]];
    if (!s.need_solve || s.singular || (s.phase != PH_DC && s.phase != PH_TRAN)) return;
  }
  double sum = 0.0;
  for (int t = L.l_ptr[i] + sub; t < L.l_ptr[i + 1]; t += 8) sum += L.lu[L.l_pos[t]] * L.y[L.l_col[t]];
  for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
  if (sub == 0) L.y[i] = b[L.row_of_step[i]] - sum;
}

// z[k] = (y[k] - sum_j U(k,j) z[j]) / U(k,k);  x[col_of_step[k]] = z[k]
__global__ void k_lu_usolve_level(LUDev L, double *__restrict__ x, const int *rows, int count,
                                  const CircState *cs, int masked) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int sub = threadIdx.x & 7;
  if (g >= count) return;
  const int k = rows[g];
  if (masked) {
    const CircState &s = cs[L.circ_of_step[k]];
    if (!s.need_solve || s.singular || (s.phase != PH_DC && s.phase != PH_TRAN)) return;
  }
  double sum = 0.0;
  for (int t = L.u_ptr[k] + sub; t < L.u_ptr[k + 1]; t += 8) sum += L.lu[L.u_pos[t]] * L.y[L.u_col[t]];
  for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
  if (sub == 0) {
    const double z = (L.y[k] - sum) / L.lu[L.diag[k]];
    L.y[k] = z;
    x[L.col_of_step[k]] = z;
  }
}

void launch_lu_factor_k(cudaStream_t st, const LUDev &L, const double *vals, CircState *cs, int masked,
                        double pivot_tol) {
  const int nl = (int)L.h_f_lvl.size() - 1;
  for (int l = 0; l < nl; ++l) {
    const int cnt = L.h_f_lvl[l + 1] - L.h_f_lvl[l];
    if (cnt <= 0) continue;
    const int threads = 128;
    const int blocks = (cnt * 32 + threads - 1) / threads;
    k_lu_factor_level<<<blocks, threads, 0, st>>>(L, vals, L.f_cols + L.h_f_lvl[l], cnt, cs, masked,
                                                  pivot_tol);
  }
}

void launch_lu_solve_k(cudaStream_t st, const LUDev &L, const double *b, double *x, const CircState *cs,
                       int masked) {
  const int threads = 128;
  const int nl = (int)L.h_l_lvl.size() - 1;
  for (int l = 0; l < nl; ++l) {
    const int cnt = L.h_l_lvl[l + 1] - L.h_l_lvl[l];
    if (cnt <= 0) continue;
    k_lu_lsolve_level<<<(cnt * 8 + threads - 1) / threads, threads, 0, st>>>(L, b, L.l_rows + L.h_l_lvl[l],
                                                                             cnt, cs, masked);
  }
  const int nu = (int)L.h_u_lvl.size() - 1;
  for (int l = 0; l < nu; ++l) {
    const int cnt = L.h_u_lvl[l + 1] - L.h_u_lvl[l];
    if (cnt <= 0) continue;
    k_lu_usolve_level<<<(cnt * 8 + threads - 1) / threads, threads, 0, st>>>(L, x, L.u_rows + L.h_u_lvl[l],
                                                                             cnt, cs, masked);
  }
}

}  // namespace xg
