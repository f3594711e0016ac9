// xg_lu.cu — sparse LU refactorization and triangular solves on the frozen
// pattern (sm_103a).
//
// Replaces the KLU numeric factorization + solve that Xyce runs on every
// Newton iteration (src/LinearAlgebraServicesPKG/N_LAS_AmesosSolver.C:358-396).
// Pivots are frozen by the host analysis (xg_symbolic.cpp).  Each sweep runs
// on a grouped schedule:
//   hubs   — items without dependencies that many others need (e.g. a supply
//            node's column), one CTA each;
//   groups — dependency-closed sets of columns/rows, one CTA each (64-512
//            threads, chosen by the analysis), a CTA barrier between local
//            levels (one ring of a Monte-Carlo batch is one group: its whole
//            factorization stays in one CTA).  A group's values — and, where
//            that costs no residency, its update metadata — are staged in
//            shared memory, walked there and written back once; solve groups
//            stage their rows' entries and their slice of y.  A group whose
//            circuit has no LU work this tick returns at once;
//   top    — what remains (the upper separators): pulled in parallel, then
//            factored right-looking in one CTA or a launch pair per level.
// Factorization is left-looking per column: load A'(:,j); for each U(k,j), k
// ascending: col_j -= L(:,k) U(k,j); threshold test of the diagonal against
// the updated column (kRuntimePivotTol; failures raise a breakdown flag and
// the host re-pivots); L(:,j) /= U(j,j).  Short columns run on one thread
// each when many groups run at once (GB300's FP64 pipe issues a warp-wide
// instruction at the same cost with 1 or 32 active lanes), else on a warp;
// long ones use the whole CTA.  Zero tests and pivot maxima run on the
// integer pipe.  The solves are row-oriented gathers (no atomics): a thread
// per short row, 8 lanes or the whole CTA for longer ones.  The U solve runs
// the factorization schedule backwards.
#include <cuda_runtime.h>

#include <algorithm>

#include <mutex>
#include <string>

#include "xg_internal.h"
#include "xg_lu_dev.cuh"

namespace xg {

constexpr int kGroupThreads = 512;  // largest group CTA (the analysis picks 64..512)

// The level pointers of a group's levels lv0 .. lv1 (at most kStagedLevels
// levels) copied into shared memory lvp[0 .. lv1 - lv0], so that the level
// loop does not wait on a global load per level; more levels are read in
// place.  Returns the array to index by lv - lv0; the caller's barrier
// after its staging makes the copy visible.
constexpr int kStagedLevels = 128;

// 1-D bulk copies (the TMA's cp.async.bulk) of contiguous global ranges into
// this CTA's shared memory, completing on one mbarrier.  Addresses and sizes
// are multiples of 16 bytes (the callers copy int4 arrays).
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long *mbar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void *dst, const void *src, unsigned bytes,
                                             unsigned long long *mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(mbar))
               : "memory");
}
// Waits (at most max_polls polls) for the mbarrier's phase 0 to complete.
__device__ __forceinline__ bool mbar_wait0(unsigned long long *mbar, int max_polls) {
  for (int i = 0; i < max_polls; ++i) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_addr(mbar))
        : "memory");
    if (done) return true;
  }
  return false;
}
constexpr int kBulkWaitPolls = 1 << 22;  // far beyond any copy's time; a timeout is reported as a breakdown
__device__ __forceinline__ const int *stage_levels(const SchedDev &S, int lv0, int lv1, int *lvp) {
  if (lv1 - lv0 > kStagedLevels) return S.lvl_ptr + lv0;
  for (int k = threadIdx.x; k <= lv1 - lv0; k += blockDim.x) lvp[k] = S.lvl_ptr[lv0 + k];
  return lvp;
}

void launch_lu_solve_k(cudaStream_t st, const LUDev &L, const double *b, double *x, const CircState *cs,
                       int masked);

// ---- factorization ----------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_factor_hubs(LUDev L, const double *__restrict__ vals, CircState *cs,
                                                     int masked, double pivot_tol) {
  __shared__ double sm[32];
  const int j = L.fs.items[blockIdx.x];
  if (!factor_active(L, cs, masked, j)) return;
  factor_column<true, T>(L, vals, j, cs, masked, pivot_tol, sm);
}

template <typename T>
__device__ void factor_group(const LUDev &L, const double *__restrict__ vals, CircState *cs, int masked,
                             double pivot_tol, double *sm, int g) {
  const SchedDev &S = L.fs;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  // one circuit's group (not idle: tested by the caller) or the top: test
  // the columns of the top and of groups that mix circuits only
  const bool multi = masked && (g >= S.n_groups || !L.fs_gcirc || L.fs_gcirc[g] < 0);
  for (int lv = S.grp_lvl[g]; lv < S.grp_lvl[g + 1]; ++lv) {
    const int b = S.lvl_ptr[lv], e = S.lvl_ptr[lv + 1];
    bool any_long = false;
    for (int t = b + (int)threadIdx.x; t < e; t += (int)blockDim.x) {
      const int j = S.items[t];
      if (S.is_thread[j] && (!multi || factor_active(L, cs, masked, j)))
        factor_column_t<T>(L, vals, j, cs, masked, pivot_tol, nullptr, L.grp_soff, L.umeta);
    }
    for (int t = b + warp; t < e; t += nwarps) {
      const int j = S.items[t];
      if (S.is_long[j]) { any_long = true; continue; }
      if (S.is_thread[j]) continue;
      if (!multi || factor_active(L, cs, masked, j)) factor_column<false, T>(L, vals, j, cs, masked, pivot_tol, sm);
    }
    if (__syncthreads_or(any_long)) {
      for (int t = b; t < e; ++t) {
        const int j = S.items[t];
        if (!S.is_long[j] || !(!multi || factor_active(L, cs, masked, j))) continue;
        factor_column<true, T>(L, vals, j, cs, masked, pivot_tol, sm);
        __syncthreads();
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) k_factor_groups(LUDev L, const double *__restrict__ vals, CircState *cs,
                                                        int masked, double pivot_tol, int top) {
  __shared__ double sm[32];
  if (!top && factor_group_idle(L, cs, masked, L.fs_gcirc, (int)blockIdx.x)) return;
  factor_group<T>(L, vals, cs, masked, pivot_tol, sm, top ? L.fs.n_groups : (int)blockIdx.x);
}

// ---- top of the factorization: pull, then right-looking -------------------
// When every L row of a top column is itself a top step (the analysis checks
// it; the top holds the upper separators of the nested dissection), the top
// columns first pull, in parallel (one warp each), the updates of every
// sub-tree column — all factored by then — and then one CTA factors the top
// right-looking in step order: pivot test and scaling of column k, then the
// rank-1 update of every column j with U(k, j) != 0 (a warp per U entry,
// lanes over L(:, k)).  One barrier pair per top column replaces the
// per-(column, row) barriers of the left-looking walk.
template <typename T>
__global__ void __launch_bounds__(256) k_top_pull(LUDev L, const double *__restrict__ vals, CircState *cs,
                                                   int masked) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (w >= L.n_top_rl) return;  // warp-uniform
  const int j = L.top_items[w];
  if (!factor_active(L, cs, masked, j)) return;
  T *lu = lu_of<T>(L);
  const int p0 = L.cp[j], p1 = L.cp[j + 1], pd = L.diag[j];
  for (int p = p0 + lane; p < p1; p += 32) {
    const int s = L.src[p];
    lu[p] = (s >= 0) ? (T)vals[s] : (T)0;
  }
  __syncwarp();
  bool lost = false;
  for (int p = p0; p < pd; ++p) {
    const int k = L.ri[p];
    if (L.is_top[k]) continue;  // the top's own updates come right-looking
    const T ukj = lu[p];
    if (ukj != (T)0) {
      const int q0 = L.diag[k] + 1, q1 = L.cp[k + 1];
      const int *tgt = L.upd_pos + L.upd_off[p];
      for (int q = q0 + lane; q < q1; q += 32) {
        const int pos = tgt[q - q0];
        if (pos > p && pos < p1) lu[pos] -= lu[q] * ukj;
        else lost = true;
      }
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, lost) && lane == 0) {
    atomicCAS(L.breakdown, 0, j + 1);
    if (masked) cs[L.circ_of_step[j]].singular = 1;
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) k_top_rl(LUDev L, CircState *cs, int masked, double pivot_tol) {
  __shared__ double sm[32];
  T *lu = lu_of<T>(L);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int t = 0; t < L.n_top_rl; ++t) {
    const int k = L.top_items[t];
    if (!factor_active(L, cs, masked, k)) continue;  // uniform: every thread reads the same flags
    const int pd = L.diag[k], p1 = L.cp[k + 1];
    double amax = 0.0;
    for (int p = pd + threadIdx.x; p < p1; p += blockDim.x) amax = fmax(amax, fabs((double)lu[p]));
    amax = team_max<true>(amax, sm);
    const double d = (double)lu[pd];
    const bool urow = L.u_ptr[k + 1] > L.u_ptr[k];
    const double tol = L.exempt[k] ? pivot_tol * L.pscale[k] : pivot_tol;
    const bool bad = (urow && !(fabs(d) >= tol * amax)) || !(fabs(d) > 0.0) || isinf(d);
    if (bad) {
      if (threadIdx.x == 0) {
        atomicCAS(L.breakdown, 0, k + 1);
        if (masked) cs[L.circ_of_step[k]].singular = 1;
      }
      if (!masked) return;  // uniform
      __syncthreads();      // the circuit's later columns see it singular and are skipped
      continue;
    }
    const T inv = (T)1 / lu[pd];
    for (int p = pd + 1 + threadIdx.x; p < p1; p += blockDim.x) lu[p] *= inv;
    __syncthreads();
    const int q0 = pd + 1, nl = p1 - q0;
    if (nl > 0) {
      for (int e = L.u_ptr[k] + warp; e < L.u_ptr[k + 1]; e += nwarps) {
        const int p = L.u_pos[e];  // U(k, j) in column j
        const int j = L.u_col[e];
        const T ukj = lu[p];
        if (ukj == (T)0) continue;
        const int *tgt = L.upd_pos + L.upd_off[p];
        const int cend = L.cp[j + 1];
        bool lost = false;
        for (int q = lane; q < nl; q += 32) {
          const int pos = tgt[q];
          if (pos > p && pos < cend) lu[pos] -= lu[q0 + q] * ukj;
          else lost = true;
        }
        if (__any_sync(0xffffffffu, lost) && lane == 0) {
          atomicCAS(L.breakdown, 0, j + 1);
          if (masked) cs[L.circ_of_step[j]].singular = 1;
        }
      }
    }
    __syncthreads();
  }
}

// Level-synchronous right-looking top on all SMs.  Level l: (1) every pivot
// column of the level (independent of each other) is tested and scaled, a
// warp each; (2) every target column j that receives updates from pivots of
// the level is updated by one warp, which applies its pivots' rank-1 terms
// one after the other (deterministic, no atomics), lanes over L(:, k).
template <typename T>
__global__ void __launch_bounds__(256) k_toplv_pivot(LUDev L, int lv, CircState *cs, int masked, double pivot_tol) {
  const int lane = threadIdx.x & 31;
  const int t = L.tlv_item_ptr[lv] + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (t >= L.tlv_item_ptr[lv + 1]) return;  // warp-uniform
  const int k = L.tlv_items[t];
  if (!factor_active(L, cs, masked, k)) return;
  T *lu = lu_of<T>(L);
  const int pd = L.diag[k], p1 = L.cp[k + 1];
  double amax = 0.0;
  for (int p = pd + lane; p < p1; p += 32) amax = fmax(amax, fabs((double)lu[p]));
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  const double d = (double)lu[pd];
  const bool urow = L.u_ptr[k + 1] > L.u_ptr[k];
  const double tol = L.exempt[k] ? pivot_tol * L.pscale[k] : pivot_tol;
  const bool bad = (urow && !(fabs(d) >= tol * amax)) || !(fabs(d) > 0.0) || isinf(d);
  if (bad) {
    if (lane == 0) {
      atomicCAS(L.breakdown, 0, k + 1);
      if (masked) cs[L.circ_of_step[k]].singular = 1;
    }
    return;
  }
  const T inv = (T)1 / lu[pd];
  for (int p = pd + 1 + lane; p < p1; p += 32) lu[p] *= inv;
}

template <typename T>
__global__ void __launch_bounds__(256) k_toplv_update(LUDev L, int lv, CircState *cs, int masked) {
  const int lane = threadIdx.x & 31;
  const int g = L.tlv_grp_ptr[lv] + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (g >= L.tlv_grp_ptr[lv + 1]) return;  // warp-uniform
  T *lu = lu_of<T>(L);
  const int j = L.tgrp_col[g], cend = L.cp[j + 1];
  bool lost = false;
  for (int e = L.tgrp_ptr[g]; e < L.tgrp_ptr[g + 1]; ++e) {
    const int k = L.tgrp_k[e];
    if (!factor_active(L, cs, masked, k)) continue;  // warp-uniform
    const int p = L.tgrp_pos[e];  // U(k, j)
    const T ukj = lu[p];
    if (ukj != (T)0) {
      const int q0 = L.diag[k] + 1, nl = L.cp[k + 1] - q0;
      const int *tgt = L.upd_pos + L.upd_off[p];
      for (int q = lane; q < nl; q += 32) {
        const int pos = tgt[q];
        if (pos > p && pos < cend) lu[pos] -= lu[q0 + q] * ukj;
        else lost = true;
      }
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, lost) && lane == 0) {
    atomicCAS(L.breakdown, 0, j + 1);
    if (masked) cs[L.circ_of_step[j]].singular = 1;
  }
}

// ---- factor groups staged in shared memory --------------------------------
// A group's columns are loaded from A once, factored left-looking in shared
// memory (the dependent chain of each update step reads U(k, j) and scatters
// into column j at shared-memory latency), and written back once.  L columns
// of hubs (outside every group) are read from global memory.
// A column of a group whose update metadata is staged too (mcol: the
// group's column records, ment: their U entries, mtg: update targets; all
// in shared memory).  TEAM lanes (1 = a thread per column, 32 = a warp).
struct FMeta {
  const int4 *col, *ent;
  const int *eptr, *tgt;
};
template <int TEAM, typename T>
__device__ void factor_column_m(const LUDev &L, int j, int r, CircState *cs, int masked, double pivot_tol,
                                double *sm, T *S, const FMeta &M) {
  const int lane = TEAM == 1 ? 0 : (int)(threadIdx.x & 31);
  const int4 col = M.col[r];  // value offset, entries, diagonal offset, pivot-test flag
  T *cj = S + col.x;
  const T *glu = lu_of<T>(L);
  bool lost = false;
  for (int u = M.eptr[r]; u < M.eptr[r + 1]; ++u) {
    const int4 en = M.ent[u];  // L source, count, target offset, position of U(k, j)
    const T ukj = cj[en.w];
    if (nz(ukj)) {
      const T *lk = en.x >= 0 ? S + en.x : glu + (-en.x - 1);
      const int *tg = M.tgt + en.z;
      for (int q = lane; q < en.y; q += TEAM) {
        const int pos = tg[q];
        if (pos > en.w && pos < col.y) cj[pos] -= lk[q] * ukj;
        else lost = true;
      }
    }
    if (TEAM > 1) __syncwarp();
  }
  unsigned long long ak = 0;
  for (int p = col.z + lane; p < col.y; p += TEAM) ak = umax64(ak, mag_key(cj[p]));
  if (TEAM > 1) {
    ak = team_max_key<false>(ak, sm);
    lost = team_any<false>(lost);
  }
  const double tol = col.w == 2 ? pivot_tol * L.pscale[j] : pivot_tol;
  if (!pivot_ok_u(L, j, cs, masked, tol, (double)cj[col.z], key_value<T>(ak), lost, lane == 0, col.w != 0))
    return;
  const T inv = (T)1 / cj[col.z];
  for (int p = col.z + 1 + lane; p < col.y; p += TEAM) cj[p] *= inv;
}

template <typename T>
__global__ void __launch_bounds__(kGroupThreads) k_factor_groups_s(LUDev L, const double *__restrict__ vals,
                                                                    CircState *cs, int masked, double pivot_tol,
                                                                    int cap) {
  extern __shared__ __align__(16) unsigned char smraw_lu[];
  T *S = reinterpret_cast<T *>(smraw_lu);
  __shared__ double sm[32];
  __shared__ int lvp[kStagedLevels + 1];
  __shared__ __align__(8) unsigned long long mbar;
  const SchedDev &SD = L.fs;
  const int g = blockIdx.x;
  if (factor_group_idle(L, cs, masked, L.fs_gcirc, g)) return;
  // a group of one circuit that is not idle refactors every column (its
  // circuit's state is tested once, above); a group that mixes circuits
  // tests each column's
  const bool multi = masked && (!L.fs_gcirc || L.fs_gcirc[g] < 0);
  if (L.grp_snz[g] > cap) {  // too large for the buffer: factor in place in global memory
    factor_group<T>(L, vals, cs, masked, pivot_tol, sm, g);
    return;
  }
  const int it0 = SD.lvl_ptr[SD.grp_lvl[g]], it1 = SD.lvl_ptr[SD.grp_lvl[g + 1]];
  if (it0 >= it1) return;
  const int lv0 = SD.grp_lvl[g];
  const int *lp = stage_levels(SD, lv0, SD.grp_lvl[g + 1], lvp);
  // a group of one circuit is active or not as a whole; packed tiny groups
  // may mix circuits, so every item is tested
  // load the group's columns from A (warp per column)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int t = it0 + warp; t < it1; t += nwarps) {
    const int j = SD.items[t], p0 = L.cp[j], p1 = L.cp[j + 1], o = L.grp_soff[j];
    for (int p = p0 + lane; p < p1; p += 32) {
      const int s = L.src[p];
      S[o + (p - p0)] = (s >= 0) ? (T)vals[s] : (T)0;
    }
  }
  const int mbytes = (L.fm_on && L.fm_gbytes) ? L.fm_gbytes[g] : 0;
  if (mbytes > 0) {
    // the update metadata of the group, after the values (16-byte aligned)
    unsigned char *mraw = smraw_lu + ((size_t)L.grp_snz[g] * sizeof(T) + 15) / 16 * 16;
    const int R = it1 - it0, u0 = L.fm_eptr[it0], U = L.fm_eptr[it1] - u0;
    const int t0 = L.fm_tptr[g], TG = L.fm_tptr[g + 1] - t0;
    FMeta M;
    int4 *mcol = reinterpret_cast<int4 *>(mraw);
    int4 *ment = mcol + R;
    int *mep = reinterpret_cast<int *>(ment + U);
    int *mtg = mep + R + 1;
    // the column records and their update entries (contiguous int4 ranges)
    // by two bulk copies; the offsets and the targets by plain loads meanwhile
    if (threadIdx.x == 0) mbar_init(&mbar);
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect(&mbar, 16u * (unsigned)(R + U));
      bulk_to_smem(mcol, L.fm_col + it0, 16u * (unsigned)R, &mbar);
      if (U > 0) bulk_to_smem(ment, L.fm_ent + u0, 16u * (unsigned)U, &mbar);
    }
    for (int r = threadIdx.x; r <= R; r += blockDim.x) mep[r] = L.fm_eptr[it0 + r] - u0;
    for (int q = threadIdx.x; q < TG; q += blockDim.x) mtg[q] = L.fm_tgt[t0 + q];
    M.col = mcol; M.ent = ment; M.eptr = mep; M.tgt = mtg;
    const bool landed = mbar_wait0(&mbar, kBulkWaitPolls);
    if (!__syncthreads_and(landed)) {
      // the copies did not land in time: report a breakdown (the host
      // re-analyses and refactors) rather than factor from unfilled memory
      if (threadIdx.x == 0) atomicCAS(L.breakdown, 0, it0 + 1);
      mbar_wait0(&mbar, kBulkWaitPolls);
      return;
    }
    for (int lv = SD.grp_lvl[g]; lv < SD.grp_lvl[g + 1]; ++lv) {
      const int b = lp[lv - lv0], e = lp[lv - lv0 + 1];
      for (int t = b + (int)threadIdx.x; t < e; t += (int)blockDim.x) {
        const int j = SD.items[t];
        if (SD.is_thread[j] && (!multi || factor_active(L, cs, masked, j)))
          factor_column_m<1, T>(L, j, t - it0, cs, masked, pivot_tol, sm, S, M);
      }
      for (int t = b + warp; t < e; t += nwarps) {
        const int j = SD.items[t];
        if (SD.is_thread[j] || !(!multi || factor_active(L, cs, masked, j))) continue;
        factor_column_m<32, T>(L, j, t - it0, cs, masked, pivot_tol, sm, S, M);
      }
      __syncthreads();
    }
  } else {
    // the update records of the group's columns (read level by level below,
    // in a chain of dependent loads) are pulled into L1 first; a prefetch
    // holds no register and no shared memory
    for (int t = it0 + (int)threadIdx.x; t < it1; t += (int)blockDim.x) {
      const int j = SD.items[t];
      const int4 *u0 = L.umeta + L.cp[j], *u1 = L.umeta + L.diag[j];
      for (const int4 *u = u0; u < u1; u += 8) asm volatile("prefetch.global.L1 [%0];" ::"l"(u));
    }
    // every column staged before any is read (a column's thread or warp
    // need not be the warp that staged it)
    __syncthreads();
    for (int lv = SD.grp_lvl[g]; lv < SD.grp_lvl[g + 1]; ++lv) {
      const int b = lp[lv - lv0], e = lp[lv - lv0 + 1];
      bool any_long = false;
      for (int t = b + (int)threadIdx.x; t < e; t += (int)blockDim.x) {
        const int j = SD.items[t];
        if (SD.is_thread[j] && (!multi || factor_active(L, cs, masked, j)))
          factor_column_t<T>(L, vals, j, cs, masked, pivot_tol, S, L.grp_soff, L.umeta);
      }
      for (int t = b + warp; t < e; t += nwarps) {
        const int j = SD.items[t];
        if (SD.is_long[j]) { any_long = true; continue; }
        if (SD.is_thread[j] || !(!multi || factor_active(L, cs, masked, j))) continue;
        factor_column_s<false, T>(L, j, cs, masked, pivot_tol, sm, S, L.grp_soff, L.umeta);
      }
      if (__syncthreads_or(any_long)) {
        for (int t = b; t < e; ++t) {
          const int j = SD.items[t];
          if (!SD.is_long[j] || !(!multi || factor_active(L, cs, masked, j))) continue;
          factor_column_s<true, T>(L, j, cs, masked, pivot_tol, sm, S, L.grp_soff, L.umeta);
          __syncthreads();
        }
      }
    }
  }
  __syncthreads();
  // write the factored columns back (the solves and the top read them); a
  // group that mixes circuits writes only the columns it factored, so the
  // factors of a circuit that is not refactoring stay as they are
  T *lu = lu_of<T>(L);
  for (int t = it0 + warp; t < it1; t += nwarps) {
    const int j = SD.items[t], p0 = L.cp[j], p1 = L.cp[j + 1], o = L.grp_soff[j];
    if (multi && !factor_active(L, cs, masked, j)) continue;
    for (int p = p0 + lane; p < p1; p += 32) lu[p] = S[o + (p - p0)];
  }
}

// ---- L solve (L schedule, forward) ------------------------------------------
__global__ void k_lsolve_hubs(LUDev L, const double *__restrict__ b, const CircState *cs, int masked) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L.ls.n_hub) return;
  const int i = L.ls.items[t];
  if (!item_active(L, cs, masked, i)) return;
  L.y[i] = b[L.row_of_step[i]];  // hubs have no L entries
}


template <typename T>
__device__ void lsolve_group(const LUDev &L, const double *__restrict__ b, const CircState *cs, int masked, int g,
                             double *sm) {
  const SchedDev &S = L.ls;
  const T *lu = lu_of<T>(L);
  const int team = threadIdx.x >> 3, nteams = blockDim.x >> 3, sub = threadIdx.x & 7;
  for (int lv = S.grp_lvl[g]; lv < S.grp_lvl[g + 1]; ++lv) {
    const int bb = S.lvl_ptr[lv], e = S.lvl_ptr[lv + 1];
    bool any_long = false;
    // short rows: a thread each
    for (int t = bb + (int)threadIdx.x; t < e; t += (int)blockDim.x) {
      const int i = S.items[t];
      if (!S.is_thread[i] || !item_active(L, cs, masked, i)) continue;
      const int q0 = L.l_ptr[i];
      const double sum = row_dot_t<T>(lu, L.l_pos, L.l_col, L.y, q0, L.l_ptr[i + 1] - q0);
      L.y[i] = b[L.row_of_step[i]] - sum;
    }
    // the others: teams of 8 lanes stride over the level; the loop bound is
    // warp-uniform
    for (int t0 = bb; t0 < e; t0 += nteams) {
      const int t = t0 + team;
      bool act = false;
      int i = 0;
      if (t < e) {
        i = S.items[t];
        if (S.is_long[i]) any_long = true;
        else act = !S.is_thread[i] && item_active(L, cs, masked, i);
      }
      if (__any_sync(0xffffffffu, act)) {
        double sum = 0.0;
        if (act)
          for (int q = L.l_ptr[i] + sub; q < L.l_ptr[i + 1]; q += 8)
            sum += (double)lu[L.l_pos[q]] * L.y[L.l_col[q]];
        for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
        if (act && sub == 0) L.y[i] = b[L.row_of_step[i]] - sum;
      }
    }
    if (__syncthreads_or(any_long)) {
      for (int t = bb; t < e; ++t) {
        const int i = S.items[t];
        if (!S.is_long[i] || !item_active(L, cs, masked, i)) continue;
        solve_row<true, true, T, false>(L, b, nullptr, i, threadIdx.x, sm);
        __syncthreads();
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kGroupThreads) k_lsolve_groups(LUDev L, const double *__restrict__ b,
                                                                  const CircState *cs, int masked, int top) {
  __shared__ double sm[32];
  if (!top && group_idle(L, cs, masked, L.ls_gcirc, (int)blockIdx.x)) return;
  lsolve_group<T>(L, b, cs, masked, top ? L.ls.n_groups : (int)blockIdx.x, sm);
}

// A group's L solve staged in shared memory: its rows' entries (values and
// buffer slots) and its slice of y are loaded once, coalesced; each level
// then reads only shared memory (a thread per row), and y is written back
// at the end.  Groups over the buffer run the global-memory path.
template <typename T>
__global__ void __launch_bounds__(kGroupThreads) k_lsolve_groups_s(LUDev L, const double *__restrict__ b,
                                                                    const CircState *cs, int masked) {
  extern __shared__ __align__(16) unsigned char smraw_sv[];
  __shared__ double sm[32];
  __shared__ int lvp[kStagedLevels + 1];
  const SchedDev &S = L.ls;
  const int g = blockIdx.x;
  if (group_idle(L, cs, masked, L.ls_gcirc, g)) return;
  if (L.ls_gbytes[g] == 0) {
    lsolve_group<T>(L, b, cs, masked, g, sm);
    return;
  }
  const T *lu = lu_of<T>(L);
  const int it0 = S.lvl_ptr[S.grp_lvl[g]], it1 = S.lvl_ptr[S.grp_lvl[g + 1]], R = it1 - it0;
  const int e0 = L.ls_eptr[it0], E = L.ls_eptr[it1] - e0;
  double *yv = reinterpret_cast<double *>(smraw_sv);
  double *ev = yv + R;
  double *xv = ev + E;  // y of an entry's column outside the group (final before this launch)
  int *es = reinterpret_cast<int *>(xv + E);
  int *ep = es + E;
  int *act = ep + R + 1;
  const int lv0 = S.grp_lvl[g];
  const int *lp = stage_levels(S, lv0, S.grp_lvl[g + 1], lvp);
  for (int r = threadIdx.x; r <= R; r += blockDim.x) {
    ep[r] = L.ls_eptr[it0 + r] - e0;
    if (r < R) {
      const int i = S.items[it0 + r];
      act[r] = item_active(L, cs, masked, i) ? 1 : 0;
      yv[r] = b[L.row_of_step[i]];
    }
  }
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    ev[e] = (double)lu[L.ls_epos[e0 + e]];
    const int src = L.ls_esrc[e0 + e];
    es[e] = src;
    if (src < 0) xv[e] = L.y[-src - 1];
  }
  __syncthreads();
  for (int lv = S.grp_lvl[g]; lv < S.grp_lvl[g + 1]; ++lv) {
    const int r0 = lp[lv - lv0] - it0, r1 = lp[lv - lv0 + 1] - it0;
    for (int r = r0 + (int)threadIdx.x; r < r1; r += (int)blockDim.x) {
      if (!act[r]) continue;
      double sum = 0.0;
      for (int q = ep[r]; q < ep[r + 1]; ++q) {
        const int src = es[q];
        sum += ev[q] * (src >= 0 ? yv[src] : xv[q]);
      }
      yv[r] -= sum;
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x)
    if (act[r]) L.y[S.items[it0 + r]] = yv[r];
}

// ---- U solve (factor schedule, backward) ------------------------------------
template <typename T, bool ACC>
__device__ void usolve_group(const LUDev &L, double *__restrict__ x, const CircState *cs, int masked, int g,
                             double *sm) {
  const SchedDev &S = L.fs;
  const T *lu = lu_of<T>(L);
  const int team = threadIdx.x >> 3, nteams = blockDim.x >> 3, sub = threadIdx.x & 7;
  for (int lv = S.grp_lvl[g + 1] - 1; lv >= S.grp_lvl[g]; --lv) {
    const int bb = S.lvl_ptr[lv], e = S.lvl_ptr[lv + 1];
    bool any_long = false;
    for (int t = bb + (int)threadIdx.x; t < e; t += (int)blockDim.x) {
      const int k = S.items[t];
      if (!S.is_thread_rev[k] || !item_active(L, cs, masked, k)) continue;
      const int q0 = L.u_ptr[k];
      const double sum = row_dot_t<T>(lu, L.u_pos, L.u_col, L.y, q0, L.u_ptr[k + 1] - q0);
      const double z = (L.y[k] - sum) / (double)lu[L.diag[k]];
      L.y[k] = z;
      if (ACC) x[L.col_of_step[k]] += z;
      else x[L.col_of_step[k]] = z;
    }
    for (int t0 = bb; t0 < e; t0 += nteams) {
      const int t = t0 + team;
      bool act = false;
      int k = 0;
      if (t < e) {
        k = S.items[t];
        if (S.is_long_rev[k]) any_long = true;
        else act = !S.is_thread_rev[k] && item_active(L, cs, masked, k);
      }
      if (__any_sync(0xffffffffu, act)) {
        double sum = 0.0;
        if (act)
          for (int q = L.u_ptr[k] + sub; q < L.u_ptr[k + 1]; q += 8)
            sum += (double)lu[L.u_pos[q]] * L.y[L.u_col[q]];
        for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
        if (act && sub == 0) {
          const double z = (L.y[k] - sum) / (double)lu[L.diag[k]];
          L.y[k] = z;
          if (ACC) x[L.col_of_step[k]] += z;
          else x[L.col_of_step[k]] = z;
        }
      }
    }
    if (__syncthreads_or(any_long)) {
      for (int t = bb; t < e; ++t) {
        const int k = S.items[t];
        if (!S.is_long_rev[k] || !item_active(L, cs, masked, k)) continue;
        solve_row<false, true, T, ACC>(L, nullptr, x, k, threadIdx.x, sm);
        __syncthreads();
      }
    }
  }
}

template <typename T, bool ACC>
__global__ void __launch_bounds__(kGroupThreads) k_usolve_groups(LUDev L, double *__restrict__ x,
                                                                  const CircState *cs, int masked, int top) {
  __shared__ double sm[32];
  if (!top && group_idle(L, cs, masked, L.fs_gcirc, (int)blockIdx.x)) return;
  usolve_group<T, ACC>(L, x, cs, masked, top ? L.fs.n_groups : (int)blockIdx.x, sm);
}

// The U solve of a group staged in shared memory (the factor schedule run
// backwards; see k_lsolve_groups_s): y and the diagonal of the group's rows
// and the entries of their U rows are loaded once.
template <typename T, bool ACC>
__global__ void __launch_bounds__(kGroupThreads) k_usolve_groups_s(LUDev L, double *__restrict__ x,
                                                                    const CircState *cs, int masked) {
  extern __shared__ __align__(16) unsigned char smraw_sv[];
  __shared__ double sm[32];
  __shared__ int lvp[kStagedLevels + 1];
  const SchedDev &S = L.fs;
  const int g = blockIdx.x;
  if (group_idle(L, cs, masked, L.fs_gcirc, g)) return;
  if (L.us_gbytes[g] == 0) {
    usolve_group<T, ACC>(L, x, cs, masked, g, sm);
    return;
  }
  const T *lu = lu_of<T>(L);
  const int it0 = S.lvl_ptr[S.grp_lvl[g]], it1 = S.lvl_ptr[S.grp_lvl[g + 1]], R = it1 - it0;
  const int e0 = L.us_eptr[it0], E = L.us_eptr[it1] - e0;
  double *yv = reinterpret_cast<double *>(smraw_sv);
  double *dv = yv + R;
  double *ev = dv + R;
  double *xv = ev + E;  // y of an entry's column outside the group (final before this launch)
  int *es = reinterpret_cast<int *>(xv + E);
  int *ep = es + E;
  int *act = ep + R + 1;
  const int lv0 = S.grp_lvl[g];
  const int *lp = stage_levels(S, lv0, S.grp_lvl[g + 1], lvp);
  for (int r = threadIdx.x; r <= R; r += blockDim.x) {
    ep[r] = L.us_eptr[it0 + r] - e0;
    if (r < R) {
      const int k = S.items[it0 + r];
      act[r] = item_active(L, cs, masked, k) ? 1 : 0;
      yv[r] = L.y[k];
      dv[r] = (double)lu[L.diag[k]];
    }
  }
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    ev[e] = (double)lu[L.us_epos[e0 + e]];
    const int src = L.us_esrc[e0 + e];
    es[e] = src;
    if (src < 0) xv[e] = L.y[-src - 1];
  }
  __syncthreads();
  for (int lv = S.grp_lvl[g + 1] - 1; lv >= S.grp_lvl[g]; --lv) {
    const int r0 = lp[lv - lv0] - it0, r1 = lp[lv - lv0 + 1] - it0;
    for (int r = r0 + (int)threadIdx.x; r < r1; r += (int)blockDim.x) {
      if (!act[r]) continue;
      double sum = 0.0;
      for (int q = ep[r]; q < ep[r + 1]; ++q) {
        const int src = es[q];
        sum += ev[q] * (src >= 0 ? yv[src] : xv[q]);
      }
      yv[r] = (yv[r] - sum) / dv[r];
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    if (!act[r]) continue;
    const int k = S.items[it0 + r];
    L.y[k] = yv[r];
    if (ACC) x[L.col_of_step[k]] += yv[r];
    else x[L.col_of_step[k]] = yv[r];
  }
}

template <typename T, bool ACC>
__global__ void __launch_bounds__(256) k_usolve_hubs(LUDev L, double *__restrict__ x, const CircState *cs,
                                                     int masked) {
  __shared__ double sm[32];
  const int k = L.fs.items[blockIdx.x];
  if (!item_active(L, cs, masked, k)) return;
  solve_row<false, true, T, ACC>(L, nullptr, x, k, threadIdx.x, sm);
}

// ---- the tops of the solves, one level per launch on all SMs --------------
// (large tops: the upper separators give hundreds of levels that one CTA
// would walk alone).  A warp per row; the level's rows are independent.
template <typename T>
__global__ void __launch_bounds__(256) k_lsolve_level(LUDev L, int lv, const double *__restrict__ b,
                                                      const CircState *cs, int masked) {
  const int lane = threadIdx.x & 31;
  const int t = L.ls.lvl_ptr[lv] + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (t >= L.ls.lvl_ptr[lv + 1]) return;  // warp-uniform
  const int i = L.ls.items[t];
  if (!item_active(L, cs, masked, i)) return;
  const T *lu = lu_of<T>(L);
  double sum = 0.0;
  for (int q = L.l_ptr[i] + lane; q < L.l_ptr[i + 1]; q += 32) sum += (double)lu[L.l_pos[q]] * L.y[L.l_col[q]];
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) L.y[i] = b[L.row_of_step[i]] - sum;
}

template <typename T, bool ACC>
__global__ void __launch_bounds__(256) k_usolve_level(LUDev L, int lv, double *__restrict__ x, const CircState *cs,
                                                      int masked) {
  const int lane = threadIdx.x & 31;
  const int t = L.fs.lvl_ptr[lv] + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (t >= L.fs.lvl_ptr[lv + 1]) return;  // warp-uniform
  const int k = L.fs.items[t];
  if (!item_active(L, cs, masked, k)) return;
  const T *lu = lu_of<T>(L);
  double sum = 0.0;
  for (int q = L.u_ptr[k] + lane; q < L.u_ptr[k + 1]; q += 32) sum += (double)lu[L.u_pos[q]] * L.y[L.u_col[q]];
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) {
    const double z = (L.y[k] - sum) / (double)lu[L.diag[k]];
    L.y[k] = z;
    if (ACC) x[L.col_of_step[k]] += z;
    else x[L.col_of_step[k]] = z;
  }
}

// ---- FP64 residual of a refined solve ---------------------------------------
// r = b - A x over the rows of active circuits, A in the context's CSR order
// (IRSolver's residual step, src/LinearAlgebraServicesPKG/N_LAS_IRSolver.C:482-540).
// One 8-lane team per row.
__global__ void __launch_bounds__(256) k_ir_residual(LUDev L, const double *__restrict__ b,
                                                     const double *__restrict__ x, const CircState *cs,
                                                     int masked) {
  const int row = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 3);
  const int sub = threadIdx.x & 7;
  const bool in = row < L.n;
  bool act = in;
  if (in && masked) {
    const CircState &s = cs[L.a_circ[row]];
    act = s.need_solve && !s.singular && (s.phase == PH_DC || s.phase == PH_TRAN);
  }
  double sum = 0.0;
  if (act)
    for (int e = L.a_rp[row] + sub; e < L.a_rp[row + 1]; e += 8) sum += L.a_vals[e] * x[L.a_ci[e]];
  for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, 8);
  if (act && sub == 0) L.ir_r[row] = b[row] - sum;
}

// ---- allocation-free solve --------------------------------------------------
// Scratch of xg_lu_solve_noalloc: the intermediate vector y of L y = P b, in a
// file-scope device array that every GPU loading the library holds until the
// process exits (kNoAllocMaxN doubles = 2 MiB).  All calls share it.
static __device__ __align__(256) double g_noalloc_y[kNoAllocMaxN];

namespace {
std::mutex g_noalloc_mu;
double *g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

// Device address of the scratch on `device` (which must be current); looked
// up once per device with cudaGetSymbolAddress — a host-side reference to
// g_noalloc_y is not a device address.
int noalloc_scratch(int device, double **out, std::string &err) {
  if (device < 0 || device >= kNoAllocMaxDevices) {
    err = "device ordinal out of range for the allocation-free scratch";
    return XG_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_y);
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress(g_noalloc_y): ") + cudaGetErrorString(e);
      return XG_ERR_CUDA;
    }
    g_noalloc_ptr[device] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[device];
  return XG_OK;
}

// The triangular solves of launch_lu_solve_k with the static scratch in place
// of the analysis' y vector (unmasked: every row is solved).
void launch_lu_solve_noalloc_k(cudaStream_t st, LUDev L, double *scratch, const double *b, double *x,
                               const CircState *cs) {
  L.y = scratch;
  launch_lu_solve_k(st, L, b, x, cs, 0);
}

// ---- launchers --------------------------------------------------------------
template <typename T>
static void factor_sweeps(cudaStream_t st, const LUDev &L, const double *vals, CircState *cs, int masked,
                          double pivot_tol) {
  if (L.fs.n_hub > 0) k_factor_hubs<T><<<L.fs.n_hub, 256, 0, st>>>(L, vals, cs, masked, pivot_tol);
  if (L.fs.n_groups > 0) {
    // groups of up to kGroupSmemBytes factor in shared memory; the buffer is
    // sized for the largest of them, larger groups factor in global memory
    const int w = sizeof(T) == 4 ? 1 : 0;
    const int fit = L.grp_fit[w];
    const size_t smem = std::max((size_t)fit * sizeof(T), L.fm_on ? (size_t)L.fm_smem[w] : (size_t)0);
    if (L.grp_snz && fit > 0)
      k_factor_groups_s<T><<<L.fs.n_groups, L.fs_threads, smem, st>>>(L, vals, cs, masked, pivot_tol, fit);
    else
      k_factor_groups<T><<<L.fs.n_groups, L.fs_threads, 0, st>>>(L, vals, cs, masked, pivot_tol, 0);
  }
  if (L.fs.n_top_items > 0) {
    if (L.n_top_rl > 0) {
      const long long threads = (long long)L.n_top_rl * 32;
      k_top_pull<T><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(L, vals, cs, masked);
      if (L.n_top_lv > 0 && L.h_tlv_item_ptr) {
        for (int lv = 0; lv < L.n_top_lv; ++lv) {
          const int ni = L.h_tlv_item_ptr[lv + 1] - L.h_tlv_item_ptr[lv];
          const int ng = L.h_tlv_grp_ptr[lv + 1] - L.h_tlv_grp_ptr[lv];
          if (ni > 0) k_toplv_pivot<T><<<(ni + 7) / 8, 256, 0, st>>>(L, lv, cs, masked, pivot_tol);
          if (ng > 0) k_toplv_update<T><<<(ng + 7) / 8, 256, 0, st>>>(L, lv, cs, masked);
        }
      } else {
        k_top_rl<T><<<1, 1024, 0, st>>>(L, cs, masked, pivot_tol);
      }
    } else {
      k_factor_groups<T><<<1, 1024, 0, st>>>(L, vals, cs, masked, pivot_tol, 1);
    }
  }
}

// Opt-in of the staged kernels to their largest buffers: beyond 48 KB of
// dynamic plus static shared memory a launch needs it, and the staged solve
// kernels' own static arrays sit on top of buffers of up to kSolveSmemBytes.
int lu_prepare_k() {
  const int solve_bytes = kSolveSmemBytes + 4096;
  auto set = [](const void *f, int bytes) {
    return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
  };
  if (!set((const void *)k_factor_groups_s<double>, kGroupSmemBytes) ||
      !set((const void *)k_factor_groups_s<float>, kGroupSmemBytes) ||
      !set((const void *)k_lsolve_groups_s<double>, solve_bytes) ||
      !set((const void *)k_lsolve_groups_s<float>, solve_bytes) ||
      !set((const void *)k_usolve_groups_s<double, false>, solve_bytes) ||
      !set((const void *)k_usolve_groups_s<double, true>, solve_bytes) ||
      !set((const void *)k_usolve_groups_s<float, false>, solve_bytes) ||
      !set((const void *)k_usolve_groups_s<float, true>, solve_bytes))
    return XG_ERR_CUDA;
  return XG_OK;
}

void launch_lu_factor_k(cudaStream_t st, const LUDev &L, const double *vals, CircState *cs, int masked,
                        double pivot_tol) {
  if (L.mixed) factor_sweeps<float>(st, L, vals, cs, masked, pivot_tol);
  else factor_sweeps<double>(st, L, vals, cs, masked, pivot_tol);
}

// One forward + backward sweep: x = (LU)^-1 b, or x += (LU)^-1 b (ACC).
template <typename T, bool ACC>
static void solve_sweeps(cudaStream_t st, const LUDev &L, const double *b, double *x, const CircState *cs,
                         int masked) {
  if (L.ls.n_hub > 0) k_lsolve_hubs<<<(L.ls.n_hub + 255) / 256, 256, 0, st>>>(L, b, cs, masked);
  if (L.ls.n_groups > 0) {
    if (L.ls_smem > 0)
      k_lsolve_groups_s<T><<<L.ls.n_groups, L.ls_threads, L.ls_smem, st>>>(L, b, cs, masked);
    else
      k_lsolve_groups<T><<<L.ls.n_groups, L.ls_threads, 0, st>>>(L, b, cs, masked, 0);
  }
  if (L.ls.n_top_items > 0) {
    if (L.h_ls_lvl_ptr) {
      for (int lv = L.ls_top_lo; lv < L.ls_top_hi; ++lv) {
        const int nr = L.h_ls_lvl_ptr[lv + 1] - L.h_ls_lvl_ptr[lv];
        if (nr > 0) k_lsolve_level<T><<<(nr + 7) / 8, 256, 0, st>>>(L, lv, b, cs, masked);
      }
    } else {
      k_lsolve_groups<T><<<1, kGroupThreads, 0, st>>>(L, b, cs, masked, 1);
    }
  }
  if (L.fs.n_top_items > 0) {
    if (L.h_fs_lvl_ptr) {
      for (int lv = L.fs_top_hi - 1; lv >= L.fs_top_lo; --lv) {
        const int nr = L.h_fs_lvl_ptr[lv + 1] - L.h_fs_lvl_ptr[lv];
        if (nr > 0) k_usolve_level<T, ACC><<<(nr + 7) / 8, 256, 0, st>>>(L, lv, x, cs, masked);
      }
    } else {
      k_usolve_groups<T, ACC><<<1, kGroupThreads, 0, st>>>(L, x, cs, masked, 1);
    }
  }
  if (L.fs.n_groups > 0) {
    if (L.us_smem > 0)
      k_usolve_groups_s<T, ACC><<<L.fs.n_groups, L.us_threads, L.us_smem, st>>>(L, x, cs, masked);
    else
      k_usolve_groups<T, ACC><<<L.fs.n_groups, L.us_threads, 0, st>>>(L, x, cs, masked, 0);
  }
  if (L.fs.n_hub > 0) k_usolve_hubs<T, ACC><<<L.fs.n_hub, 256, 0, st>>>(L, x, cs, masked);
}

// FP64: one solve.  FP32 factors: one solve, then n_refine steps of
// r = b - A x (FP64), x += (LU)^-1 r.
void launch_lu_solve_k(cudaStream_t st, const LUDev &L, const double *b, double *x, const CircState *cs,
                       int masked) {
  if (!L.mixed) {
    solve_sweeps<double, false>(st, L, b, x, cs, masked);
    return;
  }
  solve_sweeps<float, false>(st, L, b, x, cs, masked);
  const unsigned blocks = (unsigned)(((size_t)L.n * 8 + 255) / 256);
  for (int k = 0; k < L.n_refine; ++k) {
    k_ir_residual<<<blocks, 256, 0, st>>>(L, b, x, cs, masked);
    solve_sweeps<float, true>(st, L, L.ir_r, x, cs, masked);
  }
}

}  // namespace xg
