// xg_mlp.cu — learned Newton predictor: a per-node MLP 5 -> 64 -> 64 -> 1
// (sm_103a).  No counterpart in the reference: it hooks the predictor of
// WorkingIntegrationMethod::obtainPredictor
// (src/TimeIntegrationPKG/N_TIA_WorkingIntegrationMethod.C:176), whose
// polynomial guess (OneStep::obtainPredictor, N_TIA_OneStep.C:135-175) it
// corrects.  Full Newton to the unchanged tolerances still decides every
// step; a per-circuit rule falls back to the polynomial predictor when the
// learned guess raises the Newton iteration count.
//
// Layers 1 and 2 (and the dH1 = dZ2 W2^T product of the backward pass) run
// on the tensor cores: warp-level mma.sync m16n8k16, BF16 operands, FP32
// accumulation, 16 node rows per warp.  The accumulator fragments of one
// layer are repacked in registers as the A fragments of the next (the C
// layout of two adjacent 16x8 tiles is the A layout of one 16x16 tile).
// Weight gradients are FP32 sums over the rows (SIMT, shared memory);
// Adam keeps FP32 master weights and refreshes the BF16 copies.
//
// Parameter vector (FP32 master, xg_mlp_* entry points):
//   W1[5][64] | b1[64] | W2[64][64] (in x out) | b2[64] | w3[64] | b3
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "xg_internal.h"

namespace xg {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + D (16x8 f32)
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared-memory copy of the network (BF16 operands, FP32 vectors).
struct MlpSmem {
  __nv_bfloat16 w1t[kMlpHid][kMlpInPad];   // [n][k]: B operand of layer 1
  __nv_bfloat16 w2t[kMlpHid][kMlpHid];     // [n][k]: B operand of layer 2 (W2^T)
  __nv_bfloat16 w2[kMlpHid][kMlpHid];      // [k][n]: B operand of dH1 = dZ2 W2^T
  float b1[kMlpHid], b2[kMlpHid], w3[kMlpHid];
  float b3, in_shift[kMlpIn], in_scale[kMlpIn], out_shift, out_scale;
};

__device__ void mlp_load_smem(const MlpDev &P, MlpSmem &S) {
  const __nv_bfloat16 *w1t = reinterpret_cast<const __nv_bfloat16 *>(P.w1t);
  const __nv_bfloat16 *w2t = reinterpret_cast<const __nv_bfloat16 *>(P.w2t);
  const __nv_bfloat16 *w2 = reinterpret_cast<const __nv_bfloat16 *>(P.w2);
  for (int i = threadIdx.x; i < kMlpHid * kMlpInPad; i += blockDim.x) (&S.w1t[0][0])[i] = w1t[i];
  for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x) {
    (&S.w2t[0][0])[i] = w2t[i];
    (&S.w2[0][0])[i] = w2[i];
  }
  for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
    S.b1[i] = P.theta[kMlpOffB1 + i];
    S.b2[i] = P.theta[kMlpOffB2 + i];
    S.w3[i] = P.theta[kMlpOffW3 + i];
  }
  if (threadIdx.x == 0) {
    S.b3 = P.theta[kMlpOffB3];
    for (int i = 0; i < kMlpIn; ++i) { S.in_shift[i] = P.norm[i]; S.in_scale[i] = P.norm[kMlpIn + i]; }
    S.out_shift = P.norm[2 * kMlpIn];
    S.out_scale = P.norm[2 * kMlpIn + 1];
  }
  __syncthreads();
}

// Warp forward pass over 16 rows.  Lane (g = lane/4, t = lane%4) supplies the
// standardized features fx[0..4] of rows g and g+8 and receives:
//   h1[j][0..3], h2[j][0..3]: post-tanh activations in accumulator layout
//     (tile j covers hidden columns 8j..8j+7; [0],[1] row g cols 8j+2t,+1;
//     [2],[3] row g+8),
//   y[0], y[1]: network outputs of rows g and g+8 (all four lanes of a group).
__device__ __forceinline__ void mlp_forward_warp(const MlpSmem &S, const float (&fg)[kMlpIn],
                                                 const float (&fg8)[kMlpIn], float (&h1)[8][4],
                                                 float (&h2)[8][4], float (&y)[2]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  // layer 1: A = X (16 x 16, features 0..4, zero padded)
  auto feat = [&](const float (&f)[kMlpIn], int k) { return k < kMlpIn ? f[k] : 0.0f; };
  uint32_t a[4];
  a[0] = pack_bf16(feat(fg, 2 * t), feat(fg, 2 * t + 1));
  a[1] = pack_bf16(feat(fg8, 2 * t), feat(fg8, 2 * t + 1));
  a[2] = 0u;
  a[3] = 0u;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const int n = 8 * j + g;
    const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w1t[n][2 * t]);
    const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w1t[n][2 * t + 8]);
    mma16816(c, a, b0, b1);
    const int col = 8 * j + 2 * t;
    h1[j][0] = tanhf(c[0] + S.b1[col]);
    h1[j][1] = tanhf(c[1] + S.b1[col + 1]);
    h1[j][2] = tanhf(c[2] + S.b1[col]);
    h1[j][3] = tanhf(c[3] + S.b1[col + 1]);
  }
  // layer 2: A fragments of k-block kb from tiles 2kb, 2kb+1
  uint32_t a2[4][4];
#pragma unroll
  for (int kb = 0; kb < 4; ++kb) {
    a2[kb][0] = pack_bf16(h1[2 * kb][0], h1[2 * kb][1]);
    a2[kb][1] = pack_bf16(h1[2 * kb][2], h1[2 * kb][3]);
    a2[kb][2] = pack_bf16(h1[2 * kb + 1][0], h1[2 * kb + 1][1]);
    a2[kb][3] = pack_bf16(h1[2 * kb + 1][2], h1[2 * kb + 1][3]);
  }
  float p0 = 0.f, p1 = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const int n = 8 * j + g;
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
      const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w2t[n][16 * kb + 2 * t]);
      const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w2t[n][16 * kb + 2 * t + 8]);
      mma16816(c, a2[kb], b0, b1);
    }
    const int col = 8 * j + 2 * t;
    h2[j][0] = tanhf(c[0] + S.b2[col]);
    h2[j][1] = tanhf(c[1] + S.b2[col + 1]);
    h2[j][2] = tanhf(c[2] + S.b2[col]);
    h2[j][3] = tanhf(c[3] + S.b2[col + 1]);
    // layer 3 partial dot products (FP32)
    p0 += h2[j][0] * S.w3[col] + h2[j][1] * S.w3[col + 1];
    p1 += h2[j][2] * S.w3[col] + h2[j][3] * S.w3[col + 1];
  }
  p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
  p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
  p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
  p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
  y[0] = p0 + S.b3;
  y[1] = p1 + S.b3;
}

// ---- inference inside the transient tick ------------------------------------
// After k_history has written the polynomial predictor xn0 of every step
// attempt, rows of circuits whose learned predictor is on start Newton from
//   x = xn0 + s * (out_shift + out_scale * MLP(features)),
// where s = |d1| + |d2| + |d3| + kMlpScaleFloor (d1 = x_n - x_{n-1},
// d2 = x_{n-1} - x_{n-2}, d3 = x_{n-2} - x_{n-3}) is the node's recent motion
// and the features are (d1 / s, d2 / s, d3 / s, x_n, log(h_{n+1} / h_n)),
// standardized by in_shift / in_scale: a node at rest keeps its polynomial
// guess (rows with s < kMlpActive are not corrected).  xn0 itself stays the polynomial predictor, so the predictor-
// corrector error estimate (OneStep, N_TIA_OneStep.C:1584-1640) and the step
// control are those of the reference.  Branch currents keep the polynomial guess.
__global__ void __launch_bounds__(128) k_ml_predict(DevArrays d, int n) {
  __shared__ MlpSmem S;
  mlp_load_smem(d.mlp, S);
  const int warp_row0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 16;
  if (warp_row0 >= n) return;  // warp-uniform
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int rows[2] = {warp_row0 + g, warp_row0 + g + 8};
  bool use[2];
  float f[2][kMlpIn];
  double scale[2] = {0.0, 0.0};
  for (int q = 0; q < 2; ++q) {
    const int r = rows[q];
    use[q] = false;
    for (int k = 0; k < kMlpIn; ++k) f[q][k] = 0.f;
    if (r < n && !d.is_branch[r]) {
      const CircState &s = d.cs[d.circ_of_row[r]];
      if (s.start_step && s.phase == PH_TRAN && s.ml_use && s.lastTimeStep > 0.0) {
        const double d1 = d.mlh1[r], d2 = d.mlh2[r], d3 = d.mlh3[r];
        const double sc = fabs(d1) + fabs(d2) + fabs(d3) + kMlpScaleFloor;
        if (sc < kMlpActive) continue;  // a node at rest keeps the polynomial guess
        use[q] = true;
        scale[q] = sc;
        const double raw[kMlpIn] = {d1 / sc, d2 / sc, d3 / sc, d.xcurr[r], log(s.h / s.lastTimeStep)};
        for (int k = 0; k < kMlpIn; ++k) f[q][k] = (float)((raw[k] - S.in_shift[k]) * S.in_scale[k]);
      }
    }
  }
  if (!__any_sync(0xffffffffu, use[0] || use[1])) return;
  float h1[8][4], h2[8][4], y[2];
  mlp_forward_warp(S, f[0], f[1], h1, h2, y);
  if (t != 0) return;
  for (int q = 0; q < 2; ++q) {
    if (!use[q]) continue;
    const int r = rows[q];
    const double corr = scale[q] * ((double)S.out_shift + (double)S.out_scale * (double)y[q]);
    d.x[r] = d.xn0[r] + corr;
  }
}

// Per-circuit gate of the learned predictor (one thread per circuit, before
// k_ml_predict): after each step attempt that ended, compare its Newton
// iteration count with the running mean of polynomial-predictor steps; a
// learned step that needed more iterations turns the learned predictor off
// for kMlBackoff steps, after which it is tried again.
__global__ void k_ml_gate(DevArrays d, int ncirc, int enabled) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncirc) return;
  CircState &s = d.cs[c];
  if (!s.start_step || s.phase != PH_TRAN) return;
  if (s.ml_pending) {  // the attempt that just ended used s.ml_use
    const double it = (double)s.last_iters;
    if (s.ml_use) {
      s.ml_steps++;
      s.ml_iters += s.last_iters;
      if (s.plain_steps > 0 && it > s.plain_ema + 0.5) s.ml_backoff = kMlBackoff;
    } else {
      s.plain_ema = (s.plain_steps == 0) ? it : 0.9 * s.plain_ema + 0.1 * it;
      s.plain_steps++;
      s.plain_iters += s.last_iters;
    }
  }
  s.ml_pending = 1;
  int use = enabled && s.accepted >= 4;
  if (use && s.ml_backoff > 0) { s.ml_backoff--; use = 0; }
  s.ml_use = use;
}

void launch_ml_predict_k(cudaStream_t st, const DevArrays &d, int n, int ncirc, int enabled) {
  k_ml_gate<<<(ncirc + 127) / 128, 128, 0, st>>>(d, ncirc, enabled);
  if (enabled) {
    const int warps = (n + 15) / 16;
    k_ml_predict<<<(warps + 3) / 4, 128, 0, st>>>(d, n);
  }
}

// ---- training -----------------------------------------------------------------
// Gradient of L = 0.5 / N * sum_r (MLP(x_r) - y_r)^2 over N standardized
// samples (features x[N][5] row-major, targets y[N], already standardized).
// Persistent blocks of 4 warps walk 64-row tiles; each thread owns fixed
// entries of the gradient vector and adds them to grad (FP32) once.
constexpr int kMlpGradThreads = 128;

struct GradSmem {
  MlpSmem S;
  float xs[64][kMlpIn];
  float h1s[64][kMlpHid], h2s[64][kMlpHid], dz2s[64][kMlpHid], dz1s[64][kMlpHid];
  float dys[64];
};

__global__ void __launch_bounds__(kMlpGradThreads) k_mlp_grad(MlpDev P, const float *__restrict__ X,
                                                               const float *__restrict__ Y, int N, float invN,
                                                               float *grad, float *loss) {
  extern __shared__ __align__(16) unsigned char smraw[];
  GradSmem &G = *reinterpret_cast<GradSmem *>(smraw);
  MlpSmem &S = G.S;
  auto &xs = G.xs;
  auto &h1s = G.h1s;
  auto &h2s = G.h2s;
  auto &dz2s = G.dz2s;
  auto &dz1s = G.dz1s;
  auto &dys = G.dys;
  mlp_load_smem(P, S);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  // owned gradient entries: W2 (4096) -> 32 each; W1 (320) -> up to 3; b1|b2|w3 (192) -> up to 2; b3
  float aW2[32], aW1[3] = {0.f, 0.f, 0.f}, aV[2] = {0.f, 0.f}, aB3 = 0.f, aL = 0.f;
#pragma unroll
  for (int m = 0; m < 32; ++m) aW2[m] = 0.f;
  const int ntiles = (N + 63) / 64;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int r0 = tile * 64 + warp * 16;
    float f[2][kMlpIn], tgt[2];
    bool valid[2];
    for (int q = 0; q < 2; ++q) {
      const int r = r0 + g + 8 * q;
      valid[q] = r < N;
      for (int k = 0; k < kMlpIn; ++k) f[q][k] = valid[q] ? X[(size_t)r * kMlpIn + k] : 0.f;
      tgt[q] = valid[q] ? Y[r] : 0.f;
    }
    float h1[8][4], h2[8][4], y[2];
    mlp_forward_warp(S, f[0], f[1], h1, h2, y);
    float dy[2];
    for (int q = 0; q < 2; ++q) {
      const float e = valid[q] ? (y[q] - tgt[q]) : 0.f;
      dy[q] = e * invN;
      if (t == 0) aL += 0.5f * e * e * invN;
    }
    // dZ2 = dy w3 (1 - h2^2), in accumulator layout
    float dz2[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = 8 * j + 2 * t;
      dz2[j][0] = dy[0] * S.w3[col] * (1.f - h2[j][0] * h2[j][0]);
      dz2[j][1] = dy[0] * S.w3[col + 1] * (1.f - h2[j][1] * h2[j][1]);
      dz2[j][2] = dy[1] * S.w3[col] * (1.f - h2[j][2] * h2[j][2]);
      dz2[j][3] = dy[1] * S.w3[col + 1] * (1.f - h2[j][3] * h2[j][3]);
    }
    // dH1 = dZ2 W2^T on the tensor cores: K = layer-2 outputs, N = layer-2 inputs
    uint32_t ad[4][4];
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
      ad[kb][0] = pack_bf16(dz2[2 * kb][0], dz2[2 * kb][1]);
      ad[kb][1] = pack_bf16(dz2[2 * kb][2], dz2[2 * kb][3]);
      ad[kb][2] = pack_bf16(dz2[2 * kb + 1][0], dz2[2 * kb + 1][1]);
      ad[kb][3] = pack_bf16(dz2[2 * kb + 1][2], dz2[2 * kb + 1][3]);
    }
    const int lr = warp * 16;  // this warp's rows in the tile
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const int nn = 8 * j + g;  // layer-2 input index (column of dH1)
#pragma unroll
      for (int kb = 0; kb < 4; ++kb) {
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w2[nn][16 * kb + 2 * t]);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w2[nn][16 * kb + 2 * t + 8]);
        mma16816(c, ad[kb], b0, b1);
      }
      const int col = 8 * j + 2 * t;
      dz1s[lr + g][col] = c[0] * (1.f - h1[j][0] * h1[j][0]);
      dz1s[lr + g][col + 1] = c[1] * (1.f - h1[j][1] * h1[j][1]);
      dz1s[lr + g + 8][col] = c[2] * (1.f - h1[j][2] * h1[j][2]);
      dz1s[lr + g + 8][col + 1] = c[3] * (1.f - h1[j][3] * h1[j][3]);
      h1s[lr + g][col] = h1[j][0]; h1s[lr + g][col + 1] = h1[j][1];
      h1s[lr + g + 8][col] = h1[j][2]; h1s[lr + g + 8][col + 1] = h1[j][3];
      h2s[lr + g][col] = h2[j][0]; h2s[lr + g][col + 1] = h2[j][1];
      h2s[lr + g + 8][col] = h2[j][2]; h2s[lr + g + 8][col + 1] = h2[j][3];
      dz2s[lr + g][col] = dz2[j][0]; dz2s[lr + g][col + 1] = dz2[j][1];
      dz2s[lr + g + 8][col] = dz2[j][2]; dz2s[lr + g + 8][col + 1] = dz2[j][3];
    }
    if (t == 0) {
      for (int q = 0; q < 2; ++q) {
        dys[lr + g + 8 * q] = dy[q];
        for (int k = 0; k < kMlpIn; ++k) xs[lr + g + 8 * q][k] = f[q][k];
      }
    }
    __syncthreads();
    // weight gradients over the tile's 64 rows (FP32)
#pragma unroll 4
    for (int m = 0; m < 32; ++m) {
      const int idx = tid + kMlpGradThreads * m, k = idx >> 6, nn = idx & 63;
      float s = 0.f;
      for (int r = 0; r < 64; ++r) s += h1s[r][k] * dz2s[r][nn];
      aW2[m] += s;
    }
    for (int m = 0; m < 3; ++m) {
      const int idx = tid + kMlpGradThreads * m;
      if (idx >= kMlpIn * kMlpHid) break;
      const int i = idx >> 6, k = idx & 63;
      float s = 0.f;
      for (int r = 0; r < 64; ++r) s += xs[r][i] * dz1s[r][k];
      aW1[m] += s;
    }
    for (int m = 0; m < 2; ++m) {
      const int idx = tid + kMlpGradThreads * m;  // 0..191: b1 | b2 | w3
      if (idx >= 3 * kMlpHid) break;
      const int part = idx >> 6, k = idx & 63;
      float s = 0.f;
      for (int r = 0; r < 64; ++r)
        s += (part == 0) ? dz1s[r][k] : (part == 1) ? dz2s[r][k] : dys[r] * h2s[r][k];
      aV[m] += s;
    }
    if (tid == 0) {
      float s = 0.f;
      for (int r = 0; r < 64; ++r) s += dys[r];
      aB3 += s;
    }
    __syncthreads();
  }
#pragma unroll 4
  for (int m = 0; m < 32; ++m) atomicAdd(&grad[kMlpOffW2 + tid + kMlpGradThreads * m], aW2[m]);
  for (int m = 0; m < 3; ++m) {
    const int idx = tid + kMlpGradThreads * m;
    if (idx < kMlpIn * kMlpHid) atomicAdd(&grad[kMlpOffW1 + idx], aW1[m]);
  }
  for (int m = 0; m < 2; ++m) {
    const int idx = tid + kMlpGradThreads * m;
    if (idx >= 3 * kMlpHid) break;
    const int part = idx >> 6, k = idx & 63;
    const int off = (part == 0) ? kMlpOffB1 : (part == 1) ? kMlpOffB2 : kMlpOffW3;
    atomicAdd(&grad[off + k], aV[m]);
  }
  if (tid == 0) atomicAdd(&grad[kMlpOffB3], aB3);
  for (int o = 16; o > 0; o >>= 1) aL += __shfl_xor_sync(0xffffffffu, aL, o);
  if (lane == 0) atomicAdd(loss, aL);
}

// Adam on the FP32 master vector, then the BF16 operand copies.
__global__ void k_mlp_adam(MlpDev P, const float *__restrict__ grad, float *m1, float *m2, float lr, float b1c,
                           float b2c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  const float gr = grad[i];
  const float a = 0.9f * m1[i] + 0.1f * gr, b = 0.999f * m2[i] + 0.001f * gr * gr;
  m1[i] = a;
  m2[i] = b;
  P.theta[i] -= lr * (a / b1c) / (sqrtf(b / b2c) + 1e-8f);
}

// BF16 operand copies of the master weights: w1t[n][k] = W1[k][n] (k < 5, else
// 0), w2t[n][k] = W2[k][n], w2[k][n] = W2[k][n].
__global__ void k_mlp_refresh(MlpDev P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  __nv_bfloat16 *w1t = reinterpret_cast<__nv_bfloat16 *>(P.w1t);
  __nv_bfloat16 *w2t = reinterpret_cast<__nv_bfloat16 *>(P.w2t);
  __nv_bfloat16 *w2 = reinterpret_cast<__nv_bfloat16 *>(P.w2);
  if (i < kMlpHid * kMlpInPad) {
    const int n = i / kMlpInPad, k = i % kMlpInPad;
    w1t[i] = __float2bfloat16_rn(k < kMlpIn ? P.theta[kMlpOffW1 + k * kMlpHid + n] : 0.f);
  }
  if (i < kMlpHid * kMlpHid) {
    const int n = i / kMlpHid, k = i % kMlpHid;
    w2t[i] = __float2bfloat16_rn(P.theta[kMlpOffW2 + k * kMlpHid + n]);
    w2[i] = __float2bfloat16_rn(P.theta[kMlpOffW2 + i]);
  }
}

// Forward only, for checks: out[r] = MLP(X[r]) (standardized units).
__global__ void __launch_bounds__(128) k_mlp_forward(MlpDev P, const float *__restrict__ X, int N, float *out) {
  __shared__ MlpSmem S;
  mlp_load_smem(P, S);
  const int r0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 16;
  if (r0 >= N) return;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float f[2][kMlpIn];
  for (int q = 0; q < 2; ++q) {
    const int r = r0 + g + 8 * q;
    for (int k = 0; k < kMlpIn; ++k) f[q][k] = (r < N) ? X[(size_t)r * kMlpIn + k] : 0.f;
  }
  float h1[8][4], h2[8][4], y[2];
  mlp_forward_warp(S, f[0], f[1], h1, h2, y);
  if (t == 0)
    for (int q = 0; q < 2; ++q) {
      const int r = r0 + g + 8 * q;
      if (r < N) out[r] = y[q];
    }
}

void launch_mlp_refresh_k(cudaStream_t st, const MlpDev &P) {
  k_mlp_refresh<<<(kMlpHid * kMlpHid + 255) / 256, 256, 0, st>>>(P);
}

int launch_mlp_grad_k(cudaStream_t st, const MlpDev &P, const float *X, const float *Y, int N, float *grad,
                      float *loss, int sm_count) {
  const int tiles = (N + 63) / 64;
  const int blocks = tiles < 2 * sm_count ? tiles : 2 * sm_count;
  const size_t smem = sizeof(GradSmem);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return XG_ERR_CUDA;
  if (blocks > 0)
    k_mlp_grad<<<blocks, kMlpGradThreads, smem, st>>>(P, X, Y, N, 1.0f / (float)(N > 0 ? N : 1), grad, loss);
  return XG_OK;
}

void launch_mlp_adam_k(cudaStream_t st, const MlpDev &P, const float *grad, float *m1, float *m2, float lr,
                       float b1c, float b2c) {
  k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(P, grad, m1, m2, lr, b1c, b2c);
}

void launch_mlp_forward_k(cudaStream_t st, const MlpDev &P, const float *X, int N, float *out) {
  const int warps = (N + 15) / 16;
  if (warps > 0) k_mlp_forward<<<(warps + 3) / 4, 128, 0, st>>>(P, X, N, out);
}

}  // namespace xg
