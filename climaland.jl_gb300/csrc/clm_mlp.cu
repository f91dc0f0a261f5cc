// MLP kernels of the learned Newton initial guess: training (forward +
// backward in one kernel, Adam), prediction, and the per-step guess.
//
// All GEMMs are BF16 x BF16 -> FP32 on the tensor cores through
// mma.sync.m16n8k16 (operand fragments built from shared memory or repacked
// from the previous layer's accumulators). A CTA of four warps owns 64 rows
// (16 per warp). Weight gradients are reduced per CTA with the same MMA
// (transposed activations staged in shared memory) and added to a global
// FP32 gradient with atomics; Adam keeps FP32 master weights.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "clm_column.cuh"
#include "clm_mlp.cuh"

namespace clm {
namespace mlp {

constexpr int kRows = 64;   // rows per CTA
constexpr int kWarps = 4;
constexpr int kSR = kRows + 8;  // padded row length of row-indexed (transposed) tiles

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low 16 bits)
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ void mma(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// Shared-memory image of the weights: transposed (WT[n][k], k contiguous:
// B operands of the forward GEMMs), BF16, padded rows; biases and the
// standardisation in FP32. Inference kernels stage only this.
struct Weights {
  __nv_bfloat16 W1T[kMlpHidden][kMlpInPad + 8];
  __nv_bfloat16 W2T[kMlpHidden][kMlpHidden + 8];
  __nv_bfloat16 W3T[kMlpOut][kMlpHidden + 8];
  float b1[kMlpHidden], b2[kMlpHidden], b3[kMlpOut];
  float in_mean[kMlpIn], in_istd[kMlpIn], out_mean[kMlpOut], out_std[kMlpOut];
};

// Training adds the row-major weights (W[k][n], n contiguous: B operands of
// the backward GEMMs dY W^T) and the CTA's transposed activations.
struct Smem : Weights {
  __nv_bfloat16 W2r[kMlpHidden][kMlpHidden + 8];
  __nv_bfloat16 W3r[kMlpHidden][kMlpOutPad + 8];
  __nv_bfloat16 XT[kMlpInPad][kSR];
  __nv_bfloat16 H1T[kMlpHidden][kSR];
  __nv_bfloat16 H2T[kMlpHidden][kSR];
  __nv_bfloat16 dA1T[kMlpHidden][kSR];
  __nv_bfloat16 dA2T[kMlpHidden][kSR];
  __nv_bfloat16 dYT[kMlpOutPad][kSR];
  // per-warp staging of 16 rows of raw inputs
  float xs[kWarps][16][kMlpInPad];
};

// Inference (prediction, in-step guess): eight warps of 16 rows each.
constexpr int kInferWarps = 8;
struct InferSmem : Weights {
  float xs[kInferWarps][16][kMlpInPad];
};

__device__ void stage_forward(Weights& S, const float* __restrict__ P, const float* __restrict__ norm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < kMlpInPad * kMlpHidden; i += nt) {
    const int k = i / kMlpHidden, n = i % kMlpHidden;
    S.W1T[n][k] = __float2bfloat16_rn(P[kMlpW1 + i]);
  }
  for (int i = tid; i < kMlpHidden * kMlpHidden; i += nt) {
    const int k = i / kMlpHidden, n = i % kMlpHidden;
    S.W2T[n][k] = __float2bfloat16_rn(P[kMlpW2 + i]);
  }
  for (int i = tid; i < kMlpHidden * kMlpOut; i += nt) {
    const int k = i / kMlpOut, n = i % kMlpOut;
    S.W3T[n][k] = __float2bfloat16_rn(P[kMlpW3 + i]);
  }
  for (int i = tid; i < kMlpHidden; i += nt) {
    S.b1[i] = P[kMlpB1 + i];
    S.b2[i] = P[kMlpB2 + i];
  }
  for (int i = tid; i < kMlpOut; i += nt) {
    S.b3[i] = P[kMlpB3 + i];
    S.out_mean[i] = norm[2 * kMlpIn + i];
    S.out_std[i] = norm[2 * kMlpIn + kMlpOut + i];
  }
  for (int i = tid; i < kMlpIn; i += nt) {
    S.in_mean[i] = norm[i];
    const float sd = norm[kMlpIn + i];
    S.in_istd[i] = sd > 1e-20f ? 1.0f / sd : 0.0f;
  }
}

__device__ void stage_weights(Smem& S, const float* __restrict__ P, const float* __restrict__ norm) {
  stage_forward(S, P, norm);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < kMlpHidden * kMlpHidden; i += nt) {
    const int k = i / kMlpHidden, n = i % kMlpHidden;
    S.W2r[k][n] = __float2bfloat16_rn(P[kMlpW2 + i]);
  }
  for (int i = tid; i < kMlpHidden * kMlpOutPad; i += nt) {
    const int k = i / kMlpOutPad, n = i % kMlpOutPad;
    S.W3r[k][n] = __float2bfloat16_rn(n < kMlpOut ? P[kMlpW3 + k * kMlpOut + n] : 0.0f);
  }
}

// Forward pass of one warp's 16 rows given their A fragments (5 k-chunks of
// the standardised inputs). Leaves the pre-activations in A1, A2 and the
// standardised outputs in Y (accumulator layout).
struct Fwd {
  float A1[8][4], A2[8][4], Y[5][4];
};

__device__ __forceinline__ void forward16(const Weights& S, const uint32_t xf[5][4], Fwd& F,
                                          uint32_t h1f[4][4], uint32_t h2f[4][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  // layer 1
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = S.b1[8 * j + 2 * t], b1 = S.b1[8 * j + 2 * t + 1];
    F.A1[j][0] = b0; F.A1[j][1] = b1; F.A1[j][2] = b0; F.A1[j][3] = b1;
#pragma unroll
    for (int kk = 0; kk < 5; ++kk)
      mma(F.A1[j], xf[kk], ld32(&S.W1T[8 * j + g][16 * kk + 2 * t]),
          ld32(&S.W1T[8 * j + g][16 * kk + 2 * t + 8]));
  }
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const float* c0 = F.A1[2 * kk];
    const float* c1 = F.A1[2 * kk + 1];
    h1f[kk][0] = pack2(gelu(c0[0]), gelu(c0[1]));
    h1f[kk][1] = pack2(gelu(c0[2]), gelu(c0[3]));
    h1f[kk][2] = pack2(gelu(c1[0]), gelu(c1[1]));
    h1f[kk][3] = pack2(gelu(c1[2]), gelu(c1[3]));
  }
  // layer 2
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = S.b2[8 * j + 2 * t], b1 = S.b2[8 * j + 2 * t + 1];
    F.A2[j][0] = b0; F.A2[j][1] = b1; F.A2[j][2] = b0; F.A2[j][3] = b1;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
      mma(F.A2[j], h1f[kk], ld32(&S.W2T[8 * j + g][16 * kk + 2 * t]),
          ld32(&S.W2T[8 * j + g][16 * kk + 2 * t + 8]));
  }
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const float* c0 = F.A2[2 * kk];
    const float* c1 = F.A2[2 * kk + 1];
    h2f[kk][0] = pack2(gelu(c0[0]), gelu(c0[1]));
    h2f[kk][1] = pack2(gelu(c0[2]), gelu(c0[3]));
    h2f[kk][2] = pack2(gelu(c1[0]), gelu(c1[1]));
    h2f[kk][3] = pack2(gelu(c1[2]), gelu(c1[3]));
  }
  // output layer
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const float b0 = S.b3[8 * j + 2 * t], b1 = S.b3[8 * j + 2 * t + 1];
    F.Y[j][0] = b0; F.Y[j][1] = b1; F.Y[j][2] = b0; F.Y[j][3] = b1;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
      mma(F.Y[j], h2f[kk], ld32(&S.W3T[8 * j + g][16 * kk + 2 * t]),
          ld32(&S.W3T[8 * j + g][16 * kk + 2 * t + 8]));
  }
}

// A fragments of 16 staged rows xs[16][kMlpInPad] (raw features):
// standardise and pack (feature columns >= kMlpIn are zero).
__device__ __forceinline__ void input_fragments(const Weights& S, const float (*xs)[kMlpInPad],
                                                uint32_t xf[5][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  auto val = [&](int r, int f) -> float {
    return f < kMlpIn ? (xs[r][f] - S.in_mean[f]) * S.in_istd[f] : 0.0f;
  };
#pragma unroll
  for (int kk = 0; kk < 5; ++kk) {
    const int c = 16 * kk + 2 * t;
    xf[kk][0] = pack2(val(g, c), val(g, c + 1));
    xf[kk][1] = pack2(val(g + 8, c), val(g + 8, c + 1));
    xf[kk][2] = pack2(val(g, c + 8), val(g, c + 9));
    xf[kk][3] = pack2(val(g + 8, c + 8), val(g + 8, c + 9));
  }
}

// ---------------------------------------------------------------------------
// training: forward + backward for rows [row0, row0 + nrows) of (X, Y)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kWarps * 32)
    train_kernel(const float* __restrict__ P, const float* __restrict__ norm,
                 const float* __restrict__ X, const float* __restrict__ Yt, int64_t row0,
                 int nrows, float* __restrict__ grads, float* __restrict__ loss_sum) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  stage_weights(S, P, norm);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int cta_row = blockIdx.x * kRows;
  // raw rows of this warp into xs (zero beyond nrows)
  for (int i = lane; i < 16 * kMlpInPad; i += 32) {
    const int r = i / kMlpInPad, f = i % kMlpInPad;
    const int row = cta_row + 16 * warp + r;
    S.xs[warp][r][f] = (row < nrows && f < kMlpIn) ? X[(row0 + row) * kMlpIn + f] : 0.0f;
  }
  __syncthreads();
  uint32_t xf[5][4], h1f[4][4], h2f[4][4];
  input_fragments(S, S.xs[warp], xf);
  // XT (standardised inputs, transposed) for dW1
  for (int i = lane; i < 16 * kMlpInPad; i += 32) {
    const int r = i % 16, f = i / 16;
    const float x = f < kMlpIn ? (S.xs[warp][r][f] - S.in_mean[f]) * S.in_istd[f] : 0.0f;
    S.XT[f][16 * warp + r] = __float2bfloat16_rn(x);
  }
  Fwd F;
  forward16(S, xf, F, h1f, h2f);
  const int rA = 16 * warp + g, rB = rA + 8;  // CTA-local rows of this thread
  const bool vA = cta_row + rA < nrows, vB = cta_row + rB < nrows;
  // store H1T, H2T
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = 8 * j + 2 * t;
    S.H1T[c][rA] = __float2bfloat16_rn(gelu(F.A1[j][0]));
    S.H1T[c + 1][rA] = __float2bfloat16_rn(gelu(F.A1[j][1]));
    S.H1T[c][rB] = __float2bfloat16_rn(gelu(F.A1[j][2]));
    S.H1T[c + 1][rB] = __float2bfloat16_rn(gelu(F.A1[j][3]));
    S.H2T[c][rA] = __float2bfloat16_rn(gelu(F.A2[j][0]));
    S.H2T[c + 1][rA] = __float2bfloat16_rn(gelu(F.A2[j][1]));
    S.H2T[c][rB] = __float2bfloat16_rn(gelu(F.A2[j][2]));
    S.H2T[c + 1][rB] = __float2bfloat16_rn(gelu(F.A2[j][3]));
  }
  // loss and dY (standardised targets), mean over the batch
  const float scale = 2.0f / (float)nrows;
  float dY[5][4];
  float lsum = 0.0f;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int o = 8 * j + 2 * t + (q & 1);
      const int r = (q < 2) ? rA : rB;
      const bool valid = (q < 2) ? vA : vB;
      float d = 0.0f;
      if (valid) {
        const float tgt = (Yt[(row0 + cta_row + r) * kMlpOut + o] - S.out_mean[o]) / S.out_std[o];
        const float e = F.Y[j][q] - tgt;
        lsum += e * e;
        d = scale * e;
      }
      dY[j][q] = d;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
  if (lane == 0) atomicAdd(loss_sum, lsum);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int c = 8 * j + 2 * t;
    S.dYT[c][rA] = __float2bfloat16_rn(j < 5 ? dY[j][0] : 0.0f);
    S.dYT[c + 1][rA] = __float2bfloat16_rn(j < 5 ? dY[j][1] : 0.0f);
    S.dYT[c][rB] = __float2bfloat16_rn(j < 5 ? dY[j][2] : 0.0f);
    S.dYT[c + 1][rB] = __float2bfloat16_rn(j < 5 ? dY[j][3] : 0.0f);
  }
  // dH2 = dY W3^T (k = output, 3 chunks of 16; outputs >= 40 are zero)
  uint32_t dyf[3][4];
#pragma unroll
  for (int kk = 0; kk < 3; ++kk) {
    const int j0 = 2 * kk, j1 = 2 * kk + 1;
    dyf[kk][0] = pack2(dY[j0][0], dY[j0][1]);
    dyf[kk][1] = pack2(dY[j0][2], dY[j0][3]);
    dyf[kk][2] = j1 < 5 ? pack2(dY[j1][0], dY[j1][1]) : 0u;
    dyf[kk][3] = j1 < 5 ? pack2(dY[j1][2], dY[j1][3]) : 0u;
  }
  float dA2[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    dA2[j][0] = dA2[j][1] = dA2[j][2] = dA2[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 3; ++kk)
      mma(dA2[j], dyf[kk], ld32(&S.W3r[8 * j + g][16 * kk + 2 * t]),
          ld32(&S.W3r[8 * j + g][16 * kk + 2 * t + 8]));
#pragma unroll
    for (int q = 0; q < 4; ++q) dA2[j][q] *= gelu_grad(F.A2[j][q]);
  }
  uint32_t da2f[4][4];
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    da2f[kk][0] = pack2(dA2[2 * kk][0], dA2[2 * kk][1]);
    da2f[kk][1] = pack2(dA2[2 * kk][2], dA2[2 * kk][3]);
    da2f[kk][2] = pack2(dA2[2 * kk + 1][0], dA2[2 * kk + 1][1]);
    da2f[kk][3] = pack2(dA2[2 * kk + 1][2], dA2[2 * kk + 1][3]);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = 8 * j + 2 * t;
    S.dA2T[c][rA] = __float2bfloat16_rn(dA2[j][0]);
    S.dA2T[c + 1][rA] = __float2bfloat16_rn(dA2[j][1]);
    S.dA2T[c][rB] = __float2bfloat16_rn(dA2[j][2]);
    S.dA2T[c + 1][rB] = __float2bfloat16_rn(dA2[j][3]);
  }
  // dH1 = dA2 W2^T
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
      mma(d, da2f[kk], ld32(&S.W2r[8 * j + g][16 * kk + 2 * t]),
          ld32(&S.W2r[8 * j + g][16 * kk + 2 * t + 8]));
    const int c = 8 * j + 2 * t;
    S.dA1T[c][rA] = __float2bfloat16_rn(d[0] * gelu_grad(F.A1[j][0]));
    S.dA1T[c + 1][rA] = __float2bfloat16_rn(d[1] * gelu_grad(F.A1[j][1]));
    S.dA1T[c][rB] = __float2bfloat16_rn(d[2] * gelu_grad(F.A1[j][2]));
    S.dA1T[c + 1][rB] = __float2bfloat16_rn(d[3] * gelu_grad(F.A1[j][3]));
  }
  __syncthreads();
  // weight gradients: dW = act^T dA over the CTA's 64 rows (4 k-chunks).
  // Output tiles: dW1 5x8, dW2 4x8, dW3 4x5 (m16 x n8), spread over warps.
  const int nt1 = 5 * 8, nt2 = 4 * 8, nt3 = 4 * 5;
  for (int tile = warp; tile < nt1 + nt2 + nt3; tile += kWarps) {
    const __nv_bfloat16(*Am)[kSR];
    const __nv_bfloat16(*Bm)[kSR];
    int mt, ntile, ldo, base;
    if (tile < nt1) {
      Am = S.XT; Bm = S.dA1T; mt = tile / 8; ntile = tile % 8; ldo = kMlpHidden; base = kMlpW1;
    } else if (tile < nt1 + nt2) {
      const int u = tile - nt1;
      Am = S.H1T; Bm = S.dA2T; mt = u / 8; ntile = u % 8; ldo = kMlpHidden; base = kMlpW2;
    } else {
      const int u = tile - nt1 - nt2;
      Am = S.H2T; Bm = S.dYT; mt = u / 5; ntile = u % 5; ldo = kMlpOut; base = kMlpW3;
    }
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      uint32_t a[4];
      a[0] = ld32(&Am[16 * mt + g][16 * kk + 2 * t]);
      a[1] = ld32(&Am[16 * mt + g + 8][16 * kk + 2 * t]);
      a[2] = ld32(&Am[16 * mt + g][16 * kk + 2 * t + 8]);
      a[3] = ld32(&Am[16 * mt + g + 8][16 * kk + 2 * t + 8]);
      mma(c, a, ld32(&Bm[8 * ntile + g][16 * kk + 2 * t]), ld32(&Bm[8 * ntile + g][16 * kk + 2 * t + 8]));
    }
    const int m0 = 16 * mt + g, n0 = 8 * ntile + 2 * t;
    atomicAdd(&grads[base + m0 * ldo + n0], c[0]);
    atomicAdd(&grads[base + m0 * ldo + n0 + 1], c[1]);
    atomicAdd(&grads[base + (m0 + 8) * ldo + n0], c[2]);
    atomicAdd(&grads[base + (m0 + 8) * ldo + n0 + 1], c[3]);
  }
  // bias gradients: column sums of dA1, dA2, dY over the rows
  for (int i = threadIdx.x; i < 2 * kMlpHidden + kMlpOut; i += blockDim.x) {
    const __nv_bfloat16* row;
    int dst;
    if (i < kMlpHidden) { row = S.dA1T[i]; dst = kMlpB1 + i; }
    else if (i < 2 * kMlpHidden) { row = S.dA2T[i - kMlpHidden]; dst = kMlpB2 + i - kMlpHidden; }
    else { row = S.dYT[i - 2 * kMlpHidden]; dst = kMlpB3 + i - 2 * kMlpHidden; }
    float sum = 0.0f;
    for (int r = 0; r < kRows; ++r) sum += __bfloat162float(row[r]);
    atomicAdd(&grads[dst], sum);
  }
}

// Adam with bias correction; clears the gradient for the next step.
__global__ void adam_kernel(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M,
                            float* __restrict__ V, int n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.0f - b1) * g;
  const float v = b2 * V[i] + (1.0f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  P[i] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
  G[i] = 0.0f;
}

// ---------------------------------------------------------------------------
// prediction on raw feature rows (de-standardised outputs)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kInferWarps * 32)
    predict_kernel(const float* __restrict__ P, const float* __restrict__ norm,
                   const float* __restrict__ X, int64_t nrows, float* __restrict__ Yout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
  stage_forward(S, P, norm);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  for (int64_t r0 = (int64_t)(blockIdx.x * kInferWarps + warp) * 16; r0 < nrows;
       r0 += (int64_t)gridDim.x * kInferWarps * 16) {
    for (int i = lane; i < 16 * kMlpInPad; i += 32) {
      const int r = i / kMlpInPad, f = i % kMlpInPad;
      S.xs[warp][r][f] = (r0 + r < nrows && f < kMlpIn) ? X[(r0 + r) * kMlpIn + f] : 0.0f;
    }
    __syncwarp();
    uint32_t xf[5][4], h1f[4][4], h2f[4][4];
    input_fragments(S, S.xs[warp], xf);
    Fwd F;
    forward16(S, xf, F, h1f, h2f);
#pragma unroll
    for (int j = 0; j < 5; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int o = 8 * j + 2 * t + (q & 1);
        const int64_t r = r0 + g + (q < 2 ? 0 : 8);
        if (r < nrows) Yout[r * kMlpOut + o] = F.Y[j][q] * S.out_std[o] + S.out_mean[o];
      }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// features of the handle's columns (original order) and the in-step guess
// ---------------------------------------------------------------------------
__global__ void features_kernel(StepArgs A, double t, double dt, float* __restrict__ X) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.L.stride || A.L.col_n[s] != kMlpLayers) return;
  const int tile = s / kTile, lane = s % kTile;
  const int64_t base = A.L.tile_off[tile] + lane;
  Col<double> v{A.v + base, kTile}, ti{A.ti + base, kTile}, e{A.e + base, kTile};
  float f[kMlpIn];
  column_features(A, s, A.L.perm[s], v, ti, e, t, dt, f);
  float* out = X + (int64_t)A.L.perm[s] * kMlpIn;
  for (int i = 0; i < kMlpIn; ++i) out[i] = f[i];
}

// guess[0][cell] = delta vartheta_l, guess[1][cell] = delta rho_e_int
// (internal layout), for every 20-layer column: the column's previous
// increment (its state now minus `prev`, the state at the previous guess)
// plus the network's predicted change of the increment; `prev` then takes
// the current state. A warp takes 16 columns; its two half-warps build the
// features of layers 0-9 and 10-19.
__global__ void __launch_bounds__(kInferWarps * 32)
    guess_kernel(StepArgs A, const float* __restrict__ P, const float* __restrict__ norm,
                 StepClock clk, float* __restrict__ guess, double* __restrict__ prev) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
  stage_forward(S, P, norm);
  __syncthreads();
  const double t = clk.start(), dt = clk.step();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
  const int64_t nci = A.L.ncells_int;
  const int nrows = A.L.stride;
  const int half = lane >> 4;
  constexpr int kHalf = kMlpLayers / 2;
  for (int r0 = (blockIdx.x * kInferWarps + warp) * 16; r0 < nrows;
       r0 += gridDim.x * kInferWarps * 16) {
    {
      const int s = r0 + (lane & 15);
      float* xr = S.xs[warp][lane & 15];
      if (A.L.col_n[s] == kMlpLayers) {
        const int64_t base = A.L.tile_off[s / kTile] + s % kTile;
        Col<double> v{A.v + base, kTile}, ti{A.ti + base, kTile}, e{A.e + base, kTile};
        column_features(A, s, A.L.perm[s], v, ti, e, t, dt, xr, half * kHalf, (half + 1) * kHalf,
                        half == 1);
      } else {
        for (int f = half; f < kMlpIn; f += 2) xr[f] = S.in_mean[f];
      }
      if (half == 0)
        for (int f = kMlpIn; f < kMlpInPad; ++f) xr[f] = 0.0f;
    }
    __syncwarp();
    uint32_t xf[5][4], h1f[4][4], h2f[4][4];
    input_fragments(S, S.xs[warp], xf);
    Fwd F;
    forward16(S, xf, F, h1f, h2f);
#pragma unroll
    for (int j = 0; j < 5; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int o = 8 * j + 2 * t4 + (q & 1);
        const int s = r0 + g + (q < 2 ? 0 : 8);
        if (A.L.col_n[s] != kMlpLayers) continue;
        const int k = o % kMlpLayers;
        const int64_t cell = A.L.tile_off[s / kTile] + (int64_t)k * kTile + s % kTile;
        const int64_t slot = (o < kMlpLayers ? 0 : nci) + cell;
        const double cur = o < kMlpLayers ? A.v[cell] : A.e[cell];
        const double inc = cur - prev[slot];
        prev[slot] = cur;
        guess[slot] = (float)(inc + (double)(F.Y[j][q] * S.out_std[o] + S.out_mean[o]));
      }
    __syncwarp();
  }
}

}  // namespace mlp

size_t mlp_smem_bytes() { return sizeof(mlp::Smem); }

cudaError_t mlp_train_step(const float* P, const float* norm, const float* X, const float* Y,
                           int64_t row0, int nrows, float* grads, float* loss_sum, cudaStream_t st) {
  const size_t sm = sizeof(mlp::Smem);
  cudaError_t e = cudaFuncSetAttribute(mlp::train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  mlp::train_kernel<<<(nrows + mlp::kRows - 1) / mlp::kRows, mlp::kWarps * 32, sm, st>>>(
      P, norm, X, Y, row0, nrows, grads, loss_sum);
  return cudaGetLastError();
}

cudaError_t mlp_adam(float* P, float* G, float* M, float* V, int step, float lr, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
  const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
  mlp::adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(P, G, M, V, kMlpParams, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

// Persistent grid: resident CTAs of the inference kernels (all SMs).
template <typename K>
static int infer_grid(K kernel, size_t sm, int64_t rows) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, mlp::kInferWarps * 32, sm);
  const int64_t need = (rows + 16 * mlp::kInferWarps - 1) / (16 * mlp::kInferWarps);
  int64_t grid = (int64_t)(per > 0 ? per : 1) * (nsm > 0 ? nsm : 1);
  if (grid > need) grid = need;
  return grid < 1 ? 1 : (int)grid;
}

cudaError_t mlp_predict(const float* P, const float* norm, const float* X, int64_t nrows, float* Y,
                        cudaStream_t st) {
  const size_t sm = sizeof(mlp::InferSmem);
  cudaError_t e = cudaFuncSetAttribute(mlp::predict_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = infer_grid(mlp::predict_kernel, sm, nrows);
  mlp::predict_kernel<<<grid, mlp::kInferWarps * 32, sm, st>>>(P, norm, X, nrows, Y);
  return cudaGetLastError();
}

cudaError_t mlp_features(const StepArgs& A, double t, double dt, float* X, cudaStream_t st) {
  mlp::features_kernel<<<(A.L.stride + 127) / 128, 128, 0, st>>>(A, t, dt, X);
  return cudaGetLastError();
}

// Kernel attribute and persistent grid of the guess kernel: set up once
// (clm_load_mlp), so the per-step launch makes no other runtime call and can
// be captured in a CUDA graph.
cudaError_t mlp_guess_setup(int64_t rows, int* grid) {
  const size_t sm = sizeof(mlp::InferSmem);
  cudaError_t e = cudaFuncSetAttribute(mlp::guess_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  *grid = infer_grid(mlp::guess_kernel, sm, rows);
  return cudaGetLastError();
}

cudaError_t mlp_guess(const StepArgs& A, const float* P, const float* norm, const StepClock& clk,
                      float* guess, double* prev, int grid, cudaStream_t st) {
  mlp::guess_kernel<<<grid, mlp::kInferWarps * 32, sizeof(mlp::InferSmem), st>>>(A, P, norm, clk, guess, prev);
  return cudaGetLastError();
}

}  // namespace clm
