// pbf_mlp.cuh — device pieces of the learned start's MLP shared by the
// training/inference kernels (pbf_learned.cu) and the fused feature + network
// pass of the step (pbf_passes.cuh): flat parameter layout, bf16 packing, the
// mma.sync.m16n8k16 wrapper, SiLU, weight staging and the 16-row forward tile.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"
#include "pbf_params.h"

namespace pbf {
namespace mlp {

constexpr int kIn = 8, kH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + kIn * kH, OFF_W2 = OFF_B1 + kH, OFF_B2 = OFF_W2 + kH * kH,
              OFF_W3 = OFF_B2 + kH, OFF_B3 = OFF_W3 + kH, kParams = OFF_B3 + 1;
static_assert(kParams == PBF_MLP_PARAMS, "flat parameter layout");

constexpr int kW1S = 24;  // bf16 row stride of W1^T in smem (16 + 8 pad)
constexpr int kW2S = 72;  // bf16 row stride of 64-wide tiles (64 + 8 pad)

using Norm = MLPNorm;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// sigmoid(z) = (1 + tanh(z/2)) / 2 with the hardware tanh approximation
// (tanh.approx.f32, one MUFU instruction; absolute error ~ 2^-11, below the
// bf16 rounding the activations get next).
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sigmoid_f(float z) { return fmaf(0.5f, tanh_fast(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu_f(float z) { return z * sigmoid_f(z); }
__device__ __forceinline__ float dsilu_f(float z) {
  float s = sigmoid_f(z);
  return s * (1.0f + z * (1.0f - s));
}

// Stage W1^T (bf16, k padded to 16), W2^T and optionally W2 into shared memory.
__device__ __forceinline__ void stage_weights(const float* __restrict__ P, uint16_t* sW1t, uint16_t* sW2t, uint16_t* sW2) {
  for (int q = threadIdx.x; q < kH * 16; q += blockDim.x) {
    int n = q / 16, k = q % 16;
    float w = (k < kIn) ? P[OFF_W1 + k * kH + n] : 0.0f;
    __nv_bfloat16 b = __float2bfloat16_rn(w);
    sW1t[n * kW1S + k] = *reinterpret_cast<uint16_t*>(&b);
  }
  for (int q = threadIdx.x; q < kH * kH; q += blockDim.x) {
    int k = q / kH, n = q % kH;  // W2[k][n]
    __nv_bfloat16 b = __float2bfloat16_rn(P[OFF_W2 + q]);
    uint16_t u = *reinterpret_cast<uint16_t*>(&b);
    sW2t[n * kW2S + k] = u;
    if (sW2) sW2[k * kW2S + n] = u;
  }
}

// Forward pass of one 16-row tile held by a warp.  x: normalised inputs of
// rows g and g+8, features 2t and 2t+1 (the A fragment columns this lane
// holds).  Returns z1/z2 pre-activations (for the backward pass), the bf16
// A fragments of h1, and y for rows g and g+8 in every lane of the group.
struct Fwd {
  float z1[8][4];
  float z2[8][4];
  uint32_t a2[4][4];  // h1 as A fragments (k-steps of layer 2)
  float h2[8][4];     // bf16-rounded h2
  float y0, y8;
};

__device__ __forceinline__ void forward_tile(const float (&xg)[2], const float (&x8)[2], const uint16_t* sW1t,
                                             const uint16_t* sW2t, const float* sB1, const float* sB2,
                                             const float* sW3, float b3, Fwd& F) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t a1[4] = {pack_bf16(xg[0], xg[1]), pack_bf16(x8[0], x8[1]), 0u, 0u};
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    int n = 8 * j + g;
    uint32_t b0 = *reinterpret_cast<const uint32_t*>(sW1t + n * kW1S + 2 * t);
    uint32_t b1 = *reinterpret_cast<const uint32_t*>(sW1t + n * kW1S + 8 + 2 * t);
    float c0 = sB1[8 * j + 2 * t], c1 = sB1[8 * j + 2 * t + 1];
    float d[4] = {c0, c1, c0, c1};
    mma16816(d, a1, b0, b1);
#pragma unroll
    for (int q = 0; q < 4; ++q) F.z1[j][q] = d[q];
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    F.a2[s][0] = pack_bf16(silu_f(F.z1[2 * s][0]), silu_f(F.z1[2 * s][1]));
    F.a2[s][1] = pack_bf16(silu_f(F.z1[2 * s][2]), silu_f(F.z1[2 * s][3]));
    F.a2[s][2] = pack_bf16(silu_f(F.z1[2 * s + 1][0]), silu_f(F.z1[2 * s + 1][1]));
    F.a2[s][3] = pack_bf16(silu_f(F.z1[2 * s + 1][2]), silu_f(F.z1[2 * s + 1][3]));
  }
  float yg = 0.0f, y8 = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    int n = 8 * j + g;
    float c0 = sB2[8 * j + 2 * t], c1 = sB2[8 * j + 2 * t + 1];
    float d[4] = {c0, c1, c0, c1};
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      uint32_t b0 = *reinterpret_cast<const uint32_t*>(sW2t + n * kW2S + 16 * s + 2 * t);
      uint32_t b1 = *reinterpret_cast<const uint32_t*>(sW2t + n * kW2S + 16 * s + 8 + 2 * t);
      mma16816(d, F.a2[s], b0, b1);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      F.z2[j][q] = d[q];
      F.h2[j][q] = bf16_round(silu_f(d[q]));
    }
    float w0 = sW3[8 * j + 2 * t], w1 = sW3[8 * j + 2 * t + 1];
    yg += F.h2[j][0] * w0 + F.h2[j][1] * w1;
    y8 += F.h2[j][2] * w0 + F.h2[j][3] * w1;
  }
  yg += __shfl_xor_sync(0xffffffffu, yg, 1);
  yg += __shfl_xor_sync(0xffffffffu, yg, 2);
  y8 += __shfl_xor_sync(0xffffffffu, y8, 1);
  y8 += __shfl_xor_sync(0xffffffffu, y8, 2);
  F.y0 = yg + b3;
  F.y8 = y8 + b3;
}

__device__ __forceinline__ void load_inputs(const float* __restrict__ feat, const Norm& nm, uint32_t rows,
                                            uint32_t r0, float (&xg)[2], float (&x8)[2]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t ra = r0 + g, rb = r0 + g + 8;
  float2 fa = (ra < rows) ? *reinterpret_cast<const float2*>(feat + 8 * (size_t)ra + 2 * t) : make_float2(0.f, 0.f);
  float2 fb = (rb < rows) ? *reinterpret_cast<const float2*>(feat + 8 * (size_t)rb + 2 * t) : make_float2(0.f, 0.f);
  int k0 = 2 * t, k1 = 2 * t + 1;
  xg[0] = (ra < rows) ? (fa.x - nm.mean[k0]) * nm.inv_std[k0] : 0.0f;
  xg[1] = (ra < rows) ? (fa.y - nm.mean[k1]) * nm.inv_std[k1] : 0.0f;
  x8[0] = (rb < rows) ? (fb.x - nm.mean[k0]) * nm.inv_std[k0] : 0.0f;
  x8[1] = (rb < rows) ? (fb.y - nm.mean[k1]) * nm.inv_std[k1] : 0.0f;
}

}  // namespace mlp
}  // namespace pbf
