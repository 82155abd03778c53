// pbf_device.cuh — device math of the PBF substep: SPH kernels, the jittered
// wall clamp and the volume-map interpolation.
//
// Included by the two pass translation units: pbf_passes_exact.cu is compiled
// with -fmad=false, so every a*b+c below rounds twice exactly like the CPU
// restatement and the results are bit-identical to it; pbf_passes_fast.cu
// lets the compiler form FMAs.  Every formula keeps the operation order of the
// reference WGSL it restates (cited per function).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_params.h"

namespace pbf {

#ifdef PBF_FAST_MATH
constexpr bool kFast = true;
#else
constexpr bool kFast = false;
#endif

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ f3 divs(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }

// ---- SPH kernels (src/simulator/PBF/shader/common.ts:1-40) -----------------------
// poly6: coef * (h^2 - r^2)^3 for r <= h
__device__ __forceinline__ float poly6(const SimParams& p, float rl) {
  float t = p.h2 - rl * rl;
  float x = (rl <= p.h) ? (t * t * t) : 0.0f;
  return p.poly6 * x;
}
// spiky gradient: coef * (h - r)^2 * r/|r|, zero direction at r == 0
__device__ __forceinline__ f3 spiky_grad(const SimParams& p, f3 d, float rl) {
  float t = p.h - rl;
  float x = (rl <= p.h) ? (t * t) : 0.0f;
  f3 n = (rl > 0.0f) ? divs(d, rl) : mk(0.f, 0.f, 0.f);
  return (p.spiky * x) * n;
}
// Akinci cohesion spline times r/|r|
__device__ __forceinline__ f3 cohesion(const SimParams& p, f3 d, float rl) {
  float a = p.h - rl;
  float a3 = a * a * a;
  float b3 = rl * rl * rl;
  float t = a3 * b3;
  float res = (rl > p.half_h) ? t : fmaf(2.0f, t, p.coh_bias);
  res = (rl <= p.h) ? res : 0.0f;
  f3 n = (rl > 0.0f) ? divs(d, rl) : mk(0.f, 0.f, 0.f);
  return (p.coh * res) * n;
}

// One particle pair: offset d, |d|^2, |d| and 1/|d| (0 at d = 0).  Exact mode
// evaluates |d| = sqrt(d.d) and divides like the reference; fast mode uses
// rsqrt and multiplies by the reciprocal.
struct Pair {
  f3 d;
  float r2, rl, ir;
};
// 1 / sqrt(x) by the hardware approximation (rsqrt.approx.ftz.f32, one MUFU
// instruction): the fast mode's pair distance.  A squared distance below the
// normal range (|d| < 1e-19, only the pair of a particle with itself in
// practice, where r^2 = 0) gives +inf; make_pair_of zeroes r^2 = 0 itself.
__device__ __forceinline__ float frsqrt_fast(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ Pair make_pair_of(f3 d) {
  Pair q;
  q.d = d;
  q.r2 = dot3(d, d);
  if (kFast) {
    q.ir = (q.r2 > 0.0f) ? frsqrt_fast(q.r2) : 0.0f;
    q.rl = q.r2 * q.ir;
  } else {
    q.rl = sqrtf(q.r2);
    q.ir = 0.0f;
  }
  return q;
}
// The same pair with the library's rsqrtf in fast mode (exact mode: as
// make_pair_of): the XSPH pass runs faster with it (0.1265 against 0.1310 ms
// at 2^20), the other passes with frsqrt_fast.
__device__ __forceinline__ Pair make_pair_of_lib(f3 d) {
  if (!kFast) return make_pair_of(d);
  Pair q;
  q.d = d;
  q.r2 = dot3(d, d);
  q.ir = (q.r2 > 0.0f) ? rsqrtf(q.r2) : 0.0f;
  q.rl = q.r2 * q.ir;
  return q;
}
__device__ __forceinline__ float poly6_p(const SimParams& p, const Pair& q) {
  if (kFast) {
    float t = p.h2 - q.r2;
    return (q.r2 <= p.h2) ? p.poly6 * (t * t * t) : 0.0f;
  }
  return poly6(p, q.rl);
}
__device__ __forceinline__ f3 spiky_p(const SimParams& p, const Pair& q) {
  if (kFast) {
    float t = p.h - q.rl;
    float x = (q.rl <= p.h) ? (t * t) : 0.0f;
    return (p.spiky * x * q.ir) * q.d;
  }
  return spiky_grad(p, q.d, q.rl);
}
__device__ __forceinline__ f3 cohesion_p(const SimParams& p, const Pair& q) {
  if (kFast) {
    float a = p.h - q.rl;
    float t = (a * a * a) * (q.rl * q.rl * q.rl);
    float res = (q.rl > p.half_h) ? t : fmaf(2.0f, t, p.coh_bias);
    res = (q.rl <= p.h) ? res : 0.0f;
    return (p.coh * res * q.ir) * q.d;
  }
  return cohesion(p, q.d, q.rl);
}
// 1 / x by the hardware approximation (rcp.approx.ftz.f32, one MUFU
// instruction, about 1 ulp): the fast mode's reciprocal.
__device__ __forceinline__ float frcp_fast(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// a / b: IEEE division in exact mode, reciprocal-multiply in fast mode.
__device__ __forceinline__ float fdiv(float a, float b) { return kFast ? a * frcp_fast(b) : a / b; }
__device__ __forceinline__ f3 fdiv3(f3 a, float b) {
  if (kFast) {
    float r = frcp_fast(b);
    return r * a;
  }
  return divs(a, b);
}

// ---- wall clamp with jitter (common.ts:43-67) ------------------------------------
// The reference's random3 is fract(sin(dot(.)) * 43758.5453); that value depends
// on the last bits of a large-argument sin, which no two sin implementations
// agree on.  The default mode replaces it with an integer hash of the float
// bits ("lowbias32" finaliser, C. Wellons), identical on every device and host.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ float hash2(float a, float b) {
  uint32_t h = mix32(__float_as_uint(a) ^ mix32(__float_as_uint(b) + 0x9e3779b9U));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float sinhash(float a, float b) {
  float d = a * 12.9898f + b * 78.233f;
  float s = sinf(d) * 43758.5453f;
  return s - floorf(s);
}
__device__ __forceinline__ f3 clamp_rand(const SimParams& p, f3 q) {
  float r0, r1, r2;
  if (p.jitter_mode == 1) {
    r0 = sinhash(q.y, q.z);
    r1 = sinhash(q.x, q.z);
    r2 = sinhash(q.x, q.y);
  } else {
    r0 = hash2(q.y, q.z);
    r1 = hash2(q.x, q.z);
    r2 = hash2(q.x, q.y);
  }
  // each product and sum rounded once in both precision modes (no
  // contraction into FMAs): the clamp bounds of the reference
  f3 rv = mk(__fmul_rn(p.jitter, r0), __fmul_rn(p.jitter, r1), __fmul_rn(p.jitter, r2));
  f3 lo = mk(__fadd_rn(p.dmin[0], rv.x), __fadd_rn(p.dmin[1], rv.y), __fadd_rn(p.dmin[2], rv.z));
  f3 hi = mk(__fsub_rn(p.dmax[0], rv.x), __fsub_rn(p.dmax[1], rv.y), __fsub_rn(p.dmax[2], rv.z));
  return mk(fmaxf(fminf(q.x, hi.x), lo.x), fmaxf(fminf(q.y, hi.y), lo.y), fmaxf(fminf(q.z, hi.z), lo.z));
}

// ---- hash grid ---------------------------------------------------------------------
// Cell of a point: floor((x - origin) * cells_per_length), clamped into the
// grid (neighborShader.ts:28-29 computes floor(x * D) on the unit cube).
__device__ __forceinline__ int cell_axis(float x, float o, float inv, int d) {
  int c = (int)floorf((x - o) * inv);
  return min(max(c, 0), d - 1);
}
__device__ __forceinline__ uint32_t cell_key(int cx, int cy, int cz, const GridParams& g) {
  return g.key_base + (uint32_t)cx * (uint32_t)(g.dim[1] * g.dim[2]) + (uint32_t)cy * (uint32_t)g.dim[2] +
         (uint32_t)cz;
}

// ---- volume map (src/simulator/boundary/discreteFieldShader.ts:1-192) ---------------
// 32-node cubic serendipity hexahedron.  Node order per cell: corners
// (i,j,k),(i+1,j,k),(i,j+1,k),(i+1,j+1,k), then the same at k+1; x-edge nodes
// (e, z-side, y-side); y-edge nodes (e, x-side, z-side); z-edge nodes
// (e, y-side, x-side) — the grouping of the reference's valvec0..valvec7.
struct CellLoc {
  int i, j, k;
  f3 s;
};
__device__ __forceinline__ CellLoc field_locate(const FieldParams& f, f3 x) {
  float q[3] = {x.x, x.y, x.z};
  int c[3];
  float s[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float u = (q[a] - f.origin[a]) * f.scale[a];
    float fl = floorf(u);
    int ci = (int)fl;
    ci = min(max(ci, 0), f.res[a] - 1);
    c[a] = ci;
    s[a] = 2.0f * (u - fl) - 1.0f;
  }
  return CellLoc{c[0], c[1], c[2], mk(s[0], s[1], s[2])};
}

__host__ __device__ __forceinline__ void cell_nodes(const FieldParams& f, int i, int j, int k, bool quirk,
                                                    uint32_t* idx) {
  const uint32_t nx = f.res[0], ny = f.res[1], nz = f.res[2];
  const uint32_t nc = (nx + 1) * (ny + 1) * (nz + 1);
  const uint32_t nex = 2 * nx * (ny + 1) * (nz + 1);
  const uint32_t ney = (nx + 1) * 2 * ny * (nz + 1);
#define PBF_C(kk, jj, ii) (((uint32_t)(kk) * (ny + 1) + (uint32_t)(jj)) * (nx + 1) + (uint32_t)(ii))
#define PBF_EX(kk, jj, e) (nc + ((uint32_t)(kk) * (ny + 1) + (uint32_t)(jj)) * (2 * nx) + (uint32_t)(e))
#define PBF_EY(ii, kk, e) (nc + nex + ((uint32_t)(ii) * (nz + 1) + (uint32_t)(kk)) * (2 * ny) + (uint32_t)(e))
#define PBF_EZ(jj, ii, e) (nc + nex + ney + ((uint32_t)(jj) * (nx + 1) + (uint32_t)(ii)) * (2 * nz) + (uint32_t)(e))
  int i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
  idx[0] = PBF_C(k, j, i); idx[1] = PBF_C(k, j, i + 1); idx[2] = PBF_C(k, j + 1, i); idx[3] = PBF_C(k, j + 1, i + 1);
  idx[4] = PBF_C(k + 1, j, i); idx[5] = PBF_C(k + 1, j, i + 1); idx[6] = PBF_C(k + 1, j + 1, i); idx[7] = PBF_C(k + 1, j + 1, i + 1);
  idx[8] = PBF_EX(k, j, i2); idx[9] = PBF_EX(k, j, i2 + 1); idx[10] = PBF_EX(k + 1, j, i2); idx[11] = PBF_EX(k + 1, j, i2 + 1);
  idx[12] = PBF_EX(k, j + 1, i2); idx[13] = PBF_EX(k, j + 1, i2 + 1); idx[14] = PBF_EX(k + 1, j + 1, i2); idx[15] = PBF_EX(k + 1, j + 1, i2 + 1);
  idx[16] = PBF_EY(i, k, j2); idx[17] = PBF_EY(i, k, j2 + 1); idx[18] = PBF_EY(i + 1, k, j2); idx[19] = PBF_EY(i + 1, k, j2 + 1);
  idx[20] = PBF_EY(i, k + 1, j2); idx[21] = PBF_EY(i, k + 1, j2 + 1); idx[22] = PBF_EY(i + 1, k + 1, j2); idx[23] = PBF_EY(i + 1, k + 1, j2 + 1);
  idx[24] = PBF_EZ(j, i, k2); idx[25] = PBF_EZ(j, i, k2 + 1); idx[26] = PBF_EZ(j + 1, i, k2); idx[27] = PBF_EZ(j + 1, i, k2 + 1);
  idx[28] = PBF_EZ(j, i + 1, k2); idx[29] = PBF_EZ(j, i + 1, k2 + 1); idx[30] = PBF_EZ(j + 1, i + 1, k2); idx[31] = PBF_EZ(j + 1, i + 1, k2 + 1);
#undef PBF_C
#undef PBF_EX
#undef PBF_EY
#undef PBF_EZ
  if (quirk) {
    // The reference's volume interpolation reads x-edge (k+1,.,i2) twice
    // (discreteFieldShader.ts:146-147) and z-edge k2 in place of k2+1 (:152-153).
    idx[11] = idx[10];
    idx[15] = idx[14];
    idx[25] = idx[24];
    idx[27] = idx[26];
    idx[29] = idx[28];
    idx[31] = idx[30];
  }
}

// The node quirk of cell_nodes applied to the 32 volume values of a packed
// block (stored in the plain node order): the same values the quirked node
// indices would read.
__device__ __forceinline__ void volume_quirk_values(float* v) {
  v[11] = v[10];
  v[15] = v[14];
  v[25] = v[24];
  v[27] = v[26];
  v[29] = v[28];
  v[31] = v[30];
}

// Packed block of the field cell (i,j,k), or null when the map has no
// blocks or the cell has none (its nodes are then gathered).
__device__ __forceinline__ const float4* field_block(const FieldParams& f, const FieldBlocks& fb, int i, int j,
                                                     int k) {
  if (!fb.cell) return nullptr;
  const uint32_t c = __ldg(fb.cell + f.flag_off + ((size_t)k * f.res[1] + j) * f.res[0] + i);
  return c == kNoBlock ? nullptr : fb.nodes + (size_t)c * 16u;
}

// kN node values (a multiple of 4) from a packed block.
template <int kN>
__device__ __forceinline__ void block_values(const float4* blk, float* val) {
#pragma unroll
  for (int q = 0; q < kN / 4; ++q) {
    const float4 v = __ldg(blk + q);
    val[4 * q] = v.x;
    val[4 * q + 1] = v.y;
    val[4 * q + 2] = v.z;
    val[4 * q + 3] = v.w;
  }
}

// Shape functions and local gradients.  Corner: (1/64)(1+-x)(1+-y)(1+-z)(9|s|^2-19).
// Edge along u at u = -1/3 (e=0) / +1/3 (e=1): (9/64)(1-u^2)(1+3 sigma u)(1+-v)(1+-w).
__device__ __forceinline__ void shape32(f3 s, float* N, f3* dN) {
  const float c1 = (float)(1.0 / 64.0), c9 = (float)(9.0 / 64.0);
  float x = s.x, y = s.y, z = s.z;
  float x2 = x * x, y2 = y * y, z2 = z * z;
  float r2 = x2 + y2 + z2;
  float mx = 1.0f - x, px = 1.0f + x, my = 1.0f - y, py = 1.0f + y, mz = 1.0f - z, pz = 1.0f + z;
  float q = 9.0f * r2 - 19.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    int a = c & 1, b = (c >> 1) & 1, e = (c >> 2) & 1;
    float lx = a ? px : mx, ly = b ? py : my, lz = e ? pz : mz;
    float sx = a ? 1.0f : -1.0f, sy = b ? 1.0f : -1.0f, sz = e ? 1.0f : -1.0f;
    float pr = lx * ly * lz;
    N[c] = c1 * pr * q;
    dN[c].x = c1 * (sx * ly * lz * q + pr * (18.0f * x));
    dN[c].y = c1 * (sy * lx * lz * q + pr * (18.0f * y));
    dN[c].z = c1 * (sz * lx * ly * q + pr * (18.0f * z));
  }
  float su[3] = {x, y, z};
  float fsq[3] = {1.0f - x2, 1.0f - y2, 1.0f - z2};
  float fm[3] = {mx, my, mz}, fp[3] = {px, py, pz};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const int av = (ax + 1) % 3, aw = (ax + 2) % 3;
    float u = su[ax];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int e = n & 1, wside = (n >> 1) & 1, vside = (n >> 2) & 1;
      float sg = e ? 1.0f : -1.0f;
      float lin = 1.0f + 3.0f * sg * u;
      float fv = vside ? fp[av] : fm[av];
      float fw = wside ? fp[aw] : fm[aw];
      float sv = vside ? 1.0f : -1.0f;
      float sw = wside ? 1.0f : -1.0f;
      float g = fsq[ax] * lin;
      float vw = fv * fw;
      float dn_u = c9 * vw * (-2.0f * u * lin + 3.0f * sg * fsq[ax]);
      float dn_v = c9 * g * (sv * fw);
      float dn_w = c9 * g * (fv * sw);
      int slot = 8 + ax * 8 + n;
      N[slot] = c9 * g * vw;
      float d3[3];
      d3[ax] = dn_u;
      d3[av] = dn_v;
      d3[aw] = dn_w;
      dN[slot] = mk(d3[0], d3[1], d3[2]);
    }
  }
}

// 32-term weighted sums in the reduction order of discreteFieldShader.ts:155-159.
__device__ __forceinline__ float sum32(const float* w, const float* v) {
  float d[8];
#pragma unroll
  for (int g = 0; g < 8; ++g)
    d[g] = w[4 * g] * v[4 * g] + w[4 * g + 1] * v[4 * g + 1] + w[4 * g + 2] * v[4 * g + 2] + w[4 * g + 3] * v[4 * g + 3];
  float s0 = d[0] + d[4], s1 = d[1] + d[5], s2 = d[2] + d[6], s3 = d[3] + d[7];
  return s0 + s1 + s2 + s3;
}
__device__ __forceinline__ f3 sum32v(const f3* w, const float* v) {
  f3 g[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    f3 a = v[4 * q] * w[4 * q];
    a = a + v[4 * q + 1] * w[4 * q + 1];
    a = a + v[4 * q + 2] * w[4 * q + 2];
    a = a + v[4 * q + 3] * w[4 * q + 3];
    g[q] = a;
  }
  f3 lo = ((g[0] + g[1]) + g[2]) + g[3];
  f3 hi = ((g[4] + g[5]) + g[6]) + g[7];
  return lo + hi;
}

// Interpolated SDF value only (the learned start's boundary feature).
__device__ __forceinline__ float boundary_distance(const FieldParams& f, const float* __restrict__ sdf, f3 x) {
  CellLoc L = field_locate(f, x);
  uint32_t idx[32];
  cell_nodes(f, L.i, L.j, L.k, false, idx);
  if (f.trilinear) {
    float tx = (L.s.x + 1.0f) * 0.5f, ty = (L.s.y + 1.0f) * 0.5f, tz = (L.s.z + 1.0f) * 0.5f;
    float d = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      int a = q & 1, b = (q >> 1) & 1, e = (q >> 2) & 1;
      float wx = a ? tx : 1.0f - tx, wy = b ? ty : 1.0f - ty, wz = e ? tz : 1.0f - tz;
      d = d + wx * wy * wz * __ldg(sdf + idx[q]);
    }
    return d;
  }
  float N[32];
  f3 dN[32];
  float val[32];
  shape32(L.s, N, dN);
#pragma unroll
  for (int q = 0; q < 32; ++q) val[q] = __ldg(sdf + idx[q]);
  return sum32(N, val);
}

// Node values of one field cell for the boundary sample: gathered from the
// node arrays by the cell's node indices, or read from its packed block.
struct NodeGather {
  const FieldParams& f;
  const float* __restrict__ sdf;
  const float* __restrict__ vol;
  int i, j, k;
  __device__ __forceinline__ void sdf_values(float* v, int n) const {
    uint32_t idx[32];
    cell_nodes(f, i, j, k, false, idx);
#pragma unroll
    for (int q = 0; q < n; ++q) v[q] = __ldg(sdf + idx[q]);
  }
  __device__ __forceinline__ void vol_values(float* v, int n) const {
    uint32_t idx[32];
    cell_nodes(f, i, j, k, f.quirk != 0, idx);  // the quirk touches edge nodes only (n == 8 reads corners)
#pragma unroll
    for (int q = 0; q < n; ++q) v[q] = __ldg(vol + idx[q]);
  }
};
struct NodeBlock {
  const float4* blk;
  int quirk;
  __device__ __forceinline__ void sdf_values(float* v, int n) const {
    if (n == 8) block_values<8>(blk, v);
    else block_values<32>(blk, v);
  }
  __device__ __forceinline__ void vol_values(float* v, int n) const {
    if (n == 8) {
      block_values<8>(blk + 8, v);
    } else {
      block_values<32>(blk + 8, v);
      if (quirk) volume_quirk_values(v);
    }
  }
};

// BoundaryVolume pass for one particle (src/simulator/PBF/shader/boundaryVolume.ts:31-55)
// from the cell located at x: returns (x_b, V_b) or zero when the particle is
// outside the band 0 < d < h; dist_out (optional) receives the interpolated
// SDF (boundary_distance's value).  Src supplies the node values.
template <class Src>
__device__ __forceinline__ float4 boundary_sample_from(const SimParams& p, const FieldParams& f, const CellLoc& L,
                                                       const Src& src, f3 x, float* dist_out) {
  float dist, volume;
  f3 grad;
  if (f.trilinear) {
    float tx = (L.s.x + 1.0f) * 0.5f, ty = (L.s.y + 1.0f) * 0.5f, tz = (L.s.z + 1.0f) * 0.5f;
    float c8[8];
    src.sdf_values(c8, 8);
    dist = 0.0f;
    f3 g = mk(0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      int a = q & 1, b = (q >> 1) & 1, e = (q >> 2) & 1;
      float wx = a ? tx : 1.0f - tx, wy = b ? ty : 1.0f - ty, wz = e ? tz : 1.0f - tz;
      float sx = a ? 1.0f : -1.0f, sy = b ? 1.0f : -1.0f, sz = e ? 1.0f : -1.0f;
      float v = c8[q];
      dist = dist + wx * wy * wz * v;
      g = g + mk(sx * wy * wz * v, wx * sy * wz * v, wx * wy * sz * v);
    }
    grad = mk(0.5f * f.gscale[0] * g.x, 0.5f * f.gscale[1] * g.y, 0.5f * f.gscale[2] * g.z);
    if (dist_out) *dist_out = dist;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (dist > 0.0f && dist < p.h && len3(grad) > 1e-9f) {
      src.vol_values(c8, 8);
      volume = 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        int a = q & 1, b = (q >> 1) & 1, e = (q >> 2) & 1;
        float wx = a ? tx : 1.0f - tx, wy = b ? ty : 1.0f - ty, wz = e ? tz : 1.0f - tz;
        volume = volume + wx * wy * wz * c8[q];
      }
      if (volume > 0.0f) {
        f3 n = divs(grad, len3(grad));
        float d = fmaxf(dist + 0.5f * p.r, 2.0f * p.r);
        out = f4(x - d * n, volume);
      }
    }
    return out;
  }
  float N[32];
  f3 dN[32];
  float val[32];
  shape32(L.s, N, dN);
  src.sdf_values(val, 32);
  dist = sum32(N, val);
  f3 g = sum32v(dN, val);
  grad = mk(f.gscale[0] * g.x, f.gscale[1] * g.y, f.gscale[2] * g.z);
  if (dist_out) *dist_out = dist;
  float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
  if (dist > 0.0f && dist < p.h && len3(grad) > 1e-9f) {
    src.vol_values(val, 32);
    volume = sum32(N, val);
    if (volume > 0.0f) {
      f3 n = divs(grad, len3(grad));
      float d = fmaxf(dist + 0.5f * p.r, 2.0f * p.r);
      out = f4(x - d * n, volume);
    }
  }
  return out;
}

// The boundary sample with the nodes gathered from the node arrays.
__device__ __forceinline__ float4 boundary_sample(const SimParams& p, const FieldParams& f, const float* __restrict__ sdf,
                                                  const float* __restrict__ vol, f3 x, float* dist_out = nullptr) {
  const CellLoc L = field_locate(f, x);
  return boundary_sample_from(p, f, L, NodeGather{f, sdf, vol, L.i, L.j, L.k}, x, dist_out);
}
static __device__ __noinline__ float4 boundary_sample_gather(const SimParams& p, const FieldParams& f,
                                                             const float* __restrict__ sdf,
                                                             const float* __restrict__ vol, f3 x, float* dist_out) {
  return boundary_sample(p, f, sdf, vol, x, dist_out);
}

// The boundary sample from the cell's packed block (FieldBlocks): two
// 128-byte lines per field instead of 32 scattered nodes.  A cell without a
// block (not flagged; the band never lists one) takes the gather path.
__device__ __forceinline__ float4 boundary_sample_packed(const SimParams& p, const FieldParams& f,
                                                         const FieldBlocks& fb, const float* __restrict__ sdf,
                                                         const float* __restrict__ vol, f3 x, float* dist_out) {
  const CellLoc L = field_locate(f, x);
  const float4* blk = field_block(f, fb, L.i, L.j, L.k);
  if (!blk) return boundary_sample_gather(p, f, sdf, vol, x, dist_out);
  return boundary_sample_from(p, f, L, NodeBlock{blk, f.quirk}, x, dist_out);
}

}  // namespace pbf
