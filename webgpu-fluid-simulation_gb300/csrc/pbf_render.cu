// pbf_render.cu — screen-space fluid buffers as CUDA kernels: the particle
// sprites of ParicleRasterizer (src/renderer/filteredParticleFluid/
// paricleRasterizer.ts:170-204, shader/depthPassShader.ts,
// shader/volumePassShader.ts) and the narrow-range filter of TextureFilter
// (textureFilter.ts:129-160, shader/filterPassShader.ts).
//
// Rasterisation is restated for camera-facing sprites.  The view matrix is
// affine and the projection has no x/y shear, so a sprite (the particle's
// camera-space centre plus (+-hs, +-hs, 0, 0)) projects to an axis-aligned
// rectangle whose corners share clip z and w.  It is clipped away whole
// unless 0 <= z_clip <= w_clip with w_clip > 0.  A pixel is covered when its
// centre lies in the rectangle (left/top edges in, right/bottom out), and
// the sprite's uv there is the centre's position across the rectangle
// (perspective-correct interpolation reduces to linear at constant w).
//
// Depth pass: the fragment at uv has n.xy = 2 uv - 1, is discarded when
// |n.xy|^2 > 1, and otherwise lies on the sphere of radius R in front of the
// centre: z = c.z + sqrt(1 - |n.xy|^2) R.  Its depth (clip z / clip w,
// clamped to [0, 1]) must beat the depth buffer ('greater', reverse-Z) and
// all other fragments of the pixel; equal depths keep the first particle
// drawn, i.e. the lowest index.  One 64-bit atomicMax per fragment on
// (depth bits, ~index) decides it, so the result does not depend on thread
// order.  The winner's eye depth -z / w goes to the depth map (0 elsewhere)
// and its depth to the depth buffer.
//
// Fragment n.xy: uv is the pixel centre's position across the rectangle,
// n = 2 uv - 1, evaluated as one fused multiply-add per axis from per-sprite
// constants (sx = 2 / (x1 - x0), ox = (0.5 - x0) sx - 1; likewise in y from
// the bottom edge).  A sprite's fragments are skipped where a bound of its
// depths cannot beat the pixel's key, which changes nothing in the result.
//
// Volume pass: sprites of half-side R on the half-resolution target add
// exp(-2 |n.xy|^2), evaluated as the product exp(-2 nx^2) exp(-2 ny^2) of
// per-column and per-row factors.  The sum is kept in 64-bit fixed point
// with 40 fraction bits, where every float term in [2^-3, 2) is exact, so
// the sum is exact and order-free; it is rounded to float once.  The
// exponential is this file's own (splat_exp), so the CPU restatement can
// produce the same bits.
//
// The filter is the reference's narrow-range filter, separable, x then y,
// with its sample window of 32 + 32 texels per 32-texel block: the centre it
// reads for texel p is p - (16 - filterSize/2), so filter sizes below 32
// shift the image as the reference's shader does.  Reads outside the image
// clamp to the edge (the robust-access behaviour of WGSL textureLoad under
// coordinate clamping).  The x pass writes a cleared temporary where its
// centre is positive; the y pass writes the depth map where the
// temporary's centre is positive and leaves the other texels as they were.
//
// This unit is compiled with -fmad=false: every float operation rounds as
// written, fused multiply-adds only where written (__fmaf_rn), which the CPU
// restatement reproduces with fmaf.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"

namespace {

constexpr int kMaxHalf = 16;          // MaxFilterSize 32 >> 1
constexpr int kFilterX = 128;         // texels per block of the x pass
constexpr int kFilterYRows = 64;      // rows per block of the y pass
constexpr double kFix = 1099511627776.0;  // 2^40

__constant__ float c_gauss[kMaxHalf + 1];

struct Cam {
  float v[16];  // view, column-major
  float p[16];  // projection, column-major
};

// A sprite on one target: its covered pixels and the affine maps from pixel
// index to the fragment's n.xy = 2 uv - 1 (uv measured from the rectangle's
// left and bottom edges at the pixel centre): nx = i sx + ox, ny = j sy + oy.
struct Sprite {
  int i0, i1, j0, j1;  // covered pixels [i0, i1) x [j0, j1)
  float sx, ox, sy, oy;
  float cz, cw;        // camera-space z and w of the centre
  uint32_t dmax;       // bits of an upper bound of the fragment depths (depth sprites)
};

__device__ inline void mat_vec(const float* m, float x, float y, float z, float w, float o[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) o[r] = ((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w;
}

__device__ inline int pixel_edge(float f, int size) {
  // first pixel whose centre i + 0.5 is >= f, clamped to [0, size]
  const float e = fminf(fmaxf(f - 0.5f, -1.0f), (float)size);
  return min(max((int)ceilf(e), 0), size);
}

// The sprite of half-side hs around the camera-space centre c on a W x H
// target; false when it is clipped away or covers no pixel centre.
__device__ inline bool make_sprite(const Cam& C, const float c[4], float hs, int W, int H, Sprite& s) {
  float bl[4], tr[4];
  mat_vec(C.p, c[0] + (-hs), c[1] + (-hs), c[2], c[3], bl);
  mat_vec(C.p, c[0] + hs, c[1] + hs, c[2], c[3], tr);
  if (!(bl[3] > 0.0f) || !(bl[2] >= 0.0f) || !(bl[2] <= bl[3])) return false;
  const float fw = (float)W, fh = (float)H;
  const float fx0 = 0.5f * (bl[0] / bl[3] + 1.0f) * fw;
  const float fx1 = 0.5f * (tr[0] / tr[3] + 1.0f) * fw;
  const float fyb = 0.5f * (-(bl[1] / bl[3]) + 1.0f) * fh;
  const float fyt = 0.5f * (-(tr[1] / tr[3]) + 1.0f) * fh;
  if (!(fx1 != fx0) || !(fyb != fyt)) return false;
  s.i0 = pixel_edge(fminf(fx0, fx1), W);
  s.i1 = pixel_edge(fmaxf(fx0, fx1), W);
  s.j0 = pixel_edge(fminf(fyt, fyb), H);
  s.j1 = pixel_edge(fmaxf(fyt, fyb), H);
  const float ax = 2.0f / (fx1 - fx0), ay = 2.0f / (fyb - fyt);
  s.sx = ax;
  s.ox = __fmaf_rn(0.5f - fx0, ax, -1.0f);
  s.sy = -ay;
  s.oy = __fmaf_rn(fyb - 0.5f, ay, -1.0f);
  s.cz = c[2];
  s.cw = c[3];
  return s.i0 < s.i1 && s.j0 < s.j1;
}

// |n.xy|^2 of the sprite's fragment at pixel (i, j).
__device__ inline float sprite_r2(const Sprite& s, int i, int j) {
  const float nx = __fmaf_rn((float)i, s.sx, s.ox), ny = __fmaf_rn((float)j, s.sy, s.oy);
  return __fmaf_rn(nx, nx, ny * ny);
}

// [0, 1] depth of camera-space z (w = the centre's w).
__device__ inline float depth_of(const Cam& C, float z, float w) {
  const float d = __fmaf_rn(C.p[10], z, C.p[14] * w) / __fmaf_rn(C.p[11], z, C.p[15] * w);
  return d > 0.0f ? fminf(d, 1.0f) : 0.0f;
}

// Depth-pass fragment: camera z of the sphere point and its [0, 1] depth.
__device__ inline float sprite_depth(const Cam& C, const Sprite& s, float r2, float R, float& z) {
  z = __fmaf_rn(sqrtf(1.0f - r2), R, s.cz);
  return depth_of(C, z, s.cw);
}

// An upper bound of the depths of a depth sprite's fragments.  Their z lie
// in [c.z, zt = c.z + R] (sqrt(1 - r2) is in [0, 1] and the rounded fma is
// monotone in it).  With a positive denominator on that interval, a
// numerator that does not fall and a denominator that does not rise as z
// grows (p10 >= 0 >= p11: the reverse-Z perspective) make every rounded
// non-negative depth at most the depth at zt, and negative depths clamp to
// 0; the mirror case bounds them by the depth at c.z.  Otherwise there is no
// bound (all ones).
__device__ inline uint32_t depth_bound(const Cam& C, float cz, float cw, float R) {
  const float zt = __fmaf_rn(1.0f, R, cz);
  const float d0 = __fmaf_rn(C.p[11], cz, C.p[15] * cw), d1 = __fmaf_rn(C.p[11], zt, C.p[15] * cw);
  if (!(d0 > 0.0f && d1 > 0.0f)) return 0xffffffffu;
  if (C.p[10] >= 0.0f && C.p[11] <= 0.0f) return __float_as_uint(depth_of(C, zt, cw));
  if (C.p[10] <= 0.0f && C.p[11] >= 0.0f) return __float_as_uint(depth_of(C, cz, cw));
  return 0xffffffffu;
}

// v * 2^40 as an integer, exactly, for a float v in [2^-3, 2): its 24-bit
// significand shifted by (biased exponent - 110).
__device__ inline unsigned long long fix40(float v) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t e = (b >> 23) & 0xffu;
  return (unsigned long long)((b & 0x7fffffu) | 0x800000u) << (e - 110u);
}

// exp(x) for x in [-2, 0]: Cody-Waite reduction x = k ln2 + r with ln 2 in
// two parts (the high part has 16 significant bits, so k * hi is exact for
// |k| <= 3), then exp(r) by its Taylor series to degree 8 in Horner form with
// fused multiply-adds (|r| <= 0.35: truncation below 3e-10), scaled by 2^k.
__device__ inline float splat_exp(float x) {
  const float k = floorf(__fmaf_rn(x, 1.44269502f, 0.5f));
  const float r = __fmaf_rn(-k, 1.42860677e-6f, __fmaf_rn(-k, 0.693145751953125f, x));
  float p = 2.48015873e-5f;              // 1/8!
  p = __fmaf_rn(p, r, 1.98412698e-4f);   // 1/7!
  p = __fmaf_rn(p, r, 1.38888889e-3f);   // 1/6!
  p = __fmaf_rn(p, r, 8.33333333e-3f);   // 1/5!
  p = __fmaf_rn(p, r, 4.16666667e-2f);   // 1/4!
  p = __fmaf_rn(p, r, 1.66666667e-1f);   // 1/3!
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  return p * __uint_as_float((uint32_t)((int)k + 127) << 23);   // 2^k (k in [-3, 0])
}

__device__ inline uint32_t depth_bits(float d) { return __float_as_uint(d); }

__global__ void k_init(const float* scene, unsigned long long* keys, unsigned long long* acc, int W, int H, int W2,
                       int H2) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= W) return;
  const size_t p = (size_t)y * W + x;
  float s = scene ? scene[p] : 0.0f;
  s = s > 0.0f ? fminf(s, 1.0f) : 0.0f;
  keys[p] = ((unsigned long long)depth_bits(s) << 32) | 0xffffffffull;
  if (x < W2 && y < H2) acc[(size_t)y * W2 + x] = 0ull;
}

// Sprites are set up one per lane (32 particles per warp) in shared memory;
// the warp then walks them one by one with its lanes spread over each
// sprite's pixels: for sprites up to 32 pixels wide, floor(32 / width) rows
// per step (lane -> row lane / width by a 16-bit reciprocal, exact for lane
// and width up to 32), else 32 columns per step.  Every lane takes part in
// every step (frag receives whether its pixel is inside the sprite), so the
// fragment code may use warp-wide votes and shuffles.
struct SpriteSlot {
  Sprite s[2];   // depth, volume
  uint32_t ok;   // bit 0: depth sprite visible, bit 1: volume sprite visible
};

// ceil(2^16 / w) for w = 1 .. 32
__constant__ uint32_t c_recip16[33] = {0,    65536, 32768, 21846, 16384, 13108, 10923, 9363, 8192, 7282, 6554,
                                       5958, 5462,  5042,  4682,  4370,  4096,  3856,  3641, 3450, 3277, 3121,
                                       2979, 2850,  2731,  2622,  2521,  2428,  2341,  2260, 2185, 2115, 2048};

template <typename Frag>
__device__ inline void walk_sprite(const Sprite& s, uint32_t lane, Frag frag) {
  const int w = s.i1 - s.i0;
  if (w <= 32) {
    const uint32_t m = c_recip16[w];
    const int rows = (int)((32u * m) >> 16);
    const int lr = (int)((lane * m) >> 16), lc = (int)lane - lr * w;
    for (int jb = s.j0; jb < s.j1; jb += rows) {
      const int j = jb + lr;
      frag(s.i0 + lc, j, lr < rows && j < s.j1);
    }
  } else {
    for (int j = s.j0; j < s.j1; ++j)
      for (int ib = s.i0; ib < s.i1; ib += 32) frag(ib + (int)lane, j, ib + (int)lane < s.i1);
  }
}

// exp(-2 n^2) of a fragment coordinate n: the volume term exp(-2 |n|^2) is
// the product of the x and y factors.
__device__ inline float gauss_axis(float n) { return splat_exp((n * n) * -2.0f); }

constexpr int kQueue = 64;  // per-warp queue of depth fragments that pass the bound test

// Depth fragments that may win are queued (pixel, sprite) per warp and
// evaluated 32 at a time with all lanes busy: the full fragment (square root,
// division, key, atomicMax) runs only for them.
__device__ inline void depth_fragments(const Cam& C, const SpriteSlot* slots, const uint32_t* qij, const uint8_t* qk,
                                       uint32_t count, uint32_t lane, uint32_t base, float R, int W,
                                       unsigned long long* keys) {
  if (lane >= count) return;
  const uint32_t e = qij[lane], k = qk[lane];
  const int i = (int)(e & 0xffffu), j = (int)(e >> 16);
  const Sprite& s = slots[k].s[0];
  const float r2 = sprite_r2(s, i, j);
  if (r2 > 1.0f) return;
  float z;
  const float d = sprite_depth(C, s, r2, R, z);
  const unsigned long long key = ((unsigned long long)__float_as_uint(d) << 32) | (0xffffffffull - (base + k));
  unsigned long long* kp = keys + (size_t)j * W + i;
  if (key > *(volatile unsigned long long*)kp) atomicMax(kp, key);
}

__global__ void __launch_bounds__(256) k_splat(Cam C, const float4* __restrict__ pos, uint32_t n, float R, int W, int H,
                                               int W2, int H2, unsigned long long* keys, unsigned long long* acc) {
  __shared__ SpriteSlot slots[8][32];
  __shared__ uint32_t qij[8][kQueue];
  __shared__ uint8_t qk[8][kQueue];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t base = warp * 32; base < n; base += warps * 32) {
    const uint32_t q = base + lane;
    SpriteSlot& mine = slots[wib][lane];
    mine.ok = 0;
    if (q < n) {
      const float4 x = pos[q];
      float c[4];
      mat_vec(C.v, x.x, x.y, x.z, 1.0f, c);
      if (make_sprite(C, c, 0.5f * R, W, H, mine.s[0])) {
        mine.ok |= 1u;
        mine.s[0].dmax = depth_bound(C, c[2], c[3], R);
      }
      if (make_sprite(C, c, R, W2, H2, mine.s[1])) mine.ok |= 2u;
    }
    __syncwarp();
    const uint32_t cnt = min(32u, n - base);
    uint32_t qn = 0;  // queued depth fragments (warp-uniform)
    for (uint32_t k = 0; k < cnt; ++k) {
      const SpriteSlot& sl = slots[wib][k];
      const uint32_t ok = sl.ok;
      if (ok & 1u) {
        const Sprite s = sl.s[0];
        const unsigned long long bound = ((unsigned long long)s.dmax << 32) | (0xffffffffull - (base + k));
        walk_sprite(s, lane, [&](int i, int j, bool in) {
          // only fragments whose sprite bound beats the pixel's current key can win
          const bool pass = in && bound > *(volatile unsigned long long*)(keys + (size_t)j * W + i);
          const unsigned m = __ballot_sync(0xffffffffu, pass);
          if (pass) {
            const uint32_t at = qn + __popc(m & lt);
            qij[wib][at] = ((uint32_t)j << 16) | (uint32_t)i;
            qk[wib][at] = (uint8_t)k;
          }
          qn += __popc(m);
          if (qn >= 32) {
            __syncwarp();
            depth_fragments(C, slots[wib], qij[wib], qk[wib], 32, lane, base, R, W, keys);
            __syncwarp();
            qn -= 32;
            if (lane < qn) {
              qij[wib][lane] = qij[wib][32 + lane];
              qk[wib][lane] = qk[wib][32 + lane];
            }
            __syncwarp();
          }
        });
      }
      if (ok & 2u) {
        const Sprite s = sl.s[1];
        // per-lane axis factors: this lane's column (narrow sprites) and row j0 + lane
        const int w = s.i1 - s.i0, h = s.j1 - s.j0;
        float ex = 0.0f, ey = 0.0f;
        if (w <= 32) {
          const uint32_t m = c_recip16[w];
          const int lc = (int)lane - (int)((lane * m) >> 16) * w;
          ex = gauss_axis(__fmaf_rn((float)(s.i0 + lc), s.sx, s.ox));
        }
        if (h <= 32) ey = gauss_axis(__fmaf_rn((float)(s.j0 + (int)lane), s.sy, s.oy));
        walk_sprite(s, lane, [&](int i, int j, bool in) {
          float fy = __shfl_sync(0xffffffffu, ey, (j - s.j0) & 31);
          if (!in) return;
          const float r2 = sprite_r2(s, i, j);
          if (r2 > 1.0f) return;
          if (h > 32) fy = gauss_axis(__fmaf_rn((float)j, s.sy, s.oy));
          const float fx = w <= 32 ? ex : gauss_axis(__fmaf_rn((float)i, s.sx, s.ox));
          atomicAdd(acc + (size_t)j * W2 + i, fix40(fx * fy));
        });
      }
    }
    __syncwarp();
    depth_fragments(C, slots[wib], qij[wib], qk[wib], qn, lane, base, R, W, keys);
    __syncwarp();
  }
}

// Per pixel: the winning fragment's eye depth (recomputed from its index),
// the updated depth buffer, and the volume map.
__global__ void k_resolve(Cam C, const float4* __restrict__ pos, float R, int W, int H, int W2, int H2,
                          const unsigned long long* keys, const unsigned long long* acc, float* depth, float* scene,
                          float* volume) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= W) return;
  const size_t p = (size_t)y * W + x;
  const unsigned long long key = keys[p];
  float s0 = scene ? scene[p] : 0.0f;
  s0 = s0 > 0.0f ? fminf(s0, 1.0f) : 0.0f;
  float out = 0.0f;
  if ((uint32_t)(key >> 32) != depth_bits(s0)) {
    const uint32_t q = 0xffffffffu - (uint32_t)key;
    const float4 xq = pos[q];
    float c[4];
    mat_vec(C.v, xq.x, xq.y, xq.z, 1.0f, c);
    Sprite s;
    make_sprite(C, c, 0.5f * R, W, H, s);
    float z;
    sprite_depth(C, s, sprite_r2(s, x, y), R, z);
    out = -z / s.cw;
    if (scene) scene[p] = __uint_as_float((uint32_t)(key >> 32));
  }
  depth[p] = out;
  if (x < W2 && y < H2) {
    const size_t p2 = (size_t)y * W2 + x;
    volume[p2] = (float)((double)acc[p2] * (1.0 / kFix));
  }
}

// The narrow-range filter for one texel given its window v[0 .. 2 half]
// (centre v[half]); false when the centre is not positive (no write).
__device__ inline bool narrow_range(const float* v, int stride, int half, float threshold, float mu, float& result) {
  const float center = v[half * stride];
  if (!(center > 0.0f)) return false;
  float value_sum = center, weight_sum = 1.0f;
  float lo = center - threshold, hi = center + threshold;
  const float bound_high = center + mu;
  for (int i = 1; i <= half; ++i) {
    float a = v[(half - i) * stride], b = v[(half + i) * stride];
    const float g = c_gauss[i];
    if (a < lo || b < lo) continue;
    a = a > hi ? bound_high : a;
    b = b > hi ? bound_high : b;
    lo = fminf(lo, fminf(a, b) - threshold);
    hi = fmaxf(hi, fmaxf(a, b) + threshold);
    weight_sum += g * 2.0f;
    value_sum += (a + b) * g;
  }
  result = value_sum / weight_sum;
  return true;
}

__global__ void __launch_bounds__(kFilterX) k_filter_x(const float* __restrict__ src, float* __restrict__ dst, int W,
                                                      int H, int half, float threshold, float mu) {
  __shared__ float row[kFilterX + 2 * kMaxHalf];
  const int x0 = blockIdx.x * kFilterX, y = blockIdx.y;
  const float* s = src + (size_t)y * W;
  for (int k = threadIdx.x; k < kFilterX + 2 * kMaxHalf; k += kFilterX)
    row[k] = s[min(max(x0 - kMaxHalf + k, 0), W - 1)];
  __syncthreads();
  const int x = x0 + threadIdx.x;
  if (x >= W) return;
  float r;
  dst[(size_t)y * W + x] = narrow_range(row + threadIdx.x, 1, half, threshold, mu, r) ? r : 0.0f;
}

__global__ void __launch_bounds__(256) k_filter_y(const float* __restrict__ src, float* __restrict__ dst, int W, int H,
                                                  int half, float threshold, float mu) {
  __shared__ float col[kFilterYRows + 2 * kMaxHalf][33];
  const int x = blockIdx.x * 32 + threadIdx.x, y0 = blockIdx.y * kFilterYRows;
  const int xc = min(x, W - 1);
  for (int k = threadIdx.y; k < kFilterYRows + 2 * kMaxHalf; k += 8)
    col[k][threadIdx.x] = src[(size_t)min(max(y0 - kMaxHalf + k, 0), H - 1) * W + xc];
  __syncthreads();
  if (x >= W) return;
  for (int q = threadIdx.y; q < kFilterYRows; q += 8) {
    const int y = y0 + q;
    if (y >= H) break;
    float r;
    if (narrow_range(&col[q][threadIdx.x], 33, half, threshold, mu, r)) dst[(size_t)y * W + x] = r;
  }
}

}  // namespace

struct pbf_renderer {
  int W = 0, H = 0, W2 = 0, H2 = 0;
  pbf_render_options opt{};
  pbf_camera cam{};
  bool has_cam = false;
  float gauss[kMaxHalf + 1] = {};
  float* depth = nullptr;
  float* temp = nullptr;
  float* volume = nullptr;
  unsigned long long* keys = nullptr;
  unsigned long long* acc = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  float ms[2] = {0.0f, 0.0f};
};

namespace {

void release(pbf_renderer* r) {
  cudaFree(r->depth);
  cudaFree(r->temp);
  cudaFree(r->volume);
  cudaFree(r->keys);
  cudaFree(r->acc);
  for (auto& e : r->ev)
    if (e) cudaEventDestroy(e);
}

// Gaussian weights of filterPassShader.ts: sigma = (filterSize >> 1) / 2,
// weight_i = exp(-i^2 * 0.5 / sigma^2) with the argument formed in float.
void gauss_table(uint32_t filter_size, float* g) {
  const int half = (int)(filter_size >> 1);
  const float sigma = (float)half * 0.5f;
  const float k = 0.5f / (sigma * sigma);
  for (int i = 0; i <= kMaxHalf; ++i) {
    const float arg = -(float)(i * i) * k;
    g[i] = (i <= half && half > 0) ? (float)std::exp((double)arg) : 0.0f;
  }
}

// TextureFilter.execute: x pass img -> temp, y pass temp -> img.
cudaError_t launch_filter(const float* gauss, float* img, float* temp, int W, int H, uint32_t filter_size, float R,
                          cudaStream_t st) {
  if (filter_size < 2) return cudaSuccess;
  cudaError_t e = cudaMemcpyToSymbolAsync(c_gauss, gauss, sizeof(float) * (kMaxHalf + 1), 0, cudaMemcpyHostToDevice,
                                          st);
  if (e != cudaSuccess) return e;
  const int half = (int)(filter_size >> 1);
  k_filter_x<<<dim3((unsigned)((W + kFilterX - 1) / kFilterX), (unsigned)H), kFilterX, 0, st>>>(img, temp, W, H, half,
                                                                                              R * 5.0f, R);
  k_filter_y<<<dim3((unsigned)((W + 31) / 32), (unsigned)((H + kFilterYRows - 1) / kFilterYRows)), dim3(32, 8), 0,
               st>>>(temp, img, W, H, half, R * 5.0f, R);
  return cudaGetLastError();
}

bool finite16(const float* m) {
  for (int q = 0; q < 16; ++q)
    if (!std::isfinite(m[q])) return false;
  return true;
}

}  // namespace

extern "C" {

int pbf_renderer_create(uint32_t width, uint32_t height, pbf_renderer** out) {
  if (!out || width < 2 || height < 2 || width > 16384 || height > 16384) return PBF_EINVAL;
  *out = nullptr;
  pbf_renderer* r = new pbf_renderer();
  r->W = (int)width;
  r->H = (int)height;
  r->W2 = (int)(width / 2);  // fluidVolumeMap: canvas size / 2
  r->H2 = (int)(height / 2);
  // RenderingOptions defaults of the reference (src/common/config.ts:14-20)
  r->opt.mode = 0;
  r->opt.filter_size = 32;
  r->opt.particle_radius = 0.02f;
  r->opt.opacity = 0.25f;
  r->opt.tint_color[0] = 6.0f / 255.0f;
  r->opt.tint_color[1] = 105.0f / 255.0f;
  r->opt.tint_color[2] = 217.0f / 255.0f;
  const size_t px = (size_t)width * height, px2 = (size_t)r->W2 * r->H2;
  cudaError_t e = cudaMalloc(&r->depth, px * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&r->temp, px * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&r->volume, px2 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&r->keys, px * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&r->acc, px2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(r->depth, 0, px * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(r->volume, 0, px2 * sizeof(float));
  for (auto& ev : r->ev)
    if (e == cudaSuccess) e = cudaEventCreate(&ev);
  if (e != cudaSuccess) {
    release(r);
    delete r;
    return PBF_ECUDA;
  }
  pbf_renderer_set_config(r, &r->opt);
  *out = r;
  return PBF_OK;
}

int pbf_renderer_destroy(pbf_renderer* r) {
  if (!r) return PBF_EINVAL;
  cudaDeviceSynchronize();
  release(r);
  delete r;
  return PBF_OK;
}

int pbf_renderer_set_config(pbf_renderer* r, const pbf_render_options* o) {
  if (!r || !o || o->filter_size > 2 * kMaxHalf || !(o->particle_radius > 0.0f) ||
      !std::isfinite(o->particle_radius))
    return PBF_EINVAL;
  r->opt = *o;
  gauss_table(o->filter_size, r->gauss);
  return PBF_OK;
}

int pbf_renderer_set_camera(pbf_renderer* r, const pbf_camera* c) {
  if (!r || !c || !finite16(c->view) || !finite16(c->projection)) return PBF_EINVAL;
  const float* v = c->view;
  const float* p = c->projection;
  if (v[3] != 0.0f || v[7] != 0.0f || v[11] != 0.0f || v[15] != 1.0f) return PBF_EINVAL;  // affine view
  // projection without x/y shear: x_clip from (x, z), y_clip from (y, z), z_clip and w_clip from z
  if (p[1] != 0.0f || p[2] != 0.0f || p[3] != 0.0f || p[4] != 0.0f || p[6] != 0.0f || p[7] != 0.0f) return PBF_EINVAL;
  r->cam = *c;
  r->has_cam = true;
  return PBF_OK;
}

int pbf_render(pbf_renderer* r, const float* d_positions, uint32_t n, float* d_scene_depth, void* stream) {
  if (!r || (!d_positions && n) || !r->has_cam || n > 0xfffffffeu) return PBF_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  Cam C;
  std::memcpy(C.v, r->cam.view, sizeof(C.v));
  std::memcpy(C.p, r->cam.projection, sizeof(C.p));
  const float R = r->opt.particle_radius;
  const float4* pos = (const float4*)d_positions;
  cudaEventRecord(r->ev[0], st);
  const dim3 rows((unsigned)((r->W + 255) / 256), (unsigned)r->H);
  k_init<<<rows, 256, 0, st>>>(d_scene_depth, r->keys, r->acc, r->W, r->H, r->W2, r->H2);
  if (n) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)n + 255) / 256, (uint64_t)sms * 8);
    k_splat<<<blocks, 256, 0, st>>>(C, pos, n, R, r->W, r->H, r->W2, r->H2, r->keys, r->acc);
  }
  k_resolve<<<rows, 256, 0, st>>>(C, pos, R, r->W, r->H, r->W2, r->H2, r->keys, r->acc, r->depth, d_scene_depth,
                                  r->volume);
  cudaEventRecord(r->ev[1], st);
  if (launch_filter(r->gauss, r->depth, r->temp, r->W, r->H, r->opt.filter_size, R, st) != cudaSuccess)
    return PBF_ECUDA;
  cudaEventRecord(r->ev[2], st);
  if (cudaGetLastError() != cudaSuccess) return PBF_ECUDA;
  if (cudaEventSynchronize(r->ev[2]) != cudaSuccess) return PBF_ECUDA;
  cudaEventElapsedTime(&r->ms[0], r->ev[0], r->ev[1]);
  cudaEventElapsedTime(&r->ms[1], r->ev[1], r->ev[2]);
  return PBF_OK;
}

int pbf_texture_filter(const pbf_render_options* o, float* d_texture, uint32_t width, uint32_t height, void* stream) {
  if (!o || (!d_texture && width && height) || o->filter_size > 2 * kMaxHalf || !(o->particle_radius > 0.0f) ||
      !std::isfinite(o->particle_radius) || width > 65536 || height > 65536)
    return PBF_EINVAL;
  if (o->filter_size < 2 || width == 0 || height == 0) return PBF_OK;
  cudaStream_t st = (cudaStream_t)stream;
  float g[kMaxHalf + 1];
  gauss_table(o->filter_size, g);
  float* temp = nullptr;
  if (cudaMallocAsync(&temp, (size_t)width * height * sizeof(float), st) != cudaSuccess) return PBF_ECUDA;
  cudaError_t e = launch_filter(g, d_texture, temp, (int)width, (int)height, o->filter_size, o->particle_radius, st);
  cudaFreeAsync(temp, st);
  // the weights table is read from a host array by an asynchronous copy
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? PBF_OK : PBF_ECUDA;
}

int pbf_render_simulation(pbf_renderer* r, pbf_handle* h, float* d_scene_depth) {
  if (!r || !h) return PBF_EINVAL;
  return pbf_render(r, pbf_position_device(h), pbf_particle_count(h), d_scene_depth, pbf_stream(h));
}

const float* pbf_renderer_map_device(const pbf_renderer* r, uint32_t which) {
  if (!r) return nullptr;
  return which == PBF_RENDER_DEPTH ? r->depth : which == PBF_RENDER_VOLUME ? r->volume : nullptr;
}

int pbf_renderer_map_size(const pbf_renderer* r, uint32_t which, uint32_t* width, uint32_t* height) {
  if (!r || !width || !height || which > PBF_RENDER_VOLUME) return PBF_EINVAL;
  *width = (uint32_t)(which == PBF_RENDER_DEPTH ? r->W : r->W2);
  *height = (uint32_t)(which == PBF_RENDER_DEPTH ? r->H : r->H2);
  return PBF_OK;
}

int pbf_renderer_copy_map(const pbf_renderer* r, uint32_t which, float* host, size_t bytes) {
  uint32_t w, h;
  if (!host || pbf_renderer_map_size(r, which, &w, &h)) return PBF_EINVAL;
  if (bytes != (size_t)w * h * sizeof(float)) return PBF_EINVAL;
  return cudaMemcpy(host, pbf_renderer_map_device(r, which), bytes, cudaMemcpyDeviceToHost) == cudaSuccess
             ? PBF_OK
             : PBF_ECUDA;
}

int pbf_renderer_timings(const pbf_renderer* r, float ms[2]) {
  if (!r || !ms) return PBF_EINVAL;
  ms[0] = r->ms[0];
  ms[1] = r->ms[1];
  return PBF_OK;
}

}  // extern "C"
