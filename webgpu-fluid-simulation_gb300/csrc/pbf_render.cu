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
// Volume pass: sprites of half-side R on the half-resolution target add
// exp(-2 |n.xy|^2).  The sum is kept in 64-bit fixed point with 40
// fraction bits, where every float term in [e^-2, 1] is exact, so the sum
// is exact and order-free; it is rounded to float once.  The exponential is
// this file's own (splat_exp), so the CPU restatement can produce the same
// bits.
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
// written, which the CPU restatement reproduces.
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

struct Sprite {
  float fx0, fx1;  // framebuffer x of the left / right edge
  float fyt, fyb;  // framebuffer y of the top / bottom edge
  int i0, i1, j0, j1;  // covered pixels [i0, i1) x [j0, j1)
  float cz, cw;    // camera-space z and w of the centre
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

// The sprite of half-side hs around the particle on a W x H target; false
// when it is clipped away.
__device__ inline bool make_sprite(const Cam& C, const float c[4], float hs, int W, int H, Sprite& s) {
  float bl[4], tr[4];
  mat_vec(C.p, c[0] + (-hs), c[1] + (-hs), c[2], c[3], bl);
  mat_vec(C.p, c[0] + hs, c[1] + hs, c[2], c[3], tr);
  if (!(bl[3] > 0.0f) || !(bl[2] >= 0.0f) || !(bl[2] <= bl[3])) return false;
  const float fw = (float)W, fh = (float)H;
  s.fx0 = 0.5f * (bl[0] / bl[3] + 1.0f) * fw;
  s.fx1 = 0.5f * (tr[0] / tr[3] + 1.0f) * fw;
  s.fyb = 0.5f * (-(bl[1] / bl[3]) + 1.0f) * fh;
  s.fyt = 0.5f * (-(tr[1] / tr[3]) + 1.0f) * fh;
  if (!(s.fx1 != s.fx0) || !(s.fyb != s.fyt)) return false;
  s.i0 = pixel_edge(fminf(s.fx0, s.fx1), W);
  s.i1 = pixel_edge(fmaxf(s.fx0, s.fx1), W);
  s.j0 = pixel_edge(fminf(s.fyt, s.fyb), H);
  s.j1 = pixel_edge(fmaxf(s.fyt, s.fyb), H);
  s.cz = c[2];
  s.cw = c[3];
  return s.i0 < s.i1 && s.j0 < s.j1;
}

// |n.xy|^2 of the sprite's fragment at pixel (i, j).
__device__ inline float sprite_r2(const Sprite& s, int i, int j) {
  const float uvx = (((float)i + 0.5f) - s.fx0) / (s.fx1 - s.fx0);
  const float uvy = (s.fyb - ((float)j + 0.5f)) / (s.fyb - s.fyt);
  const float nx = uvx * 2.0f - 1.0f, ny = uvy * 2.0f - 1.0f;
  return nx * nx + ny * ny;
}

// Depth-pass fragment: camera z of the sphere point and its [0, 1] depth.
__device__ inline float sprite_depth(const Cam& C, const Sprite& s, float r2, float R, float& z) {
  const float nz = sqrtf(1.0f - r2);
  z = s.cz + nz * R;
  const float w = s.cw + 0.0f * R;
  const float d = (C.p[10] * z + C.p[14] * w) / (C.p[11] * z + C.p[15] * w);
  return d > 0.0f ? fminf(d, 1.0f) : 0.0f;
}

// exp(x) for x in [-2, 0]: Cody-Waite reduction x = k ln2 + r with ln 2 in
// two parts (the high part has 16 significant bits, so k * hi is exact for
// |k| <= 3), then exp(r) by its Taylor series to degree 8 in Horner form
// (|r| <= 0.35: truncation below 3e-10), scaled by 2^k.
__host__ __device__ inline float splat_exp(float x) {
  const float k = floorf(x * 1.44269502f + 0.5f);
  const float r = (x - k * 0.693145751953125f) - k * 1.42860677e-6f;
  float p = 2.48015873e-5f;           // 1/8!
  p = p * r + 1.98412698e-4f;         // 1/7!
  p = p * r + 1.38888889e-3f;         // 1/6!
  p = p * r + 8.33333333e-3f;         // 1/5!
  p = p * r + 4.16666667e-2f;         // 1/4!
  p = p * r + 1.66666667e-1f;         // 1/3!
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  const int e = (int)k + 127;         // 2^k as a float (k in [-3, 0])
  uint32_t bits = (uint32_t)e << 23;
  float scale;
  memcpy(&scale, &bits, 4);
  return p * scale;
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

// One warp per particle: the depth sprite on the full target, then the
// volume sprite on the half-resolution target.
__global__ void __launch_bounds__(256) k_splat(Cam C, const float4* __restrict__ pos, uint32_t n, float R, int W, int H,
                                               int W2, int H2, unsigned long long* keys, unsigned long long* acc) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += warps) {
    const float4 x = pos[q];
    float c[4];
    mat_vec(C.v, x.x, x.y, x.z, 1.0f, c);
    Sprite s;
    if (make_sprite(C, c, 0.5f * R, W, H, s)) {
      const int w = s.i1 - s.i0, cnt = w * (s.j1 - s.j0);
      const unsigned long long low = 0xffffffffull - q;
      for (int t = lane; t < cnt; t += 32) {
        const int i = s.i0 + t % w, j = s.j0 + t / w;
        const float r2 = sprite_r2(s, i, j);
        if (r2 > 1.0f) continue;
        float z;
        const float d = sprite_depth(C, s, r2, R, z);
        const unsigned long long key = ((unsigned long long)depth_bits(d) << 32) | low;
        unsigned long long* k = keys + (size_t)j * W + i;
        if (key > *(volatile unsigned long long*)k) atomicMax(k, key);
      }
    }
    if (make_sprite(C, c, R, W2, H2, s)) {
      const int w = s.i1 - s.i0, cnt = w * (s.j1 - s.j0);
      for (int t = lane; t < cnt; t += 32) {
        const int i = s.i0 + t % w, j = s.j0 + t / w;
        const float r2 = sprite_r2(s, i, j);
        if (r2 > 1.0f) continue;
        const float v = splat_exp(-r2 * 2.0f);
        atomicAdd(acc + (size_t)j * W2 + i, (unsigned long long)((double)v * kFix));
      }
    }
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
    out = -z / (s.cw + 0.0f * R);
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
    const unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)n * 32 + 255) / 256, (uint64_t)sms * 8 * 32);
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
