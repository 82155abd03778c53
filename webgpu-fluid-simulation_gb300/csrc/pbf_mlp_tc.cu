// pbf_mlp_tc.cu — inference of the learned start's network (8 -> 64 -> 64 -> 1,
// SiLU, BF16 weights and activations, FP32 accumulation) on the 5th-generation
// tensor cores: tcgen05.mma with both operands in shared memory and the
// accumulators in tensor memory (TMEM), read back with tcgen05.ld.
//
// One CTA of 1024 threads per SM holds the weights once and runs eight
// independent tile pipelines, one per warpgroup: warpgroup g walks its own
// 128-row tiles (persistent grid), thread t of the warpgroup serving row t.
// Each pipeline has its own operand tiles, its own mbarrier, a named barrier
// of 128 threads, and TMEM columns 64 g .. 64 g + 63 (layer 2 reuses layer
// 1's columns once they have been read), so an SM keeps eight tiles in
// flight.  (Four CTAs of two pipelines each, the same resources per SM,
// entered in waves about 10 us apart, each after the previous wave's weight
// staging; one CTA per SM stages the weights once and starts every pipeline
// together.)  Per tile:
//   1. each thread normalises its row's 8 features into bf16 and stores them
//      in columns 0..7 of the pipeline's X tile (K = 16); columns 8 and 9
//      hold the constant 1, the rest 0;
//   2. the warpgroup's first thread issues D = X W1' (M=128, N=64, K=16),
//      where rows 8 and 9 of W1' carry b1 split into two bf16 parts (hi and
//      the remainder lo), so D = X W1 + b1 to about 2^-16 relative; it
//      commits to the pipeline's mbarrier;
//   3. every thread loads its row of D (tcgen05.ld), applies SiLU, rounds to
//      bf16 and stores the row of H1 into the pipeline's H tile;
//   4. D = H1 W2 (four K=16 steps) + X B2 (one step; B2's only non-zero rows
//      8 and 9 carry b2 hi/lo against X's constant columns), into the same
//      columns;
//   5. every thread loads its row of D, applies SiLU, rounds to bf16 and
//      stores H2 over H1;
//   6. D = H2 W3' + X B3 (M=128, N=16): columns 0 and 1 of W3' hold w3 hi and
//      lo, B3 carries b3 hi/lo, so y = D[0] + D[1]; lambda_hat = y lam_scale.
// The rounding points of the activations are those of the mma.sync kernels
// (pbf_learned.cu); the biases and the last layer are summed by the tensor
// cores in FP32.
//
// Operand layout: the canonical K-major layout without swizzling: 8-row x
// 16-byte core matrices stored contiguously (128 B), core matrices adjacent
// in K at LBO = 128 B, adjacent 8-row groups at SBO = (K / 8) * 128 B.
#include <algorithm>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"
#include "pbf_kernels.h"
#include "pbf_mlp.cuh"

namespace pbf {
namespace {

using namespace mlp;

constexpr int kTcRows = 128;                     // rows per tile (UMMA M)
constexpr int kTcPipes = 8;                      // tile pipelines (warpgroups) per CTA
constexpr int kTcThreads = 128 * kTcPipes;       // one CTA per SM
constexpr uint32_t kTmemCols = 64u * kTcPipes;   // pipeline g: columns 64 g .. 64 g + 63
constexpr uint32_t kWaitPolls = 1u << 24;

struct TcSmem {
  alignas(128) uint8_t a1[kTcPipes][kTcRows * 16 * 2];  // X per pipeline: 128 x 16 bf16
  alignas(128) uint8_t a2[kTcPipes][kTcRows * 64 * 2];  // H1, then H2, per pipeline: 128 x 64 bf16
  alignas(128) uint8_t b1[64 * 16 * 2];          // W1'^T: 64 x 16 bf16 (N x K), b1 in K rows 8, 9
  alignas(128) uint8_t b2[64 * 64 * 2];          // W2^T: 64 x 64 bf16
  alignas(128) uint8_t b2b[64 * 16 * 2];         // b2 in K rows 8, 9 (against X's ones): 64 x 16
  alignas(128) uint8_t b3[16 * 64 * 2];          // W3'^T: 16 x 64, w3 hi / lo in N rows 0, 1
  alignas(128) uint8_t b3b[16 * 16 * 2];         // b3 hi / lo in N row 0, K rows 8, 9
  alignas(8) uint64_t mbar[kTcPipes];
  uint32_t tmem;
  uint32_t failed[kTcPipes];  // per pipeline: a completion wait gave up
};

// Byte offset of element (row, k) in a K-major canonical tile with kk K elements.
__device__ __forceinline__ uint32_t canon(uint32_t row, uint32_t k, uint32_t kk) {
  return (row >> 3) * (kk / 8u) * 128u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, LBO, SBO (all >> 4), version 1
// (bits 46-47), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr uint32_t idesc_of(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}
constexpr uint32_t kIdesc64 = idesc_of(64), kIdesc16 = idesc_of(16);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// Bounded wait for the mbarrier phase; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (uint32_t i = 0; i < kWaitPolls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
    if (i > 32) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Two consecutive TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float& a, float& b) {
  uint32_t r0, r1;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  a = __uint_as_float(r0);
  b = __uint_as_float(r1);
}

// SiLU(z) = z sigmoid(z) = h + h tanh(h) with h = z / 2 (one tanh.approx).
__device__ __forceinline__ float silu_h(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_fast(h), h);
}

// Splits of a float into two bf16 parts: hi = bf16(x), lo = bf16(x - hi).
__device__ __forceinline__ __nv_bfloat16 bf_hi(float x) { return __float2bfloat16_rn(x); }
__device__ __forceinline__ __nv_bfloat16 bf_lo(float x) {
  return __float2bfloat16_rn(x - __bfloat162float(__float2bfloat16_rn(x)));
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// Barrier of one pipeline's 128 threads (named barriers 1 .. kTcPipes).
__device__ __forceinline__ void pipe_sync(uint32_t wg) {
  asm volatile("bar.sync %0, 128;" ::"r"(1u + wg) : "memory");
}

__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_infer_tc(const float* __restrict__ P, Norm nm,
                                                            const float* __restrict__ feat, uint32_t rows,
                                                            float* __restrict__ lambda, float* __restrict__ lam_sum,
                                                            const float4* __restrict__ xs, float4* __restrict__ xl,
                                                            uint32_t* err, LateBoundary lb) {
  extern __shared__ __align__(128) uint8_t tc_raw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(tc_raw);
  const uint32_t tid = threadIdx.x, warp = tid >> 5, row = tid & 127u, wg = tid >> 7;
  // weights into the canonical layouts; X's constant columns (8, 9: one) set once
  const __nv_bfloat16 z16 = __float2bfloat16_rn(0.0f);
  for (uint32_t q = tid; q < 64u * 16u; q += kTcThreads) {
    const uint32_t n = q / 16u, k = q % 16u;
    __nv_bfloat16 w = z16, wb = z16;
    if (k < (uint32_t)kIn) {
      w = __float2bfloat16_rn(P[OFF_W1 + k * kH + n]);
    } else if (k == 8) {
      w = bf_hi(P[OFF_B1 + n]);
      wb = bf_hi(P[OFF_B2 + n]);
    } else if (k == 9) {
      w = bf_lo(P[OFF_B1 + n]);
      wb = bf_lo(P[OFF_B2 + n]);
    }
    *reinterpret_cast<__nv_bfloat16*>(sm.b1 + canon(n, k, 16)) = w;
    *reinterpret_cast<__nv_bfloat16*>(sm.b2b + canon(n, k, 16)) = wb;
  }
  for (uint32_t q = tid; q < 64u * 64u; q += kTcThreads) {
    const uint32_t k = q / 64u, n = q % 64u;  // W2[k][n]
    *reinterpret_cast<__nv_bfloat16*>(sm.b2 + canon(n, k, 64)) = __float2bfloat16_rn(P[OFF_W2 + q]);
  }
  for (uint32_t q = tid; q < 16u * 64u; q += kTcThreads) {
    const uint32_t n = q / 64u, k = q % 64u;
    const float w = P[OFF_W3 + k];
    *reinterpret_cast<__nv_bfloat16*>(sm.b3 + canon(n, k, 64)) = n == 0 ? bf_hi(w) : n == 1 ? bf_lo(w) : z16;
  }
  for (uint32_t q = tid; q < 16u * 16u; q += kTcThreads) {
    const uint32_t n = q / 16u, k = q % 16u;
    const float b = P[OFF_B3];
    *reinterpret_cast<__nv_bfloat16*>(sm.b3b + canon(n, k, 16)) =
        (n == 0 && k == 8) ? bf_hi(b) : (n == 0 && k == 9) ? bf_lo(b) : z16;
  }
  st_shared_v4(smem_u32(sm.a1[wg] + canon(row, 8, 16)), pack_bf16(1.0f, 1.0f), 0u, 0u, 0u);
  const uint32_t mbar = smem_u32(&sm.mbar[wg]);
  if (row == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    sm.failed[wg] = 0u;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t dcol = sm.tmem + 64u * wg;                // this pipeline's accumulator
  const uint32_t lane_base = (32u * (warp & 3u)) << 16;    // this warp's TMEM lanes
  const uint64_t a1d = smem_desc(smem_u32(sm.a1[wg]), 128, 256);
  const uint64_t b1d = smem_desc(smem_u32(sm.b1), 128, 256);
  const uint64_t b2bd = smem_desc(smem_u32(sm.b2b), 128, 256);
  const uint64_t b3bd = smem_desc(smem_u32(sm.b3b), 128, 256);
  const uint32_t a2 = smem_u32(sm.a2[wg]), b2 = smem_u32(sm.b2), b3 = smem_u32(sm.b3);
  uint32_t phase = 0;
  const uint32_t tiles = (rows + kTcRows - 1) / kTcRows;
  const uint32_t first = (uint32_t)kTcPipes * blockIdx.x + wg, step = (uint32_t)kTcPipes * gridDim.x;
  // the next tile's feature row (and x* when the output is packed), loaded
  // one tile ahead
  float4 nf0 = make_float4(0.f, 0.f, 0.f, 0.f), nf1 = nf0, nx = nf0, nb = nf0;
  float nsd = 0.0f;
  auto fetch = [&](uint32_t tile) {
    const uint32_t rr = tile * kTcRows + row;
    if (tile < tiles && rr < rows) {
      nf0 = reinterpret_cast<const float4*>(feat)[2 * (size_t)rr];
      nf1 = reinterpret_cast<const float4*>(feat)[2 * (size_t)rr + 1];
      if (xl) nx = xs[rr];
      if (lb.bdata) {
        nb = lb.bdata[rr];
        nsd = lb.bsdf[rr];
      }
    }
  };
  fetch(first);
  for (uint32_t tile = first; tile < tiles; tile += step) {
    const uint32_t r = tile * kTcRows + row;
    const bool valid = r < rows;
    // 1. X row: normalised features in bf16
    {
      float x[8];
      if (valid) {
        float f[8] = {nf0.x, nf0.y, nf0.z, nf0.w, nf1.x, nf1.y, nf1.z, nf1.w};
        if (lb.bdata) {  // the boundary terms of features 0, 5 and 6 (LateBoundary)
          float dens = f[0];
          if (nb.w != 0.0f) {
            const float dx = nx.x - nb.x, dy = nx.y - nb.y, dz = nx.z - nb.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            const float t = lb.h2 - r2;
            dens = dens + nb.w * ((r2 <= lb.h2) ? lb.poly6 * (t * t * t) : 0.0f);
          }
          f[0] = dens - 1.0f;
          f[5] = fminf(nsd, 2.0f * lb.h) / lb.h;
          f[6] = nb.w / lb.V;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = (f[k] - nm.mean[k]) * nm.inv_std[k];
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = 0.0f;
      }
      st_shared_v4(smem_u32(sm.a1[wg] + canon(row, 0, 16)), pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]),
                   pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
    }
    const float4 xr = nx;
    fetch(tile + step);  // in flight while this tile is computed
    fence_async_smem();
    fence_before_sync();
    pipe_sync(wg);
    fence_after_sync();
    // a failure flagged before this barrier is seen by every thread of the
    // pipeline, so they leave together
    if (*(volatile uint32_t*)&sm.failed[wg]) break;
    // 2. D = X W1 + b1
    if (row == 0) {
      mma_f16(dcol, a1d, b1d, kIdesc64, 0u);
      mma_commit(mbar);
    }
    bool ok = mbar_wait(mbar, phase);
    phase ^= 1u;
    fence_after_sync();
    // 3. and 5.: this row of D -> bf16(SiLU(D)) into the H tile, 32 columns at a time
    auto act = [&]() {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        float v[32];
        tmem_ld32(dcol + lane_base + 32u * half, v);
#pragma unroll
        for (int kb = 0; kb < 4; ++kb) {
          const int j = 8 * kb;
          st_shared_v4(a2 + canon(row, 32 * half + 8 * kb, 64), pack_bf16(silu_h(v[j]), silu_h(v[j + 1])),
                       pack_bf16(silu_h(v[j + 2]), silu_h(v[j + 3])), pack_bf16(silu_h(v[j + 4]), silu_h(v[j + 5])),
                       pack_bf16(silu_h(v[j + 6]), silu_h(v[j + 7])));
        }
      }
      fence_async_smem();
      fence_before_sync();
      pipe_sync(wg);
      fence_after_sync();
    };
    act();
    // 4. D = H1 W2 + b2 (four K = 16 steps and the bias step), over layer 1's columns
    if (row == 0) {
#pragma unroll
      for (uint32_t ks = 0; ks < 4; ++ks)
        mma_f16(dcol, smem_desc(a2 + 256u * ks, 128, 1024), smem_desc(b2 + 256u * ks, 128, 1024), kIdesc64,
                ks > 0 ? 1u : 0u);
      mma_f16(dcol, a1d, b2bd, kIdesc64, 1u);
      mma_commit(mbar);
    }
    ok = mbar_wait(mbar, phase) && ok;
    phase ^= 1u;
    fence_after_sync();
    act();
    // 6. y = H2 w3 + b3 (N = 16; columns 0 and 1 hold the hi and lo parts)
    if (row == 0) {
#pragma unroll
      for (uint32_t ks = 0; ks < 4; ++ks)
        mma_f16(dcol, smem_desc(a2 + 256u * ks, 128, 1024), smem_desc(b3 + 256u * ks, 128, 1024), kIdesc16,
                ks > 0 ? 1u : 0u);
      mma_f16(dcol, a1d, b3bd, kIdesc16, 1u);
      mma_commit(mbar);
    }
    ok = mbar_wait(mbar, phase) && ok;
    phase ^= 1u;
    fence_after_sync();
    if (!ok) atomicOr(&sm.failed[wg], 1u);
    float y0, y1;
    tmem_ld2(dcol + lane_base, y0, y1);
    const float y = y0 + y1;
    // the next tile's layer 1 overwrites these columns only after this barrier
    fence_before_sync();
    if (valid) {
      const float l = y * nm.lam_scale;
      if (xl) {
        xl[r] = make_float4(xr.x, xr.y, xr.z, l);
      } else {
        lambda[r] = l;
      }
      if (lam_sum) lam_sum[r] = l;
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(sm.tmem), "r"(kTmemCols) : "memory");
  }
  if (tid == 0 && err) {
    uint32_t f = 0;
    for (int g = 0; g < kTcPipes; ++g) f |= sm.failed[g];
    if (f) atomicOr(err, PBF_DEVERR_MMA_TIMEOUT);
  }
}


// ---- training: forward + backward on the tensor cores --------------------------------
//
// One CTA of 128 threads (one warpgroup), thread t serving row t of each
// 128-row tile, TMEM holding every accumulator (512 columns: one CTA per SM):
//   columns   0- 63  z1 = X W1 + b1            (kept for the backward pass)
//   columns  64-127  z2 = H1 W2 + b2           (kept for the backward pass)
//   columns 128-143  y  = H2 w3 + b3           (hi / lo columns 0, 1)
//   columns 160-223  dH1 = dZ2 W2^T
//   columns 256-319  [dW2; db2]  accumulated over the CTA's tiles
//   columns 320-383  [dW1; db1]  accumulated over the CTA's tiles
//   columns 384-399  [dw3; db3]  accumulated over the CTA's tiles
// The weight and bias gradients are products over the tile's rows: their A
// operands are the transposed activations H1^T, X^T, H2^T (M = 128: the
// hidden / input units, then one row of ones that turns the same product
// into the bias gradient; the rows past it are never written, as the
// accumulator rows they feed are never read) and their B operands dZ2^T, dZ1^T and
// dy (N x K = rows), each written by its row's thread into column t of a
// K-major tile.  dy is split into bf16 hi / lo rows, so dw3 and db3 keep
// about 2^-16 relative accuracy; the other products take their operands in
// bf16 at the rounding points of the mma.sync kernel (X, W, H1, H2, dZ2,
// dZ1).  All operands are K-major, no swizzle, as in k_mlp_infer_tc.
constexpr uint32_t kGrTmemCols = 512;
constexpr uint32_t kColZ1 = 0, kColZ2 = 64, kColY = 128, kColDH1 = 160, kColG1 = 256, kColG2 = 320, kColG3 = 384;

struct GrSmem {
  alignas(128) uint8_t x1[128 * 16 * 2];    // X rows (K = 16: 8 features, ones at 8, 9)
  alignas(128) uint8_t hA[128 * 64 * 2];    // H1 rows, then H2 rows, then dZ2 rows
  alignas(128) uint8_t tH1[128 * 128 * 2];  // A of [dW2; db2]: H1^T, ones (row 64); rows 65+ unused
  alignas(128) uint8_t tX[128 * 128 * 2];   // A of [dW1; db1]: X^T, ones (row 8); rows 9+ unused
  alignas(128) uint8_t tH2[128 * 128 * 2];  // A of [dw3; db3]: H2^T, ones (row 64); rows 65+ unused
  alignas(128) uint8_t tDZ2[64 * 128 * 2];  // B: dZ2^T (N = 64 x K = rows)
  alignas(128) uint8_t tDZ1[64 * 128 * 2];  // B: dZ1^T
  alignas(128) uint8_t tDY[16 * 128 * 2];   // B: dy hi (N row 0), lo (row 1); rows 2+ unused
  alignas(128) uint8_t b1[64 * 16 * 2];     // W1'^T with b1 hi / lo in K rows 8, 9
  alignas(128) uint8_t b2[64 * 64 * 2];     // W2^T (N = out, K = in)
  alignas(128) uint8_t b2b[64 * 16 * 2];    // b2 hi / lo in K rows 8, 9
  alignas(128) uint8_t b3[16 * 64 * 2];     // w3 hi / lo in N rows 0, 1
  alignas(128) uint8_t b3b[16 * 16 * 2];    // b3 hi / lo in N row 0, K rows 8, 9
  alignas(128) uint8_t b2t[64 * 64 * 2];    // W2 (N = in, K = out): B of dH1 = dZ2 W2^T
  float w3[64];                             // w3 in FP32 (dZ2's factor)
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  uint32_t failed;
};

__device__ __forceinline__ void st_bf16(uint8_t* tile, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + off) = __float2bfloat16_rn(v);
}

// All threads' shared-memory writes visible to the tensor cores, then thread
// 0 issues `issue()` and commits; everyone waits for the MMAs (bounded).
template <class F>
__device__ __forceinline__ bool gr_mma_step(GrSmem& sm, uint32_t mbar, uint32_t& phase, F&& issue) {
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (threadIdx.x == 0) {
    issue();
    mma_commit(mbar);
  }
  const bool ok = mbar_wait(mbar, phase);
  phase ^= 1u;
  fence_after_sync();
  return ok;
}

__global__ void __launch_bounds__(128, 1) k_mlp_grad_tc(const float* __restrict__ P, Norm nm,
                                                      const float* __restrict__ feat,
                                                      const float* __restrict__ target, uint32_t rows,
                                                      float inv_batch, float* __restrict__ G,
                                                      float* __restrict__ loss, uint32_t* err) {
  extern __shared__ __align__(128) uint8_t gr_raw[];
  GrSmem& sm = *reinterpret_cast<GrSmem*>(gr_raw);
  const uint32_t tid = threadIdx.x, warp = tid >> 5, row = tid;
  const __nv_bfloat16 z16 = __float2bfloat16_rn(0.0f);
  // weights (as in k_mlp_infer_tc) and the transposed W2
  for (uint32_t q = tid; q < 64u * 16u; q += 128u) {
    const uint32_t n = q / 16u, k = q % 16u;
    __nv_bfloat16 w = z16, wb = z16;
    if (k < (uint32_t)kIn) {
      w = __float2bfloat16_rn(P[OFF_W1 + k * kH + n]);
    } else if (k == 8) {
      w = bf_hi(P[OFF_B1 + n]);
      wb = bf_hi(P[OFF_B2 + n]);
    } else if (k == 9) {
      w = bf_lo(P[OFF_B1 + n]);
      wb = bf_lo(P[OFF_B2 + n]);
    }
    *reinterpret_cast<__nv_bfloat16*>(sm.b1 + canon(n, k, 16)) = w;
    *reinterpret_cast<__nv_bfloat16*>(sm.b2b + canon(n, k, 16)) = wb;
  }
  for (uint32_t q = tid; q < 64u * 64u; q += 128u) {
    const uint32_t i = q / 64u, j = q % 64u;  // W2[i][j]: in i, out j
    const __nv_bfloat16 w = __float2bfloat16_rn(P[OFF_W2 + q]);
    *reinterpret_cast<__nv_bfloat16*>(sm.b2 + canon(j, i, 64)) = w;
    *reinterpret_cast<__nv_bfloat16*>(sm.b2t + canon(i, j, 64)) = w;
  }
  for (uint32_t q = tid; q < 16u * 64u; q += 128u) {
    const uint32_t n = q / 64u, k = q % 64u;
    const float w = P[OFF_W3 + k];
    *reinterpret_cast<__nv_bfloat16*>(sm.b3 + canon(n, k, 64)) = n == 0 ? bf_hi(w) : n == 1 ? bf_lo(w) : z16;
  }
  for (uint32_t q = tid; q < 16u * 16u; q += 128u) {
    const uint32_t n = q / 16u, k = q % 16u;
    const float b = P[OFF_B3];
    *reinterpret_cast<__nv_bfloat16*>(sm.b3b + canon(n, k, 16)) =
        (n == 0 && k == 8) ? bf_hi(b) : (n == 0 && k == 9) ? bf_lo(b) : z16;
  }
  // constant parts of the gradient operands: the ones rows (row 64 of H1^T
  // and H2^T, row 8 of X^T) that turn the products into bias gradients.
  // The data rows are rewritten for every tile.  The rows below them (and
  // dy's rows 2..15) are not written: they only reach accumulator rows
  // (columns of [dw3; db3]) that are never read.  Thread t writes the
  // 16-byte unit of elements k = 8 (t % 16) .. + 7 of one ones row.
  if (tid < 48u) {
    const uint32_t ones2 = pack_bf16(1.0f, 1.0f);
    uint8_t* tile = tid < 16u ? sm.tH1 : tid < 32u ? sm.tH2 : sm.tX;
    const uint32_t m = tid < 32u ? 64u : 8u, k = 8u * (tid % 16u);
    st_shared_v4(smem_u32(tile + canon(m, k, 128)), ones2, ones2, ones2, ones2);
  }
  if (tid < 64u) sm.w3[tid] = P[OFF_W3 + tid];
  st_shared_v4(smem_u32(sm.x1 + canon(row, 8, 16)), pack_bf16(1.0f, 1.0f), 0u, 0u, 0u);
  const uint32_t mbar = smem_u32(&sm.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    sm.failed = 0u;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem)),
                 "r"(kGrTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tm = sm.tmem;
  const uint32_t lane_base = (32u * warp) << 16;
  const uint64_t x1d = smem_desc(smem_u32(sm.x1), 128, 256);
  const uint64_t b1d = smem_desc(smem_u32(sm.b1), 128, 256);
  const uint64_t b2bd = smem_desc(smem_u32(sm.b2b), 128, 256);
  const uint64_t b3bd = smem_desc(smem_u32(sm.b3b), 128, 256);
  const uint32_t hA = smem_u32(sm.hA), b2 = smem_u32(sm.b2), b3 = smem_u32(sm.b3), b2t = smem_u32(sm.b2t);
  const uint32_t tH1 = smem_u32(sm.tH1), tX = smem_u32(sm.tX), tH2 = smem_u32(sm.tH2);
  const uint32_t tDZ2 = smem_u32(sm.tDZ2), tDZ1 = smem_u32(sm.tDZ1), tDY = smem_u32(sm.tDY);
  uint32_t phase = 0;
  bool ok = true;
  float lsum = 0.0f;
  uint32_t done_tiles = 0;
  const uint32_t tiles = (rows + 127u) / 128u;
  for (uint32_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++done_tiles) {
    const uint32_t r = tile * 128u + row;
    const bool valid = r < rows;
    float x[8], t = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = valid ? (feat[8 * (size_t)r + k] - nm.mean[k]) * nm.inv_std[k] : 0.0f;
    if (valid) t = target[r] / nm.lam_scale;
    st_shared_v4(smem_u32(sm.x1 + canon(row, 0, 16)), pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]),
                 pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
#pragma unroll
    for (int k = 0; k < 8; ++k) st_bf16(sm.tX, canon(k, row, 128), x[k]);
    // z1 = X W1 + b1
    ok = gr_mma_step(sm, mbar, phase, [&] { mma_f16(tm + kColZ1, x1d, b1d, kIdesc64, 0u); }) && ok;
    // H1 rows (layer 2's A) and H1^T (dW2's A)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tmem_ld32(tm + lane_base + kColZ1 + 32u * half, v);
#pragma unroll
      for (int kb = 0; kb < 4; ++kb) {
        const int j = 8 * kb;
        float h[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) h[e] = silu_h(v[j + e]);
        st_shared_v4(hA + canon(row, 32 * half + j, 64), pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]),
                     pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]));
#pragma unroll
        for (int e = 0; e < 8; ++e) st_bf16(sm.tH1, canon(32 * half + j + e, row, 128), h[e]);
      }
    }
    // z2 = H1 W2 + b2
    ok = gr_mma_step(sm, mbar, phase, [&] {
      for (uint32_t ks = 0; ks < 4; ++ks)
        mma_f16(tm + kColZ2, smem_desc(hA + 256u * ks, 128, 1024), smem_desc(b2 + 256u * ks, 128, 1024), kIdesc64,
                ks > 0 ? 1u : 0u);
      mma_f16(tm + kColZ2, x1d, b2bd, kIdesc64, 1u);
    }) && ok;
    // H2 rows (layer 3's A) and H2^T (dw3's A)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tmem_ld32(tm + lane_base + kColZ2 + 32u * half, v);
#pragma unroll
      for (int kb = 0; kb < 4; ++kb) {
        const int j = 8 * kb;
        float h[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) h[e] = silu_h(v[j + e]);
        st_shared_v4(hA + canon(row, 32 * half + j, 64), pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]),
                     pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]));
#pragma unroll
        for (int e = 0; e < 8; ++e) st_bf16(sm.tH2, canon(32 * half + j + e, row, 128), h[e]);
      }
    }
    // y = H2 w3 + b3
    ok = gr_mma_step(sm, mbar, phase, [&] {
      for (uint32_t ks = 0; ks < 4; ++ks)
        mma_f16(tm + kColY, smem_desc(hA + 256u * ks, 128, 1024), smem_desc(b3 + 256u * ks, 128, 1024), kIdesc16,
                ks > 0 ? 1u : 0u);
      mma_f16(tm + kColY, x1d, b3bd, kIdesc16, 1u);
    }) && ok;
    float y0, y1;
    tmem_ld2(tm + lane_base + kColY, y0, y1);
    const float err_y = valid ? (y0 + y1) - t : 0.0f;
    lsum += err_y * err_y;
    const float dy = 2.0f * err_y * inv_batch;
    st_bf16(sm.tDY, canon(0, row, 128), dy);
    st_bf16(sm.tDY, canon(1, row, 128), dy - __bfloat162float(__float2bfloat16_rn(dy)));
    // dZ2 = dy w3 silu'(z2): rows (dH1's A) and transposed (dW2's B)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tmem_ld32(tm + lane_base + kColZ2 + 32u * half, v);
#pragma unroll
      for (int kb = 0; kb < 4; ++kb) {
        const int j = 8 * kb;
        float d[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) d[e] = dy * sm.w3[32 * half + j + e] * dsilu_f(v[j + e]);
        st_shared_v4(hA + canon(row, 32 * half + j, 64), pack_bf16(d[0], d[1]), pack_bf16(d[2], d[3]),
                     pack_bf16(d[4], d[5]), pack_bf16(d[6], d[7]));
#pragma unroll
        for (int e = 0; e < 8; ++e) st_bf16(sm.tDZ2, canon(32 * half + j + e, row, 128), d[e]);
      }
    }
    // dH1 = dZ2 W2^T
    ok = gr_mma_step(sm, mbar, phase, [&] {
      for (uint32_t ks = 0; ks < 4; ++ks)
        mma_f16(tm + kColDH1, smem_desc(hA + 256u * ks, 128, 1024), smem_desc(b2t + 256u * ks, 128, 1024),
                kIdesc64, ks > 0 ? 1u : 0u);
    }) && ok;
    // dZ1 = dH1 silu'(z1), transposed (dW1's B)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float g[32], z[32];
      tmem_ld32(tm + lane_base + kColDH1 + 32u * half, g);
      tmem_ld32(tm + lane_base + kColZ1 + 32u * half, z);
#pragma unroll
      for (int e = 0; e < 32; ++e) st_bf16(sm.tDZ1, canon(32 * half + e, row, 128), g[e] * dsilu_f(z[e]));
    }
    // the gradient products over the tile's rows, accumulated across tiles
    const uint32_t acc0 = done_tiles > 0 ? 1u : 0u;
    ok = gr_mma_step(sm, mbar, phase, [&] {
      for (uint32_t ks = 0; ks < 8; ++ks) {
        const uint32_t a = ks > 0 ? 1u : acc0;
        mma_f16(tm + kColG1, smem_desc(tH1 + 256u * ks, 128, 2048), smem_desc(tDZ2 + 256u * ks, 128, 2048), kIdesc64,
                a);
        mma_f16(tm + kColG2, smem_desc(tX + 256u * ks, 128, 2048), smem_desc(tDZ1 + 256u * ks, 128, 2048), kIdesc64,
                a);
        mma_f16(tm + kColG3, smem_desc(tH2 + 256u * ks, 128, 2048), smem_desc(tDY + 256u * ks, 128, 2048), kIdesc16,
                a);
      }
    }) && ok;
    ok = !__syncthreads_or(!ok);
  }
  if (!ok) {
    // a completion wait gave up: let the MMAs in flight finish (bounded)
    // before TMEM is read or released
    mbar_wait(mbar, phase);
    if (tid == 0 && err) atomicOr(err, PBF_DEVERR_MMA_TIMEOUT);
  } else if (done_tiles > 0) {
    // row m of the accumulators: [dW2; db2], [dW1; db1], [dw3; db3]
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tmem_ld32(tm + lane_base + kColG1 + 32u * half, v);
      if (row < 64u) {
#pragma unroll
        for (int e = 0; e < 32; ++e) atomicAdd(G + OFF_W2 + row * kH + 32 * half + e, v[e]);
      } else if (row == 64u) {
#pragma unroll
        for (int e = 0; e < 32; ++e) atomicAdd(G + OFF_B2 + 32 * half + e, v[e]);
      }
      tmem_ld32(tm + lane_base + kColG2 + 32u * half, v);
      if (row < (uint32_t)kIn) {
#pragma unroll
        for (int e = 0; e < 32; ++e) atomicAdd(G + OFF_W1 + row * kH + 32 * half + e, v[e]);
      } else if (row == (uint32_t)kIn) {
#pragma unroll
        for (int e = 0; e < 32; ++e) atomicAdd(G + OFF_B1 + 32 * half + e, v[e]);
      }
    }
    float g0, g1;
    tmem_ld2(tm + lane_base + kColG3, g0, g1);
    if (row < 64u) atomicAdd(G + OFF_W3 + row, g0 + g1);
    else if (row == 64u) atomicAdd(G + OFF_B3, g0 + g1);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((tid & 31u) == 0) atomicAdd(loss, lsum);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(kGrTmemCols) : "memory");
  }
}
}  // namespace

// The tile buffers of the eight pipelines and the weights (about 175 KB) in
// dynamic shared memory; one CTA per SM holds all 512 TMEM columns.
constexpr int kTcSmem = (int)sizeof(TcSmem);

cudaError_t launch_mlp_infer_tc(const float* d_params, const pbf_mlp& model, const float* d_feat, uint32_t rows,
                                float* d_lambda, float* d_lam_sum, cudaStream_t st, const float4* d_xs, float4* d_xl,
                                uint32_t* d_err, LateBoundary lb) {
  if (rows == 0) return cudaSuccess;
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // dynamic shared memory above the 48 KB default needs the opt-in
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    // one CTA per SM: it allocates all 512 TMEM columns
    per_sm = 1;
    if (e != cudaSuccess) {
      sms = 0;
      return e;
    }
  }
  Norm nm;
  for (int k = 0; k < kIn; ++k) {
    nm.mean[k] = model.feat_mean[k];
    nm.inv_std[k] = model.feat_inv_std[k];
  }
  nm.lam_scale = model.lam_scale;
  const uint32_t tiles = (rows + kTcRows - 1) / kTcRows;
  // one resident wave, kTcPipes tile pipelines per CTA
  const uint32_t grid =
      std::min<uint32_t>((tiles + kTcPipes - 1) / kTcPipes, (uint32_t)sms * (uint32_t)per_sm);
  k_mlp_infer_tc<<<grid, kTcThreads, kTcSmem, st>>>(d_params, nm, d_feat, rows, d_lambda, d_lam_sum, d_xs, d_xl,
                                                    d_err, lb);
  return cudaGetLastError();
}

cudaError_t launch_mlp_grad_tc(const float* d_params, const pbf_mlp& model, const float* d_feat,
                               const float* d_target, uint32_t rows, float* d_grad, float* d_loss, uint32_t* d_err,
                               cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GrSmem));
    if (e != cudaSuccess) {
      sms = 0;
      return e;
    }
  }
  Norm nm;
  for (int k = 0; k < kIn; ++k) {
    nm.mean[k] = model.feat_mean[k];
    nm.inv_std[k] = model.feat_inv_std[k];
  }
  nm.lam_scale = model.lam_scale;
  const uint32_t tiles = (rows + 127u) / 128u;
  // one CTA per SM at most: each holds all 512 TMEM columns
  const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)sms);
  k_mlp_grad_tc<<<grid, 128, sizeof(GrSmem), st>>>(d_params, nm, d_feat, d_target, rows, 1.0f / (float)rows,
                                                   d_grad, d_loss, d_err);
  return cudaGetLastError();
}

}  // namespace pbf
