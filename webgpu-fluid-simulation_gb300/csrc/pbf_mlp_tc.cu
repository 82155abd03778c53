// pbf_mlp_tc.cu — inference of the learned start's network (8 -> 64 -> 64 -> 1,
// SiLU, BF16 weights and activations, FP32 accumulation) on the 5th-generation
// tensor cores: tcgen05.mma with both operands in shared memory and the
// accumulators in tensor memory (TMEM), read back with tcgen05.ld.
//
// A CTA of 256 threads (two warpgroups) owns TMEM lanes 0..127 and walks
// 128-row tiles (persistent grid).  Thread t serves row t % 128; warp w reads
// lanes 32 (w % 4) .. + 31, and warpgroup g takes accumulator columns
// 32 g .. 32 g + 31 of each layer, so both warpgroups share every epilogue:
//   1. each thread normalises its row's 8 features into bf16 (K padded to 16)
//      and stores them in the A tile (shared memory);
//   2. one thread issues D1 = X W1 (M=128, N=64, K=16) into TMEM columns
//      0..63 and commits to an mbarrier;
//   3. every thread loads its row of D1 (tcgen05.ld), adds b1, applies SiLU,
//      rounds to bf16 and stores the row of H1 into the second A tile;
//   4. one thread issues D2 = H1 W2 (four K=16 steps) into columns 64..127;
//   5. every thread loads its row of D2, adds b2, applies SiLU, rounds to
//      bf16 and forms y = w3 . h2 + b3; lambda_hat = y * lam_scale.
// The rounding points are those of the mma.sync kernels (pbf_learned.cu).
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

constexpr int kTcRows = 128;        // rows per tile (UMMA M)
constexpr int kTcThreads = 256;     // two threads per row (one per warpgroup)
constexpr uint32_t kTmemCols = 128; // D1: columns 0..63, D2: 64..127
constexpr uint32_t kWaitPolls = 1u << 24;

struct TcSmem {
  alignas(128) uint8_t a1[kTcRows * 16 * 2];  // X: 128 x 16 bf16
  alignas(128) uint8_t a2[kTcRows * 64 * 2];  // H1: 128 x 64 bf16
  alignas(128) uint8_t b1[64 * 16 * 2];       // W1^T: 64 x 16 bf16 (N x K)
  alignas(128) uint8_t b2[64 * 64 * 2];       // W2^T: 64 x 64 bf16
  float bias1[64], bias2[64], w3[64];
  float ypart[kTcRows];  // warpgroup 1's half of w3 . h2 per row
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  uint32_t failed;
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
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
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

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__global__ void __launch_bounds__(kTcThreads) k_mlp_infer_tc(const float* __restrict__ P, Norm nm,
                                                            const float* __restrict__ feat, uint32_t rows,
                                                            float* __restrict__ lambda, float* __restrict__ lam_sum,
                                                            const float4* __restrict__ xs, float4* __restrict__ xl,
                                                            uint32_t* err) {
  __shared__ TcSmem sm;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, row = tid & 127u, wg = tid >> 7;
  // weights into the canonical layouts, K padding of X set to zero once
  for (uint32_t q = tid; q < 64u * 16u; q += kTcThreads) {
    const uint32_t n = q / 16u, k = q % 16u;
    const float w = (k < (uint32_t)kIn) ? P[OFF_W1 + k * kH + n] : 0.0f;
    *reinterpret_cast<__nv_bfloat16*>(sm.b1 + canon(n, k, 16)) = __float2bfloat16_rn(w);
  }
  for (uint32_t q = tid; q < 64u * 64u; q += kTcThreads) {
    const uint32_t k = q / 64u, n = q % 64u;  // W2[k][n]
    *reinterpret_cast<__nv_bfloat16*>(sm.b2 + canon(n, k, 64)) = __float2bfloat16_rn(P[OFF_W2 + q]);
  }
  for (uint32_t q = tid; q < 64u; q += kTcThreads) {
    sm.bias1[q] = P[OFF_B1 + q];
    sm.bias2[q] = P[OFF_B2 + q];
    sm.w3[q] = P[OFF_W3 + q];
  }
  if (wg == 0) st_shared_v4(smem_u32(sm.a1 + canon(row, 8, 16)), 0u, 0u, 0u, 0u);
  const uint32_t mbar = smem_u32(&sm.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    sm.failed = 0u;
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
  const uint32_t tmem = sm.tmem;
  const uint32_t lane_base = (32u * (warp & 3u)) << 16;
  const float b3 = P[OFF_B3];
  const uint64_t a1d = smem_desc(smem_u32(sm.a1), 128, 256);
  const uint64_t b1d = smem_desc(smem_u32(sm.b1), 128, 256);
  uint32_t phase = 0;
  const uint32_t tiles = (rows + kTcRows - 1) / kTcRows;
  // the next tile's feature row, loaded one tile ahead (warpgroup 0)
  float4 nf0 = make_float4(0.f, 0.f, 0.f, 0.f), nf1 = nf0;
  auto fetch = [&](uint32_t tile) {
    const uint32_t rr = tile * kTcRows + row;
    if (wg == 0 && tile < tiles && rr < rows) {
      nf0 = reinterpret_cast<const float4*>(feat)[2 * (size_t)rr];
      nf1 = reinterpret_cast<const float4*>(feat)[2 * (size_t)rr + 1];
    }
  };
  fetch(blockIdx.x);
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    if (sm.failed) break;  // uniform: read after the previous tile's barriers
    const uint32_t r = tile * kTcRows + row;
    const bool valid = r < rows;
    // 1. X row: normalised features in bf16
    if (wg == 0) {
      float x[8];
      if (valid) {
        const float f[8] = {nf0.x, nf0.y, nf0.z, nf0.w, nf1.x, nf1.y, nf1.z, nf1.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = (f[k] - nm.mean[k]) * nm.inv_std[k];
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = 0.0f;
      }
      st_shared_v4(smem_u32(sm.a1 + canon(row, 0, 16)), pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]),
                   pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
    }
    fetch(tile + gridDim.x);  // in flight while this tile is computed
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    // 2. D1 = X W1
    if (tid == 0 && !sm.failed) {
      mma_f16(tmem, a1d, b1d, 0u);
      mma_commit(mbar);
    }
    if (!mbar_wait(mbar, phase)) atomicOr(&sm.failed, 1u);
    phase ^= 1u;
    fence_after_sync();
    // 3. H1 row = bf16(SiLU(D1 + b1)), this warpgroup's 32 columns
    {
      float v[32];
      tmem_ld32(tmem + lane_base + 32u * wg, v);
#pragma unroll
      for (int kb = 0; kb < 4; ++kb) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = 8 * kb + 2 * e, c = 32 * (int)wg + j;
          w[e] = pack_bf16(silu_f(v[j] + sm.bias1[c]), silu_f(v[j + 1] + sm.bias1[c + 1]));
        }
        st_shared_v4(smem_u32(sm.a2 + canon(row, 32 * wg + 8 * kb, 64)), w[0], w[1], w[2], w[3]);
      }
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    // 4. D2 = H1 W2 (four K = 16 steps)
    if (tid == 0 && !sm.failed) {
#pragma unroll
      for (uint32_t ks = 0; ks < 4; ++ks) {
        mma_f16(tmem + 64u, smem_desc(smem_u32(sm.a2) + 256u * ks, 128, 1024),
                smem_desc(smem_u32(sm.b2) + 256u * ks, 128, 1024), ks > 0 ? 1u : 0u);
      }
      mma_commit(mbar);
    }
    if (!mbar_wait(mbar, phase)) atomicOr(&sm.failed, 1u);
    phase ^= 1u;
    fence_after_sync();
    // 5. y = w3 . bf16(SiLU(D2 + b2)) + b3: each warpgroup its 32 columns,
    //    warpgroup 1 hands its half to warpgroup 0
    float y = wg == 0 ? b3 : 0.0f;
    {
      float v[32];
      tmem_ld32(tmem + lane_base + 64u + 32u * wg, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int c = 32 * (int)wg + j;
        y = fmaf(bf16_round(silu_f(v[j] + sm.bias2[c])), sm.w3[c], y);
      }
    }
    if (wg == 1) sm.ypart[row] = y;
    fence_before_sync();
    __syncthreads();
    if (wg == 0 && valid) {
      y += sm.ypart[row];
      const float l = y * nm.lam_scale;
      if (xl) {
        const float4 x = xs[r];
        xl[r] = make_float4(x.x, x.y, x.z, l);
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
  if (tid == 0 && sm.failed && err) atomicOr(err, PBF_DEVERR_MMA_TIMEOUT);
}

}  // namespace

// Dynamic shared memory requested on top of the static tile buffers so that
// at most four CTAs share an SM (4 x 128 TMEM columns = the SM's 512).
constexpr int kTcPadSmem = 24 * 1024;

cudaError_t launch_mlp_infer_tc(const float* d_params, const pbf_mlp& model, const float* d_feat, uint32_t rows,
                                float* d_lambda, float* d_lam_sum, cudaStream_t st, const float4* d_xs, float4* d_xl,
                                uint32_t* d_err) {
  if (rows == 0) return cudaSuccess;
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // static + dynamic shared memory above the 48 KB default needs the opt-in
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcPadSmem);
    // the whole L1/shared array as shared memory, so four CTAs fit
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    // four CTAs per SM: the TMEM limit (4 x 128 of 512 columns), which the
    // padded shared memory also enforces
    per_sm = 4;
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
  const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)sms * (uint32_t)per_sm);  // one resident wave
  k_mlp_infer_tc<<<grid, kTcThreads, kTcPadSmem, st>>>(d_params, nm, d_feat, rows, d_lambda, d_lam_sum, d_xs, d_xl,
                                                       d_err);
  return cudaGetLastError();
}

}  // namespace pbf
