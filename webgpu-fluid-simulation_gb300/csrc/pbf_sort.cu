// pbf_sort.cu — integer pipeline of the neighbour search: single-pass
// decoupled look-back exclusive scan, counting-sort scatter, stable
// within-cell order by particle id, the stable LSD radix sort of the
// stand-alone search, state gather, id-order export and the per-step
// metrics reduction.
//
// Reference counterparts (relative to the reference root):
//   ExclusiveScan.execute + scanShader.ts  src/simulator/neighbor/exclusiveScan.ts:134-166,
//                                          src/simulator/neighbor/scanShader.ts:16-107
//   ParticleInsert / CountingSort          src/simulator/neighbor/neighborShader.ts:24-60
// The reference's within-cell order is the order its atomicAdd calls happened
// to return; here it is defined as particle-id order (the sequential
// semantics), which the sort below reproduces exactly whatever order the
// warp-aggregated atomics ran in.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"
#include "pbf_device.cuh"
#include "pbf_kernels.h"

namespace pbf {

namespace {
constexpr uint32_t kFull = 0xffffffffu;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048 elements per tile
static_assert(kScanTile == (int)kScanTileElements, "scan tile size");
constexpr uint32_t kFlagAggregate = 1u, kFlagPrefix = 2u;
constexpr uint32_t kSpinLimit = 1u << 22;             // ~ tens of ms at worst, then give up

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pack(uint32_t flag, uint32_t value) {
  return ((unsigned long long)flag << 32) | value;
}

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* total, uint32_t* warp_sums) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t w = (lane < nw) ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) warp_sums[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  uint32_t warp_excl = (warp == 0) ? 0u : warp_sums[warp - 1];
  *total = warp_sums[(blockDim.x >> 5) - 1];
  return warp_excl + x - v;
}

// Single-pass scan: tiles take ids from a counter in launch order, publish
// their aggregate, look back over predecessors (bounded waits) and publish
// the inclusive prefix.  Status words pack (flag << 32 | value).
__global__ void __launch_bounds__(kScanThreads) k_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                       size_t n, unsigned long long* status, uint32_t* counter,
                                                       uint32_t* err) {
  __shared__ uint32_t s_items[kScanTile + kScanTile / 32];
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_prefix;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const size_t base = (size_t)tile * kScanTile;
  // striped coalesced load, padded transpose to blocked order
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int li = k * kScanThreads + threadIdx.x;
    size_t gi = base + li;
    s_items[li + (li >> 5)] = (gi < n) ? __ldg(in + gi) : 0u;
  }
  __syncthreads();
  uint32_t items[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int li = threadIdx.x * kScanItems + k;
    items[k] = s_items[li + (li >> 5)];
    sum += items[k];
  }
  uint32_t total;
  uint32_t texcl = block_exclusive(sum, &total, s_warp);
  // look-back
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    uint32_t prefix = 0;
    if (tile == 0) {
      if (lane == 0) st_release_u64(status + 0, pack(kFlagPrefix, total));
    } else {
      if (lane == 0) st_release_u64(status + tile, pack(kFlagAggregate, total));
      long pred = (long)tile - 1;
      bool done = false;
      while (!done) {
        long idx = pred - lane;
        unsigned long long w = pack(kFlagPrefix, 0);  // lanes past tile 0 read as an empty prefix
        uint32_t spins = 0;
        if (idx >= 0) {
          w = ld_acquire_u64(status + idx);
          while ((uint32_t)(w >> 32) == 0u) {
            if (++spins > kSpinLimit) {
              atomicOr(err, (uint32_t)PBF_DEVERR_SCAN_TIMEOUT);
              w = pack(kFlagPrefix, 0);
              break;
            }
            __nanosleep(32);
            w = ld_acquire_u64(status + idx);
          }
        }
        uint32_t flag = (uint32_t)(w >> 32), val = (uint32_t)w;
        uint32_t pmask = __ballot_sync(kFull, flag == kFlagPrefix);
        // lanes up to (and including) the nearest prefix contribute
        int stop = pmask ? (__ffs(pmask) - 1) : 31;
        uint32_t contrib = (lane <= stop) ? val : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(kFull, contrib, o);
        prefix += contrib;
        if (pmask) done = true;
        pred -= 32;
      }
      if (lane == 0) st_release_u64(status + tile, pack(kFlagPrefix, prefix + total));
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  uint32_t run = s_prefix + texcl;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int li = threadIdx.x * kScanItems + k;
    s_items[li + (li >> 5)] = run;
    run += items[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int li = k * kScanThreads + threadIdx.x;
    size_t gi = base + li;
    if (gi < n) out[gi] = s_items[li + (li >> 5)];
  }
}

// ---- counting-sort scatter (CountingSort, neighborShader.ts:49-60) -----------------
__global__ void __launch_bounds__(256) k_scatter(uint32_t n, const uint32_t* __restrict__ key,
                                                 const uint32_t* __restrict__ rank, const uint32_t* __restrict__ cell_start,
                                                 const uint32_t* __restrict__ ids, uint32_t* __restrict__ perm_raw,
                                                 uint32_t* __restrict__ id_raw) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  uint32_t k = key[s];
  uint32_t dst = __ldg(cell_start + k) + rank[s];
  perm_raw[dst] = s;
  id_raw[dst] = ids ? __ldg(ids + s) : s;
}

// ---- stable within-cell order ------------------------------------------------------
// One thread per sorted position q: the entry scattered there ranks itself
// by particle id among its cell's entries and moves to cell_start + rank.
// The work follows the particles (sum over cells of count^2), not the cell
// count, so empty cells cost nothing.  Cells above kRankMax entries go to
// the block radix path (the thread at the cell's first position lists it).
constexpr uint32_t kRankMax = 1024;

__global__ void __launch_bounds__(256) k_cellfix(uint32_t n, const uint32_t* __restrict__ key,
                                                 const uint32_t* __restrict__ cell_count,
                                                 const uint32_t* __restrict__ cell_start,
                                                 const uint32_t* __restrict__ perm_raw,
                                                 const uint32_t* __restrict__ id_raw, uint32_t* __restrict__ perm,
                                                 uint32_t* big_list, uint32_t* big_count) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const uint32_t s = perm_raw[q];
  const uint32_t c = __ldg(key + s);
  const uint32_t cnt = __ldg(cell_count + c);
  if (cnt == 1) {
    perm[q] = s;
    return;
  }
  const uint32_t st = __ldg(cell_start + c);
  if (cnt > kRankMax) {
    if (q == st) big_list[atomicAdd(big_count, 1u)] = c;
    return;
  }
  const uint32_t my = id_raw[q];
  uint32_t r = 0;
  for (uint32_t m = 0; m < cnt; ++m) r += (__ldg(id_raw + st + m) < my) ? 1u : 0u;
  perm[st + r] = s;
}

// Block LSD radix sort (8-bit digits) of one very full cell by particle id;
// stable because tiles are processed in order and ranks within a tile follow
// thread order.
constexpr int kRadixThreads = 256;
__global__ void __launch_bounds__(kRadixThreads) k_bigcell(const uint32_t* __restrict__ big_list,
                                                           const uint32_t* __restrict__ big_count,
                                                           const uint32_t* __restrict__ cell_count,
                                                           const uint32_t* __restrict__ cell_start,
                                                           uint32_t* __restrict__ perm_raw, uint32_t* __restrict__ id_raw,
                                                           uint32_t* __restrict__ perm, uint32_t* __restrict__ tmp_slot,
                                                           uint32_t* __restrict__ tmp_id, int passes) {
  __shared__ uint32_t s_base[256];
  __shared__ uint32_t s_wcount[kRadixThreads / 32][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t nb = *big_count;
  for (uint32_t bi = blockIdx.x; bi < nb; bi += gridDim.x) {
    const uint32_t c = big_list[bi];
    const uint32_t cnt = cell_count[c], st = cell_start[c];
    // ping-pong between the cell's own segments of (perm_raw, id_raw) and (tmp_slot, tmp_id);
    // the last pass writes the slots straight into perm.
    uint32_t* src_slot = perm_raw + st;
    uint32_t* src_id = id_raw + st;
    for (int pass = 0; pass < passes; ++pass) {
      const int shift = 8 * pass;
      const bool even = (pass & 1) == 0;
      uint32_t* dst_slot = (even ? tmp_slot : perm_raw) + st;
      uint32_t* dst_id = (even ? tmp_id : id_raw) + st;
      if (pass == passes - 1) dst_slot = perm + st;
      // histogram
      for (int d = tid; d < 256; d += kRadixThreads) s_base[d] = 0;
      __syncthreads();
      for (uint32_t e = tid; e < cnt; e += kRadixThreads) atomicAdd(&s_base[(src_id[e] >> shift) & 255u], 1u);
      __syncthreads();
      if (tid == 0) {
        uint32_t run = 0;
        for (int d = 0; d < 256; ++d) {
          uint32_t v = s_base[d];
          s_base[d] = run;
          run += v;
        }
      }
      __syncthreads();
      for (uint32_t t0 = 0; t0 < cnt; t0 += kRadixThreads) {
        for (int q = tid; q < (kRadixThreads / 32) * 256; q += kRadixThreads) (&s_wcount[0][0])[q] = 0;
        __syncthreads();
        uint32_t e = t0 + tid;
        bool valid = e < cnt;
        uint32_t d = valid ? ((src_id[e] >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(kFull, d);
        uint32_t lrank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lrank == 0) s_wcount[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
          uint32_t r = s_base[d] + lrank;
          for (int w = 0; w < warp; ++w) r += s_wcount[w][d];
          dst_slot[r] = src_slot[e];
          dst_id[r] = src_id[e];
        }
        __syncthreads();
        for (int dd = tid; dd < 256; dd += kRadixThreads) {
          uint32_t add = 0;
          for (int w = 0; w < kRadixThreads / 32; ++w) add += s_wcount[w][dd];
          s_base[dd] += add;
        }
        __syncthreads();
      }
      src_slot = dst_slot;
      src_id = dst_id;
      __syncthreads();
    }
  }
}

// ---- stable LSD radix sort by cell key of points in particle-id order ---------------
// The stand-alone search receives its points in id order, so a stable sort
// of the ids by cell key yields the order with every cell's particles in id
// order: no within-cell pass, and skewed cell occupancy costs nothing extra.
// Each pass over a digit is reduce-then-scan: every tile of 3072 records
// counts its digits (written digit-major, count[d * tiles + tile]); one
// exclusive scan of that matrix gives each (digit, tile) run its global
// place; then every tile ranks its records by digit in shared memory (stable
// in input order) and writes each digit's run there.  Reads and writes are
// coalesced, and no tile waits on another.
constexpr int kOsThreads = 256;
constexpr int kOsItems = 12;
constexpr int kOsTile = kOsThreads * kOsItems;  // 3072 records per tile
constexpr int kOsWarps = kOsThreads / 32;
constexpr int kOsMaxRadix = 256;

// Lanes of the warp holding the same digit (valid lanes only): one ballot per
// digit bit.
template <int kWidth>
__device__ __forceinline__ unsigned digit_peers(uint32_t d, bool valid) {
  unsigned peers = __ballot_sync(kFull, valid);
#pragma unroll
  for (int b = 0; b < kWidth; ++b) {
    const unsigned m = __ballot_sync(kFull, (d >> b) & 1u);
    peers &= ((d >> b) & 1u) ? m : ~m;
  }
  return peers;
}

// Cell key of every point (ParticleInsert).
__global__ void __launch_bounds__(256) k_cell_keys(GridParams g, const float4* __restrict__ pos, uint32_t n,
                                                   uint32_t* __restrict__ key) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const float4 x = __ldg(pos + s);
    const int cx = cell_axis(x.x, g.origin[0], g.inv_cell[0], g.dim[0]);
    const int cy = cell_axis(x.y, g.origin[1], g.inv_cell[1], g.dim[1]);
    const int cz = cell_axis(x.z, g.origin[2], g.inv_cell[2], g.dim[2]);
    key[s] = cell_key(cx, cy, cz, g);
  }
}

// Digit counts of one tile, digit-major (per-warp counters in shared memory,
// summed at the end).
template <int kWidth>
__global__ void __launch_bounds__(kOsThreads) k_tile_digits(uint32_t n, const uint32_t* __restrict__ kin,
                                                            uint32_t* __restrict__ count, uint32_t tiles, int shift) {
  constexpr uint32_t kRadix = 1u << kWidth, kMask = kRadix - 1u;
  __shared__ uint32_t s_cnt[kOsWarps][kRadix];
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  for (uint32_t d = tid; d < kOsWarps * kRadix; d += kOsThreads) (&s_cnt[0][0])[d] = 0u;
  const uint32_t t0 = blockIdx.x * (uint32_t)kOsTile;
  uint32_t d[kOsItems];
#pragma unroll
  for (int i = 0; i < kOsItems; ++i) {
    const uint32_t idx = t0 + (uint32_t)i * kOsThreads + tid;
    d[i] = idx < n ? (__ldg(kin + idx) >> shift) & kMask : kRadix;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kOsItems; ++i)
    if (d[i] < kRadix) atomicAdd(&s_cnt[warp][d[i]], 1u);
  __syncthreads();
  for (uint32_t dd = tid; dd < kRadix; dd += kOsThreads) {
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < kOsWarps; ++w) c += s_cnt[w][dd];
    count[(size_t)dd * tiles + blockIdx.x] = c;
  }
}

// One pass over the digit (key >> shift) & (2^kWidth - 1): place[d * tiles +
// tile] is where the tile's run of digit d starts.  vin == nullptr: the values
// are the input positions (particle ids).  cell_count (the last pass only):
// the written keys are in final order, so each run of equal keys a warp
// writes is added to its cell's count once.
template <int kWidth>
__global__ void __launch_bounds__(kOsThreads, 4) k_radix_pass(uint32_t n, const uint32_t* __restrict__ kin,
                                                              const uint32_t* __restrict__ vin,
                                                              uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                              const uint32_t* __restrict__ place, uint32_t tiles,
                                                              int shift, uint32_t* cell_count) {
  constexpr uint32_t kRadix = 1u << kWidth, kMask = kRadix - 1u;
  __shared__ uint32_t s_key[kOsTile];
  __shared__ uint32_t s_val[kOsTile];
  __shared__ uint32_t s_wcnt[kOsWarps][kRadix];  // per-warp digit counts, then offsets over warps
  __shared__ uint32_t s_loc[kRadix];             // digit counts of the tile, then their exclusive scan
  __shared__ uint32_t s_glob[kRadix];            // global place of the tile's first record of each digit
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t tile = blockIdx.x;
  for (uint32_t i = tid; i < kOsWarps * kRadix; i += kOsThreads) (&s_wcnt[0][0])[i] = 0u;
  for (uint32_t d = tid; d < kRadix; d += kOsThreads) s_glob[d] = __ldg(place + (size_t)d * tiles + tile);
  const uint32_t t0 = tile * (uint32_t)kOsTile;
  // warp w holds records t0 + 512 w .. + 511; round i is records 32 i .. 32 i + 31 of it
  const uint32_t w0 = t0 + warp * (32u * kOsItems) + lane;
  uint32_t k[kOsItems], v[kOsItems], r[kOsItems];
#pragma unroll
  for (int i = 0; i < kOsItems; ++i) {
    const uint32_t idx = w0 + 32u * i;
    const bool valid = idx < n;
    k[i] = valid ? __ldg(kin + idx) : 0xffffffffu;
    v[i] = valid ? (vin ? __ldg(vin + idx) : idx) : 0u;
  }
  __syncthreads();
  // stable ranks within the warp, round by round in input order: the lowest
  // lane of each digit group adds the group to the warp's counter and passes
  // the old count on (shared-memory atomics keep the rounds in order)
  uint32_t* wc = s_wcnt[warp];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int i = 0; i < kOsItems; ++i) {
    const bool valid = w0 + 32u * i < n;
    const uint32_t d = (k[i] >> shift) & kMask;
    const unsigned peers = digit_peers<kWidth>(d, valid);
    const int leader = __ffs(peers) - 1;
    uint32_t before = 0u;
    if (valid && (int)lane == leader) before = atomicAdd(wc + d, (uint32_t)__popc(peers));
    before = __shfl_sync(kFull, before, leader & 31);
    r[i] = before + (uint32_t)__popc(peers & lt);
  }
  __syncthreads();
  // per digit: offsets over the warps and the tile's count
  if (tid < kRadix) {
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kOsWarps; ++w) {
      const uint32_t c = s_wcnt[w][tid];
      s_wcnt[w][tid] = cnt;
      cnt += c;
    }
    s_loc[tid] = cnt;
  }
  __syncthreads();
  // exclusive scan of the tile's digit counts (warp 0)
  if (warp == 0) {
    constexpr uint32_t kPer = (kRadix + 31u) / 32u;
    uint32_t loc[kPer];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < kPer; ++j) {
      const uint32_t d = lane * kPer + j;
      loc[j] = d < kRadix ? s_loc[d] : 0u;
      sum += loc[j];
    }
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if ((int)lane >= o) x += y;
    }
    uint32_t run = x - sum;
#pragma unroll
    for (uint32_t j = 0; j < kPer; ++j) {
      const uint32_t d = lane * kPer + j;
      if (d < kRadix) s_loc[d] = run;
      run += loc[j];
    }
  }
  __syncthreads();
  // records to their tile-sorted place in shared memory
#pragma unroll
  for (int i = 0; i < kOsItems; ++i) {
    if (w0 + 32u * i < n) {
      const uint32_t d = (k[i] >> shift) & kMask;
      const uint32_t lp = s_loc[d] + s_wcnt[warp][d] + r[i];
      s_key[lp] = k[i];
      s_val[lp] = v[i];
    }
  }
  __syncthreads();
  // each digit's run to its global place: consecutive j, consecutive addresses
  const uint32_t in_tile = (n - t0) < (uint32_t)kOsTile ? (n - t0) : (uint32_t)kOsTile;
#pragma unroll 4
  for (uint32_t j0 = 0; j0 < in_tile; j0 += kOsThreads) {
    const uint32_t j = j0 + tid;
    const bool valid = j < in_tile;
    const uint32_t kk = valid ? s_key[j] : 0xffffffffu;
    if (valid) {
      const uint32_t d = (kk >> shift) & kMask;
      const uint32_t p = s_glob[d] + (j - s_loc[d]);
      if (p < n) {
        kout[p] = kk;
        vout[p] = s_val[j];
      }
    }
    if (cell_count) {  // a warp's 32 consecutive records: one add per run of equal keys
      const uint32_t up = __shfl_up_sync(kFull, kk, 1);
      const bool start = valid && (lane == 0u || up != kk);
      const unsigned starts = __ballot_sync(kFull, start);
      const unsigned valid_mask = __ballot_sync(kFull, valid);
      if (start) {
        const unsigned later = starts & ~((2u << lane) - 1u);
        const uint32_t end = later ? (uint32_t)(__ffs(later) - 1) : (uint32_t)(32 - __clz(valid_mask));
        atomicAdd(cell_count + kk, end - lane);
      }
    }
  }
}

// particleSortIndex: the place of each particle within its cell, by particle
// id.  Four sorted positions a thread (vector loads keep more reads in flight
// ahead of the scattered stores).
__global__ void __launch_bounds__(256) k_rank_sorted(uint32_t n, const uint32_t* __restrict__ skey,
                                                     const uint32_t* __restrict__ order,
                                                     const uint32_t* __restrict__ cell_start,
                                                     uint32_t* __restrict__ rank_out) {
  const uint32_t q0 = 4u * (blockIdx.x * blockDim.x + threadIdx.x);
  if (q0 >= n) return;
  if (q0 + 4u <= n) {
    const uint4 k = __ldg(reinterpret_cast<const uint4*>(skey + q0));
    const uint4 o = __ldg(reinterpret_cast<const uint4*>(order + q0));
    const uint32_t s0 = __ldg(cell_start + k.x), s1 = __ldg(cell_start + k.y), s2 = __ldg(cell_start + k.z),
                   s3 = __ldg(cell_start + k.w);
    rank_out[o.x] = q0 - s0;
    rank_out[o.y] = q0 + 1u - s1;
    rank_out[o.z] = q0 + 2u - s2;
    rank_out[o.w] = q0 + 3u - s3;
  } else {
    for (uint32_t q = q0; q < n; ++q) rank_out[order[q]] = q - __ldg(cell_start + skey[q]);
  }
}

// ---- gather of the particle state into the new order -------------------------------
__global__ void __launch_bounds__(256) k_gather(uint32_t n, const uint32_t* __restrict__ perm,
                                                const float4* __restrict__ pos_in, const float4* __restrict__ xs_in,
                                                const uint32_t* __restrict__ id_in, float4* __restrict__ pos_out,
                                                float4* __restrict__ xs_out, uint32_t* __restrict__ id_out,
                                                const float* __restrict__ f_in, float* __restrict__ f_out) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t o = perm[t];
  pos_out[t] = __ldg(pos_in + o);
  xs_out[t] = __ldg(xs_in + o);
  id_out[t] = id_in ? __ldg(id_in + o) : o;  // no id array: the input order is the id order
  if (f_in) f_out[t] = __ldg(f_in + o);
}

__global__ void __launch_bounds__(256) k_gather_cb(uint32_t n, const uint32_t* __restrict__ perm,
                                                   const float4* __restrict__ pos_in,
                                                   const float4* __restrict__ xs_in,
                                                   const uint32_t* __restrict__ id_in,
                                                   const uint32_t* __restrict__ key_in, float4* __restrict__ pos_out,
                                                   float4* __restrict__ xs_out, uint32_t* __restrict__ id_out,
                                                   uint32_t* __restrict__ skey_out, float4* __restrict__ xs0_out,
                                                   const float* __restrict__ f_in, float* __restrict__ f_out) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t o = perm[t];
  pos_out[t] = __ldg(pos_in + o);
  const float4 x = __ldg(xs_in + o);
  xs_out[t] = x;
  xs0_out[t] = x;
  skey_out[t] = __ldg(key_in + o);
  id_out[t] = id_in ? __ldg(id_in + o) : o;
  if (f_in) f_out[t] = __ldg(f_in + o);
}

__global__ void k_scatter_f4(uint32_t n, const uint32_t* __restrict__ id, const float4* __restrict__ src,
                             float4* __restrict__ dst) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  dst[id[t]] = src[t];
}
__global__ void k_scatter_w(uint32_t n, const uint32_t* __restrict__ id, const float4* __restrict__ src,
                            float* __restrict__ dst) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  dst[id[t]] = src[t].w;
}
__global__ void k_scatter_u32(uint32_t n, const uint32_t* __restrict__ id, const uint32_t* __restrict__ src,
                              uint32_t* __restrict__ dst) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  dst[id[t]] = src[t];
}
__global__ void k_list_to_ids(uint32_t total, const uint32_t* __restrict__ list, const uint32_t* __restrict__ id,
                              uint32_t* __restrict__ out) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= total) return;
  out[q] = id[list[q]];
}
__global__ void k_copy_runs(uint32_t n, const uint32_t* __restrict__ slot_off, const uint32_t* __restrict__ id_off,
                            const uint32_t* __restrict__ ids, const uint32_t* __restrict__ src, uint32_t* __restrict__ dst) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t b = slot_off[t], e = slot_off[t + 1], o = id_off[ids[t]];
  for (uint32_t q = b; q < e; ++q) dst[o + (q - b)] = src[q];
}
// ---- metrics --------------------------------------------------------------------------
__device__ __forceinline__ void atomic_max_pos_float(float* addr, float v) {
  // v >= 0: the int ordering of non-negative floats matches their value ordering
  atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}
__global__ void __launch_bounds__(256) k_metrics(SimParams p, FieldParams f, const float* __restrict__ sdf,
                                                 const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                 const uint32_t* __restrict__ nbr_count, uint32_t n, float* accum_f,
                                                 double* accum_d, uint32_t* accum_u) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  float comp = 0.f, aerr = 0.f;
  double ke = 0.0, serr = 0.0, scomp = 0.0;
  uint32_t bad = 0, pen = 0, nb = 0;
  if (t < n) {
    if (nbr_count) nb = nbr_count[t];
    float4 x = pos[t];
    float4 v = vel[t];
    bool fin = isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
    if (!fin) {
      bad = 1;
    } else {
      float e = x.w / p.rho0 - 1.0f;
      comp = fmaxf(0.0f, e);
      aerr = fabsf(e);
      serr = aerr;
      scomp = comp;
      ke = 0.5 * (double)p.m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
      if (f.loaded && sdf) {
        CellLoc L = field_locate(f, mk(x.x, x.y, x.z));
        uint32_t idx[32];
        cell_nodes(f, L.i, L.j, L.k, false, idx);
        float N[32];
        f3 dN[32];
        float val[32];
        shape32(L.s, N, dN);
        for (int q = 0; q < 32; ++q) val[q] = sdf[idx[q]];
        if (sum32(N, val) < 0.0f) pen = 1;
      }
    }
  }
  // warp reduce then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    comp = fmaxf(comp, __shfl_xor_sync(kFull, comp, o));
    aerr = fmaxf(aerr, __shfl_xor_sync(kFull, aerr, o));
    ke += __shfl_xor_sync(kFull, ke, o);
    serr += __shfl_xor_sync(kFull, serr, o);
    scomp += __shfl_xor_sync(kFull, scomp, o);
    bad += __shfl_xor_sync(kFull, bad, o);
    pen += __shfl_xor_sync(kFull, pen, o);
    nb += __shfl_xor_sync(kFull, nb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos_float(accum_f + 0, comp);
    atomic_max_pos_float(accum_f + 1, aerr);
    atomicAdd(accum_d + 0, serr);
    atomicAdd(accum_d + 1, ke);
    atomicAdd(accum_d + 2, scomp);
    atomicAdd(accum_u + 0, bad);
    atomicAdd(accum_u + 1, pen);
    atomicAdd(accum_u + 2, nb);
  }
}

inline unsigned blocks_for(size_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

RadixPlan radix_plan(uint32_t cells, size_t n) {
  RadixPlan r;
  uint32_t bits = 1;
  while (bits < 32 && (1ull << bits) < (uint64_t)cells) ++bits;
  r.passes = (int)((bits + 7) / 8);
  r.width = (int)((bits + (uint32_t)r.passes - 1) / (uint32_t)r.passes);
  r.tiles = (n + kOsTile - 1) / kOsTile;
  return r;
}

namespace {
size_t round256(size_t b) { return (b + 255) / 256 * 256; }
}  // namespace

// Scratch: the digit-major count matrix, its scan and the scan's own scratch.
size_t radix_scratch_bytes(size_t n) {
  size_t tiles = (n + kOsTile - 1) / kOsTile;
  if (tiles == 0) tiles = 1;
  const size_t m = tiles * kOsMaxRadix;
  return 2 * round256(m * sizeof(uint32_t)) + scan_scratch_bytes(m);
}

cudaError_t launch_radix_sort_idorder(GridParams g, const float4* pos, uint32_t n, uint32_t* keys, uint32_t* skeys,
                                      uint32_t* order, uint32_t* const tmp_k[2], uint32_t* const tmp_v[2],
                                      void* scratch, uint32_t* err, cudaStream_t st, cudaEvent_t after_keys,
                                      uint32_t* cell_count) {
  cudaError_t e = cudaSuccess;
  if (n == 0) return after_keys ? cudaEventRecord(after_keys, st) : cudaSuccess;
  const RadixPlan plan = radix_plan(g.cells, n);
  const uint32_t radix = 1u << plan.width;
  const size_t m = plan.tiles * radix;
  char* sc = reinterpret_cast<char*>(scratch);
  uint32_t* count = reinterpret_cast<uint32_t*>(sc);
  uint32_t* place = reinterpret_cast<uint32_t*>(sc + round256(plan.tiles * kOsMaxRadix * sizeof(uint32_t)));
  void* scan_scr = sc + 2 * round256(plan.tiles * kOsMaxRadix * sizeof(uint32_t));
  unsigned blocks = (unsigned)((n + 255) / 256);
  if (blocks > 152u * 8u) blocks = 152u * 8u;
  k_cell_keys<<<blocks, 256, 0, st>>>(g, pos, n, keys);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (after_keys && (e = cudaEventRecord(after_keys, st)) != cudaSuccess) return e;
  for (int p = 0; p < plan.passes; ++p) {
    const bool last = p == plan.passes - 1;
    const uint32_t* kin = p == 0 ? keys : tmp_k[(p - 1) & 1];
    const uint32_t* vin = p == 0 ? nullptr : tmp_v[(p - 1) & 1];
    uint32_t* kout = last ? skeys : tmp_k[p & 1];
    uint32_t* vout = last ? order : tmp_v[p & 1];
    const int shift = p * plan.width;
    const unsigned grid = (unsigned)plan.tiles;
    const uint32_t tl = (uint32_t)plan.tiles;
    switch (plan.width) {
#define PBF_RADIX_WIDTH(W)                                                              \
  case W:                                                                               \
    k_tile_digits<W><<<grid, kOsThreads, 0, st>>>(n, kin, count, tl, shift);            \
    if ((e = cudaGetLastError()) != cudaSuccess) return e;                              \
    if ((e = launch_exclusive_scan(count, place, m, scan_scr, err, st)) != cudaSuccess) \
      return e;                                                                         \
    k_radix_pass<W><<<grid, kOsThreads, 0, st>>>(n, kin, vin, kout, vout, place, tl, shift, last ? cell_count : nullptr); \
    break;
      PBF_RADIX_WIDTH(1)
      PBF_RADIX_WIDTH(2)
      PBF_RADIX_WIDTH(3)
      PBF_RADIX_WIDTH(4)
      PBF_RADIX_WIDTH(5)
      PBF_RADIX_WIDTH(6)
      PBF_RADIX_WIDTH(7)
      PBF_RADIX_WIDTH(8)
#undef PBF_RADIX_WIDTH
      default:
        return cudaErrorInvalidValue;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_cell_offsets(uint32_t cells, const uint32_t* cell_count, uint32_t* cell_start, void* scan_scratch,
                                uint32_t* err, cudaStream_t st) {
  return launch_exclusive_scan(cell_count, cell_start, (size_t)cells + 1, scan_scratch, err, st);
}

cudaError_t launch_rank_sorted(uint32_t n, const uint32_t* skeys, const uint32_t* order, const uint32_t* cell_start,
                               uint32_t* rank_out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint32_t threads = (n + 3u) / 4u;
  k_rank_sorted<<<(threads + 255u) / 256u, 256, 0, st>>>(n, skeys, order, cell_start, rank_out);
  return cudaGetLastError();
}

size_t scan_scratch_bytes(size_t n) {
  size_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 0) tiles = 1;
  return 256 + tiles * sizeof(unsigned long long);
}

cudaError_t launch_exclusive_scan(const uint32_t* in, uint32_t* out, size_t n, void* scratch, uint32_t* err,
                                  cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  size_t tiles = (n + kScanTile - 1) / kScanTile;
  cudaError_t e = cudaMemsetAsync(scratch, 0, scan_scratch_bytes(n), st);
  if (e != cudaSuccess) return e;
  uint32_t* counter = reinterpret_cast<uint32_t*>(scratch);
  unsigned long long* status = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(scratch) + 256);
  k_scan<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, status, counter, err);
  return cudaGetLastError();
}

// Self-test of the look-back's bounded wait: one CTA of a two-tile scan,
// started as tile 1 (the tile counter is preset), so tile 0's status word,
// which nothing writes, is what it waits for.  The wait gives up after
// kSpinLimit polls, flags PBF_DEVERR_SCAN_TIMEOUT in *err and the kernel
// completes.  Every access stays inside the two tiles' buffers.
cudaError_t launch_scan_timeout_selftest(uint32_t* err, cudaStream_t st) {
  const size_t n = 2 * (size_t)kScanTile;
  uint32_t *in = nullptr, *out = nullptr;
  void* scratch = nullptr;
  cudaError_t e = cudaMallocAsync(&in, n * sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&out, n * sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&scratch, scan_scratch_bytes(n), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(in, 0, n * sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, scan_scratch_bytes(n), st);
  const uint32_t one = 1u;
  uint32_t* counter = reinterpret_cast<uint32_t*>(scratch);
  if (e == cudaSuccess) e = cudaMemcpyAsync(counter, &one, sizeof(one), cudaMemcpyHostToDevice, st);
  unsigned long long* status = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(scratch) + 256);
  if (e == cudaSuccess) {
    k_scan<<<1, kScanThreads, 0, st>>>(in, out, n, status, counter, err);
    e = cudaGetLastError();
  }
  // the host value copied above must outlive the copy
  cudaError_t e2 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2;
  cudaFreeAsync(in, st);
  cudaFreeAsync(out, st);
  cudaFreeAsync(scratch, st);
  e2 = cudaStreamSynchronize(st);
  return e == cudaSuccess ? e2 : e;
}

cudaError_t launch_sort_by_cell(GridParams g, uint32_t n, const uint32_t* ids, SortBuffers& b, uint32_t id_bits,
                                cudaStream_t st) {
  cudaError_t e = launch_exclusive_scan(b.cell_count, b.cell_start, (size_t)g.cells + 1, b.scan_scratch, b.err, st);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  k_scatter<<<blocks_for(n, 256), 256, 0, st>>>(n, b.key, b.rank, b.cell_start, ids, b.perm_raw, b.id_raw);
  e = cudaMemsetAsync(b.big_count, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_cellfix<<<blocks_for(n, 256), 256, 0, st>>>(n, b.key, b.cell_count, b.cell_start, b.perm_raw, b.id_raw, b.perm,
                                                 b.big_list, b.big_count);
  int passes = (int)((id_bits + 7) / 8);
  if (passes < 1) passes = 1;
  k_bigcell<<<152, kRadixThreads, 0, st>>>(b.big_list, b.big_count, b.cell_count, b.cell_start, b.perm_raw, b.id_raw,
                                           b.perm, b.tmp_a, b.tmp_b, passes);
  return cudaGetLastError();
}

cudaError_t launch_gather_state(uint32_t n, const uint32_t* perm, const float4* pos_in, const float4* xs_in,
                                const uint32_t* id_in, float4* pos_out, float4* xs_out, uint32_t* id_out,
                                cudaStream_t st, const float* f_in, float* f_out) {
  if (n == 0) return cudaSuccess;
  k_gather<<<blocks_for(n, 256), 256, 0, st>>>(n, perm, pos_in, xs_in, id_in, pos_out, xs_out, id_out, f_in, f_out);
  return cudaGetLastError();
}

cudaError_t launch_gather_state_cb(uint32_t n, const uint32_t* perm, const float4* pos_in, const float4* xs_in,
                                   const uint32_t* id_in, const uint32_t* key_in, float4* pos_out, float4* xs_out,
                                   uint32_t* id_out, uint32_t* skey_out, float4* xs0_out, cudaStream_t st,
                                   const float* f_in, float* f_out) {
  if (n == 0) return cudaSuccess;
  k_gather_cb<<<blocks_for(n, 256), 256, 0, st>>>(n, perm, pos_in, xs_in, id_in, key_in, pos_out, xs_out, id_out,
                                                  skey_out, xs0_out, f_in, f_out);
  return cudaGetLastError();
}

cudaError_t launch_scatter_by_id(uint32_t n, const uint32_t* id, const float4* src, float4* dst, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_scatter_f4<<<blocks_for(n, 256), 256, 0, st>>>(n, id, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_scatter_w_by_id(uint32_t n, const uint32_t* id, const float4* src, float* dst, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_scatter_w<<<blocks_for(n, 256), 256, 0, st>>>(n, id, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_scatter_by_id_u32(uint32_t n, const uint32_t* id, const uint32_t* src, uint32_t* dst,
                                     cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_scatter_u32<<<blocks_for(n, 256), 256, 0, st>>>(n, id, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_list_to_ids(uint32_t total, const uint32_t* list, const uint32_t* id, uint32_t* out,
                               cudaStream_t st) {
  if (total == 0) return cudaSuccess;
  k_list_to_ids<<<blocks_for(total, 256), 256, 0, st>>>(total, list, id, out);
  return cudaGetLastError();
}
cudaError_t launch_copy_runs(uint32_t n, const uint32_t* slot_off, const uint32_t* id_off, const uint32_t* ids,
                             const uint32_t* src, uint32_t* dst, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_copy_runs<<<blocks_for(n, 256), 256, 0, st>>>(n, slot_off, id_off, ids, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_metrics(SimParams p, FieldParams f, const float* sdf, const float4* pos, const float4* vel,
                           const uint32_t* nbr_count, uint32_t n, float* accum_f, double* accum_d, uint32_t* accum_u,
                           cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_metrics<<<blocks_for(n, 256), 256, 0, st>>>(p, f, sdf, pos, vel, nbr_count, n, accum_f, accum_d, accum_u);
  return cudaGetLastError();
}

}  // namespace pbf
