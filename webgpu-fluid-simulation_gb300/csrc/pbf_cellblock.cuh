// pbf_cellblock.cuh — the neighbour passes as cell-block kernels.
//
// Included by pbf_passes.cuh inside namespace pbf::PBF_NS (compiled in both
// the exact and the fast unit).  Same passes as the list kernels above —
// LambdaCalculation, ConstrainSolve + Apply, AttributeUpdate,
// VorticityConfinement, XSPH (pressureConstrain.ts:31-179,
// attributeUpdate.ts:25-59, vorticityConfinement.ts:25-66, XSPH.ts:31-92) —
// with a different way of reaching the neighbours:
//
//  - One CTA takes a tile of kCbT consecutive slots.  Slots are sorted by
//    cell key and keys are z-fastest, so the tile is one or a few column
//    segments: runs of slots in the same (x, y) cell column, each over a
//    range of z cells.
//  - For every segment, the 3 x 3 neighbouring columns' slot runs over the
//    segment's z range widened by the search reach are staged into shared
//    memory: one 1-D bulk copy (cp.async.bulk, global -> shared, completion
//    counted on one mbarrier) per run and field.  The tile's 27-cell halo
//    then sits in shared memory: no neighbour list is read from HBM.
//  - Each slot walks its own 9 windows (its neighbourhood's runs) inside the
//    staged runs, in key order and then slot order — the reference's
//    neighbour order (neighborShader.ts:121-149 visits the 27 cells x, y, z
//    from -1 to 1 and each cell in sorted order) — and keeps the neighbours
//    found at search time (the predicted positions x*_0, as the reference's
//    lists do):
//      kMemMask: a 32-bit mask per window written by the cell-block build
//                (bit k: the k-th candidate of the window is a neighbour;
//                candidates past the 32nd are tested against x*_0 from
//                global memory, flagged per window);
//      kMemTest: no neighbour structure at all: every candidate's staged
//                x*_0 is tested, |x*_0,i - x*_0,j|^2 <= h^2, as the search
//                does.
//    Both give the list's neighbour set in the list's order, and the sums go
//    through the same per-pass add() as the list walks, so exact mode stays
//    bit-identical to the CPU restatement.
//  - A tile whose segments or staged records exceed the shared-memory plan
//    (more than kCbMaxSeg columns, or more records than the capacity) walks
//    the same windows from global memory instead: same order, same results.
#pragma once

namespace cbk {
constexpr int kT = 128;                    // slots per tile = threads per CTA
constexpr int kMaxSeg = 8;                 // column segments per staged tile
constexpr int kMaxRuns = 9 * kMaxSeg;      // 3 x 3 runs per segment
constexpr uint32_t kPolls = 1u << 22;      // bounded mbarrier wait
}  // namespace cbk

enum { kMemMask = 0, kMemTest = 1 };

struct CbShared {
  unsigned long long bar;
  int seg_cx[cbk::kMaxSeg], seg_cy[cbk::kMaxSeg], seg_zlo[cbk::kMaxSeg], seg_zhi[cbk::kMaxSeg];
  uint32_t run_slot0[cbk::kMaxRuns];
  uint32_t run_off[cbk::kMaxRuns + 1];
  int col[cbk::kT];
  int wcnt[cbk::kT / 32];
  uint32_t wsum[cbk::kT / 32];
};

// The slot a thread owns in its tile.
struct CbSlot {
  uint32_t t;
  bool valid;
  int seg, cx, cy, cz;
};

__device__ __forceinline__ uint32_t cb_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cb_mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cb_smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void cb_mbar_expect(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(cb_smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared; both addresses 16-byte aligned, bytes a
// multiple of 16 (whole float4 records).
__device__ __forceinline__ void cb_bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   cb_smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(cb_smem_u32(bar))
               : "memory");
}
// Bounded wait for phase `phase` of the mbarrier; false when it gave up.
__device__ __forceinline__ bool cb_mbar_wait(unsigned long long* bar, uint32_t phase) {
  const uint32_t a = cb_smem_u32(bar);
  for (uint32_t i = 0; i < cbk::kPolls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
    if (i > 16) __nanosleep(32);
  }
  return false;
}

__device__ __forceinline__ void decode_key(const GridParams& g, uint32_t key, int& cx, int& cy, int& cz) {
  const uint32_t k = key - g.key_base;
  const uint32_t dz = (uint32_t)g.dim[2], dy = (uint32_t)g.dim[1];
  const uint32_t col = k / dz;
  cz = (int)(k - col * dz);
  cx = (int)(col / dy);
  cy = (int)(col - (uint32_t)cx * dy);
}

// Tile set-up: each thread's slot and cell, the tile's column segments, the
// 9 staged runs per segment and their bulk copies into `rec` (kF fields of
// A.cap records each).  Returns whether the halo was staged (uniform over
// the CTA); when it was not, the tile walks global memory.  Every thread of
// the CTA calls it.
template <int kF>
__device__ __forceinline__ bool cb_stage(CbShared& S, float4* rec, const float4* const* src, const CbArgs& A,
                                         CbSlot& me) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const GridParams& g = A.g;
  me.t = blockIdx.x * cbk::kT + tid;
  me.valid = me.t < A.n;
  me.cx = me.cy = me.cz = 0;
  int col = -1;
  if (me.valid) {
    decode_key(g, __ldg(A.skey + me.t), me.cx, me.cy, me.cz);
    col = me.cx * g.dim[1] + me.cy;
  }
  S.col[tid] = col;
  __syncthreads();
  const int prev = tid ? S.col[tid - 1] : -1;
  const int next = tid + 1 < cbk::kT ? S.col[tid + 1] : -1;
  const bool start = me.valid && col != prev;
  const bool last = me.valid && col != next;
  const unsigned bal = __ballot_sync(0xffffffffu, start);
  if (lane == 0) S.wcnt[w] = __popc(bal);
  __syncthreads();
  int before = 0, nseg = 0;
#pragma unroll
  for (int k = 0; k < cbk::kT / 32; ++k) {
    const int c = S.wcnt[k];
    before += (k < w) ? c : 0;
    nseg += c;
  }
  me.seg = before + __popc(bal & (0xffffffffu >> (31 - lane))) - 1;
  if (nseg == 0 || nseg > cbk::kMaxSeg) return false;
  if (start) {
    S.seg_cx[me.seg] = me.cx;
    S.seg_cy[me.seg] = me.cy;
    S.seg_zlo[me.seg] = me.cz;
  }
  if (last) S.seg_zhi[me.seg] = me.cz;
  __syncthreads();
  const int nruns = 9 * nseg;
  uint32_t len = 0;
  if (tid < nruns) {
    const int sg = tid / 9, q = tid - 9 * sg;
    const int x = S.seg_cx[sg] + q / 3 - 1, y = S.seg_cy[sg] + q % 3 - 1;
    uint32_t b = 0;
    if (x >= 0 && y >= 0 && x < g.dim[0] && y < g.dim[1]) {
      const int zl = max(S.seg_zlo[sg] - g.reach_z, 0), zh = min(S.seg_zhi[sg] + g.reach_z, g.dim[2] - 1);
      b = __ldg(A.cell_start + cell_key(x, y, zl, g));
      len = __ldg(A.cell_start + cell_key(x, y, zh, g) + 1) - b;
    }
    S.run_slot0[tid] = b;
  }
  // exclusive scan of the run lengths (nruns <= 72 < kT)
  uint32_t incl = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) S.wsum[w] = incl;
  __syncthreads();
  uint32_t base = 0;
#pragma unroll
  for (int k = 0; k < cbk::kT / 32; ++k) base += (k < w) ? S.wsum[k] : 0u;
  if (tid < nruns) S.run_off[tid] = base + incl - len;
  if (tid == nruns - 1) S.run_off[nruns] = base + incl;
  if (tid == 0) cb_mbar_init(&S.bar);
  __syncthreads();
  const uint32_t total = S.run_off[nruns];
  if (total > A.cap) return false;
  if (tid == 0) cb_mbar_expect(&S.bar, total * 16u * (uint32_t)kF);
  __syncthreads();
  if (tid < nruns && len) {
#pragma unroll
    for (int f = 0; f < kF; ++f)
      cb_bulk_g2s(rec + (size_t)f * A.cap + S.run_off[tid], src[f] + S.run_slot0[tid], len * 16u, &S.bar);
  }
  const bool done = cb_mbar_wait(&S.bar, 0);
  if (__syncthreads_or(!done)) {
    // the copies did not complete in time: report, give the copies in flight
    // a second bounded wait before the shared memory is left, and walk
    // global memory instead
    if (tid == 0) atomicOr(A.err, PBF_DEVERR_STAGE_TIMEOUT);
    cb_mbar_wait(&S.bar, 0);
    __syncthreads();
    return false;
  }
  return true;
}

// Global loads of the walk: read-only path, or L2-coherent (kC) for data a
// kernel rewrites between grid-wide barriers (the fallback solve).
template <bool kC>
__device__ __forceinline__ float4 cb_ldg(const float4* p) {
  if constexpr (kC) return __ldcg(p);
  return __ldg(p);
}

// The pass fields of one neighbour.
template <int kP>
struct CbRec {
  float4 v[kP];
};

// Visits slot me.t's neighbours in the reference order and calls
// fn(const CbRec<kP>&) with the kP pass fields of each (field 0 of the
// staged records is x*_0 when membership is tested).  Returns the neighbour
// count.  The next window's bounds (and mask) are loaded while the current
// one is walked; inside a window the neighbours go in batches of four —
// four record loads in flight, then four add()s — as the list walk does.
template <bool kStaged, int kMemb, int kP, bool kC, class Fn>
__device__ __forceinline__ uint32_t cb_walk(const SimParams& p, const CbArgs& A, const CbShared* S, const float4* rec,
                                            const float4* const* src, const CbSlot& me, Fn&& fn) {
  constexpr int kOff = kMemb == kMemTest ? 1 : 0;
  const GridParams& g = A.g;
  uint32_t ovf = 0;
  if constexpr (kMemb == kMemMask) ovf = __ldg(A.ovf + me.t);
  f3 x0i = mk(0.f, 0.f, 0.f);
  if (kMemb == kMemTest || ovf) x0i = xyz(cb_ldg<kC>(A.xs0 + me.t));
  auto window = [&](int q, Run& r, uint32_t& m) {
    r = run_of(g, A.cell_start, me.cx, me.cy, me.cz, q / 3 - 1, q % 3 - 1);
    m = 0u;
    if constexpr (kMemb == kMemMask) m = (r.b != r.e) ? __ldg(A.mask + (size_t)q * A.n + me.t) : 0u;
  };
  auto load = [&](uint32_t j, int base) {
    CbRec<kP> r;
#pragma unroll
    for (int f = 0; f < kP; ++f) {
      if constexpr (kStaged)
        r.v[f] = rec[(size_t)(f + kOff) * A.cap + (uint32_t)((int)j + base)];
      else
        r.v[f] = cb_ldg<kC>(src[f + kOff] + j);
    }
    return r;
  };
  auto x0_of = [&](uint32_t j, int base) -> f3 {
    if constexpr (kStaged && kMemb == kMemTest) return xyz(rec[(uint32_t)((int)j + base)]);
    return xyz(cb_ldg<kC>(A.xs0 + j));
  };
  uint32_t cnt = 0;
  Run r;
  uint32_t m;
  window(0, r, m);
#pragma unroll 1
  for (int q = 0; q < 9; ++q) {
    Run rn{0u, 0u};
    uint32_t mn = 0u;
    if (q < 8) window(q + 1, rn, mn);
    int base = 0;  // shared-memory record index of slot j: j + base
    if constexpr (kStaged) {
      const int ri = me.seg * 9 + q;
      base = (int)S->run_off[ri] - (int)S->run_slot0[ri];
    }
    if constexpr (kMemb == kMemMask) {
      while (m) {
        uint32_t j[4];
        bool v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          v[k] = m != 0u;
          j[k] = r.b + (v[k] ? (uint32_t)__ffs(m) - 1u : 0u);
          m &= m - 1u;
        }
        CbRec<kP> rr[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (v[k]) rr[k] = load(j[k], base);
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (v[k]) {
            fn(rr[k]);
            ++cnt;
          }
      }
      if ((ovf >> q) & 1u) {  // candidates past the mask: tested at x*_0
        for (uint32_t j = r.b + 32u; j < r.e; ++j)
          if (within_h(p, xyz(cb_ldg<kC>(A.xs0 + j)) - x0i)) {
            fn(load(j, base));
            ++cnt;
          }
      }
    } else {
      for (uint32_t j0 = r.b; j0 < r.e; j0 += 4u) {
        bool v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint32_t j = j0 + (uint32_t)k;
          v[k] = j < r.e && within_h(p, x0_of(j < r.e ? j : j0, base) - x0i);
        }
        CbRec<kP> rr[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (v[k]) rr[k] = load(j0 + (uint32_t)k, base);
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (v[k]) {
            fn(rr[k]);
            ++cnt;
          }
      }
    }
    r = rn;
    m = mn;
  }
  return cnt;
}

// Runs the walk from shared memory when the tile was staged, else from
// global memory (the same visits in the same order).
template <int kMemb, int kP, class Fn>
__device__ __forceinline__ uint32_t cb_visit(bool staged, const SimParams& p, const CbArgs& A, const CbShared& S,
                                             const float4* rec, const float4* const* src, const CbSlot& me,
                                             Fn&& fn) {
  if (staged) return cb_walk<true, kMemb, kP, false>(p, A, &S, rec, src, me, fn);
  return cb_walk<false, kMemb, kP, false>(p, A, &S, rec, src, me, fn);
}

// Fields a pass stages: x*_0 first when membership is tested, then its own.
template <int kMemb, int kP>
struct CbSrc {
  static constexpr int kOff = kMemb == kMemTest ? 1 : 0;
  static constexpr int kF = kOff + kP;
  const float4* a[kF];
  __device__ __forceinline__ CbSrc(const CbArgs& A, const float4* f0, const float4* f1 = nullptr,
                                   const float4* f2 = nullptr) {
    if constexpr (kOff == 1) a[0] = A.xs0;
    const float4* f[3] = {f0, f1, f2};
#pragma unroll
    for (int k = 0; k < kP; ++k) a[kOff + k] = f[k];
  }
};

extern __shared__ float4 cb_dyn[];

// The cell-block search: per slot, the 9 windows' membership masks (bit k of
// mask[q][t]: candidate k of window q is within h at x*_0; candidates past
// 32 flagged in ovf[t] bit q), the neighbour count and, with kFeat, the
// learned start's features (as k_nbr_build_feat).
template <bool kFeat>
__global__ void __launch_bounds__(cbk::kT) k_cb_build(SimParams p, CbArgs A, uint32_t* __restrict__ mask,
                                                      uint16_t* __restrict__ ovf_out,
                                                      uint32_t* __restrict__ nbr_count, int have_field,
                                                      const float4* __restrict__ bdata, SolverAux a) {
  __shared__ CbShared S;
  const float4* const src[1] = {A.xs0};
  CbSlot me;
  const bool staged = cb_stage<1>(S, cb_dyn, src, A, me);
  if (!me.valid) return;
  const GridParams& g = A.g;
  const f3 xi = xyz(__ldg(A.xs0 + me.t));
  uint32_t cnt = 0, ovf = 0;
  float w = 0.0f;  // sum of (h^2 - r^2)^3 over the neighbours (features)
  int q = 0;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy, ++q) {
      const Run r = run_of(g, A.cell_start, me.cx, me.cy, me.cz, dx, dy);
      int base = 0;
      if (staged && r.b != r.e) {
        const int ri = me.seg * 9 + q;
        base = (int)S.run_off[ri] - (int)S.run_slot0[ri];
      }
      uint32_t m = 0;
      for (uint32_t j = r.b; j < r.e; ++j) {
        const float4 xj = staged ? cb_dyn[(uint32_t)((int)j + base)] : __ldg(A.xs0 + j);
        const f3 d = xyz(xj) - xi;
        const float r2 = dist2_rn(d);
        if (r2 <= p.h2) {
          const uint32_t k = j - r.b;
          if (k < 32u)
            m |= 1u << k;
          else
            ovf |= 1u << q;
          ++cnt;
          if constexpr (kFeat) {
            const float c = p.h2 - r2;
            w = w + c * c * c;
          }
        }
      }
      mask[(size_t)q * A.n + me.t] = m;
    }
  ovf_out[me.t] = (uint16_t)ovf;
  nbr_count[me.t] = cnt;
  if constexpr (kFeat) {
    const float dens_fluid = p.V * (p.poly6 * w);
    float dens = dens_fluid, vb = 0.0f;
    if (have_field) {
      float4 bd = bdata[me.t];
      vb = bd.w;
      if (bd.w != 0.0f) dens = dens + bd.w * poly6_p(p, make_pair_of(xi - xyz(bd)));
    }
    const float4 xo = a.pos[me.t];
    const f3 vi = p.inv_dt * (xi - xyz(xo));
    float sd = a.bsdf ? fminf(a.bsdf[me.t], 2.0f * p.h) : 2.0f * p.h;
    a.feat[2 * me.t] = make_float4(dens - 1.0f, a.lam_prev ? a.lam_prev[me.t] : 0.0f, (float)cnt,
                                   len3(vi) * p.dt / p.h);
    a.feat[2 * me.t + 1] =
        make_float4(divergence_feature(p, xo, dens_fluid), sd / p.h, vb / p.V, a.substep_index);
  }
}

template <int kMemb, int kMode>
__global__ void __launch_bounds__(cbk::kT, 8) k_cb_lambda(SimParams p, CbArgs A, int have_field,
                                                       const float4* __restrict__ bdata,
                                                       const float4* __restrict__ xs, float4* __restrict__ xl,
                                                       SolverAux a) {
  __shared__ CbShared S;
  if (a.guard && *a.guard == 0) return;
  constexpr bool kStats = kMode == 2;
  const CbSrc<kMemb, 1> s(A, xs);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 1>::kF>(S, cb_dyn, s.a, A, me);
  unsigned cmax = 0u, csum = 0u, ccnt = 0u;
  if (me.valid) {
    LamSum acc;
    acc.init(xyz(xs[me.t]));
    const uint32_t cnt =
        cb_visit<kMemb, 1>(staged, p, A, S, cb_dyn, s.a, me, [&](const CbRec<1>& r) { acc.add(p, r.v[0]); });
    const float vsum = lambda_finish<kStats ? 0 : kMode, false>(p, have_field, bdata, xl, a, me.t, acc, cnt);
    if constexpr (kStats) compression_add(cmax, csum, ccnt, vsum * p.V);
  }
  if constexpr (kStats) compression_flush(a.stats, cmax, csum, ccnt);
}

template <int kMemb>
__global__ void __launch_bounds__(cbk::kT, 8) k_cb_deltap(SimParams p, CbArgs A, SolverAux a, int have_field,
                                                       const float4* __restrict__ xl,
                                                       const float4* __restrict__ bdata, float4* __restrict__ xs_out,
                                                       float4* __restrict__ dp_out) {
  __shared__ CbShared S;
  if (a.guard && *a.guard == 0) return;
  if (a.need && *a.need == 0) {  // the adaptive test found this iteration unneeded: copy x* through
    const uint32_t t = blockIdx.x * cbk::kT + threadIdx.x;
    if (t < A.n) xs_out[t] = a.xs_in[t];
    return;
  }
  const CbSrc<kMemb, 1> s(A, xl);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 1>::kF>(S, cb_dyn, s.a, A, me);
  if (!me.valid) return;
  DpSum acc;
  acc.init(xl[me.t]);
  cb_visit<kMemb, 1>(staged, p, A, S, cb_dyn, s.a, me, [&](const CbRec<1>& r) { acc.add(p, r.v[0]); });
  const f3 dp = deltap_finish<false>(p, have_field, bdata, me.t, acc);
  if (dp_out) dp_out[me.t] = f4(dp, 0.0f);
  const f3 xn = clamp_rand(p, acc.xi + dp);
  xs_out[me.t] = f4(xn, 0.0f);
  if (a.band.list) band_mark<false>(p, a.band, a.tab, me.t, xn);
}

template <int kMemb>
__global__ void __launch_bounds__(cbk::kT, 8) k_cb_density(SimParams p, CbArgs A, SolverAux a,
                                                        const float4* __restrict__ xs, float4* __restrict__ pos,
                                                        float4* __restrict__ vel, uint32_t* __restrict__ nbr_count) {
  __shared__ CbShared S;
  if (a.guard && *a.guard == 0) return;
  const CbSrc<kMemb, 1> s(A, xs);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 1>::kF>(S, cb_dyn, s.a, A, me);
  unsigned cmax = 0u, csum = 0u, ccnt = 0u;
  if (me.valid) {
    DensSum acc;
    acc.init(xyz(xs[me.t]));
    const uint32_t cnt =
        cb_visit<kMemb, 1>(staged, p, A, S, cb_dyn, s.a, me, [&](const CbRec<1>& r) { acc.add(p, r.v[0]); });
    if (nbr_count) nbr_count[me.t] = cnt;
    const float vsum = density_finish<false>(p, pos, vel, me.t, acc);
    if (a.stats) compression_add(cmax, csum, ccnt, vsum * p.V);
  }
  if (a.stats) compression_flush(a.stats, cmax, csum, ccnt);
}

template <int kMemb>
__global__ void __launch_bounds__(cbk::kT, 6) k_cb_vorticity(SimParams p, CbArgs A, const float4* __restrict__ pos,
                                                          const float4* __restrict__ vel, float4* __restrict__ omega,
                                                          float4* __restrict__ normal) {
  __shared__ CbShared S;
  const CbSrc<kMemb, 2> s(A, pos, vel);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 2>::kF>(S, cb_dyn, s.a, A, me);
  if (!me.valid) return;
  VortSum acc;
  acc.init(xyz(pos[me.t]), xyz(vel[me.t]));
  cb_visit<kMemb, 2>(staged, p, A, S, cb_dyn, s.a, me, [&](const CbRec<2>& r) { acc.add(p, r.v[0], r.v[1]); });
  vorticity_finish(p, omega, normal, me.t, acc);
}

template <int kMemb>
__global__ void __launch_bounds__(cbk::kT, 6) k_cb_xsph(SimParams p, CbArgs A, const float4* __restrict__ pos,
                                                     const float4* __restrict__ vel,
                                                     const float4* __restrict__ omega,
                                                     const float4* __restrict__ normal, float4* __restrict__ acc_out) {
  __shared__ CbShared S;
  const CbSrc<kMemb, 3> s(A, pos, vel, normal);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 3>::kF>(S, cb_dyn, s.a, A, me);
  if (!me.valid) return;
  XsphSum acc;
  acc.init(pos[me.t], xyz(vel[me.t]), xyz(normal[me.t]));
  cb_visit<kMemb, 3>(staged, p, A, S, cb_dyn, s.a, me,
                     [&](const CbRec<3>& r) { acc.add(p, r.v[0], r.v[1], r.v[2]); });
  xsph_finish(p, acc_out, me.t, acc, xyz(omega[me.t]));
}

template <int kMemb>
__global__ void __launch_bounds__(cbk::kT, 6) k_cb_vorticity_split(SimParams p, CbArgs A,
                                                                const float4* __restrict__ pos,
                                                                const float4* __restrict__ vel,
                                                                float4* __restrict__ omega,
                                                                float4* __restrict__ normal,
                                                                float4* __restrict__ visc,
                                                                float4* __restrict__ coh_sum) {
  __shared__ CbShared S;
  const CbSrc<kMemb, 2> s(A, pos, vel);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 2>::kF>(S, cb_dyn, s.a, A, me);
  if (!me.valid) return;
  VortSplitSum acc;
  acc.init(pos[me.t], xyz(vel[me.t]));
  cb_visit<kMemb, 2>(staged, p, A, S, cb_dyn, s.a, me, [&](const CbRec<2>& r) { acc.add(p, r.v[0], r.v[1]); });
  vorticity_split_finish(p, omega, normal, visc, coh_sum, me.t, acc);
}

template <int kMemb>
__global__ void __launch_bounds__(cbk::kT, 6) k_cb_xsph_split(SimParams p, CbArgs A, const float4* __restrict__ pos,
                                                           const float4* __restrict__ omega,
                                                           const float4* __restrict__ normal,
                                                           const float4* __restrict__ visc,
                                                           const float4* __restrict__ coh_sum,
                                                           float4* __restrict__ acc_out) {
  __shared__ CbShared S;
  const CbSrc<kMemb, 2> s(A, pos, normal);
  CbSlot me;
  const bool staged = cb_stage<CbSrc<kMemb, 2>::kF>(S, cb_dyn, s.a, A, me);
  if (!me.valid) return;
  XsphSplitSum acc;
  acc.init(pos[me.t], xyz(normal[me.t]));
  cb_visit<kMemb, 2>(staged, p, A, S, cb_dyn, s.a, me, [&](const CbRec<2>& r) { acc.add(p, r.v[0], r.v[1]); });
  xsph_split_finish(p, acc_out, me.t, acc, xyz(omega[me.t]), visc[me.t], coh_sum[me.t]);
}

// ---- the learned start's fallback solve on the cell-block search -------------------------
// Visitors of the fallback's walks (one add() per neighbour).
struct LamAdd {
  LamSum* acc;
  const SimParams* p;
  __device__ __forceinline__ void operator()(const CbRec<1>& r) const { acc->add(*p, r.v[0]); }
};
struct DpAdd {
  DpSum* acc;
  const SimParams* p;
  __device__ __forceinline__ void operator()(const CbRec<1>& r) const { acc->add(*p, r.v[0]); }
};
struct DensAdd {
  DensSum* acc;
  const SimParams* p;
  __device__ __forceinline__ void operator()(const CbRec<1>& r) const { acc->add(*p, r.v[0]); }
};

// The same phases as k_fallback_solve, each slot walking its windows from
// global memory with L2-coherent loads (the data changes between the
// kernel's grid-wide barriers).
__device__ __forceinline__ CbSlot cb_slot_of(const CbArgs& A, uint32_t t) {
  CbSlot me;
  me.t = t;
  me.valid = true;
  me.seg = 0;
  decode_key(A.g, __ldg(A.skey + t), me.cx, me.cy, me.cz);
  return me;
}

template <int kMemb>
__global__ void __launch_bounds__(256) k_cb_fallback_solve(FallbackArgs F, CbArgs A) {
  if (*F.guard == 0) return;
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const SimParams p = F.p;
  const uint32_t n = p.n, stride = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr bool kT0 = kMemb == kMemTest;  // field 0 of the walk is x*_0
  for (uint32_t t = t0; t < n; t += stride) {
    F.pos[t] = __ldcg(F.pos_old + __ldg(F.perm + t));
    const float4 x0 = __ldcg(F.xs_save + t);
    F.xs0[t] = make_float4(x0.x, x0.y, x0.z, 0.0f);
  }
  grid.sync();
  int b = 0;
  for (int it = 0; it < F.iters; ++it) {
    float4* cur = b ? F.xs1 : F.xs0;
    float4* nxt = b ? F.xs0 : F.xs1;
    if (F.f.loaded) {
      for (uint32_t t = t0; t < n; t += stride)
        boundary_slot<true>(p, F.f, F.sdf, F.vol, F.bflag, cur, F.bdata, nullptr, t);
      grid.sync();
    }
    SolverAux al{};
    al.lam_sum = F.lam_sum;
    al.lam_first = it == 0 ? 1 : 0;
    const float4* src_l[2] = {kT0 ? A.xs0 : cur, cur};
    for (uint32_t t = t0; t < n; t += stride) {
      const CbSlot me = cb_slot_of(A, t);
      LamSum acc;
      acc.init(xyz(__ldcg(cur + t)));
      const uint32_t cnt = cb_walk<false, kMemb, 1, true>(p, A, nullptr, nullptr, src_l, me, LamAdd{&acc, &p});
      lambda_finish<0, true>(p, F.f.loaded, F.bdata, F.xl, al, t, acc, cnt);
    }
    grid.sync();
    const float4* src_d[2] = {kT0 ? A.xs0 : F.xl, F.xl};
    for (uint32_t t = t0; t < n; t += stride) {
      const CbSlot me = cb_slot_of(A, t);
      DpSum acc;
      acc.init(__ldcg(F.xl + t));
      cb_walk<false, kMemb, 1, true>(p, A, nullptr, nullptr, src_d, me, DpAdd{&acc, &p});
      const f3 dp = deltap_finish<true>(p, F.f.loaded, F.bdata, t, acc);
      nxt[t] = f4(clamp_rand(p, acc.xi + dp), 0.0f);
    }
    grid.sync();
    b = 1 - b;
  }
  float4* fin = F.final_buf ? F.xs1 : F.xs0;
  if (b != F.final_buf) {
    const float4* srcb = b ? F.xs1 : F.xs0;
    for (uint32_t t = t0; t < n; t += stride) fin[t] = __ldcg(srcb + t);
    grid.sync();
  }
  const float4* src_r[2] = {kT0 ? A.xs0 : fin, fin};
  for (uint32_t t = t0; t < n; t += stride) {
    const CbSlot me = cb_slot_of(A, t);
    DensSum acc;
    acc.init(xyz(__ldcg(fin + t)));
    cb_walk<false, kMemb, 1, true>(p, A, nullptr, nullptr, src_r, me, DensAdd{&acc, &p});
    density_finish<true>(p, F.pos, F.vel, t, acc);
  }
}

template <int kMemb>
void fill_cb_set(CbSet* c) {
  c->lambda = k_cb_lambda<kMemb, 0>;
  c->lambda_feat = k_cb_lambda<kMemb, 1>;
  c->lambda_stats = k_cb_lambda<kMemb, 2>;
  c->deltap = k_cb_deltap<kMemb>;
  c->density_velocity = k_cb_density<kMemb>;
  c->vorticity = k_cb_vorticity<kMemb>;
  c->xsph = k_cb_xsph<kMemb>;
  if constexpr (kFast) {
    c->vorticity_split = k_cb_vorticity_split<kMemb>;
    c->xsph_split = k_cb_xsph_split<kMemb>;
  } else {
    c->vorticity_split = nullptr;
    c->xsph_split = nullptr;
  }
  c->fallback = k_cb_fallback_solve<kMemb>;
}
