// pbf_passes.cuh — the floating-point passes of one PBF substep.
//
// This header is compiled twice, into namespace pbf::exact (-fmad=false) and
// pbf::fast, by pbf_passes_exact.cu / pbf_passes_fast.cu.  PBF_NS names the
// namespace.  All particle arrays are in cell-sorted slot order (the layout
// the counting-sort reorder writes); neighbour lists hold slot indices.
//
// Reference passes restated here (paths relative to the reference root):
//   predict + key + count  TimeIntegration (src/simulator/PBF/shader/timeIntegration.ts:20-32)
//                          + ParticleInsert (src/simulator/neighbor/neighborShader.ts:24-32)
//   nbr_count / nbr_list   NeighborCount / NeighborList (neighborShader.ts:101-246)
//   lambda                 BoundaryVolume (boundaryVolume.ts:26-57) + LambdaCalculation
//                          (src/simulator/PBF/shader/pressureConstrain.ts:31-85)
//   deltap                 ConstrainSolve + ConstrainApply (pressureConstrain.ts:109-179)
//   density_velocity       AttributeUpdate (attributeUpdate.ts:25-59)
//   vorticity              VorticityConfinement (vorticityConfinement.ts:25-66)
//   xsph                   XSPH + vorticity force + surface tension (XSPH.ts:31-92)
#pragma once

#include <cooperative_groups.h>

#include "pbf_device.cuh"
#include "pbf_kernels.h"

namespace pbf {
namespace PBF_NS {

constexpr uint32_t kFull = 0xffffffffu;
constexpr uint32_t kNoKey = 0xffffffffu;

// Warp-aggregated count: lanes with equal keys elect one leader that does a
// single atomicAdd for all of them; each lane's rank = leader's base + its
// position among its peers.
__device__ __forceinline__ uint32_t warp_aggregated_rank(uint32_t* cell_count, uint32_t key) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t peers = __match_any_sync(kFull, key);
  uint32_t leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader && key != kNoKey) base = atomicAdd(cell_count + key, (uint32_t)__popc(peers));
  base = __shfl_sync(kFull, base, leader);
  uint32_t lt = (1u << lane) - 1u;
  return base + (uint32_t)__popc(peers & lt);
}

__device__ __forceinline__ uint32_t key_of(const GridParams& g, f3 x) {
  int cx = cell_axis(x.x, g.origin[0], g.inv_cell[0], g.dim[0]);
  int cy = cell_axis(x.y, g.origin[1], g.inv_cell[1], g.dim[1]);
  int cz = cell_axis(x.z, g.origin[2], g.inv_cell[2], g.dim[2]);
  return cell_key(cx, cy, cz, g);
}

// Every step pass exists as a one-tile-per-CTA kernel (kLoop = false: the
// loop below runs once and compiles away) and as a persistent kernel
// (kLoop = true: a grid of a few CTAs per SM walks the tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...).  PBF_TILES keeps the bound uniform across a
// CTA, so warp collectives stay converged; PBF_SLOTS is per thread.  A
// `continue` ends the one-tile form too (the step sets the index to n).
#define PBF_TILES(n) \
  for (uint32_t tile0 = blockIdx.x * blockDim.x; tile0 < (n); tile0 = kLoop ? tile0 + gridDim.x * blockDim.x : (n))
#define PBF_SLOTS(t, n)                                                                     \
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < (n); \
       t = kLoop ? t + gridDim.x * blockDim.x : (n))

// Per-slot scene of a batch: overrides the by-value grid / domain.  The
// kernels that consult it are instantiated twice; with kBatch = false the
// lookup folds away and the single-scene code is what it was without batches.
template <bool kBatch>
__device__ __forceinline__ const SceneDesc* scene_of(const SceneTab& tab, uint32_t t) {
  if constexpr (!kBatch) return nullptr;
  return tab.scene + __ldg(tab.slot_scene + t);
}
__device__ __forceinline__ void scene_domain(SimParams& p, const SceneDesc* sd) {
  if (!sd) return;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    p.dmin[a] = sd->dmin[a];
    p.dmax[a] = sd->dmax[a];
  }
}

// y + a x with the product and the sum each rounded once (no contraction).
__device__ __forceinline__ f3 axpy_rn(float a, f3 x, f3 y) {
  return mk(__fadd_rn(y.x, __fmul_rn(a, x.x)), __fadd_rn(y.y, __fmul_rn(a, x.y)), __fadd_rn(y.z, __fmul_rn(a, x.z)));
}

// predict x* (TimeIntegration), its cell key and within-cell rank (ParticleInsert).
// x* is computed with the reference's rounding in both precision modes, so
// the neighbour search starts from the restatement's positions bit for bit
// and fast mode finds the reference's neighbour sets too.
template <bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_predict(SimParams p0, GridParams g0, SceneTab tab,
                                                 const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                 const float4* __restrict__ acc, float4* __restrict__ xs_out,
                                                 uint32_t* __restrict__ key_out, uint32_t* __restrict__ rank_out,
                                                 uint32_t* cell_count) {
  PBF_TILES(p0.n) {
    const uint32_t s = tile0 + threadIdx.x;
    uint32_t key = kNoKey;
    if (s < p0.n) {
      SimParams p = p0;
      GridParams g = g0;
      const SceneDesc* sd = scene_of<kBatch>(tab, s);
      if (sd) {
        scene_domain(p, sd);
        g = sd->grid;
      }
      f3 x = xyz(pos[s]);
      f3 v = xyz(vel[s]);
      f3 a = xyz(acc[s]);
      f3 gv = mk(0.0f + a.x, p.gy + a.y, 0.0f + a.z);
      f3 vp = axpy_rn(p.dt, gv, v);
      f3 xp = clamp_rand(p, axpy_rn(p.dt, vp, x));
      xs_out[s] = f4(xp, 0.0f);
      key = key_of(g, xp);
      key_out[s] = key;
    }
    uint32_t rank = warp_aggregated_rank(cell_count, key);
    if (s < p0.n) rank_out[s] = rank;
  }
}

// |d|^2 with the reference's rounding (x*x + y*y, then + z*z, each product
// and sum rounded once; no contraction in either compile mode) and the
// neighbour test |d|^2 <= h^2 on it: every neighbour search of the library
// and the CPU restatement then agree on the neighbour sets bit for bit.
__device__ __forceinline__ float dist2_rn(f3 d) {
  return __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z));
}
__device__ __forceinline__ bool within_h(const SimParams& p, f3 d) { return dist2_rn(d) <= p.h2; }

// Range of slots covering cells (cx+dx, cy+dy, cz-Z .. cz+Z), Z = g.reach_z:
// the neighbourhood is (2 g.reach + 1)^2 runs of consecutive keys because
// keys are z-fastest (reach 1, Z = 1: the reference's 27 cells as 9 runs).
struct Run {
  uint32_t b, e;
};
__device__ __forceinline__ Run run_of(const GridParams& g, const uint32_t* __restrict__ cell_start, int cx, int cy,
                                      int cz, int dx, int dy) {
  int x = cx + dx, y = cy + dy;
  if (x < 0 || y < 0 || x >= g.dim[0] || y >= g.dim[1]) return Run{0, 0};
  int zlo = max(cz - g.reach_z, 0), zhi = min(cz + g.reach_z, g.dim[2] - 1);
  uint32_t k0 = cell_key(x, y, zlo, g), k1 = cell_key(x, y, zhi, g) + 1u;
  return Run{__ldg(cell_start + k0), __ldg(cell_start + k1)};
}

// NeighborCount: neighbours within h of x*, self included, 27 cells in key
// order (stand-alone search; slot n receives 0 so a scan of n + 1 counts
// ends in the total).
__global__ void __launch_bounds__(256) k_nbr_count(SimParams p, GridParams g, const float4* __restrict__ xs,
                                                   const uint32_t* __restrict__ cell_start,
                                                   uint32_t* __restrict__ nbr_count) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cnt = 0;
  if (t < p.n) {
    f3 xi = xyz(xs[t]);
    int cx = cell_axis(xi.x, g.origin[0], g.inv_cell[0], g.dim[0]);
    int cy = cell_axis(xi.y, g.origin[1], g.inv_cell[1], g.dim[1]);
    int cz = cell_axis(xi.z, g.origin[2], g.inv_cell[2], g.dim[2]);
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy) {
        Run r = run_of(g, cell_start, cx, cy, cz, dx, dy);
        for (uint32_t u = r.b; u < r.e; ++u) {
          f3 d = xyz(__ldg(xs + u)) - xi;
          if (within_h(p, d)) ++cnt;
        }
      }
  }
  if (t <= p.n) nbr_count[t] = cnt;
}

// Velocity divergence feature of the learned start, -div(v') dt, by the
// continuity equation: (rho_prev - rho*) / rho* with rho* the fluid density
// at x* (V sum W) and rho_prev the particle's density after the previous
// substep (x.w / rho0); 0 before the first density pass.
__device__ __forceinline__ float divergence_feature(const SimParams& p, float4 x_prev, float dens_fluid) {
  const float prev = x_prev.w / p.rho0;
  return (prev > 0.0f && dens_fluid > 0.0f) ? (prev - dens_fluid) / dens_fluid : 0.0f;
}

// NeighborCount + NeighborList of the step in one traversal.  The list is
// interleaved by warp with a fixed slice of max_nbr entries per particle:
// neighbour q of slot t is at (t / 32) * 32 * max_nbr + 32 q + t % 32, so the
// q-th entries of a warp's 32 particles are one contiguous 128-byte segment,
// and no count pass or scan is needed to place them.  nbr_count[t] receives
// the true count; a count above max_nbr flags an overflow (the entries past
// the slice are dropped and max_seen records the largest count for growing).
// Runs are visited in key order, so entries come in increasing slot order.
template <bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_nbr_build(SimParams p, GridParams g0, SceneTab tab,
                                                   const float4* __restrict__ xs,
                                                   const uint32_t* __restrict__ cell_start, uint32_t max_nbr,
                                                   uint32_t* __restrict__ nbr_list, uint32_t* __restrict__ nbr_count,
                                                   uint32_t* max_seen, uint32_t* err) {
  PBF_TILES(p.n) {
    const uint32_t t = tile0 + threadIdx.x;
    if (t < p.n) {
      const SceneDesc* sd = scene_of<kBatch>(tab, t);
      const GridParams g = sd ? sd->grid : g0;
      f3 xi = xyz(xs[t]);
      int cx = cell_axis(xi.x, g.origin[0], g.inv_cell[0], g.dim[0]);
      int cy = cell_axis(xi.y, g.origin[1], g.inv_cell[1], g.dim[1]);
      int cz = cell_axis(xi.z, g.origin[2], g.inv_cell[2], g.dim[2]);
      uint32_t* out = nbr_list + (size_t)(t >> 5) * 32u * max_nbr + (t & 31u);
      uint32_t q = 0;
      for (int dx = -g.reach; dx <= g.reach; ++dx)
        for (int dy = -g.reach; dy <= g.reach; ++dy) {
          Run r = run_of(g, cell_start, cx, cy, cz, dx, dy);
          for (uint32_t u = r.b; u < r.e; ++u) {
            f3 d = xyz(__ldg(xs + u)) - xi;
            if (within_h(p, d)) {
              if (q < max_nbr) out[32u * q] = u;
              ++q;
            }
          }
        }
      nbr_count[t] = q;
      const unsigned m = __activemask();
      if (__any_sync(m, q > max_nbr)) {
        unsigned wmax = __reduce_max_sync(m, q);
        if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) {
          atomicMax(max_seen, wmax);
          atomicOr(err, 0x1u);
        }
      }
    }
  }
}

// The learned start's neighbour build: the same traversal, which also sums
// the fluid density at x*_0 over the neighbours it finds (poly6 from the
// squared distance the test already has: a few FMAs per hit) and writes the
// start's feature rows (a.feat, the layout the lambda pass records for
// training).  Needs the boundary sampling at x*_0 first (bdata, a.bsdf),
// unless a.late_boundary leaves the boundary terms to the network pass
// (have_field = 0, a.bsdf = null: the sampling may then run concurrently).
template <bool kLoop>
__global__ void __launch_bounds__(256) k_nbr_build_feat(SimParams p, GridParams g, const float4* __restrict__ xs,
                                                        const uint32_t* __restrict__ cell_start, uint32_t max_nbr,
                                                        uint32_t* __restrict__ nbr_list,
                                                        uint32_t* __restrict__ nbr_count, uint32_t* max_seen,
                                                        uint32_t* err, int have_field,
                                                        const float4* __restrict__ bdata, SolverAux a) {
  PBF_TILES(p.n) {
    const uint32_t t = tile0 + threadIdx.x;
    if (t < p.n) {
      const f3 xi = xyz(xs[t]);
      int cx = cell_axis(xi.x, g.origin[0], g.inv_cell[0], g.dim[0]);
      int cy = cell_axis(xi.y, g.origin[1], g.inv_cell[1], g.dim[1]);
      int cz = cell_axis(xi.z, g.origin[2], g.inv_cell[2], g.dim[2]);
      uint32_t* out = nbr_list + (size_t)(t >> 5) * 32u * max_nbr + (t & 31u);
      uint32_t q = 0;
      float w = 0.0f;  // sum of (h^2 - r^2)^3 over the neighbours
      for (int dx = -g.reach; dx <= g.reach; ++dx)
        for (int dy = -g.reach; dy <= g.reach; ++dy) {
          Run r = run_of(g, cell_start, cx, cy, cz, dx, dy);
          for (uint32_t u = r.b; u < r.e; ++u) {
            f3 d = xyz(__ldg(xs + u)) - xi;
            const float r2 = dist2_rn(d);
            if (r2 <= p.h2) {
              if (q < max_nbr) out[32u * q] = u;
              ++q;
              const float c = p.h2 - r2;
              w = w + c * c * c;
            }
          }
        }
      nbr_count[t] = q;
      const unsigned m = __activemask();
      if (__any_sync(m, q > max_nbr)) {
        unsigned wmax = __reduce_max_sync(m, q);
        if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) {
          atomicMax(max_seen, wmax);
          atomicOr(err, 0x1u);
        }
      }
      const float dens_fluid = p.V * (p.poly6 * w);
      float dens = dens_fluid, vb = 0.0f;
      if (have_field) {
        float4 bd = bdata[t];
        vb = bd.w;
        if (bd.w != 0.0f) dens = dens + bd.w * poly6_p(p, make_pair_of(xi - xyz(bd)));
      }
      const float4 xo = a.pos[t];
      const f3 vi = p.inv_dt * (xi - xyz(xo));
      float sd = a.bsdf ? fminf(a.bsdf[t], 2.0f * p.h) : 2.0f * p.h;
      float f0 = dens - 1.0f, f5 = sd / p.h, f6 = vb / p.V;
      if (a.late_boundary) {  // the network pass adds the boundary terms (LateBoundary)
        f0 = dens_fluid;
        f5 = 0.0f;
        f6 = 0.0f;
      }
      a.feat[2 * t] = make_float4(f0, a.lam_prev ? a.lam_prev[t] : 0.0f, (float)min(q, max_nbr),
                                  len3(vi) * p.dt / p.h);
      a.feat[2 * t + 1] = make_float4(divergence_feature(p, xo, dens_fluid), f5, f6, a.substep_index);
    }
  }
}

// The same build with two consecutive slots per thread.  Slots are sorted by
// cell, so slots 2k and 2k+1 usually share a cell and therefore every
// candidate run: each candidate is loaded once and tested against both
// particles (half the loads and loop overhead per test).  A pair that spans
// two cells (or scenes) walks its two neighbourhoods one after the other.
// Lists, counts and their order are those of k_nbr_build.
template <bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_nbr_build2(SimParams p, GridParams g0, SceneTab tab,
                                                    const float4* __restrict__ xs,
                                                    const uint32_t* __restrict__ cell_start, uint32_t max_nbr,
                                                    uint32_t* __restrict__ nbr_list, uint32_t* __restrict__ nbr_count,
                                                    uint32_t* max_seen, uint32_t* err) {
  const uint32_t npair = (p.n + 1u) >> 1;
  PBF_TILES(npair) {
    const uint32_t k = tile0 + threadIdx.x;
    if (k < npair) {
      const uint32_t ta = 2u * k, tb = ta + 1u;
      const bool hb = tb < p.n;
      const SceneDesc* sa = scene_of<kBatch>(tab, ta);
      const GridParams ga = sa ? sa->grid : g0;
      const f3 xa = xyz(xs[ta]);
      const int ax = cell_axis(xa.x, ga.origin[0], ga.inv_cell[0], ga.dim[0]);
      const int ay = cell_axis(xa.y, ga.origin[1], ga.inv_cell[1], ga.dim[1]);
      const int az = cell_axis(xa.z, ga.origin[2], ga.inv_cell[2], ga.dim[2]);
      uint32_t* outa = nbr_list + (size_t)(ta >> 5) * 32u * max_nbr + (ta & 31u);
      uint32_t* outb = nbr_list + (size_t)(tb >> 5) * 32u * max_nbr + (tb & 31u);
      uint32_t qa = 0, qb = 0;
      f3 xb = xa;
      bool joint = false;
      GridParams gb = ga;
      int bx = ax, by = ay, bz = az;
      if (hb) {
        const SceneDesc* sb = scene_of<kBatch>(tab, tb);
        if (sb) gb = sb->grid;
        xb = xyz(xs[tb]);
        bx = cell_axis(xb.x, gb.origin[0], gb.inv_cell[0], gb.dim[0]);
        by = cell_axis(xb.y, gb.origin[1], gb.inv_cell[1], gb.dim[1]);
        bz = cell_axis(xb.z, gb.origin[2], gb.inv_cell[2], gb.dim[2]);
        joint = cell_key(ax, ay, az, ga) == cell_key(bx, by, bz, gb);
      }
      if (joint) {
        for (int dx = -ga.reach; dx <= ga.reach; ++dx)
          for (int dy = -ga.reach; dy <= ga.reach; ++dy) {
            Run r = run_of(ga, cell_start, ax, ay, az, dx, dy);
            for (uint32_t u = r.b; u < r.e; ++u) {
              const f3 xj = xyz(__ldg(xs + u));
              const f3 da = xj - xa, db = xj - xb;
              if (within_h(p, da)) {
                if (qa < max_nbr) outa[32u * qa] = u;
                ++qa;
              }
              if (within_h(p, db)) {
                if (qb < max_nbr) outb[32u * qb] = u;
                ++qb;
              }
            }
          }
      } else {
        for (int dx = -ga.reach; dx <= ga.reach; ++dx)
          for (int dy = -ga.reach; dy <= ga.reach; ++dy) {
            Run r = run_of(ga, cell_start, ax, ay, az, dx, dy);
            for (uint32_t u = r.b; u < r.e; ++u) {
              const f3 d = xyz(__ldg(xs + u)) - xa;
              if (within_h(p, d)) {
                if (qa < max_nbr) outa[32u * qa] = u;
                ++qa;
              }
            }
          }
        if (hb) {
          for (int dx = -gb.reach; dx <= gb.reach; ++dx)
            for (int dy = -gb.reach; dy <= gb.reach; ++dy) {
              Run r = run_of(gb, cell_start, bx, by, bz, dx, dy);
              for (uint32_t u = r.b; u < r.e; ++u) {
                const f3 d = xyz(__ldg(xs + u)) - xb;
                if (within_h(p, d)) {
                  if (qb < max_nbr) outb[32u * qb] = u;
                  ++qb;
                }
              }
            }
        }
      }
      nbr_count[ta] = qa;
      if (hb) nbr_count[tb] = qb;
      const uint32_t q = max(qa, qb);
      const unsigned m = __activemask();
      if (__any_sync(m, q > max_nbr)) {
        unsigned wmax = __reduce_max_sync(m, q);
        if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) {
          atomicMax(max_seen, wmax);
          atomicOr(err, 0x1u);
        }
      }
    }
  }
}

// The same build, warp-cooperative per cell.  The 32 sorted slots of a warp
// fall into a few cells; for each cell group the warp walks the group's
// candidate runs once, 32 candidates at a time (lane = candidate, coalesced
// loads), tests each chunk against every particle of the group (its position
// broadcast by shuffle, the hits collected by ballot into the owner lane's
// mask), and each owner then appends its hits in slot order.  Lists, counts
// and their order are those of k_nbr_build.
template <bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_nbr_build_warp(SimParams p, GridParams g0, SceneTab tab,
                                                        const float4* __restrict__ xs,
                                                        const uint32_t* __restrict__ cell_start, uint32_t max_nbr,
                                                        uint32_t* __restrict__ nbr_list,
                                                        uint32_t* __restrict__ nbr_count, uint32_t* max_seen,
                                                        uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31u;
  PBF_TILES(p.n) {
    const uint32_t t = tile0 + threadIdx.x;
    const bool valid = t < p.n;
    GridParams g = g0;
    f3 xi = mk(0.f, 0.f, 0.f);
    int cx = 0, cy = 0, cz = 0;
    uint32_t key = kNoKey;
    if (valid) {
      const SceneDesc* sd = scene_of<kBatch>(tab, t);
      if (sd) g = sd->grid;
      xi = xyz(xs[t]);
      cx = cell_axis(xi.x, g.origin[0], g.inv_cell[0], g.dim[0]);
      cy = cell_axis(xi.y, g.origin[1], g.inv_cell[1], g.dim[1]);
      cz = cell_axis(xi.z, g.origin[2], g.inv_cell[2], g.dim[2]);
      key = cell_key(cx, cy, cz, g);
    }
    const unsigned peers = __match_any_sync(kFull, key);
    unsigned todo = __ballot_sync(kFull, valid);
    uint32_t* out = nbr_list + (size_t)(t >> 5) * 32u * max_nbr + lane;
    uint32_t q = 0;
    while (todo) {
      const int leader = __ffs(todo) - 1;
      const unsigned gm = __shfl_sync(kFull, peers, leader);
      todo &= ~gm;
      const int lx = __shfl_sync(kFull, cx, leader), ly = __shfl_sync(kFull, cy, leader),
                lz = __shfl_sync(kFull, cz, leader);
      GridParams gl = g0;
      if constexpr (kBatch) {  // the group's scene grid (run bounds and keys only)
        gl.dim[0] = __shfl_sync(kFull, g.dim[0], leader);
        gl.dim[1] = __shfl_sync(kFull, g.dim[1], leader);
        gl.dim[2] = __shfl_sync(kFull, g.dim[2], leader);
        gl.key_base = __shfl_sync(kFull, g.key_base, leader);
        gl.reach = __shfl_sync(kFull, g.reach, leader);
        gl.reach_z = __shfl_sync(kFull, g.reach_z, leader);
      }
      for (int dx = -gl.reach; dx <= gl.reach; ++dx)
        for (int dy = -gl.reach; dy <= gl.reach; ++dy) {
          const Run r = run_of(gl, cell_start, lx, ly, lz, dx, dy);
          for (uint32_t u0 = r.b; u0 < r.e; u0 += 32u) {
            const uint32_t u = u0 + lane;
            const bool in = u < r.e;
            const f3 c = xyz(__ldg(xs + (in ? u : u0)));
            unsigned mine = 0u;
            unsigned pm = gm;
            while (pm) {
              const int pl = __ffs(pm) - 1;
              pm &= pm - 1u;
              const f3 xp = mk(__shfl_sync(kFull, xi.x, pl), __shfl_sync(kFull, xi.y, pl),
                               __shfl_sync(kFull, xi.z, pl));
              const f3 d = c - xp;
              const unsigned hits = __ballot_sync(kFull, in && within_h(p, d));
              if ((int)lane == pl) mine = hits;
            }
            while (mine) {
              const int b = __ffs(mine) - 1;
              mine &= mine - 1u;
              if (q < max_nbr) out[32u * q] = u0 + (uint32_t)b;
              ++q;
            }
          }
        }
    }
    if (valid) nbr_count[t] = q;
    if (__any_sync(kFull, q > max_nbr)) {
      const unsigned wmax = __reduce_max_sync(kFull, q);
      if (lane == 0) {
        atomicMax(max_seen, wmax);
        atomicOr(err, 0x1u);
      }
    }
  }
}

// NeighborList: the same traversal writing slot indices at nbr_offset[t].
__global__ void __launch_bounds__(256) k_nbr_list(SimParams p, GridParams g, const float4* __restrict__ xs,
                                                  const uint32_t* __restrict__ cell_start,
                                                  const uint32_t* __restrict__ nbr_offset, uint32_t* __restrict__ nbr_list,
                                                  uint32_t capacity, uint32_t* err) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.n) return;
  if (t == 0 && nbr_offset[p.n] > capacity) atomicOr(err, 0x1u);
  f3 xi = xyz(xs[t]);
  int cx = cell_axis(xi.x, g.origin[0], g.inv_cell[0], g.dim[0]);
  int cy = cell_axis(xi.y, g.origin[1], g.inv_cell[1], g.dim[1]);
  int cz = cell_axis(xi.z, g.origin[2], g.inv_cell[2], g.dim[2]);
  uint32_t o = nbr_offset[t];
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy) {
      Run r = run_of(g, cell_start, cx, cy, cz, dx, dy);
      for (uint32_t u = r.b; u < r.e; ++u) {
        f3 d = xyz(__ldg(xs + u)) - xi;
        if (within_h(p, d)) {
          if (o < capacity) nbr_list[o] = u;
          ++o;
        }
      }
    }
}

// Loads of per-particle records.  kC = false: the read-only path (the record
// is not written during the kernel).  kC = true: L2-coherent loads, for the
// fallback solve, which rewrites positions and multipliers between its
// grid-wide barriers within one kernel.
template <bool kC>
__device__ __forceinline__ float4 ldr(const float4* p) {
  if constexpr (kC) return __ldcg(p);
  return __ldg(p);
}
template <bool kC>
__device__ __forceinline__ float4 ldo(const float4* p) {  // the slot's own record
  if constexpr (kC) return __ldcg(p);
  return *p;
}

// Visit the cnt neighbours of a slot in list order (interleaved layout:
// entry q at base + 32 q).  Neighbours go in batches of four: the batch's
// records are gathered, the next batch's indices are requested, then the
// batch is consumed, so the list read (from DRAM) of one batch overlaps the
// gathers and arithmetic of the previous one.  List entries are streamed
// (evict-first): each pass reads the list once, and the records it gathers
// stay cached.  fn(j, xj) keeps the sequential accumulation order of the
// reference loop.
template <bool kC = false, class Fn>
__device__ __forceinline__ void for_each_neighbor(const uint32_t* __restrict__ list, uint32_t base, uint32_t cnt,
                                                  const float4* xs, Fn&& fn) {
  const uint32_t* l = list + base;
  const uint32_t full = cnt & ~3u;
  uint32_t q = 0;
  if (full) {
    uint32_t j0 = __ldcs(l), j1 = __ldcs(l + 32), j2 = __ldcs(l + 64), j3 = __ldcs(l + 96);
    while (true) {
      const float4 x0 = ldr<kC>(xs + j0), x1 = ldr<kC>(xs + j1), x2 = ldr<kC>(xs + j2), x3 = ldr<kC>(xs + j3);
      const uint32_t c0 = j0, c1 = j1, c2 = j2, c3 = j3;
      q += 4;
      const bool more = q < full;
      if (more) {
        j0 = __ldcs(l + 32 * q);
        j1 = __ldcs(l + 32 * q + 32);
        j2 = __ldcs(l + 32 * q + 64);
        j3 = __ldcs(l + 32 * q + 96);
      }
      fn(c0, x0);
      fn(c1, x1);
      fn(c2, x2);
      fn(c3, x3);
      if (!more) break;
    }
  }
  for (; q < cnt; ++q) {
    uint32_t j = __ldcs(l + 32 * q);
    fn(j, ldr<kC>(xs + j));
  }
}

// The same walk gathering two records per neighbour (its x_j and a second
// per-particle float4): both loads of a batch are issued before the batch is
// consumed.  fn(j, xj, yj).  The XSPH pass uses it for (n_j, |omega_j|)
// (0.134 -> 0.131 ms at 2^20); in the vorticity pass, which is held to 64
// registers, the extra live records made it slower (0.130 -> 0.137 ms).
template <class Fn>
__device__ __forceinline__ void for_each_neighbor2(const uint32_t* __restrict__ list, uint32_t base, uint32_t cnt,
                                                   const float4* xs, const float4* ys, Fn&& fn) {
  const uint32_t* l = list + base;
  const uint32_t full = cnt & ~3u;
  uint32_t q = 0;
  if (full) {
    uint32_t j0 = __ldcs(l), j1 = __ldcs(l + 32), j2 = __ldcs(l + 64), j3 = __ldcs(l + 96);
    while (true) {
      const float4 x0 = __ldg(xs + j0), x1 = __ldg(xs + j1), x2 = __ldg(xs + j2), x3 = __ldg(xs + j3);
      const float4 y0 = __ldg(ys + j0), y1 = __ldg(ys + j1), y2 = __ldg(ys + j2), y3 = __ldg(ys + j3);
      const uint32_t c0 = j0, c1 = j1, c2 = j2, c3 = j3;
      q += 4;
      const bool more = q < full;
      if (more) {
        j0 = __ldcs(l + 32 * q);
        j1 = __ldcs(l + 32 * q + 32);
        j2 = __ldcs(l + 32 * q + 64);
        j3 = __ldcs(l + 32 * q + 96);
      }
      fn(c0, x0, y0);
      fn(c1, x1, y1);
      fn(c2, x2, y2);
      fn(c3, x3, y3);
      if (!more) break;
    }
  }
  for (; q < cnt; ++q) {
    const uint32_t j = __ldcs(l + 32 * q);
    fn(j, __ldg(xs + j), __ldg(ys + j));
  }
}

// Whether the boundary sample of a particle can be non-zero: per field cell,
// 0 when all 32 volume nodes are zero (the interpolated volume is then zero)
// or the SDF provably stays >= h over the cell; then bData = 0 exactly.
__device__ __forceinline__ bool boundary_possible(const FieldParams& f, const uint8_t* __restrict__ flag, f3 x) {
  if (!flag) return true;
  int c[3];
  float q[3] = {x.x, x.y, x.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float u = (q[a] - f.origin[a]) * f.scale[a];
    int ci = (int)floorf(u);
    c[a] = min(max(ci, 0), f.res[a] - 1);
  }
  return __ldg(flag + ((size_t)c[2] * f.res[1] + c[1]) * f.res[0] + c[0]) != 0;
}

// Slice of slot t in the interleaved list (see k_nbr_build); a count past the
// slice (an overflowed substep, already flagged) is clamped to it.
__device__ __forceinline__ void list_slice(uint32_t max_nbr, const uint32_t* __restrict__ cnt_of, uint32_t t,
                                           uint32_t& base, uint32_t& cnt) {
  base = (t >> 5) * 32u * max_nbr + (t & 31u);
  cnt = min(__ldg(cnt_of + t), max_nbr);
}

// Whether a scene (of a batch) runs solver iteration `iter`.
__device__ __forceinline__ bool iter_active(const SceneDesc* sd, int iter) {
  return !sd || (uint32_t)iter < sd->iterations;
}

// BoundaryVolume (boundaryVolume.ts:26-57) of slot t: (x_b, V_b), skipping
// the 64-node interpolation where the field cell cannot produce a sample (the
// fallback solve's boundary phase; the step samples through the band list).
template <bool kC>
__device__ __forceinline__ void boundary_slot(const SimParams& p, const FieldParams& f, const float* __restrict__ sdf0,
                                              const float* __restrict__ vol0, const uint8_t* __restrict__ bflag0,
                                              const float4* xs, float4* bdata, float* bsdf, uint32_t t) {
  f3 xi = xyz(ldo<kC>(xs + t));
  float4 bd = make_float4(0.f, 0.f, 0.f, 0.f);
  float dist = 2.0f * p.h;  // "far" for the feature when the cell cannot contribute
  if (f.loaded) {
    const float* sdf = sdf0 + f.node_off;
    const float* vol = vol0 + f.node_off;
    const uint8_t* bflag = bflag0 ? bflag0 + f.flag_off : nullptr;
    if (boundary_possible(f, bflag, xi)) bd = boundary_sample(p, f, sdf, vol, xi, bsdf ? &dist : nullptr);
  }
  bdata[t] = bd;
  if (bsdf) bsdf[t] = dist;
}

// Band test of slot t at x (see BandArgs): outside the band bData = 0 (and
// the SDF feature 2h) at once; inside, the slot joins the list (one atomic
// per warp).  Lanes that call this together must be the active ones.
template <bool kBatch>
__device__ __forceinline__ void band_mark(const SimParams& p, const BandArgs& B, const SceneTab& tab, uint32_t t,
                                          f3 x) {
  const SceneDesc* sd = scene_of<kBatch>(tab, t);
  const FieldParams& f = sd ? sd->field : B.f;
  const bool in = f.loaded && boundary_possible(f, B.flag ? B.flag + f.flag_off : nullptr, x);
  if (!in) {
    B.bdata[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (B.bsdf) B.bsdf[t] = 2.0f * p.h;
  }
  const unsigned m = __activemask();
  const unsigned b = __ballot_sync(m, in);
  if (b) {
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)(threadIdx.x & 31u) == leader) base = atomicAdd(B.count, (uint32_t)__popc(b));
    base = __shfl_sync(m, base, leader);
    if (in) B.list[base + __popc(b & ((1u << (threadIdx.x & 31u)) - 1u))] = t;
  }
}

// The band at the predicted positions x*_0 (the first boundary sampling of a
// substep; later ones are marked by delta-p).
template <bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_band(SimParams p, SceneTab tab, const float4* __restrict__ xs, BandArgs B) {
  PBF_SLOTS(t, p.n) band_mark<kBatch>(p, B, tab, t, xyz(xs[t]));
}

// BoundaryVolume for the band's slots only: a grid of resident CTAs walks the
// list (its length is known on the device only).  Also clears the count of
// the other band list, which delta-p fills next.
// Node values come from the packed blocks (FieldBlocks): every listed slot's
// field cell is flagged, so it has one.
template <bool kBatch>
__global__ void __launch_bounds__(256, 2) k_boundary_band(SimParams p, FieldParams f0, const float* __restrict__ sdf0,
                                                          const float* __restrict__ vol0, FieldBlocks fb, SceneTab tab,
                                                          const float4* __restrict__ xs, float4* __restrict__ bdata,
                                                          float* __restrict__ bsdf, const uint32_t* __restrict__ list,
                                                          const uint32_t* count, uint32_t* other_count,
                                                          const int* guard) {
  if (other_count && blockIdx.x == 0 && threadIdx.x == 0) *other_count = 0u;
  if (guard && *guard == 0) return;  // the iteration is skipped (lagged iteration control)
  const uint32_t nb = *count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    const uint32_t t = list[i];
    const SceneDesc* sd = scene_of<kBatch>(tab, t);
    const FieldParams f = sd ? sd->field : f0;
    const float* sdf = sdf0 + f.node_off;
    const float* vol = vol0 + f.node_off;
    const f3 xi = xyz(xs[t]);
    float dist;
    bdata[t] = boundary_sample_packed(p, f, fb, sdf, vol, xi, &dist);
    if (bsdf) bsdf[t] = dist;
  }
}

// Per-step density error statistics (compression max(0, V sum W - 1), fluid
// only): each thread's running max / fixed-point sum / count, reduced over
// the CTA in shared memory, one set of atomics per CTA.  Every thread of the
// CTA calls it.
__device__ __forceinline__ void compression_add(unsigned& cmax, unsigned& csum, unsigned& ccnt, float vsum_times_v) {
  const float c = fmaxf(0.0f, vsum_times_v - 1.0f);
  cmax = max(cmax, __float_as_uint(c));  // non-negative floats order as their bits
  csum += (unsigned)(fminf(c, 1.0f) * 1048576.0f);
  ++ccnt;
}
__device__ __forceinline__ void compression_flush(SolveStats* stats, unsigned cmax, unsigned csum, unsigned ccnt) {
  __shared__ unsigned s_max, s_cnt;
  __shared__ unsigned long long s_sum;
  if (threadIdx.x == 0) {
    s_max = 0u;
    s_cnt = 0u;
    s_sum = 0ull;
  }
  __syncthreads();
  cmax = __reduce_max_sync(0xffffffffu, cmax);
  csum = __reduce_add_sync(0xffffffffu, csum);
  ccnt = __reduce_add_sync(0xffffffffu, ccnt);
  if ((threadIdx.x & 31u) == 0) {
    atomicMax(&s_max, cmax);
    atomicAdd(&s_cnt, ccnt);
    atomicAdd(&s_sum, (unsigned long long)csum);
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_cnt) {
    atomicMax(&stats->max_bits, s_max);
    atomicAdd(&stats->count, s_cnt);
    atomicAdd(&stats->sum_fx, s_sum);
  }
}

// ---- per-neighbour sums of the passes --------------------------------------------
// One struct per pass holds the slot's own values and running sums; add()
// takes one neighbour's records.  The list walks and the cell-block walks
// (pbf_cellblock.cuh) call the same add(), so both evaluate the same
// arithmetic in the same (reference) order.

// LambdaCalculation's sums (pressureConstrain.ts:49-61): grad, sum |grad|^2, sum W.
struct LamSum {
  f3 xi, grad;
  float sum2, dens;
  __device__ __forceinline__ void init(f3 x) {
    xi = x;
    grad = mk(0.f, 0.f, 0.f);
    sum2 = 0.0f;
    dens = 0.0f;
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 xj) {
    Pair q = make_pair_of(xi - xyz(xj));
    f3 gk = spiky_p(p, q);
    grad = grad + gk;
    sum2 = sum2 + dot3(gk, gk);
    dens = dens + poly6_p(p, q);
  }
};
// ConstrainSolve's sum (pressureConstrain.ts:127-141) over packed (x*_j, lambda_j).
struct DpSum {
  f3 xi, pu;
  float li;
  __device__ __forceinline__ void init(float4 xli) {
    xi = xyz(xli);
    li = xli.w;
    pu = mk(0.f, 0.f, 0.f);
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 xj) {
    Pair q = make_pair_of(xi - xyz(xj));
    pu = pu + (li + xj.w) * spiky_p(p, q);
  }
};
// AttributeUpdate's density sum (attributeUpdate.ts:40-49).
struct DensSum {
  f3 xi;
  float dens;
  __device__ __forceinline__ void init(f3 x) {
    xi = x;
    dens = 0.0f;
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 xj) {
    Pair q = make_pair_of(xi - xyz(xj));
    dens = dens + poly6_p(p, q);
  }
};
// VorticityConfinement's sums (vorticityConfinement.ts:46-61): omega and the Akinci normal.
struct VortSum {
  f3 xi, vi, om, nm;
  __device__ __forceinline__ void init(f3 x, f3 v) {
    xi = x;
    vi = v;
    om = mk(0.f, 0.f, 0.f);
    nm = mk(0.f, 0.f, 0.f);
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 pj, float4 vj) {
    Pair q = make_pair_of(xi - xyz(pj));
    f3 vd = xyz(vj) - vi;
    float volume = fdiv(p.m, pj.w);
    f3 gw = spiky_p(p, q);
    om = om + volume * cross3(vd, gw);
    nm = nm + volume * gw;
  }
};
// XSPH + vorticity force + Akinci tension sums (XSPH.ts:57-81), single pass.
struct XsphSum {
  f3 xi, vi, ni, vu, eta, ten;
  float ri;
  __device__ __forceinline__ void init(float4 pi, f3 v, f3 n) {
    xi = xyz(pi);
    ri = pi.w;
    vi = v;
    ni = n;
    vu = mk(0.f, 0.f, 0.f);
    eta = mk(0.f, 0.f, 0.f);
    ten = mk(0.f, 0.f, 0.f);
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 pj, float4 vj, float4 nj) {
    float rj = pj.w;
    Pair q = make_pair_of(xi - xyz(pj));
    f3 vd = xyz(vj) - vi;
    float kij = fdiv(p.two_rho0, ri + rj);
    vu = vu + fdiv3(poly6_p(p, q) * vd, rj);
    eta = eta + fdiv3(nj.w * spiky_p(p, q), rj);  // nj: (normal_j, |omega_j|)
    f3 coh = p.m * cohesion_p(p, q);
    f3 curv = ni - xyz(nj);
    ten = ten - kij * (coh + curv);
  }
};
// Fast mode's split: the vorticity pass also sums XSPH's viscosity term and
// the cohesion part of the tension (see k_vorticity_split).
struct VortSplitSum {
  f3 xi, vi, om, nm, vu, cs;
  float ri;
  __device__ __forceinline__ void init(float4 pi, f3 v) {
    xi = xyz(pi);
    ri = pi.w;
    vi = v;
    om = mk(0.f, 0.f, 0.f);
    nm = mk(0.f, 0.f, 0.f);
    vu = mk(0.f, 0.f, 0.f);
    cs = mk(0.f, 0.f, 0.f);
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 pj, float4 vj) {
    Pair q = make_pair_of(xi - xyz(pj));
    f3 vd = xyz(vj) - vi;
    const float inv_rj = frcp_fast(pj.w);
    const float volume = p.m * inv_rj;
    f3 gw = spiky_p(p, q);
    om = om + volume * cross3(vd, gw);
    nm = nm + volume * gw;
    vu = vu + (poly6_p(p, q) * inv_rj) * vd;
    const float kij = p.two_rho0 * frcp_fast(ri + pj.w);
    cs = cs + kij * (p.m * cohesion_p(p, q));
  }
};
// ... and the XSPH pass the vorticity-force eta and the curvature part.
struct XsphSplitSum {
  f3 xi, ni, eta, cv;
  float ri;
  __device__ __forceinline__ void init(float4 pi, f3 n) {
    xi = xyz(pi);
    ri = pi.w;
    ni = n;
    eta = mk(0.f, 0.f, 0.f);
    cv = mk(0.f, 0.f, 0.f);
  }
  __device__ __forceinline__ void add(const SimParams& p, float4 pj, float4 nj) {  // nj: (normal_j, |omega_j|)
    Pair q = make_pair_of_lib(xi - xyz(pj));
    eta = eta + (nj.w * frcp_fast(pj.w)) * spiky_p(p, q);
    const float kij = p.two_rho0 * frcp_fast(ri + pj.w);
    cv = cv + kij * (ni - xyz(nj));
  }
};

// LambdaCalculation (pressureConstrain.ts:31-85).  Writes xl[t] = (x*, lambda):
// the next pass gathers a neighbour's position and multiplier in one load.
//   kMode 0: the reference pass.
//   kMode 2: the reference pass + the density error statistics (a.stats).
//   kMode 1: also writes the learned start's 8 features at x*_0 (density
//            error, previous multiplier, neighbour count, |v'| dt/h, -div(v') dt
//            by continuity, boundary SDF/h, boundary volume/V, substep index;
//            v' = (x* - x)/dt) for trace capture.

// The rest of LambdaCalculation after the neighbour sums: the boundary
// pseudo-particle, the constraint and the multiplier; writes xl[t] and the
// optional multiplier sum / features (nbr: the neighbour count); returns sum W.
template <int kMode, bool kC>
__device__ __forceinline__ float lambda_finish(const SimParams& p, int have_field, const float4* bdata, float4* xl,
                                               const SolverAux& a, uint32_t t, const LamSum& acc, uint32_t nbr) {
  constexpr bool kFeat = kMode >= 1;
  const f3 xi = acc.xi;
  f3 grad = acc.grad;
  float sum2 = acc.sum2, dens = acc.dens;
  const float vsum = dens;
  dens = dens * p.V;
  const float dens_fluid = dens;
  grad = p.V * grad;
  sum2 = sum2 * p.V2;
  float vb = 0.0f;
  if (have_field) {
    float4 bd = ldo<kC>(bdata + t);
    vb = bd.w;
    if (bd.w != 0.0f) {
      Pair q = make_pair_of(xi - xyz(bd));
      f3 gk = bd.w * spiky_p(p, q);
      grad = grad + gk;
      dens = dens + bd.w * poly6_p(p, q);
    }
  }
  float c = fmaxf(0.0f, dens - 1.0f);
  float s = dot3(grad, grad) + sum2;
  float lam = fdiv(-c, s + p.lambda_eps);
  xl[t] = f4(xi, lam);
  if (a.lam_sum) a.lam_sum[t] = a.lam_first ? lam : a.lam_sum[t] + lam;
  if (kFeat) {
    const float4 xo = a.pos[t];
    const f3 vi = p.inv_dt * (xi - xyz(xo));
    float sd = a.bsdf ? fminf(a.bsdf[t], 2.0f * p.h) : 2.0f * p.h;
    a.feat[2 * t] = make_float4(dens - 1.0f, a.lam_prev ? a.lam_prev[t] : 0.0f, (float)nbr, len3(vi) * p.dt / p.h);
    a.feat[2 * t + 1] = make_float4(divergence_feature(p, xo, dens_fluid), sd / p.h, vb / p.V, a.substep_index);
  }
  return vsum;
}

template <int kMode, bool kC>
__device__ __forceinline__ float lambda_slot(const SimParams& p, int have_field, const float4* bdata, const float4* xs,
                                            uint32_t max_nbr, const uint32_t* __restrict__ nbr_cnt,
                                            const uint32_t* __restrict__ nbr_list, float4* xl, const SolverAux& a,
                                            uint32_t t) {
  uint32_t b, e;
  list_slice(max_nbr, nbr_cnt, t, b, e);
  LamSum acc;
  acc.init(xyz(ldo<kC>(xs + t)));
  for_each_neighbor<kC>(nbr_list, b, e, xs, [&](uint32_t, float4 xj) { acc.add(p, xj); });
  return lambda_finish<kMode, kC>(p, have_field, bdata, xl, a, t, acc, e);
}

template <int kMode, bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_lambda(SimParams p, int have_field, const float4* __restrict__ bdata,
                                                const float4* __restrict__ xs, uint32_t max_nbr,
                                                const uint32_t* __restrict__ nbr_cnt,
                                                const uint32_t* __restrict__ nbr_list,
                                                float4* __restrict__ xl, SolverAux a) {
  if (a.guard && *a.guard == 0) return;
  // kMode 2: also the density error at these positions into a.stats (the
  // adaptive iteration's test; the same quantity AttributeUpdate reports)
  constexpr bool kStats = kMode == 2;
  unsigned cmax = 0u, csum = 0u, ccnt = 0u;
  PBF_SLOTS(t, p.n) {
    if (!iter_active(scene_of<kBatch>(a.tab, t), a.iter)) continue;
    const float vsum =
        lambda_slot<kStats ? 0 : kMode, false>(p, have_field, bdata, xs, max_nbr, nbr_cnt, nbr_list, xl, a, t);
    if constexpr (kStats) compression_add(cmax, csum, ccnt, vsum * p.V);
  }
  if constexpr (kStats) compression_flush(a.stats, cmax, csum, ccnt);
}

// ConstrainSolve + ConstrainApply: x*_new = clamp(x* + 0.5 * dp) into the other
// buffer; (x*_j, lambda_j) come packed from the lambda pass.  A scene of a
// batch that has finished its iterations copies its x* through (a.xs_in), so
// every scene ends in the same buffer.
// Position correction of slot t from the packed (x*, lambda) records; xi
// receives the slot's own x*.
// The rest of ConstrainSolve after the neighbour sum: the boundary term and
// the 0.5 factor (pressureConstrain.ts:142-158).
template <bool kC>
__device__ __forceinline__ f3 deltap_finish(const SimParams& p, int have_field, const float4* bdata, uint32_t t,
                                            const DpSum& acc) {
  const f3 xi = acc.xi;
  const float li = acc.li;
  f3 pu = p.V * acc.pu;
  if (have_field) {
    float4 bd = ldo<kC>(bdata + t);
    if (bd.w != 0.0f) {
      Pair q = make_pair_of(xi - xyz(bd));
      pu = pu + (bd.w * li) * spiky_p(p, q);
    }
  }
  return 0.5f * pu;
}

template <bool kC>
__device__ __forceinline__ f3 deltap_slot(const SimParams& p, int have_field, const float4* xl, const float4* bdata,
                                          uint32_t max_nbr, const uint32_t* __restrict__ nbr_cnt,
                                          const uint32_t* __restrict__ nbr_list, uint32_t t, f3& xi) {
  uint32_t b, e;
  list_slice(max_nbr, nbr_cnt, t, b, e);
  DpSum acc;
  acc.init(ldo<kC>(xl + t));
  for_each_neighbor<kC>(nbr_list, b, e, xl, [&](uint32_t, float4 xj) { acc.add(p, xj); });
  xi = acc.xi;
  return deltap_finish<kC>(p, have_field, bdata, t, acc);
}

template <bool kBatch, bool kLoop>
__global__ void __launch_bounds__(256) k_deltap(SimParams p, SolverAux a, int have_field,
                                                const float4* __restrict__ xl, const float4* __restrict__ bdata,
                                                uint32_t max_nbr, const uint32_t* __restrict__ nbr_cnt,
                                                const uint32_t* __restrict__ nbr_list,
                                                float4* __restrict__ xs_out, float4* __restrict__ dp_out) {
  if (a.guard && *a.guard == 0) return;
  const bool skip = a.need && *a.need == 0;  // the adaptive test found this iteration unneeded
  PBF_SLOTS(t, p.n) {
    if (skip || !iter_active(scene_of<kBatch>(a.tab, t), a.iter)) {
      xs_out[t] = a.xs_in[t];
      continue;
    }
    f3 xi;
    const f3 dp = deltap_slot<false>(p, have_field, xl, bdata, max_nbr, nbr_cnt, nbr_list, t, xi);
    if (dp_out) dp_out[t] = f4(dp, 0.0f);
    f3 xn;
    if constexpr (kBatch) {  // the scene's own domain (looked up after the loop: no registers held across it)
      SimParams ps = p;
      scene_domain(ps, scene_of<kBatch>(a.tab, t));
      xn = clamp_rand(ps, xi + dp);
    } else {
      xn = clamp_rand(p, xi + dp);
    }
    xs_out[t] = f4(xn, 0.0f);
    if (a.band.list) band_mark<kBatch>(p, a.band, a.tab, t, xn);
  }
}

// The rest of AttributeUpdate: rho = m sum W, v = (x* - x) / dt, x <- (x*, rho).
template <bool kC>
__device__ __forceinline__ float density_finish(const SimParams& p, float4* pos, float4* vel, uint32_t t,
                                                const DensSum& acc) {
  const f3 xi = acc.xi;
  const float vsum = acc.dens;
  const float dens = acc.dens * p.m;
  f3 xo = xyz(ldo<kC>(pos + t));
  vel[t] = f4(p.inv_dt * (xi - xo), 0.0f);
  pos[t] = f4(xi, dens);
  return vsum;
}

// AttributeUpdate of slot t; returns sum W (fluid only).
template <bool kC>
__device__ __forceinline__ float density_slot(const SimParams& p, const float4* xs, uint32_t max_nbr,
                                              const uint32_t* __restrict__ nbr_cnt,
                                              const uint32_t* __restrict__ nbr_list, float4* pos, float4* vel,
                                              uint32_t t) {
  uint32_t b, e;
  list_slice(max_nbr, nbr_cnt, t, b, e);
  DensSum acc;
  acc.init(xyz(ldo<kC>(xs + t)));
  for_each_neighbor<kC>(nbr_list, b, e, xs, [&](uint32_t, float4 xj) { acc.add(p, xj); });
  return density_finish<kC>(p, pos, vel, t, acc);
}

// AttributeUpdate: rho = m * sum W (fluid only), v = (x* - x) / dt, x <- (x*, rho).
// With a.stats, also the per-step density error (compression
// max(0, rho/rho0 - 1) = max(0, V sum W - 1)): reduced over the CTA in shared
// memory, one set of atomics per CTA.
template <bool kLoop>
__global__ void __launch_bounds__(256) k_density_velocity(SimParams p, SolverAux a, const float4* __restrict__ xs,
                                                          uint32_t max_nbr,
                                                          const uint32_t* __restrict__ nbr_cnt,
                                                          const uint32_t* __restrict__ nbr_list,
                                                          float4* __restrict__ pos, float4* __restrict__ vel) {
  if (a.guard && *a.guard == 0) return;
  unsigned cmax = 0u, csum = 0u, ccnt = 0u;
  PBF_SLOTS(t, p.n) {
    const float vsum = density_slot<false>(p, xs, max_nbr, nbr_cnt, nbr_list, pos, vel, t);
    if (a.stats) compression_add(cmax, csum, ccnt, vsum * p.V);
  }
  if (a.stats) compression_flush(a.stats, cmax, csum, ccnt);
}

// The learned start's fallback: when *guard is set, restores x and x*_0 and
// runs the plain solve (boundary, lambda, delta-p per iteration, the
// multiplier sum restarted) and AttributeUpdate, with grid-wide barriers
// between the phases; otherwise returns at once, so an unneeded fallback
// costs one launch.  Launched cooperatively with at most one resident wave of
// CTAs.  Positions and multipliers change between phases inside the kernel,
// so their loads are L2-coherent (kC = true); the arithmetic is the pass
// kernels' own (the same slot bodies).
__global__ void __launch_bounds__(256) k_fallback_solve(FallbackArgs A) {
  if (*A.guard == 0) return;
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const uint32_t n = A.p.n, stride = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t t = t0; t < n; t += stride) {
    A.pos[t] = __ldcg(A.pos_old + __ldg(A.perm + t));
    const float4 x0 = __ldcg(A.xs_save + t);
    A.xs0[t] = make_float4(x0.x, x0.y, x0.z, 0.0f);
  }
  grid.sync();
  int a = 0;
  for (int it = 0; it < A.iters; ++it) {
    float4* cur = a ? A.xs1 : A.xs0;
    float4* nxt = a ? A.xs0 : A.xs1;
    if (A.f.loaded) {
      for (uint32_t t = t0; t < n; t += stride)
        boundary_slot<true>(A.p, A.f, A.sdf, A.vol, A.bflag, cur, A.bdata, nullptr, t);
      grid.sync();
    }
    SolverAux al{};
    al.lam_sum = A.lam_sum;
    al.lam_first = it == 0 ? 1 : 0;
    for (uint32_t t = t0; t < n; t += stride)
      lambda_slot<0, true>(A.p, A.f.loaded, A.bdata, cur, A.max_nbr, A.nbr_cnt, A.nbr_list, A.xl, al, t);
    grid.sync();
    for (uint32_t t = t0; t < n; t += stride) {
      f3 xi;
      const f3 dp = deltap_slot<true>(A.p, A.f.loaded, A.xl, A.bdata, A.max_nbr, A.nbr_cnt, A.nbr_list, t, xi);
      nxt[t] = f4(clamp_rand(A.p, xi + dp), 0.0f);
    }
    grid.sync();
    a = 1 - a;
  }
  float4* fin = A.final_buf ? A.xs1 : A.xs0;
  if (a != A.final_buf) {
    const float4* src = a ? A.xs1 : A.xs0;
    for (uint32_t t = t0; t < n; t += stride) fin[t] = __ldcg(src + t);
    grid.sync();
  }
  for (uint32_t t = t0; t < n; t += stride)
    density_slot<true>(A.p, fin, A.max_nbr, A.nbr_cnt, A.nbr_list, A.pos, A.vel, t);
}

// Writes (omega, |omega|) and (h n, |omega|): the normal's w repeats |omega|
// so XSPH gathers one float4 per neighbour fewer.
__device__ __forceinline__ void vorticity_finish(const SimParams& p, float4* omega, float4* normal, uint32_t t,
                                                 const VortSum& acc) {
  const float wl = len3(acc.om);
  omega[t] = f4(acc.om, wl);
  normal[t] = f4(p.h * acc.nm, wl);
}
// XSPH's output a from its sums (XSPH.ts:82-89).
__device__ __forceinline__ void xsph_finish(const SimParams& p, float4* acc_out, uint32_t t, const XsphSum& s,
                                            f3 wi) {
  float el = len3(s.eta);
  f3 en = (el > 0.0f) ? divs(s.eta, el) : mk(0.f, 0.f, 0.f);
  float sx = p.xsph * p.inv_dt * p.m;
  f3 av = (sx * s.vu + p.vorticity * cross3(en, wi)) + p.tension * s.ten;
  acc_out[t] = f4(av, 0.0f);
}
__device__ __forceinline__ void vorticity_split_finish(const SimParams& p, float4* omega, float4* normal, float4* visc,
                                                       float4* coh_sum, uint32_t t, const VortSplitSum& s) {
  const float wl = len3(s.om);
  omega[t] = f4(s.om, wl);
  normal[t] = f4(p.h * s.nm, wl);
  visc[t] = f4(s.vu, 0.0f);
  coh_sum[t] = f4(s.cs, 0.0f);
}
__device__ __forceinline__ void xsph_split_finish(const SimParams& p, float4* acc_out, uint32_t t,
                                                  const XsphSplitSum& s, f3 wi, float4 visc_t, float4 coh_t) {
  const f3 ten = mk(0.f, 0.f, 0.f) - (xyz(coh_t) + s.cv);
  float el = len3(s.eta);
  f3 en = (el > 0.0f) ? divs(s.eta, el) : mk(0.f, 0.f, 0.f);
  float sx = p.xsph * p.inv_dt * p.m;
  f3 av = (sx * xyz(visc_t) + p.vorticity * cross3(en, wi)) + p.tension * ten;
  acc_out[t] = f4(av, 0.0f);
}

// VorticityConfinement: omega_i and the Akinci normal n_i.
template <bool kLoop>
__global__ void __launch_bounds__(256) k_vorticity(SimParams p, const float4* __restrict__ pos,
                                                   const float4* __restrict__ vel,
                                                   uint32_t max_nbr,
                                                   const uint32_t* __restrict__ nbr_cnt,
                                                   const uint32_t* __restrict__ nbr_list,
                                                   float4* __restrict__ omega, float4* __restrict__ normal) {
  PBF_SLOTS(t, p.n) {
    uint32_t b, e;
    list_slice(max_nbr, nbr_cnt, t, b, e);
    VortSum acc;
    acc.init(xyz(pos[t]), xyz(vel[t]));
    for_each_neighbor(nbr_list, b, e, pos, [&](uint32_t j, float4 pj) { acc.add(p, pj, __ldg(vel + j)); });
    vorticity_finish(p, omega, normal, t, acc);
  }
}

// XSPH viscosity + vorticity confinement force + Akinci surface tension -> a.
template <bool kLoop>
__global__ void __launch_bounds__(256, 4) k_xsph(SimParams p, const float4* __restrict__ pos,
                                                 const float4* __restrict__ vel, const float4* __restrict__ omega,
                                                 const float4* __restrict__ normal,
                                                 uint32_t max_nbr,
                                                 const uint32_t* __restrict__ nbr_cnt,
                                                 const uint32_t* __restrict__ nbr_list,
                                                 float4* __restrict__ acc) {
  PBF_SLOTS(t, p.n) {
    uint32_t b, e;
    list_slice(max_nbr, nbr_cnt, t, b, e);
    XsphSum s;
    s.init(pos[t], xyz(vel[t]), xyz(normal[t]));
    for_each_neighbor(nbr_list, b, e, pos,
                      [&](uint32_t j, float4 pj) { s.add(p, pj, __ldg(vel + j), __ldg(normal + j)); });
    xsph_finish(p, acc, t, s, xyz(omega[t]));
  }
}

// Fast mode splits XSPH's neighbour sum over the two post-solve passes: the
// vorticity pass, which already gathers x_j, rho_j and v_j, also sums the
// viscosity term u = sum W (v_j - v_i) / rho_j and the cohesion part of the
// surface tension c = sum K_ij m C(x_ij); the XSPH pass then gathers only
// (x_j, rho_j) and (n_j, |omega_j|) for eta and the curvature part.  The
// result is the reference's formula with the tension sum split in two (a
// different rounding order), so exact mode keeps the single-pass form.
template <bool kLoop>
__global__ void __launch_bounds__(256, 4) k_vorticity_split(SimParams p, const float4* __restrict__ pos,
                                                            const float4* __restrict__ vel, uint32_t max_nbr,
                                                            const uint32_t* __restrict__ nbr_cnt,
                                                            const uint32_t* __restrict__ nbr_list,
                                                            float4* __restrict__ omega, float4* __restrict__ normal,
                                                            float4* __restrict__ visc, float4* __restrict__ coh_sum) {
  PBF_SLOTS(t, p.n) {
    uint32_t b, e;
    list_slice(max_nbr, nbr_cnt, t, b, e);
    VortSplitSum s;
    s.init(pos[t], xyz(vel[t]));
    for_each_neighbor(nbr_list, b, e, pos, [&](uint32_t j, float4 pj) { s.add(p, pj, __ldg(vel + j)); });
    vorticity_split_finish(p, omega, normal, visc, coh_sum, t, s);
  }
}

template <bool kLoop>
__global__ void __launch_bounds__(256) k_xsph_split(SimParams p, const float4* __restrict__ pos,
                                                    const float4* __restrict__ omega,
                                                    const float4* __restrict__ normal,
                                                    const float4* __restrict__ visc,
                                                    const float4* __restrict__ coh_sum, uint32_t max_nbr,
                                                    const uint32_t* __restrict__ nbr_cnt,
                                                    const uint32_t* __restrict__ nbr_list, float4* __restrict__ acc) {
  PBF_SLOTS(t, p.n) {
    uint32_t b, e;
    list_slice(max_nbr, nbr_cnt, t, b, e);
    XsphSplitSum s;
    s.init(pos[t], xyz(normal[t]));
    for_each_neighbor2(nbr_list, b, e, pos, normal, [&](uint32_t, float4 pj, float4 nj) { s.add(p, pj, nj); });
    xsph_split_finish(p, acc, t, s, xyz(omega[t]), visc[t], coh_sum[t]);
  }
}

#include "pbf_cellblock.cuh"

// Launch table for this precision variant: [batch][persistent] pass sets.
template <bool B, bool P>
void fill_set(PassSet* ps) {
  ps->predict = k_predict<B, P>;
  ps->nbr_build = k_nbr_build<B, P>;
  ps->nbr_build2 = k_nbr_build2<B, P>;
  ps->nbr_build_warp = k_nbr_build_warp<B, P>;
  ps->band = k_band<B, P>;
  ps->boundary_band = k_boundary_band<B>;
  ps->lambda = k_lambda<0, B, P>;
  ps->lambda_feat = B ? nullptr : k_lambda<1, false, P>;
  ps->lambda_stats = B ? nullptr : k_lambda<2, false, P>;
  ps->nbr_build_feat = B ? nullptr : k_nbr_build_feat<P>;
  ps->deltap = k_deltap<B, P>;
  ps->density_velocity = k_density_velocity<P>;
  ps->vorticity = k_vorticity<P>;
  ps->xsph = k_xsph<P>;
  if constexpr (kFast) {
    ps->vorticity_split = k_vorticity_split<P>;
    ps->xsph_split = k_xsph_split<P>;
  } else {
    ps->vorticity_split = nullptr;
    ps->xsph_split = nullptr;
  }
}

void fill_pass_table(PassTable* tbl) {
  tbl->fallback = k_fallback_solve;
  tbl->nbr_count = k_nbr_count;
  tbl->nbr_list = k_nbr_list;
  fill_set<false, false>(&tbl->set[0][0]);
  fill_set<false, true>(&tbl->set[0][1]);
  fill_set<true, false>(&tbl->set[1][0]);
  fill_set<true, true>(&tbl->set[1][1]);
  tbl->cb_build = k_cb_build<false>;
  tbl->cb_build_feat = k_cb_build<true>;
  fill_cb_set<kMemMask>(&tbl->cb[kMemMask]);
  fill_cb_set<kMemTest>(&tbl->cb[kMemTest]);
}

}  // namespace PBF_NS
}  // namespace pbf
