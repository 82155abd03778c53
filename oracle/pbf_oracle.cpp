// pbf_oracle.cpp — CPU restatement of the reference PBF substep.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
// this file; only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
// load it, to check the GPU results or to time the method on the host.
//
// It restates, pass by pass, the WGSL of WebGPU-Fluid-Simulation in the
// order PBF.run encodes them (src/simulator/PBF/PBF.ts:398-448), on the
// particle-id layout the reference uses (no reordering of particle data):
//   TimeIntegration      src/simulator/PBF/shader/timeIntegration.ts:20-32
//   boundary_rand        src/simulator/PBF/shader/common.ts:43-67
//   ParticleInsert       src/simulator/neighbor/neighborShader.ts:24-32
//   cell scan            src/simulator/neighbor/scanShader.ts:16-107 (exact exclusive sum)
//   CountingSort         src/simulator/neighbor/neighborShader.ts:49-60
//   NeighborCount/List   src/simulator/neighbor/neighborShader.ts:101-246
//   BoundaryVolume       src/simulator/PBF/shader/boundaryVolume.ts:26-57
//   shape functions      src/simulator/boundary/discreteFieldShader.ts:15-192
//   LambdaCalculation    src/simulator/PBF/shader/pressureConstrain.ts:31-85
//   ConstrainSolve       src/simulator/PBF/shader/pressureConstrain.ts:109-158
//   ConstrainApply       src/simulator/PBF/shader/pressureConstrain.ts:172-179
//   AttributeUpdate      src/simulator/PBF/shader/attributeUpdate.ts:25-59
//   VorticityConfinement src/simulator/PBF/shader/vorticityConfinement.ts:25-66
//   XSPH                 src/simulator/PBF/shader/XSPH.ts:31-92
//   kernels              src/simulator/PBF/shader/common.ts:1-40
// The "ParticleInsert" atomicAdd order of the reference is whatever the GPU
// returns; this restatement defines it as sequential execution, i.e. ranks
// stable by particle id.
//
// Two precisions: R = float mirrors the reference's f32 arithmetic with the
// same operation order (compiled with -ffp-contract=off so no FMA is formed),
// R = double is an FP64 replica of one step.
//
// Parity status: the reference is TypeScript + WGSL and cannot run here, and
// it ships no golden vectors.  This restatement is pinned against the
// reference's own CPU self-checks (exact scan, brute-force neighbour sets,
// brute-force density, exclusiveScan.ts:193-199, neighborSearch.ts:345-372,
// PBF.ts:96-116) and against the analytic SDF of the reference's
// domain_boundary.cdm fixture; the float passes themselves are parity
// unpinned against a running reference.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/pbf_gb300.h"

namespace {

template <typename R>
struct V3 {
  R x, y, z;
};
template <typename R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> inline V3<R> add(V3<R> a, V3<R> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename R> inline V3<R> sub(V3<R> a, V3<R> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename R> inline V3<R> scl(R s, V3<R> a) { return v3(s * a.x, s * a.y, s * a.z); }
template <typename R> inline R dot3(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> inline R len3(V3<R> a) { return std::sqrt(dot3(a, a)); }
template <typename R> inline V3<R> cross3(V3<R> a, V3<R> b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename R> inline V3<R> divs(V3<R> a, R s) { return v3(a.x / s, a.y / s, a.z / s); }

// Constants the reference bakes in as WGSL consts / override constants.
template <typename R>
struct Consts {
  R h, h2, half_h, poly6, spiky, coh, coh_bias;
  R V, V2, m, two_rho0, rho0, dt, inv_dt, lambda_eps, r, jitter, gy;
  R dmin[3], dmax[3], inv_cell[3];
  int dim[3];
};

template <typename R>
Consts<R> make_consts(const pbf_config& c) {
  const double PI = 3.14159265358979323846;
  Consts<R> k;
  double h = c.kernel_radius, r = c.particle_radius;
  k.h = (R)h;
  k.h2 = (R)(h * h);
  k.half_h = (R)(0.5 * h);
  k.poly6 = (R)(315.0 / (64.0 * PI * std::pow(h, 9)));
  k.spiky = (R)(-45.0 / (PI * std::pow(h, 6)));
  k.coh = (R)(32.0 / (PI * std::pow(h, 9)));
  k.coh_bias = (R)(-std::pow(h, 6) / 64.0);
  double diam = 2.0 * r;
  double V = 0.9 * diam * diam * diam;  // SPH.ts:49
  k.V = (R)V;
  k.V2 = (R)(V * V);                    // PBF.ts:328
  k.m = (R)(V * (double)c.rest_density);  // SPH.ts:50
  k.rho0 = (R)c.rest_density;
  k.two_rho0 = (R)(2.0 * (double)c.rest_density);
  k.dt = (R)c.time_step;
  k.inv_dt = (R)(1.0 / (double)c.time_step);
  k.lambda_eps = (R)c.lambda_eps;
  k.r = (R)r;
  k.jitter = (R)c.wall_jitter;
  k.gy = (R)(-(double)c.options.gravity);
  for (int a = 0; a < 3; ++a) {
    k.dmin[a] = (R)c.domain_min[a];
    k.dmax[a] = (R)c.domain_max[a];
    double ext = (double)c.domain_max[a] - (double)c.domain_min[a];
    int d = (int)c.grid_dim[a];
    if (d == 0) d = (int)std::ceil(ext / h);
    k.dim[a] = d;
    k.inv_cell[a] = (R)((double)d / ext);
  }
  return k;
}

// ---- kernels (common.ts:1-40) -------------------------------------------------
template <typename R>
inline R poly6(const Consts<R>& k, R rl) {
  R t = k.h2 - rl * rl;
  R x = (rl <= k.h) ? (t * t * t) : (R)0;
  return k.poly6 * x;
}
template <typename R>
inline V3<R> spiky_grad(const Consts<R>& k, V3<R> d, R rl) {
  R t = k.h - rl;
  R x = (rl <= k.h) ? (t * t) : (R)0;
  V3<R> n = (rl > (R)0) ? divs(d, rl) : v3<R>(0, 0, 0);
  return scl(k.spiky * x, n);
}
template <typename R>
inline V3<R> cohesion(const Consts<R>& k, V3<R> d, R rl) {
  R a = k.h - rl;
  R a3 = a * a * a;
  R b3 = rl * rl * rl;
  R t = a3 * b3;
  R res = (rl > k.half_h) ? t : std::fma((R)2, t, k.coh_bias);
  res = (rl <= k.h) ? res : (R)0;
  V3<R> n = (rl > (R)0) ? divs(d, rl) : v3<R>(0, 0, 0);
  return scl(k.coh * res, n);
}

// ---- wall clamp with jitter (common.ts:43-67) -----------------------------------
inline uint32_t f2u(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
// Integer hash of two float bit patterns -> [0, 1).  The mixer is the
// "lowbias32" finaliser published by C. Wellons (hash-prospector).
inline uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
inline float hash2(float a, float b) {
  uint32_t h = mix32(f2u(a) ^ mix32(f2u(b) + 0x9e3779b9U));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}
inline float fractf_(float x) { return x - std::floor(x); }
inline float sinhash(float a, float b) {
  float d = a * 12.9898f + b * 78.233f;
  return fractf_(std::sin(d) * 43758.5453f);
}

template <typename R>
inline V3<R> clamp_rand(const Consts<R>& k, V3<R> p, int mode) {
  // random3: components hash (p.y,p.z), (p.x,p.z), (p.x,p.y), computed in f32
  float px = (float)p.x, py = (float)p.y, pz = (float)p.z;
  float r0, r1, r2;
  if (mode == PBF_JITTER_SIN) {
    r0 = sinhash(py, pz);
    r1 = sinhash(px, pz);
    r2 = sinhash(px, py);
  } else {
    r0 = hash2(py, pz);
    r1 = hash2(px, pz);
    r2 = hash2(px, py);
  }
  V3<R> rv = scl(k.jitter, v3<R>((R)r0, (R)r1, (R)r2));
  V3<R> lo = v3(k.dmin[0] + rv.x, k.dmin[1] + rv.y, k.dmin[2] + rv.z);
  V3<R> hi = v3(k.dmax[0] - rv.x, k.dmax[1] - rv.y, k.dmax[2] - rv.z);
  return v3(std::max(std::min(p.x, hi.x), lo.x), std::max(std::min(p.y, hi.y), lo.y),
            std::max(std::min(p.z, hi.z), lo.z));
}

// ---- volume map (discreteFieldShader.ts:1-192) ----------------------------------
struct Field {
  bool loaded = false;
  int res[3] = {0, 0, 0};
  double origin[3] = {0, 0, 0}, extent[3] = {1, 1, 1};
  std::vector<float> sdf, vol;
};

// Node index of the 32 nodes of cell (i,j,k), in the order
// corners(8) x-edges(8) y-edges(8) z-edges(8) matching the weight order below.
inline void cell_nodes(const int* G, int i, int j, int k, bool quirk_vol, long* idx) {
  const long nx = G[0], ny = G[1], nz = G[2];
  const long nc = (nx + 1) * (ny + 1) * (nz + 1);
  const long nex = 2 * nx * (ny + 1) * (nz + 1);
  const long ney = (nx + 1) * 2 * ny * (nz + 1);
  auto C = [&](long kk, long jj, long ii) { return (kk * (ny + 1) + jj) * (nx + 1) + ii; };
  auto EX = [&](long kk, long jj, long e) { return nc + (kk * (ny + 1) + jj) * (2 * nx) + e; };
  auto EY = [&](long ii, long kk, long e) { return nc + nex + (ii * (nz + 1) + kk) * (2 * ny) + e; };
  auto EZ = [&](long jj, long ii, long e) { return nc + nex + ney + (jj * (nx + 1) + ii) * (2 * nz) + e; };
  long i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
  // group 0/1: corners at k / k+1
  idx[0] = C(k, j, i); idx[1] = C(k, j, i + 1); idx[2] = C(k, j + 1, i); idx[3] = C(k, j + 1, i + 1);
  idx[4] = C(k + 1, j, i); idx[5] = C(k + 1, j, i + 1); idx[6] = C(k + 1, j + 1, i); idx[7] = C(k + 1, j + 1, i + 1);
  // group 2/3: x-edges at j / j+1
  idx[8] = EX(k, j, i2); idx[9] = EX(k, j, i2 + 1); idx[10] = EX(k + 1, j, i2); idx[11] = EX(k + 1, j, i2 + 1);
  idx[12] = EX(k, j + 1, i2); idx[13] = EX(k, j + 1, i2 + 1); idx[14] = EX(k + 1, j + 1, i2); idx[15] = EX(k + 1, j + 1, i2 + 1);
  // group 4/5: y-edges at k / k+1
  idx[16] = EY(i, k, j2); idx[17] = EY(i, k, j2 + 1); idx[18] = EY(i + 1, k, j2); idx[19] = EY(i + 1, k, j2 + 1);
  idx[20] = EY(i, k + 1, j2); idx[21] = EY(i, k + 1, j2 + 1); idx[22] = EY(i + 1, k + 1, j2); idx[23] = EY(i + 1, k + 1, j2 + 1);
  // group 6/7: z-edges at i / i+1
  idx[24] = EZ(j, i, k2); idx[25] = EZ(j, i, k2 + 1); idx[26] = EZ(j + 1, i, k2); idx[27] = EZ(j + 1, i, k2 + 1);
  idx[28] = EZ(j, i + 1, k2); idx[29] = EZ(j, i + 1, k2 + 1); idx[30] = EZ(j + 1, i + 1, k2); idx[31] = EZ(j + 1, i + 1, k2 + 1);
  if (quirk_vol) {
    // discreteFieldShader.ts:146-147 reads x-edge (k+1, ., i2) twice and
    // :152-153 reads z-edge (., ., k2) in place of k2+1.
    idx[11] = idx[10];
    idx[15] = idx[14];
    idx[25] = idx[24];
    idx[27] = idx[26];
    idx[29] = idx[28];
    idx[31] = idx[30];
  }
}

// Shape functions of the 32-node cubic serendipity hexahedron at local
// coordinates s in [-1,1]^3 and their gradients.  Corner nodes:
//   N = (1/64)(1+-x)(1+-y)(1+-z)(9(x^2+y^2+z^2) - 19)
// x-edge nodes at x = -1/3 (e=0) and +1/3 (e=1):
//   N = (9/64)(1-x^2)(1 + 3 sigma x)(1+-y)(1+-z), sigma = -1 / +1
// and cyclically for y- and z-edges.
template <typename R>
inline void shape32(V3<R> s, R* N, V3<R>* dN) {
  const R c1 = (R)(1.0 / 64.0), c9 = (R)(9.0 / 64.0);
  R x = s.x, y = s.y, z = s.z;
  R x2 = x * x, y2 = y * y, z2 = z * z;
  R r2 = x2 + y2 + z2;
  R mx = (R)1 - x, px = (R)1 + x, my = (R)1 - y, py = (R)1 + y, mz = (R)1 - z, pz = (R)1 + z;
  // corners: order (i,j,k),(i+1,j,k),(i,j+1,k),(i+1,j+1,k), then k+1
  R fx[2] = {mx, px}, fy[2] = {my, py}, fz[2] = {mz, pz};
  R sx[2] = {(R)-1, (R)1};
  R q = (R)9 * r2 - (R)19;
  for (int c = 0; c < 8; ++c) {
    int a = c & 1, b = (c >> 1) & 1, e = (c >> 2) & 1;
    R lx = fx[a], ly = fy[b], lz = fz[e];
    R p = lx * ly * lz;
    N[c] = c1 * p * q;
    dN[c].x = c1 * (sx[a] * ly * lz * q + p * ((R)18 * x));
    dN[c].y = c1 * (sx[b] * lx * lz * q + p * ((R)18 * y));
    dN[c].z = c1 * (sx[e] * lx * ly * q + p * ((R)18 * z));
  }
  // edges: for axis u with the two other axes (v, w) in the node orders of cell_nodes
  //   x-edges: (e, k-side) for j, then j+1   -> v = y (group), w = z (inner)
  //   y-edges: (e, i-side) for k, then k+1   -> v = z (group), w = x (inner)
  //   z-edges: (e, j-side) for i, then i+1   -> v = x (group), w = y (inner)
  R su[3] = {x, y, z};
  R fsq[3] = {(R)1 - x2, (R)1 - y2, (R)1 - z2};
  R fm[3] = {mx, my, mz}, fp[3] = {px, py, pz};
  for (int ax = 0; ax < 3; ++ax) {
    int av = (ax + 1) % 3, aw = (ax + 2) % 3;  // x:(y,z) y:(z,x) z:(x,y)
    R u = su[ax];
    for (int n = 0; n < 8; ++n) {
      int e = n & 1, wside = (n >> 1) & 1, vside = (n >> 2) & 1;
      R sg = e ? (R)1 : (R)-1;
      R lin = (R)1 + (R)3 * sg * u;        // 1 - 3u or 1 + 3u
      R fv = vside ? fp[av] : fm[av];
      R fw = wside ? fp[aw] : fm[aw];
      R sv = vside ? (R)1 : (R)-1;
      R sw = wside ? (R)1 : (R)-1;
      R g = fsq[ax] * lin;
      R vw = fv * fw;
      R dn_u = c9 * vw * ((R)-2 * u * lin + (R)3 * sg * fsq[ax]);
      R dn_v = c9 * g * (sv * fw);
      R dn_w = c9 * g * (fv * sw);
      int slot = 8 + ax * 8 + n;
      N[slot] = c9 * g * vw;
      R d3[3];
      d3[ax] = dn_u;
      d3[av] = dn_v;
      d3[aw] = dn_w;
      dN[slot] = v3(d3[0], d3[1], d3[2]);
    }
  }
}

// Sum of the 32 products, in the reduction order of the reference
// (discreteFieldShader.ts:155-159): per group a 4-term dot, groups g and g+4
// added, then the four pair sums left to right.
template <typename R>
inline R sum32(const R* w, const R* val) {
  R d[8];
  for (int g = 0; g < 8; ++g)
    d[g] = w[4 * g] * val[4 * g] + w[4 * g + 1] * val[4 * g + 1] + w[4 * g + 2] * val[4 * g + 2] +
           w[4 * g + 3] * val[4 * g + 3];
  R s0 = d[0] + d[4], s1 = d[1] + d[5], s2 = d[2] + d[6], s3 = d[3] + d[7];
  return s0 + s1 + s2 + s3;
}
template <typename R>
inline V3<R> sum32v(const V3<R>* w, const R* val) {
  V3<R> g[8];
  for (int q = 0; q < 8; ++q) {
    V3<R> a = scl(val[4 * q], w[4 * q]);
    a = add(a, scl(val[4 * q + 1], w[4 * q + 1]));
    a = add(a, scl(val[4 * q + 2], w[4 * q + 2]));
    a = add(a, scl(val[4 * q + 3], w[4 * q + 3]));
    g[q] = a;
  }
  V3<R> lo = add(add(add(g[0], g[1]), g[2]), g[3]);
  V3<R> hi = add(add(add(g[4], g[5]), g[6]), g[7]);
  return add(lo, hi);
}

// Node index reordering: the weight order of shape32 is corners(8), then per
// axis 8 edge nodes ordered (e, w-side, v-side); cell_nodes lists per group of
// four (the reference's valvec order).  Map weight slot -> cell_nodes slot.
// x-edges: valvec2 = (k,j,e0),(k,j,e1),(k+1,j,e0),(k+1,j,e1); valvec3 = same at j+1
//   -> n = e + 2*zside + 4*yside  : v = y, w = z  (matches shape32 for ax=0)
// y-edges: valvec4 = (i,k,e0),(i,k,e1),(i+1,k,e0),(i+1,k,e1); valvec5 = same at k+1
//   -> n = e + 2*xside + 4*zside  : v = z, w = x  (matches ax=1)
// z-edges: valvec6 = (j,i,e0),(j,i,e1),(j+1,i,e0),(j+1,i,e1); valvec7 = same at i+1
//   -> n = e + 2*yside + 4*xside  : v = x, w = y  (matches ax=2)
// so the orders coincide and no remapping is needed.

template <typename R>
struct FieldSample {
  R dist;
  V3<R> grad;
  R vol;
};

template <typename R>
inline void field_locate(const Field& f, V3<R> x, int* cell, V3<R>* s) {
  R p[3] = {x.x, x.y, x.z};
  R sl[3];
  for (int a = 0; a < 3; ++a) {
    R scale = (R)((double)f.res[a] / f.extent[a]);
    R u = (p[a] - (R)f.origin[a]) * scale;
    R fl = std::floor(u);
    int c = (int)fl;
    if (c < 0) c = 0;
    if (c > f.res[a] - 1) c = f.res[a] - 1;
    cell[a] = c;
    sl[a] = (R)2 * (u - fl) - (R)1;  // 2 fract(u) - 1
  }
  *s = v3(sl[0], sl[1], sl[2]);
}

// BoundaryVolume pass for one particle (boundaryVolume.ts:31-55).
template <typename R>
inline void boundary_sample(const Field& f, const Consts<R>& k, V3<R> x, bool quirk, bool trilinear,
                            R* out4) {
  int c[3];
  V3<R> s;
  field_locate(f, x, c, &s);
  long idx[32];
  R N[32];
  V3<R> dN[32];
  R val[32];
  R dist, vol;
  V3<R> grad;
  R gs[3];
  for (int a = 0; a < 3; ++a) gs[a] = (R)(2.0 * (double)f.res[a] / f.extent[a]);
  if (!trilinear) {
    cell_nodes(f.res, c[0], c[1], c[2], false, idx);
    shape32(s, N, dN);
    for (int q = 0; q < 32; ++q) val[q] = (R)f.sdf[idx[q]];
    dist = sum32(N, val);
    V3<R> g = sum32v(dN, val);
    grad = v3(gs[0] * g.x, gs[1] * g.y, gs[2] * g.z);
  } else {
    cell_nodes(f.res, c[0], c[1], c[2], false, idx);
    R tx = (s.x + (R)1) * (R)0.5, ty = (s.y + (R)1) * (R)0.5, tz = (s.z + (R)1) * (R)0.5;
    R w[8], dw[8][3];
    for (int q = 0; q < 8; ++q) {
      int a = q & 1, b = (q >> 1) & 1, e = (q >> 2) & 1;
      R wx = a ? tx : (R)1 - tx, wy = b ? ty : (R)1 - ty, wz = e ? tz : (R)1 - tz;
      R sx = a ? (R)1 : (R)-1, sy = b ? (R)1 : (R)-1, sz = e ? (R)1 : (R)-1;
      w[q] = wx * wy * wz;
      dw[q][0] = sx * wy * wz;
      dw[q][1] = wx * sy * wz;
      dw[q][2] = wx * wy * sz;
    }
    dist = 0;
    V3<R> g = v3<R>(0, 0, 0);
    for (int q = 0; q < 8; ++q) {
      R v = (R)f.sdf[idx[q]];
      dist = dist + w[q] * v;
      g = add(g, v3(dw[q][0] * v, dw[q][1] * v, dw[q][2] * v));
    }
    // d/du of trilinear weights is per unit local t; t = (s+1)/2 so d/dx = scale
    grad = v3((R)0.5 * gs[0] * g.x, (R)0.5 * gs[1] * g.y, (R)0.5 * gs[2] * g.z);
  }
  out4[0] = out4[1] = out4[2] = out4[3] = (R)0;
  if (dist > (R)0 && dist < k.h && len3(grad) > (R)1e-9) {
    if (!trilinear) {
      long vidx[32];
      cell_nodes(f.res, c[0], c[1], c[2], quirk, vidx);
      for (int q = 0; q < 32; ++q) val[q] = (R)f.vol[vidx[q]];
      vol = sum32(N, val);
    } else {
      R tx = (s.x + (R)1) * (R)0.5, ty = (s.y + (R)1) * (R)0.5, tz = (s.z + (R)1) * (R)0.5;
      vol = 0;
      for (int q = 0; q < 8; ++q) {
        int a = q & 1, b = (q >> 1) & 1, e = (q >> 2) & 1;
        R wx = a ? tx : (R)1 - tx, wy = b ? ty : (R)1 - ty, wz = e ? tz : (R)1 - tz;
        vol = vol + wx * wy * wz * (R)f.vol[idx[q]];
      }
    }
    if (vol > (R)0) {
      R gl = len3(grad);
      V3<R> n = divs(grad, gl);
      R d = std::max(dist + (R)0.5 * k.r, (R)2 * k.r);
      V3<R> xb = sub(x, scl(d, n));
      out4[0] = xb.x;
      out4[1] = xb.y;
      out4[2] = xb.z;
      out4[3] = vol;
    }
  }
}

// ---- the simulator --------------------------------------------------------------
template <typename R>
struct Sim {
  pbf_config cfg;
  Consts<R> k;
  Field field;
  uint32_t n = 0;
  std::vector<V3<R>> x, v, a, xs, dp, omega3, normal, bpos;
  std::vector<R> rho, lambda, omega_len, bvol;
  // neighbour search state (reference layout)
  std::vector<uint32_t> key, rank, cell_count, cell_offset, sorted, nbr_count, nbr_offset, nbr_list;

  void init(const pbf_config& c) {
    cfg = c;
    k = make_consts<R>(c);
  }
  void set_options(const pbf_options& o) {
    cfg.options = o;
    k.gy = (R)(-(double)o.gravity);
  }
  void set_particles(const float* xyzw, uint32_t count) {
    n = count;
    x.assign(n, v3<R>(0, 0, 0));
    v.assign(n, v3<R>(0, 0, 0));
    a.assign(n, v3<R>(0, 0, 0));
    xs.assign(n, v3<R>(0, 0, 0));
    dp.assign(n, v3<R>(0, 0, 0));
    omega3.assign(n, v3<R>(0, 0, 0));
    normal.assign(n, v3<R>(0, 0, 0));
    bpos.assign(n, v3<R>(0, 0, 0));
    rho.assign(n, 0);
    lambda.assign(n, 0);
    omega_len.assign(n, 0);
    bvol.assign(n, 0);
    for (uint32_t i = 0; i < n; ++i) x[i] = v3<R>((R)xyzw[4 * i], (R)xyzw[4 * i + 1], (R)xyzw[4 * i + 2]);
  }

  int cells() const { return k.dim[0] * k.dim[1] * k.dim[2]; }
  void cell_of(V3<R> p, int* c) const {
    R q[3] = {p.x, p.y, p.z};
    for (int ax = 0; ax < 3; ++ax) {
      R u = (q[ax] - k.dmin[ax]) * k.inv_cell[ax];
      int ci = (int)std::floor(u);
      if (ci < 0) ci = 0;
      if (ci > k.dim[ax] - 1) ci = k.dim[ax] - 1;
      c[ax] = ci;
    }
  }
  uint32_t key_of(const int* c) const {
    return (uint32_t)c[0] * (uint32_t)(k.dim[1] * k.dim[2]) + (uint32_t)c[1] * (uint32_t)k.dim[2] + (uint32_t)c[2];
  }

  // NeighborSearch.execute (neighborSearch.ts:270-301) on the predicted positions.
  void neighbor_search(const std::vector<V3<R>>& p, bool lists) {
    int C = cells();
    key.assign(n, 0);
    rank.assign(n, 0);
    cell_count.assign(C, 0);
    for (uint32_t i = 0; i < n; ++i) {  // ParticleInsert, sequential atomicAdd
      int c[3];
      cell_of(p[i], c);
      key[i] = key_of(c);
      rank[i] = cell_count[key[i]]++;
    }
    cell_offset.assign(C + 1, 0);  // exclusive scan (scanShader.ts), plus the total
    for (int c = 0; c < C; ++c) cell_offset[c + 1] = cell_offset[c] + cell_count[c];
    sorted.assign(n, 0);
    for (uint32_t i = 0; i < n; ++i) sorted[cell_offset[key[i]] + rank[i]] = i;  // CountingSort
    if (!lists) return;
    nbr_count.assign(n + 1, 0);
    auto visit = [&](uint32_t i, auto&& fn) {
      int c[3];
      cell_of(p[i], c);
      for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dz = -1; dz <= 1; ++dz) {
            int q[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
            if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] >= k.dim[0] || q[1] >= k.dim[1] || q[2] >= k.dim[2])
              continue;
            uint32_t ck = key_of(q);
            uint32_t s = cell_offset[ck], e = s + cell_count[ck];
            for (uint32_t t = s; t < e; ++t) {
              uint32_t j = sorted[t];
              V3<R> d = sub(p[j], p[i]);
              if (dot3(d, d) <= k.h2) fn(j);
            }
          }
    };
#pragma omp parallel for schedule(dynamic, 1024)
    for (long i = 0; i < (long)n; ++i) {  // NeighborCount
      uint32_t cnt = 0;
      visit((uint32_t)i, [&](uint32_t) { ++cnt; });
      nbr_count[i] = cnt;
    }
    nbr_offset.assign(n + 1, 0);  // particle scan over n+1 entries
    for (uint32_t i = 0; i < n; ++i) nbr_offset[i + 1] = nbr_offset[i] + nbr_count[i];
    nbr_list.assign(nbr_offset[n], 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (long i = 0; i < (long)n; ++i) {  // NeighborList
      uint32_t o = nbr_offset[i];
      visit((uint32_t)i, [&](uint32_t j) { nbr_list[o++] = j; });
    }
  }

  void substep() {
    const int jm = (int)cfg.jitter_mode;
    const bool have_field = field.loaded;
    const bool quirk = cfg.volume_quirk != 0;
    const bool tri = cfg.boundary_interp == PBF_INTERP_TRILINEAR;
    // TimeIntegration (timeIntegration.ts:25-28)
#pragma omp parallel for
    for (long i = 0; i < (long)n; ++i) {
      V3<R> g = v3<R>((R)0 + a[i].x, k.gy + a[i].y, (R)0 + a[i].z);
      V3<R> vel = add(v[i], scl(k.dt, g));
      xs[i] = clamp_rand(k, add(x[i], scl(k.dt, vel)), jm);
    }
    neighbor_search(xs, true);
    const uint32_t iters = cfg.options.iterations;
    for (uint32_t it = 0; it < iters; ++it) {
      if (have_field) {  // BoundaryVolume
#pragma omp parallel for
        for (long i = 0; i < (long)n; ++i) {
          R o[4];
          boundary_sample(field, k, xs[i], quirk, tri, o);
          bpos[i] = v3(o[0], o[1], o[2]);
          bvol[i] = o[3];
        }
      }
      // LambdaCalculation (pressureConstrain.ts:36-83)
#pragma omp parallel for
      for (long i = 0; i < (long)n; ++i) {
        V3<R> xi = xs[i];
        V3<R> grad = v3<R>(0, 0, 0);
        R sum2 = 0, dens = 0;
        for (uint32_t q = nbr_offset[i]; q < nbr_offset[i + 1]; ++q) {
          uint32_t j = nbr_list[q];
          V3<R> d = sub(xi, xs[j]);
          R rl = len3(d);
          V3<R> gk = spiky_grad(k, d, rl);
          grad = add(grad, gk);
          sum2 = sum2 + dot3(gk, gk);
          dens = dens + poly6(k, rl);
        }
        dens = dens * k.V;
        grad = scl(k.V, grad);
        sum2 = sum2 * k.V2;
        {
          V3<R> d = sub(xi, bpos[i]);
          R rl = len3(d);
          R vb = bvol[i];
          V3<R> gk = scl(vb, spiky_grad(k, d, rl));
          grad = add(grad, gk);
          dens = dens + vb * poly6(k, rl);
        }
        R cst = std::max((R)0, dens - (R)1);
        R s = dot3(grad, grad) + sum2;
        lambda[i] = -cst / (s + k.lambda_eps);
      }
      // ConstrainSolve (pressureConstrain.ts:114-156)
#pragma omp parallel for
      for (long i = 0; i < (long)n; ++i) {
        V3<R> xi = xs[i];
        R li = lambda[i];
        V3<R> pu = v3<R>(0, 0, 0);
        for (uint32_t q = nbr_offset[i]; q < nbr_offset[i + 1]; ++q) {
          uint32_t j = nbr_list[q];
          V3<R> d = sub(xi, xs[j]);
          R rl = len3(d);
          R lj = lambda[j];
          pu = add(pu, scl(li + lj, spiky_grad(k, d, rl)));
        }
        pu = scl(k.V, pu);
        {
          V3<R> d = sub(xi, bpos[i]);
          R rl = len3(d);
          pu = add(pu, scl(bvol[i] * li, spiky_grad(k, d, rl)));
        }
        dp[i] = scl((R)0.5, pu);
      }
      // ConstrainApply (pressureConstrain.ts:176-177)
#pragma omp parallel for
      for (long i = 0; i < (long)n; ++i) xs[i] = clamp_rand(k, add(xs[i], dp[i]), jm);
    }
    // AttributeUpdate (attributeUpdate.ts:30-56); the density loop reads xs only
    std::vector<R> dens_new(n);
#pragma omp parallel for
    for (long i = 0; i < (long)n; ++i) {
      V3<R> xi = xs[i];
      R dens = 0;
      for (uint32_t q = nbr_offset[i]; q < nbr_offset[i + 1]; ++q) {
        uint32_t j = nbr_list[q];
        V3<R> d = sub(xi, xs[j]);
        dens = dens + poly6(k, len3(d));
      }
      dens_new[i] = dens * k.m;
    }
#pragma omp parallel for
    for (long i = 0; i < (long)n; ++i) {
      v[i] = scl(k.inv_dt, sub(xs[i], x[i]));
      x[i] = xs[i];
      rho[i] = dens_new[i];
    }
    // VorticityConfinement (vorticityConfinement.ts:30-64)
#pragma omp parallel for
    for (long i = 0; i < (long)n; ++i) {
      V3<R> xi = x[i], vi = v[i];
      V3<R> om = v3<R>(0, 0, 0), nm = v3<R>(0, 0, 0);
      for (uint32_t q = nbr_offset[i]; q < nbr_offset[i + 1]; ++q) {
        uint32_t j = nbr_list[q];
        V3<R> d = sub(xi, x[j]);
        R rl = len3(d);
        V3<R> vd = sub(v[j], vi);
        R vol = k.m / rho[j];
        V3<R> gw = spiky_grad(k, d, rl);
        om = add(om, scl(vol, cross3(vd, gw)));
        nm = add(nm, scl(vol, gw));
      }
      omega3[i] = om;
      omega_len[i] = len3(om);
      normal[i] = scl(k.h, nm);
    }
    // XSPH + vorticity force + surface tension (XSPH.ts:36-89)
    const R cx = (R)cfg.options.xsph, cv = (R)cfg.options.vorticity, ct = (R)cfg.options.surface_tension;
#pragma omp parallel for
    for (long i = 0; i < (long)n; ++i) {
      V3<R> xi = x[i], vi = v[i], wi = omega3[i], ni = normal[i];
      R ri = rho[i];
      V3<R> vu = v3<R>(0, 0, 0), eta = v3<R>(0, 0, 0), ten = v3<R>(0, 0, 0);
      for (uint32_t q = nbr_offset[i]; q < nbr_offset[i + 1]; ++q) {
        uint32_t j = nbr_list[q];
        R rj = rho[j];
        V3<R> d = sub(xi, x[j]);
        R rl = len3(d);
        V3<R> vd = sub(v[j], vi);
        R kij = k.two_rho0 / (ri + rj);
        vu = add(vu, divs(scl(poly6(k, rl), vd), rj));
        eta = add(eta, divs(scl(omega_len[j], spiky_grad(k, d, rl)), rj));
        V3<R> coh = scl(k.m, cohesion(k, d, rl));
        V3<R> curv = sub(ni, normal[j]);
        ten = sub(ten, scl(kij, add(coh, curv)));
      }
      R el = len3(eta);
      V3<R> en = (el > (R)0) ? divs(eta, el) : v3<R>(0, 0, 0);
      R sx = cx * k.inv_dt * k.m;
      V3<R> acc = add(add(scl(sx, vu), scl(cv, cross3(en, wi))), scl(ct, ten));
      a[i] = acc;
    }
  }
};

}  // namespace

// ---- C API used by the tests (ctypes) -------------------------------------------
struct oracle_handle {
  int precision;  // 32 or 64
  Sim<float> f;
  Sim<double> d;
};

extern "C" {

oracle_handle* oracle_create(const pbf_config* cfg, int precision) {
  oracle_handle* h = new oracle_handle();
  h->precision = precision;
  if (precision == 64)
    h->d.init(*cfg);
  else
    h->f.init(*cfg);
  return h;
}
void oracle_destroy(oracle_handle* h) { delete h; }

void oracle_set_options(oracle_handle* h, const pbf_options* o) {
  if (h->precision == 64) h->d.set_options(*o); else h->f.set_options(*o);
}

void oracle_set_particles(oracle_handle* h, const float* xyzw, uint32_t n) {
  if (h->precision == 64) h->d.set_particles(xyzw, n); else h->f.set_particles(xyzw, n);
}

void oracle_set_velocities(oracle_handle* h, const float* xyzw, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    if (h->precision == 64)
      h->d.v[i] = v3<double>(xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2]);
    else
      h->f.v[i] = v3<float>(xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2]);
  }
}

void oracle_set_accelerations(oracle_handle* h, const float* xyzw, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    if (h->precision == 64)
      h->d.a[i] = v3<double>(xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2]);
    else
      h->f.a[i] = v3<float>(xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2]);
  }
}

// The last substep's neighbour search: 0 cell key per particle, 1 cell count,
// 2 cell offset (cells + 1), 3 sorted order.  Returns the array's length
// (copied when out is non-null and count matches), -1 for an unknown array.
long oracle_search_state(oracle_handle* h, int which, uint32_t* out, size_t count) {
  const std::vector<uint32_t>* v = nullptr;
  auto pick = [&](auto& sim) {
    switch (which) {
      case 0: v = &sim.key; break;
      case 1: v = &sim.cell_count; break;
      case 2: v = &sim.cell_offset; break;
      case 3: v = &sim.sorted; break;
      default: break;
    }
  };
  if (h->precision == 64) pick(h->d); else pick(h->f);
  if (!v) return -1;
  if (out && count == v->size()) std::copy(v->begin(), v->end(), out);
  return (long)v->size();
}

int oracle_set_field(oracle_handle* h, const uint32_t* res, const float* origin, const float* extent,
                     const float* sdf, const float* vol, size_t nodes) {
  Field& f = (h->precision == 64) ? h->d.field : h->f.field;
  f.loaded = true;
  for (int a = 0; a < 3; ++a) {
    f.res[a] = (int)res[a];
    f.origin[a] = origin[a];
    f.extent[a] = extent[a];
  }
  f.sdf.assign(sdf, sdf + nodes);
  f.vol.assign(vol, vol + nodes);
  return 0;
}

void oracle_substep(oracle_handle* h, uint32_t count) {
  for (uint32_t s = 0; s < count; ++s) {
    if (h->precision == 64) h->d.substep(); else h->f.substep();
  }
}

// Copy a field out as doubles (4 per particle for vector fields, 1 for scalars).
// 0 position(x,rho) 1 velocity 2 acceleration 3 predicted 4 lambda 5 boundary
// 6 omega(w,|w|) 7 normal 8 delta_p 9 neighbour count
int oracle_get_field(oracle_handle* h, int field, double* out) {
  auto run = [&](auto& S) {
    uint32_t n = S.n;
    for (uint32_t i = 0; i < n; ++i) {
      double* o = out + 4 * (size_t)i;
      auto put = [&](auto vv, double w) { o[0] = vv.x; o[1] = vv.y; o[2] = vv.z; o[3] = w; };
      switch (field) {
        case 0: put(S.x[i], S.rho[i]); break;
        case 1: put(S.v[i], 0); break;
        case 2: put(S.a[i], 0); break;
        case 3: put(S.xs[i], 0); break;
        case 4: out[i] = S.lambda[i]; break;
        case 5: put(S.bpos[i], S.bvol[i]); break;
        case 6: put(S.omega3[i], S.omega_len[i]); break;
        case 7: put(S.normal[i], 0); break;
        case 8: put(S.dp[i], 0); break;
        case 9: out[i] = S.nbr_count.empty() ? 0 : S.nbr_count[i]; break;
        default: return -1;
      }
    }
    return 0;
  };
  return (h->precision == 64) ? run(h->d) : run(h->f);
}

// Neighbour search alone on float4 positions (reference semantics, f32).
// keys[n], cell_count[C], cell_offset[C+1], order[n], rank[n]; optional
// neighbour lists: nbr_offset[n+1], and nbr_list (capacity entries).
int oracle_neighbor_search(const pbf_config* cfg, const float* xyzw, uint32_t n, uint32_t* keys,
                           uint32_t* cell_count, uint32_t* cell_offset, uint32_t* order, uint32_t* rank,
                           uint32_t* nbr_offset, uint32_t* nbr_list, uint64_t capacity, uint64_t* total) {
  Sim<float> S;
  S.init(*cfg);
  S.set_particles(xyzw, n);
  bool lists = nbr_offset != nullptr;
  S.neighbor_search(S.x, lists);
  int C = S.cells();
  if (keys) std::memcpy(keys, S.key.data(), 4 * (size_t)n);
  if (rank) std::memcpy(rank, S.rank.data(), 4 * (size_t)n);
  if (cell_count) std::memcpy(cell_count, S.cell_count.data(), 4 * (size_t)C);
  if (cell_offset) std::memcpy(cell_offset, S.cell_offset.data(), 4 * (size_t)(C + 1));
  if (order) std::memcpy(order, S.sorted.data(), 4 * (size_t)n);
  if (lists) {
    std::memcpy(nbr_offset, S.nbr_offset.data(), 4 * (size_t)(n + 1));
    uint64_t t = S.nbr_offset[n];
    if (total) *total = t;
    if (t > capacity) return 2;
    std::memcpy(nbr_list, S.nbr_list.data(), 4 * (size_t)t);
  }
  return 0;
}

int oracle_grid_cells(const pbf_config* cfg, uint32_t* dims) {
  Consts<float> k = make_consts<float>(*cfg);
  for (int a = 0; a < 3; ++a) dims[a] = (uint32_t)k.dim[a];
  return k.dim[0] * k.dim[1] * k.dim[2];
}

// Exact exclusive scan (the semantics checked by exclusiveScan.ts:193-199).
void oracle_exclusive_scan(const uint32_t* in, uint32_t* out, uint64_t n) {
  uint32_t s = 0;
  for (uint64_t i = 0; i < n; ++i) {
    out[i] = s;
    s += in[i];
  }
}

// Boundary sample of arbitrary points (BoundaryVolume pass on a point list),
// in f32 (precision 32) or f64.  out: 4 per point (x_b, V_b); raw: 5 per
// point (dist, grad, vol-unconditional) for layout checks.
int oracle_sample_field(const pbf_config* cfg, const uint32_t* res, const float* origin, const float* extent,
                        const float* sdf, const float* vol, size_t nodes, const float* pts, uint32_t n,
                        int precision, double* out) {
  Field f;
  f.loaded = true;
  for (int a = 0; a < 3; ++a) {
    f.res[a] = (int)res[a];
    f.origin[a] = origin[a];
    f.extent[a] = extent[a];
  }
  f.sdf.assign(sdf, sdf + nodes);
  f.vol.assign(vol, vol + nodes);
  bool quirk = cfg->volume_quirk != 0, tri = cfg->boundary_interp == PBF_INTERP_TRILINEAR;
  if (precision == 64) {
    Consts<double> k = make_consts<double>(*cfg);
    for (uint32_t i = 0; i < n; ++i) {
      double o[4];
      boundary_sample(f, k, v3<double>(pts[4 * i], pts[4 * i + 1], pts[4 * i + 2]), quirk, tri, o);
      for (int q = 0; q < 4; ++q) out[4 * i + q] = o[q];
    }
  } else {
    Consts<float> k = make_consts<float>(*cfg);
    for (uint32_t i = 0; i < n; ++i) {
      float o[4];
      boundary_sample(f, k, v3<float>(pts[4 * i], pts[4 * i + 1], pts[4 * i + 2]), quirk, tri, o);
      for (int q = 0; q < 4; ++q) out[4 * i + q] = o[q];
    }
  }
  return 0;
}

// Raw cubic interpolation of the SDF (value + gradient) and volume in f64.
int oracle_interpolate(const uint32_t* res, const float* origin, const float* extent, const float* sdf,
                       const float* vol, size_t nodes, const double* pts, uint32_t n, int quirk, double* out) {
  Field f;
  for (int a = 0; a < 3; ++a) {
    f.res[a] = (int)res[a];
    f.origin[a] = origin[a];
    f.extent[a] = extent[a];
  }
  for (uint32_t i = 0; i < n; ++i) {
    int c[3];
    V3<double> s;
    field_locate(f, v3<double>(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), c, &s);
    long idx[32], vidx[32];
    double N[32], val[32], vv[32];
    V3<double> dN[32];
    cell_nodes(f.res, c[0], c[1], c[2], false, idx);
    cell_nodes(f.res, c[0], c[1], c[2], quirk != 0, vidx);
    shape32(s, N, dN);
    for (int q = 0; q < 32; ++q) {
      val[q] = sdf[idx[q]];
      vv[q] = vol[vidx[q]];
    }
    double d = sum32(N, val);
    V3<double> g = sum32v(dN, val);
    double* o = out + 5 * (size_t)i;
    o[0] = d;
    o[1] = 2.0 * res[0] / extent[0] * g.x;
    o[2] = 2.0 * res[1] / extent[1] * g.y;
    o[3] = 2.0 * res[2] / extent[2] * g.z;
    o[4] = sum32(N, vv);
  }
  (void)nodes;
  return 0;
}

// Reference CPU helper PBF.computeParticleDensity (PBF.ts:96-116): brute-force
// density over all particles with the CPU kernalPoly6 (PBF.ts:16-25), in f64.
double oracle_bruteforce_density(const float* xyzw, uint32_t n, uint32_t i, double h, double mass) {
  const double PI = 3.14159265358979323846;
  double dens = 0;
  double px = xyzw[4 * i], py = xyzw[4 * i + 1], pz = xyzw[4 * i + 2];
  for (uint32_t j = 0; j < n; ++j) {
    double dx = xyzw[4 * j] - px, dy = xyzw[4 * j + 1] - py, dz = xyzw[4 * j + 2] - pz;
    double l = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (l <= h) {
      double coef = 315.0 / (64.0 * PI * std::pow(h, 9));
      double x = h * h - l * l;
      dens += coef * std::pow(x, 3);
    }
  }
  return dens * mass;
}

// Volume-map generator restated on the CPU in FP64 (same definition as
// pbf_generate_volume_map): SDF = min over shapes, V = 0.8 * Gauss-Legendre
// integral over the support ball of gamma(SDF).
static double o_sdf_shape(uint32_t kind, const double* c, const double* s, double x, double y, double z) {
  double px = x - c[0], py = y - c[1], pz = z - c[2];
  switch (kind) {
    case 0: return std::fmin(std::fmin(s[0] - std::fabs(px), s[1] - std::fabs(py)), s[2] - std::fabs(pz));
    case 1: return std::sqrt(px * px + py * py + pz * pz) - s[0];
    case 2: {
      double dr = std::sqrt(px * px + pz * pz) - s[0], dy = std::fabs(py) - s[1];
      double ax = std::fmax(dr, 0.0), ay = std::fmax(dy, 0.0);
      return std::fmin(std::fmax(dr, dy), 0.0) + std::sqrt(ax * ax + ay * ay);
    }
    case 3: {
      double q = std::sqrt(px * px + pz * pz) - s[0];
      return std::sqrt(q * q + py * py) - s[1];
    }
    case 4: {
      double qx = std::fabs(px) - s[0], qy = std::fabs(py) - s[1], qz = std::fabs(pz) - s[2];
      double ox = std::fmax(qx, 0.0), oy = std::fmax(qy, 0.0), oz = std::fmax(qz, 0.0);
      return std::sqrt(ox * ox + oy * oy + oz * oz) + std::fmin(std::fmax(qx, std::fmax(qy, qz)), 0.0);
    }
  }
  return 1e30;
}

static int gen_impl(const pbf_shape* shapes, uint32_t count, const uint32_t* res, const float* origin,
                    const float* extent, float support_radius, uint32_t quadrature, uint32_t flags,
                    const float* sdf_in, float* sdf_out, float* vol_out) {
  const double PI = 3.14159265358979323846;
  int nq = quadrature ? (int)quadrature : 12;
  std::vector<double> qx(nq), qw(nq);
  for (int i = 0; i < nq; ++i) {  // Newton on the Legendre polynomial P_nq
    double z = std::cos(PI * (i + 0.75) / (nq + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= nq; ++k) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      dp = nq * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    qx[i] = -z;
    qw[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  const double h = support_radius;
  double o[3], cell[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    o[a] = origin[a];
    cell[a] = (double)extent[a] / (double)res[a];
    hi[a] = (double)origin[a] + (double)extent[a];
  }
  const bool empty_out = (flags & 1u) != 0;
  const bool discrete = (flags & 2u) != 0;
  std::vector<float> node_sdf;  // filled below when the integrand reads the discrete map
  int ires[3] = {(int)res[0], (int)res[1], (int)res[2]};
  auto sdf_analytic = [&](double x, double y, double z) {
    double d = 1e30;
    for (uint32_t i = 0; i < count; ++i) {
      double c[3] = {shapes[i].center[0], shapes[i].center[1], shapes[i].center[2]};
      double s[3] = {shapes[i].size[0], shapes[i].size[1], shapes[i].size[2]};
      d = std::fmin(d, o_sdf_shape(shapes[i].kind, c, s, x, y, z));
    }
    return d;
  };
  auto sdf_discrete = [&](double x, double y, double z) {
    double q[3] = {x, y, z}, sl[3];
    int c[3];
    for (int a = 0; a < 3; ++a) {
      double u = (q[a] - o[a]) / cell[a];
      int ci = (int)std::floor(u);
      ci = std::min(std::max(ci, 0), ires[a] - 1);
      c[a] = ci;
      sl[a] = 2.0 * (u - (double)ci) - 1.0;
    }
    long idx[32];
    double N[32], val[32];
    V3<double> dN[32];
    cell_nodes(ires, c[0], c[1], c[2], false, idx);
    shape32(v3(sl[0], sl[1], sl[2]), N, dN);
    double acc = 0.0;
    for (int t = 0; t < 32; ++t) {
      val[t] = node_sdf[idx[t]];
      acc += N[t] * val[t];
    }
    return acc;
  };
  auto sdf = [&](double x, double y, double z) { return discrete ? sdf_discrete(x, y, z) : sdf_analytic(x, y, z); };
  auto gam = [&](double x, double y, double z) {
    if (empty_out && (x < o[0] || y < o[1] || z < o[2] || x > hi[0] || y > hi[1] || z > hi[2])) return 0.0;
    double d = sdf(x, y, z);
    if (d <= 0.0) return 1.0;
    if (d < h) {
      double q = d / h;
      if (q <= 0.5) return 6.0 * q * q * q - 6.0 * q * q + 1.0;
      double t = 1.0 - q;
      return 2.0 * t * t * t;
    }
    return 0.0;
  };
  double vsat_acc = 0.0;
  for (int a = 0; a < nq; ++a)
    for (int b = 0; b < nq; ++b)
      for (int c = 0; c < nq; ++c)
        if (qx[a] * qx[a] + qx[b] * qx[b] + qx[c] * qx[c] <= 1.0) vsat_acc += qw[a] * qw[b] * qw[c];
  const double vsat = 0.8 * vsat_acc * h * h * h;
  const long nx = res[0], ny = res[1], nz = res[2];
  // enumerate nodes in layout order
  std::vector<std::array<double, 3>> P;
  for (long k = 0; k <= nz; ++k)
    for (long j = 0; j <= ny; ++j)
      for (long i = 0; i <= nx; ++i) P.push_back({(double)i, (double)j, (double)k});
  for (long k = 0; k <= nz; ++k)
    for (long j = 0; j <= ny; ++j)
      for (long e = 0; e < 2 * nx; ++e) P.push_back({(double)(e / 2) + (double)((e % 2) + 1) / 3.0, (double)j, (double)k});
  for (long i = 0; i <= nx; ++i)
    for (long k = 0; k <= nz; ++k)
      for (long e = 0; e < 2 * ny; ++e) P.push_back({(double)i, (double)(e / 2) + (double)((e % 2) + 1) / 3.0, (double)k});
  for (long j = 0; j <= ny; ++j)
    for (long i = 0; i <= nx; ++i)
      for (long e = 0; e < 2 * nz; ++e) P.push_back({(double)i, (double)j, (double)(e / 2) + (double)((e % 2) + 1) / 3.0});
  if (discrete) {
    node_sdf.resize(P.size());
    for (size_t q = 0; q < P.size(); ++q)
      node_sdf[q] = sdf_in ? sdf_in[q]
                           : (float)sdf_analytic(o[0] + P[q][0] * cell[0], o[1] + P[q][1] * cell[1],
                                                 o[2] + P[q][2] * cell[2]);
  }
#pragma omp parallel for schedule(dynamic, 64)
  for (long q = 0; q < (long)P.size(); ++q) {
    double x = o[0] + P[q][0] * cell[0], y = o[1] + P[q][1] * cell[1], z = o[2] + P[q][2] * cell[2];
    double d = discrete ? (double)node_sdf[q] : sdf_analytic(x, y, z), v;
    if (d >= 2.0 * h) {
      v = 0.0;
    } else if (d <= -h && !empty_out) {
      v = vsat;
    } else {
      double acc = 0.0;
      for (int a = 0; a < nq; ++a)
        for (int b = 0; b < nq; ++b) {
          double wab = qw[a] * qw[b];
          for (int c = 0; c < nq; ++c) {
            if (qx[a] * qx[a] + qx[b] * qx[b] + qx[c] * qx[c] > 1.0) continue;
            acc += wab * qw[c] * gam(x + h * qx[a], y + h * qx[b], z + h * qx[c]);
          }
        }
      v = 0.8 * acc * h * h * h;
    }
    if (sdf_out) sdf_out[q] = (float)d;
    vol_out[q] = (float)v;
  }
  return 0;
}

int oracle_generate_volume_map(const pbf_shape* shapes, uint32_t count, const uint32_t* res, const float* origin,
                               const float* extent, float support_radius, uint32_t quadrature, uint32_t flags,
                               float* sdf_out, float* vol_out) {
  return gen_impl(shapes, count, res, origin, extent, support_radius, quadrature, flags, nullptr, sdf_out, vol_out);
}

int oracle_volume_from_sdf(const uint32_t* res, const float* origin, const float* extent, float support_radius,
                           uint32_t quadrature, uint32_t flags, const float* sdf, float* vol_out) {
  return gen_impl(nullptr, 0, res, origin, extent, support_radius, quadrature, flags | 2u, sdf, nullptr, vol_out);
}

// SPH.voxelizeMesh (src/simulator/SPH.ts:151-187): lattice at spacing 2r over
// the mesh's world bounding box from its minimum corner (floor(extent / 2r)
// points per axis, x slowest), a +z ray from each point in the mesh's local
// space (origin through the inverse world matrix), the nearest hit over all
// triangles of either orientation, and the point kept when the hit face's
// normal points along the ray.  Brute force over every triangle in double
// precision (the reference computes in JavaScript doubles); the inverse is
// the cofactor expansion.  Returns the kept points (x, y, z, 0) in lattice
// order.
static bool vox_invert4(const double* m, double* inv) {
  double r[16];
  r[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] -
         m[13] * m[7] * m[10];
  r[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
         m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  r[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] -
         m[12] * m[7] * m[9];
  r[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
          m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  r[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
         m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  r[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] -
         m[12] * m[3] * m[10];
  r[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
         m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  r[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
          m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  r[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] -
         m[13] * m[3] * m[6];
  r[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] +
         m[12] * m[3] * m[6];
  r[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] -
          m[12] * m[3] * m[5];
  r[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
          m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  r[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] +
         m[9] * m[3] * m[6];
  r[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] -
         m[8] * m[3] * m[6];
  r[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] +
          m[8] * m[3] * m[5];
  r[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] -
          m[8] * m[2] * m[5];
  const double det = m[0] * r[0] + m[1] * r[4] + m[2] * r[8] + m[3] * r[12];
  if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
  for (int q = 0; q < 16; ++q) inv[q] = r[q] / det;
  return true;
}

int oracle_voxelize_mesh(const float* vertices, uint32_t nv, const uint32_t* idx, uint32_t nt, const double* world,
                         double particle_radius, float* out, uint32_t capacity, uint32_t* count) {
  *count = 0;
  double W[16], M[16];
  for (int q = 0; q < 16; ++q) W[q] = world[q];
  if (!vox_invert4(W, M)) return 1;
  // Box3.expandByObject: the local vertex box's eight corners through the
  // world matrix (Box3.applyMatrix4; w = 1 for an affine matrix)
  double llo[3] = {1e300, 1e300, 1e300}, lhi[3] = {-1e300, -1e300, -1e300};
  for (uint32_t q = 0; q < nv; ++q)
    for (int a = 0; a < 3; ++a) {
      llo[a] = std::min(llo[a], (double)vertices[3 * (size_t)q + a]);
      lhi[a] = std::max(lhi[a], (double)vertices[3 * (size_t)q + a]);
    }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int corner = 0; corner < 8; ++corner) {
    const double x = (corner & 4) ? lhi[0] : llo[0], y = (corner & 2) ? lhi[1] : llo[1],
                 z = (corner & 1) ? lhi[2] : llo[2];
    const double w[3] = {W[0] * x + W[4] * y + W[8] * z + W[12], W[1] * x + W[5] * y + W[9] * z + W[13],
                         W[2] * x + W[6] * y + W[10] * z + W[14]};
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], w[a]);
      hi[a] = std::max(hi[a], w[a]);
    }
  }
  const double diam = 2.0 * particle_radius;
  uint64_t dim[3];
  for (int a = 0; a < 3; ++a) dim[a] = (uint64_t)std::floor((hi[a] - lo[a]) / diam);
  std::vector<uint8_t> in(dim[0] * dim[1] * dim[2], 0);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t id = 0; id < (int64_t)in.size(); ++id) {
    const uint64_t k = (uint64_t)id % dim[2], j = ((uint64_t)id / dim[2]) % dim[1], i = (uint64_t)id / (dim[2] * dim[1]);
    const double px = (double)i * diam + lo[0], py = (double)j * diam + lo[1], pz = (double)k * diam + lo[2];
    const double o[3] = {M[0] * px + M[4] * py + M[8] * pz + M[12], M[1] * px + M[5] * py + M[9] * pz + M[13],
                         M[2] * px + M[6] * py + M[10] * pz + M[14]};
    double best = 1e300;
    bool hit = false, along = false;
    for (uint32_t f = 0; f < nt; ++f) {
      const float* A = vertices + 3 * (size_t)idx[3 * (size_t)f];
      const float* B = vertices + 3 * (size_t)idx[3 * (size_t)f + 1];
      const float* C = vertices + 3 * (size_t)idx[3 * (size_t)f + 2];
      const double e1[3] = {(double)B[0] - A[0], (double)B[1] - A[1], (double)B[2] - A[2]};
      const double e2[3] = {(double)C[0] - A[0], (double)C[1] - A[1], (double)C[2] - A[2]};
      const double nx = e1[1] * e2[2] - e1[2] * e2[1], ny = e1[2] * e2[0] - e1[0] * e2[2],
                   nz = e1[0] * e2[1] - e1[1] * e2[0];
      // ray direction (0, 0, 1): direction . normal = nz
      double ddn = nz, sg;
      if (ddn > 0.0) {
        sg = 1.0;
      } else if (ddn < 0.0) {
        sg = -1.0;
        ddn = -ddn;
      } else {
        continue;
      }
      const double q[3] = {o[0] - A[0], o[1] - A[1], o[2] - A[2]};
      const double u = sg * (q[0] * e2[1] - q[1] * e2[0]);   // (q x e2).z
      if (u < 0.0) continue;
      const double v = sg * (e1[0] * q[1] - e1[1] * q[0]);   // (e1 x q).z
      if (v < 0.0) continue;
      if (u + v > ddn) continue;
      const double qn = -sg * (q[0] * nx + q[1] * ny + q[2] * nz);
      if (qn < 0.0) continue;
      const double t = qn / ddn;
      if (!hit || t < best) {
        best = t;
        hit = true;
        along = sg > 0.0;
      }
    }
    in[id] = (hit && along) ? 1 : 0;
  }
  uint32_t c = 0;
  for (uint64_t id = 0; id < in.size(); ++id) {
    if (!in[id]) continue;
    if (c < capacity && out) {
      const uint64_t k = id % dim[2], j = (id / dim[2]) % dim[1], i = id / (dim[2] * dim[1]);
      out[4 * (size_t)c] = (float)((double)i * diam + lo[0]);
      out[4 * (size_t)c + 1] = (float)((double)j * diam + lo[1]);
      out[4 * (size_t)c + 2] = (float)((double)k * diam + lo[2]);
      out[4 * (size_t)c + 3] = 0.0f;
    }
    ++c;
  }
  *count = c;
  return c > capacity ? 2 : 0;
}

// ---- screen-space fluid buffers (src/renderer/filteredParticleFluid) ----
// ParicleRasterizer.execute (paricleRasterizer.ts:170-204) with the sprite
// shaders depthPassShader.ts / volumePassShader.ts, then TextureFilter
// (textureFilter.ts:129-160, filterPassShader.ts), restated particle by
// particle and pixel by pixel.  Sprite geometry: the camera-space centre c =
// view * (p, 1) plus (+-hs, +-hs, 0, 0) (hs = R/2 for depth, R for volume)
// through the projection; the rectangle's framebuffer edges are
// 0.5 (ndc.x + 1) W and 0.5 (1 - ndc.y) H; pixels whose centres lie in it
// (left/top edges in) are covered; uv is the centre's position across it.
// Depth: ties of equal depth keep the lower particle index; the volume term
// is exp(-2 nx^2) exp(-2 ny^2) and its sum is exact (integer sum of the terms
// scaled by 2^40).  Filter texel reads
// clamp to the image edge.  Returns 0, or 1 for a clipped-out camera setup.
static inline void rnd_mat_vec(const float* m, float x, float y, float z, float w, float o[4]) {
  for (int r = 0; r < 4; ++r) o[r] = ((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w;
}

struct RndSprite {
  float sx, ox, sy, oy, cz, cw;
  int i0, i1, j0, j1;
};

static inline int rnd_edge(float f, int size) {
  float e = std::min(std::max(f - 0.5f, -1.0f), (float)size);
  int i = (int)std::ceil(e);
  return std::min(std::max(i, 0), size);
}

// n.xy = 2 uv - 1 at pixel (i, j): nx = i sx + ox with sx = 2 / (x1 - x0),
// ox = (0.5 - x0) sx - 1; ny = j sy + oy with sy = -2 / (yb - yt),
// oy = (yb - 0.5) (2 / (yb - yt)) - 1 (uv measured from the bottom edge).
static bool rnd_sprite(const float* P, const float c[4], float hs, int W, int H, RndSprite& s) {
  float bl[4], tr[4];
  rnd_mat_vec(P, c[0] + (-hs), c[1] + (-hs), c[2], c[3], bl);
  rnd_mat_vec(P, c[0] + hs, c[1] + hs, c[2], c[3], tr);
  if (!(bl[3] > 0.0f) || !(bl[2] >= 0.0f) || !(bl[2] <= bl[3])) return false;
  const float fx0 = 0.5f * (bl[0] / bl[3] + 1.0f) * (float)W;
  const float fx1 = 0.5f * (tr[0] / tr[3] + 1.0f) * (float)W;
  const float fyb = 0.5f * (-(bl[1] / bl[3]) + 1.0f) * (float)H;
  const float fyt = 0.5f * (-(tr[1] / tr[3]) + 1.0f) * (float)H;
  if (!(fx1 != fx0) || !(fyb != fyt)) return false;
  s.i0 = rnd_edge(std::min(fx0, fx1), W);
  s.i1 = rnd_edge(std::max(fx0, fx1), W);
  s.j0 = rnd_edge(std::min(fyt, fyb), H);
  s.j1 = rnd_edge(std::max(fyt, fyb), H);
  const float ax = 2.0f / (fx1 - fx0), ay = 2.0f / (fyb - fyt);
  s.sx = ax;
  s.ox = std::fmaf(0.5f - fx0, ax, -1.0f);
  s.sy = -ay;
  s.oy = std::fmaf(fyb - 0.5f, ay, -1.0f);
  s.cz = c[2];
  s.cw = c[3];
  return s.i0 < s.i1 && s.j0 < s.j1;
}

static inline float rnd_r2(const RndSprite& s, int i, int j) {
  const float nx = std::fmaf((float)i, s.sx, s.ox), ny = std::fmaf((float)j, s.sy, s.oy);
  return std::fmaf(nx, nx, ny * ny);
}

// exp(x), x in [-2, 0]: x = k ln2 + r (Cody-Waite, ln 2 = hi + lo with a
// 16-bit hi), Taylor series of exp(r) to degree 8 (Horner with fused
// multiply-adds), times 2^k.
static inline float rnd_exp(float x) {
  const float k = std::floor(std::fmaf(x, 1.44269502f, 0.5f));
  const float r = std::fmaf(-k, 1.42860677e-6f, std::fmaf(-k, 0.693145751953125f, x));
  const float c[9] = {1.0f, 1.0f, 0.5f, 1.66666667e-1f, 4.16666667e-2f, 8.33333333e-3f, 1.38888889e-3f,
                      1.98412698e-4f, 2.48015873e-5f};
  float p = c[8];
  for (int q = 7; q >= 0; --q) p = std::fmaf(p, r, c[q]);
  return p * std::ldexp(1.0f, (int)k);
}

static void rnd_filter_line(const float* line, int len, int stride, int half, const float* g, float threshold,
                            float mu, int pos, bool& write, float& out) {
  // texel `pos` of a line: centre at pos - (16 - half), taps +-i, reads clamped
  auto at = [&](int q) { return line[(size_t)std::min(std::max(q, 0), len - 1) * stride]; };
  const int c = pos - (16 - half);
  const float center = at(c);
  write = center > 0.0f;
  if (!write) return;
  float vs = center, ws = 1.0f, lo = center - threshold, hi = center + threshold;
  const float bh = center + mu;
  for (int i = 1; i <= half; ++i) {
    float a = at(c - i), b = at(c + i);
    if (a < lo || b < lo) continue;
    a = a > hi ? bh : a;
    b = b > hi ? bh : b;
    lo = std::min(lo, std::min(a, b) - threshold);
    hi = std::max(hi, std::max(a, b) + threshold);
    ws += g[i] * 2.0f;
    vs += (a + b) * g[i];
  }
  out = vs / ws;
}

float oracle_splat_exp(float x) { return rnd_exp(x); }

// TextureFilter.execute on one r32float image in place (x pass into a
// cleared temporary, y pass back where the temporary's centre is positive).
int oracle_narrow_range_filter(float* img, uint32_t width, uint32_t height, uint32_t filter_size, float R) {
  if (filter_size > 32) return 1;
  if (filter_size < 2) return 0;
  const int W = (int)width, H = (int)height, half = (int)(filter_size >> 1);
  const float sigma = (float)half * 0.5f, k = 0.5f / (sigma * sigma);
  float g[17] = {};
  for (int i = 0; i <= half; ++i) g[i] = (float)std::exp((double)(-(float)(i * i) * k));
  std::vector<float> temp((size_t)W * H, 0.0f);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      bool wr;
      float v = 0.0f;
      rnd_filter_line(img + (size_t)y * W, W, 1, half, g, R * 5.0f, R, x, wr, v);
      temp[(size_t)y * W + x] = wr ? v : 0.0f;
    }
  for (int x = 0; x < W; ++x)
    for (int y = 0; y < H; ++y) {
      bool wr;
      float v = 0.0f;
      rnd_filter_line(temp.data() + x, H, W, half, g, R * 5.0f, R, y, wr, v);
      if (wr) img[(size_t)y * W + x] = v;
    }
  return 0;
}

int oracle_render(const float* pos, uint32_t n, uint32_t width, uint32_t height, const float* view, const float* proj,
                  float R, uint32_t filter_size, float* scene, float* depth_out, float* volume_out) {
  const int W = (int)width, H = (int)height, W2 = W / 2, H2 = H / 2;
  std::vector<uint64_t> keys((size_t)W * H);
  std::vector<float> eye((size_t)W * H, 0.0f);
  std::vector<uint64_t> acc((size_t)W2 * H2, 0);
  auto bits = [](float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
  };
  auto clamp01 = [](float d) { return d > 0.0f ? std::min(d, 1.0f) : 0.0f; };
  for (size_t p = 0; p < keys.size(); ++p)
    keys[p] = ((uint64_t)bits(clamp01(scene ? scene[p] : 0.0f)) << 32) | 0xffffffffull;
  for (uint32_t q = 0; q < n; ++q) {
    float c[4];
    rnd_mat_vec(view, pos[4 * (size_t)q], pos[4 * (size_t)q + 1], pos[4 * (size_t)q + 2], 1.0f, c);
    RndSprite s;
    if (rnd_sprite(proj, c, 0.5f * R, W, H, s))
      for (int j = s.j0; j < s.j1; ++j)
        for (int i = s.i0; i < s.i1; ++i) {
          const float r2 = rnd_r2(s, i, j);
          if (r2 > 1.0f) continue;
          const float z = std::fmaf(std::sqrt(1.0f - r2), R, s.cz);
          const float w = s.cw;
          const float d = clamp01(std::fmaf(proj[10], z, proj[14] * w) / std::fmaf(proj[11], z, proj[15] * w));
          const uint64_t key = ((uint64_t)bits(d) << 32) | (0xffffffffull - q);
          const size_t p = (size_t)j * W + i;
          if (key > keys[p]) {
            keys[p] = key;
            eye[p] = -z / w;
          }
        }
    if (rnd_sprite(proj, c, R, W2, H2, s))
      for (int j = s.j0; j < s.j1; ++j)
        for (int i = s.i0; i < s.i1; ++i) {
          const float r2 = rnd_r2(s, i, j);
          if (r2 > 1.0f) continue;
          const float nx = std::fmaf((float)i, s.sx, s.ox), ny = std::fmaf((float)j, s.sy, s.oy);
          const float v = rnd_exp((nx * nx) * -2.0f) * rnd_exp((ny * ny) * -2.0f);
          acc[(size_t)j * W2 + i] += (uint64_t)((double)v * 1099511627776.0);
        }
  }
  for (size_t p = 0; p < keys.size(); ++p) {
    const uint32_t init = bits(clamp01(scene ? scene[p] : 0.0f));
    const bool hit = (uint32_t)(keys[p] >> 32) != init;
    depth_out[p] = hit ? eye[p] : 0.0f;
    if (hit && scene) {
      const uint32_t b = (uint32_t)(keys[p] >> 32);
      std::memcpy(&scene[p], &b, 4);
    }
  }
  for (size_t p = 0; p < acc.size(); ++p) volume_out[p] = (float)((double)acc[p] * (1.0 / 1099511627776.0));
  return oracle_narrow_range_filter(depth_out, width, height, filter_size, R) ? 1 : 0;
}

int oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void oracle_set_threads(int t) {
#ifdef _OPENMP
  omp_set_num_threads(t);
#else
  (void)t;
#endif
}

}  // extern "C"
