// pbf_volume.cu — volume-map generator (SDF + boundary volume per node) in the
// 32-node .cdm layout read by the boundary pass.
//
// The reference loads precomputed maps (src/simulator/boundary/volumeMap.ts:23-39,
// public/model/*.cdm, 20^3 cells over the unit cube).  The maps for the other
// scenes (a box container, a sphere / cylinder / torus obstacle) are built
// here: one GPU thread per node evaluates the analytic SDF and, in the band
// |SDF| < 2h, integrates the volume with an n^3 Gauss-Legendre rule in FP64.
// Compiled with -fmad=false so the CPU restatement reproduces it to the last bit.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"

namespace {

constexpr int kMaxShapes = 16;
constexpr int kMaxQuad = 32;

struct GenParams {
  int nshapes;
  uint32_t kind[kMaxShapes];
  double c[kMaxShapes][3];
  double s[kMaxShapes][3];
  int res[3];
  double origin[3], cell[3], hi[3];
  double h;
  int nq;
  double qx[kMaxQuad], qw[kMaxQuad];
  double vsat;  // 0.8 * integral of the ball (all solid)
  int outside_empty;
  int discrete;        // integrand reads the SDF through the map's own cubic interpolation
  const float* nodes;  // node SDF values (device or host pointer, matching the caller)
};

__host__ __device__ inline double sdf_shape(uint32_t kind, const double* c, const double* s, double x, double y,
                                            double z) {
  double px = x - c[0], py = y - c[1], pz = z - c[2];
  switch (kind) {
    case PBF_SHAPE_BOX_CONTAINER: {
      double d = s[0] - fabs(px);
      d = fmin(d, s[1] - fabs(py));
      d = fmin(d, s[2] - fabs(pz));
      return d;
    }
    case PBF_SHAPE_SPHERE:
      return sqrt(px * px + py * py + pz * pz) - s[0];
    case PBF_SHAPE_CYLINDER: {
      double dr = sqrt(px * px + pz * pz) - s[0];
      double dy = fabs(py) - s[1];
      double inside = fmin(fmax(dr, dy), 0.0);
      double ax = fmax(dr, 0.0), ay = fmax(dy, 0.0);
      return inside + sqrt(ax * ax + ay * ay);
    }
    case PBF_SHAPE_TORUS: {
      double q = sqrt(px * px + pz * pz) - s[0];
      return sqrt(q * q + py * py) - s[1];
    }
    case PBF_SHAPE_BOX_SOLID: {
      double qx = fabs(px) - s[0], qy = fabs(py) - s[1], qz = fabs(pz) - s[2];
      double ox = fmax(qx, 0.0), oy = fmax(qy, 0.0), oz = fmax(qz, 0.0);
      return sqrt(ox * ox + oy * oy + oz * oz) + fmin(fmax(qx, fmax(qy, qz)), 0.0);
    }
    default:
      return 1e30;
  }
}

__host__ __device__ inline double sdf_all(const GenParams& g, double x, double y, double z) {
  double d = 1e30;
  for (int i = 0; i < g.nshapes; ++i) d = fmin(d, sdf_shape(g.kind[i], g.c[i], g.s[i], x, y, z));
  return d;
}

// normalised cubic spline, C(0) = 1, zero at q >= 1
__host__ __device__ inline double cubic01(double q) {
  if (q <= 0.5) return 6.0 * q * q * q - 6.0 * q * q + 1.0;
  if (q <= 1.0) {
    double t = 1.0 - q;
    return 2.0 * t * t * t;
  }
  return 0.0;
}

// Value of the map's SDF at p through the 32-node cubic cell (FP64).
__host__ __device__ inline double sdf_interp(const GenParams& g, double x, double y, double z) {
  double q[3] = {x, y, z}, s[3];
  int c[3];
  for (int a = 0; a < 3; ++a) {
    double u = (q[a] - g.origin[a]) / g.cell[a];
    double fl = floor(u);
    int ci = (int)fl;
    if (ci < 0) ci = 0;
    if (ci > g.res[a] - 1) ci = g.res[a] - 1;
    c[a] = ci;
    s[a] = 2.0 * (u - (double)ci) - 1.0;
  }
  const uint64_t nx = g.res[0], ny = g.res[1], nz = g.res[2];
  const uint64_t nc = (nx + 1) * (ny + 1) * (nz + 1);
  const uint64_t nex = 2 * nx * (ny + 1) * (nz + 1);
  const uint64_t ney = (nx + 1) * 2 * ny * (nz + 1);
  const uint64_t i = c[0], j = c[1], k = c[2];
  double sx = s[0], sy = s[1], sz = s[2];
  double r2 = sx * sx + sy * sy + sz * sz;
  double acc = 0.0;
  for (int n = 0; n < 8; ++n) {  // corners
    int a = n & 1, b = (n >> 1) & 1, e = (n >> 2) & 1;
    double w = (1.0 / 64.0) * (a ? 1.0 + sx : 1.0 - sx) * (b ? 1.0 + sy : 1.0 - sy) * (e ? 1.0 + sz : 1.0 - sz) *
               (9.0 * r2 - 19.0);
    acc += w * (double)g.nodes[((k + e) * (ny + 1) + (j + b)) * (nx + 1) + (i + a)];
  }
  for (int n = 0; n < 8; ++n) {  // x-edges: e, z-side, y-side
    int e = n & 1, zs = (n >> 1) & 1, ys = (n >> 2) & 1;
    double w = (9.0 / 64.0) * (1.0 - sx * sx) * (1.0 + (e ? 3.0 : -3.0) * sx) * (ys ? 1.0 + sy : 1.0 - sy) *
               (zs ? 1.0 + sz : 1.0 - sz);
    acc += w * (double)g.nodes[nc + ((k + zs) * (ny + 1) + (j + ys)) * (2 * nx) + 2 * i + e];
  }
  for (int n = 0; n < 8; ++n) {  // y-edges: e, x-side, z-side
    int e = n & 1, xs = (n >> 1) & 1, zs = (n >> 2) & 1;
    double w = (9.0 / 64.0) * (1.0 - sy * sy) * (1.0 + (e ? 3.0 : -3.0) * sy) * (zs ? 1.0 + sz : 1.0 - sz) *
               (xs ? 1.0 + sx : 1.0 - sx);
    acc += w * (double)g.nodes[nc + nex + ((i + xs) * (nz + 1) + (k + zs)) * (2 * ny) + 2 * j + e];
  }
  for (int n = 0; n < 8; ++n) {  // z-edges: e, y-side, x-side
    int e = n & 1, ys = (n >> 1) & 1, xs = (n >> 2) & 1;
    double w = (9.0 / 64.0) * (1.0 - sz * sz) * (1.0 + (e ? 3.0 : -3.0) * sz) * (xs ? 1.0 + sx : 1.0 - sx) *
               (ys ? 1.0 + sy : 1.0 - sy);
    acc += w * (double)g.nodes[nc + nex + ney + ((j + ys) * (nx + 1) + (i + xs)) * (2 * nz) + 2 * k + e];
  }
  return acc;
}

__host__ __device__ inline double gamma_at(const GenParams& g, double x, double y, double z) {
  if (g.outside_empty) {
    if (x < g.origin[0] || y < g.origin[1] || z < g.origin[2] || x > g.hi[0] || y > g.hi[1] || z > g.hi[2])
      return 0.0;
  }
  double d = g.discrete ? sdf_interp(g, x, y, z) : sdf_all(g, x, y, z);
  if (d <= 0.0) return 1.0;
  if (d < g.h) return cubic01(d / g.h);
  return 0.0;
}

__host__ __device__ inline double volume_at(const GenParams& g, double x, double y, double z) {
  double acc = 0.0;
  for (int a = 0; a < g.nq; ++a) {
    double ya = g.qx[a];
    for (int b = 0; b < g.nq; ++b) {
      double yb = g.qx[b];
      double wab = g.qw[a] * g.qw[b];
      for (int c = 0; c < g.nq; ++c) {
        double yc = g.qx[c];
        if (ya * ya + yb * yb + yc * yc > 1.0) continue;
        acc += wab * g.qw[c] * gamma_at(g, x + g.h * ya, y + g.h * yb, z + g.h * yc);
      }
    }
  }
  return 0.8 * acc * g.h * g.h * g.h;
}

// Position of node `idx` in the .cdm layout (corners, x-, y-, z-edge blocks).
__host__ __device__ inline void node_position(const GenParams& g, uint64_t idx, double* p) {
  const uint64_t nx = g.res[0], ny = g.res[1], nz = g.res[2];
  const uint64_t nc = (nx + 1) * (ny + 1) * (nz + 1);
  const uint64_t nex = 2 * nx * (ny + 1) * (nz + 1);
  const uint64_t ney = (nx + 1) * 2 * ny * (nz + 1);
  double fi, fj, fk;
  if (idx < nc) {
    uint64_t i = idx % (nx + 1), r = idx / (nx + 1);
    uint64_t j = r % (ny + 1), k = r / (ny + 1);
    fi = (double)i; fj = (double)j; fk = (double)k;
  } else if (idx < nc + nex) {
    uint64_t q = idx - nc;
    uint64_t e = q % (2 * nx), r = q / (2 * nx);
    uint64_t j = r % (ny + 1), k = r / (ny + 1);
    fi = (double)(e / 2) + (double)((e % 2) + 1) / 3.0; fj = (double)j; fk = (double)k;
  } else if (idx < nc + nex + ney) {
    uint64_t q = idx - nc - nex;
    uint64_t e = q % (2 * ny), r = q / (2 * ny);
    uint64_t k = r % (nz + 1), i = r / (nz + 1);
    fj = (double)(e / 2) + (double)((e % 2) + 1) / 3.0; fk = (double)k; fi = (double)i;
  } else {
    uint64_t q = idx - nc - nex - ney;
    uint64_t e = q % (2 * nz), r = q / (2 * nz);
    uint64_t i = r % (nx + 1), j = r / (nx + 1);
    fk = (double)(e / 2) + (double)((e % 2) + 1) / 3.0; fi = (double)i; fj = (double)j;
  }
  p[0] = g.origin[0] + fi * g.cell[0];
  p[1] = g.origin[1] + fj * g.cell[1];
  p[2] = g.origin[2] + fk * g.cell[2];
}

__host__ __device__ inline void eval_node(const GenParams& g, uint64_t idx, float* sdf, float* vol) {
  double p[3];
  node_position(g, idx, p);
  double d = g.discrete ? (double)g.nodes[idx] : sdf_all(g, p[0], p[1], p[2]);
  double v;
  if (d >= 2.0 * g.h) {
    v = 0.0;
  } else if (d <= -g.h && !g.outside_empty) {
    v = g.vsat;
  } else {
    v = volume_at(g, p[0], p[1], p[2]);
  }
  *sdf = (float)d;
  *vol = (float)v;
}

__global__ void k_node_sdf(GenParams g, uint64_t nodes, float* __restrict__ sdf) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nodes) return;
  double p[3];
  node_position(g, i, p);
  sdf[i] = (float)sdf_all(g, p[0], p[1], p[2]);
}

__global__ void k_volume_map(GenParams g, uint64_t nodes, float* __restrict__ sdf, float* __restrict__ vol) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nodes) return;
  float sd;
  eval_node(g, i, &sd, vol + i);
  if (!g.discrete) sdf[i] = sd;
}

// Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on P_n.
void gauss_legendre(int n, double* x, double* w) {
  const double PI = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      if (n == 1) {
        p1 = z;
        p0 = 1.0;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = -z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace

namespace {
int run_generator(GenParams& g, uint64_t nodes, const float* sdf_in, float* sdf_out, float* vol_out) {
  float *d_sdf = nullptr, *d_vol = nullptr;
  if (cudaMalloc(&d_sdf, nodes * sizeof(float)) != cudaSuccess) return PBF_ECUDA;
  if (cudaMalloc(&d_vol, nodes * sizeof(float)) != cudaSuccess) {
    cudaFree(d_sdf);
    return PBF_ECUDA;
  }
  const unsigned blocks = (unsigned)((nodes + 127) / 128);
  cudaError_t e = cudaSuccess;
  if (g.discrete) {
    if (sdf_in)
      e = cudaMemcpy(d_sdf, sdf_in, nodes * sizeof(float), cudaMemcpyHostToDevice);
    else
      k_node_sdf<<<blocks, 128>>>(g, nodes, d_sdf);
    g.nodes = d_sdf;
  }
  if (e == cudaSuccess) {
    k_volume_map<<<blocks, 128>>>(g, nodes, d_sdf, d_vol);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && sdf_out) e = cudaMemcpy(sdf_out, d_sdf, nodes * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(vol_out, d_vol, nodes * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d_sdf);
  cudaFree(d_vol);
  return e == cudaSuccess ? PBF_OK : PBF_ECUDA;
}

int setup_grid(GenParams& g, const uint32_t res[3], const float origin[3], const float extent[3], float h,
               uint32_t quadrature, uint32_t flags, uint64_t* nodes) {
  int nq = quadrature ? (int)quadrature : 12;
  if (nq < 2 || nq > kMaxQuad || !(h > 0.0f)) return PBF_EINVAL;
  for (int a = 0; a < 3; ++a) {
    if (res[a] == 0 || res[a] > 4096 || !(extent[a] > 0.0f)) return PBF_EINVAL;
    g.res[a] = (int)res[a];
    g.origin[a] = origin[a];
    g.cell[a] = (double)extent[a] / (double)res[a];
    g.hi[a] = (double)origin[a] + (double)extent[a];
  }
  g.h = h;
  g.nq = nq;
  gauss_legendre(nq, g.qx, g.qw);
  g.outside_empty = (flags & PBF_VOLMAP_OUTSIDE_EMPTY) ? 1 : 0;
  g.discrete = (flags & PBF_VOLMAP_DISCRETE_SDF) ? 1 : 0;
  double acc = 0.0;
  for (int a = 0; a < nq; ++a)
    for (int b = 0; b < nq; ++b)
      for (int c = 0; c < nq; ++c)
        if (g.qx[a] * g.qx[a] + g.qx[b] * g.qx[b] + g.qx[c] * g.qx[c] <= 1.0) acc += g.qw[a] * g.qw[b] * g.qw[c];
  g.vsat = 0.8 * acc * g.h * g.h * g.h;
  const uint64_t nx = res[0], ny = res[1], nz = res[2];
  *nodes = (nx + 1) * (ny + 1) * (nz + 1) + 2 * nx * (ny + 1) * (nz + 1) + (nx + 1) * 2 * ny * (nz + 1) +
           (nx + 1) * (ny + 1) * 2 * nz;
  return PBF_OK;
}
}  // namespace

extern "C" int pbf_volume_from_sdf(const uint32_t res[3], const float origin[3], const float extent[3],
                                   float support_radius, uint32_t quadrature, uint32_t flags, const float* sdf,
                                   float* vol_out) {
  if (!res || !origin || !extent || !sdf || !vol_out) return PBF_EINVAL;
  GenParams g;
  std::memset(&g, 0, sizeof(g));
  uint64_t nodes = 0;
  int rc = setup_grid(g, res, origin, extent, support_radius, quadrature, flags | PBF_VOLMAP_DISCRETE_SDF, &nodes);
  if (rc) return rc;
  return run_generator(g, nodes, sdf, nullptr, vol_out);
}

extern "C" int pbf_generate_volume_map(const pbf_shape* shapes, uint32_t count, const uint32_t res[3],
                                       const float origin[3], const float extent[3], float support_radius,
                                       uint32_t quadrature, uint32_t flags, float* sdf_out, float* vol_out) {
  if (!shapes || count == 0 || count > (uint32_t)kMaxShapes || !res || !origin || !extent || !sdf_out || !vol_out)
    return PBF_EINVAL;
  if (!(support_radius > 0.0f)) return PBF_EINVAL;
  int nq = quadrature ? (int)quadrature : 12;
  if (nq < 2 || nq > kMaxQuad) return PBF_EINVAL;
  GenParams g;
  std::memset(&g, 0, sizeof(g));
  g.nshapes = (int)count;
  for (uint32_t i = 0; i < count; ++i) {
    if (shapes[i].kind > PBF_SHAPE_BOX_SOLID) return PBF_EINVAL;
    g.kind[i] = shapes[i].kind;
    for (int a = 0; a < 3; ++a) {
      g.c[i][a] = shapes[i].center[a];
      g.s[i][a] = shapes[i].size[a];
    }
  }
  uint64_t nodes = 0;
  int rc = setup_grid(g, res, origin, extent, support_radius, quadrature, flags, &nodes);
  if (rc) return rc;
  return run_generator(g, nodes, nullptr, sdf_out, vol_out);
}
