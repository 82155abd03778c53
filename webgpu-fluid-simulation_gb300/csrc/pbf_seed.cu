// pbf_seed.cu — scene seeding from a triangle mesh on the GPU: SPH.voxelizeMesh
// (src/simulator/SPH.ts:151-187).
//
// The reference places a lattice at spacing 2r over the mesh's world-space
// bounding box (three.js Box3.expandByObject: the eight corners of the local
// vertex bounding box mapped by the world matrix; the lattice starts at its
// minimum corner with floor(extent / 2r) points per axis), casts from each point a ray along +z in the mesh's local space
// (origin transformed by the inverse world matrix, direction (0, 0, 1)
// untransformed), takes the nearest hit of either face orientation
// (three-mesh-bvh raycastFirst) and keeps the point when that face points
// along the ray (normal . (0,0,1) > 0: the ray leaves the solid, so the point
// is inside).  Points are appended in (i, j, k) order, x slowest.
//
// Here every lattice point is one GPU thread.  All rays are parallel to the
// local z axis, so a triangle can only be hit by rays whose (x, y) lies in its
// xy bounding box: triangles are binned into a 2D grid of columns over the
// local xy extent (closed intervals widened by a small pad, so a triangle sits
// in every column its box touches even after rounding) and a ray tests only
// its column's list, in triangle order, so the nearest hit and its tie-break
// are those of a test over all triangles.  The ray/triangle test
// is the signed-volume (scalar triple product) form of the Moller-Trumbore
// test, in double precision like the reference's JavaScript numbers, with the
// same inclusive edges.  This unit is compiled with -fmad=false so its double
// arithmetic matches the CPU restatement operation for operation.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"
#include "pbf_kernels.h"

namespace {

struct D3 {
  double x, y, z;
};

struct MeshDev {
  const double* v;         // local vertices, 3 per vertex
  const uint32_t* tri;     // 3 indices per triangle
  const uint32_t* col_start;  // [cols + 1] start of each column's triangle list
  const uint32_t* col_tri;    // triangle ids per column
  double col_origin[2], col_max[2], col_inv[2];  // local xy extent of the mesh
  int col_dim[2];
  double inv[16];          // inverse world matrix, column-major
  double origin[3];        // lattice origin (world AABB minimum)
  double diam;
  uint32_t dim[3];
};

__host__ __device__ inline D3 sub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline D3 cross(D3 a, D3 b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Nearest hit along +z from o over triangle (a, b, c); returns false for no
// hit, else t and whether the face points along the ray.
__host__ __device__ inline bool ray_z_triangle(D3 o, D3 a, D3 b, D3 c, double& t, bool& along) {
  const D3 e1 = sub(b, a), e2 = sub(c, a), n = cross(e1, e2);
  double ddn = n.z;  // direction . normal with direction (0, 0, 1)
  double sign;
  if (ddn > 0.0) {
    sign = 1.0;
  } else if (ddn < 0.0) {
    sign = -1.0;
    ddn = -ddn;
  } else {
    return false;  // parallel
  }
  const D3 q = sub(o, a);
  const double u = sign * cross(q, e2).z;
  if (u < 0.0) return false;
  const double v = sign * cross(e1, q).z;
  if (v < 0.0) return false;
  if (u + v > ddn) return false;
  const double qn = -sign * dot(q, n);
  if (qn < 0.0) return false;  // behind the origin
  t = qn / ddn;
  along = sign > 0.0;
  return true;
}

// A seeding lattice: point (i, j, k) is ((i - shift) * diam + org[0], ...),
// evaluated in double and rounded to float once, as the host loops of
// SPH.voxelizeCube / voxelizeSphere / voxelizeMesh do; i is slowest.
struct Lattice {
  double org[3];
  double diam;
  uint32_t dim[3];
  int64_t shift;
};

__device__ inline void lattice_ijk(const Lattice& L, uint64_t id, uint32_t& i, uint32_t& j, uint32_t& k) {
  k = (uint32_t)(id % L.dim[2]);
  j = (uint32_t)((id / L.dim[2]) % L.dim[1]);
  i = (uint32_t)(id / ((uint64_t)L.dim[2] * L.dim[1]));
}

__device__ inline double lattice_rel(const Lattice& L, uint32_t i) {
  return (double)((int64_t)i - L.shift) * L.diam;
}

__device__ inline uint64_t lattice_size(const Lattice& L) { return (uint64_t)L.dim[0] * L.dim[1] * L.dim[2]; }

// SPH.voxelizeMesh's test for every lattice point: 1 = inside.
__global__ void k_mesh_flags(Lattice L, MeshDev m, uint32_t* flag) {
  const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= lattice_size(L)) return;
  uint32_t i, j, k;
  lattice_ijk(L, id, i, j, k);
  // world lattice point, then local ray origin
  const double px = lattice_rel(L, i) + L.org[0];
  const double py = lattice_rel(L, j) + L.org[1];
  const double pz = lattice_rel(L, k) + L.org[2];
  const double* M = m.inv;
  const D3 o{M[0] * px + M[4] * py + M[8] * pz + M[12], M[1] * px + M[5] * py + M[9] * pz + M[13],
             M[2] * px + M[6] * py + M[10] * pz + M[14]};
  uint32_t result = 0;
  // rays outside the (padded) local xy extent cannot meet a triangle
  if (o.x >= m.col_origin[0] && o.x <= m.col_max[0] && o.y >= m.col_origin[1] && o.y <= m.col_max[1]) {
    const int cx = min((int)floor((o.x - m.col_origin[0]) * m.col_inv[0]), m.col_dim[0] - 1);
    const int cy = min((int)floor((o.y - m.col_origin[1]) * m.col_inv[1]), m.col_dim[1] - 1);
    const uint32_t col = (uint32_t)cy * (uint32_t)m.col_dim[0] + (uint32_t)cx;
    double best = 1e300;
    bool hit = false, along = false;
    for (uint32_t q = m.col_start[col]; q < m.col_start[col + 1]; ++q) {
      const uint32_t f = m.col_tri[q];
      const uint32_t ia = m.tri[3 * f], ib = m.tri[3 * f + 1], ic = m.tri[3 * f + 2];
      const D3 a{m.v[3 * ia], m.v[3 * ia + 1], m.v[3 * ia + 2]};
      const D3 b{m.v[3 * ib], m.v[3 * ib + 1], m.v[3 * ib + 2]};
      const D3 c{m.v[3 * ic], m.v[3 * ic + 1], m.v[3 * ic + 2]};
      double t;
      bool al;
      if (ray_z_triangle(o, a, b, c, t, al) && (!hit || t < best)) {
        best = t;
        hit = true;
        along = al;
      }
    }
    result = (hit && along) ? 1u : 0u;
  }
  flag[id] = result;
}

// SPH.voxelizeSphere's test (SPH.ts:123-149): x^2 + y^2 + z^2 <= radius^2 on
// the centred lattice.
__global__ void k_sphere_flags(Lattice L, double r2, uint32_t* flag) {
  const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= lattice_size(L)) return;
  uint32_t i, j, k;
  lattice_ijk(L, id, i, j, k);
  const double x = lattice_rel(L, i), y = lattice_rel(L, j), z = lattice_rel(L, k);
  flag[id] = (x * x + y * y + z * z <= r2) ? 1u : 0u;
}

// Writes the kept points (all of them when flag is null) at out[off[id]].
__global__ void k_emit(Lattice L, const uint32_t* flag, const uint32_t* off, float4* out) {
  const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= lattice_size(L)) return;
  uint64_t dst = id;
  if (flag) {
    if (!flag[id]) return;
    dst = off[id];
  }
  uint32_t i, j, k;
  lattice_ijk(L, id, i, j, k);
  out[dst] = make_float4((float)(lattice_rel(L, i) + L.org[0]), (float)(lattice_rel(L, j) + L.org[1]),
                         (float)(lattice_rel(L, k) + L.org[2]), 0.0f);
}

// The host jitter (splitmix64 draws in particle-then-axis order) evaluated
// per draw: draw m sees the state seed + (m + 1) * golden gamma.
__global__ void k_jitter(float4* p, uint32_t n, double amplitude, uint64_t seed) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 v = p[i];
  float* c[3] = {&v.x, &v.y, &v.z};
  for (int a = 0; a < 3; ++a) {
    uint64_t z = seed + (3ull * i + a + 1) * 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    *c[a] = (float)((double)*c[a] + amplitude * (2.0 * u - 1.0));
  }
  p[i] = v;
}

__global__ void k_iota(uint32_t* ids, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ids[i] = i;
}

inline unsigned blocks_for(uint64_t n) { return (unsigned)((n + 255) / 256); }

bool invert4(const double* m, double* inv) {
  // cofactor expansion (column-major in and out)
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

// Host preparation of one mesh: validation, inverse world matrix, world
// lattice, triangle columns; device copies of the vertices (as doubles), the
// indices and the column lists.
struct MeshPrep {
  MeshDev m{};
  Lattice lat{};
  double* dv = nullptr;
  uint32_t *dt = nullptr, *ds = nullptr, *dc = nullptr;
  ~MeshPrep() {
    cudaFree(dv);
    cudaFree(dt);
    cudaFree(ds);
    cudaFree(dc);
  }
};

int prepare_mesh(const float* vertices, uint32_t vertex_count, const uint32_t* indices, uint32_t triangle_count,
                 const double* world, double particle_radius, MeshPrep& P, cudaStream_t st) {
  if (!vertices || !indices || !world || vertex_count == 0 || triangle_count == 0 || !(particle_radius > 0.0))
    return PBF_EINVAL;
  for (uint64_t q = 0; q < 3ull * triangle_count; ++q)
    if (indices[q] >= vertex_count) return PBF_EINVAL;
  double W[16], inv[16];
  for (int q = 0; q < 16; ++q) W[q] = world[q];
  // an object's world matrix is affine (bottom row 0 0 0 1)
  if (W[3] != 0.0 || W[7] != 0.0 || W[11] != 0.0 || W[15] != 1.0) return PBF_EINVAL;
  if (!invert4(W, inv)) return PBF_EINVAL;
  std::vector<double> lv(3 * (size_t)vertex_count);
  double llo[3] = {1e300, 1e300, 1e300}, lhi[3] = {-1e300, -1e300, -1e300};
  for (uint32_t q = 0; q < vertex_count; ++q)
    for (int a = 0; a < 3; ++a) {
      const double x = vertices[3 * (size_t)q + a];
      if (!std::isfinite(x)) return PBF_EINVAL;
      lv[3 * (size_t)q + a] = x;
      llo[a] = std::min(llo[a], x);
      lhi[a] = std::max(lhi[a], x);
    }
  // world AABB: the local box's eight corners through the world matrix
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
  uint64_t total = 1;
  for (int a = 0; a < 3; ++a) {
    const double d = std::floor((hi[a] - lo[a]) / diam);
    if (!(d >= 0.0) || d > 4096.0) return PBF_EINVAL;
    P.lat.dim[a] = (uint32_t)d;
    P.lat.org[a] = lo[a];
    total *= P.lat.dim[a];
  }
  P.lat.diam = diam;
  P.lat.shift = 0;
  if (total > (1ull << 30)) return PBF_EINVAL;  // lattice limit: 2^30 points per item
  if (total == 0) return PBF_OK;
  // Triangle columns over the local xy extent, about 4 triangles per column.
  // The pad (a millionth of the extent) keeps every triangle that a ray just
  // outside its exact xy box could still meet under rounding in that ray's
  // column; extra candidates never change the answer, only missing ones would.
  MeshDev& m = P.m;
  const int cd = std::max(1, std::min(1024, (int)std::sqrt((double)triangle_count / 4.0)));
  m.col_dim[0] = m.col_dim[1] = cd;
  double pad[2];
  for (int a = 0; a < 2; ++a) {
    pad[a] = 1e-6 * std::max(lhi[a] - llo[a], 1e-30) + 1e-300;
    m.col_origin[a] = llo[a] - pad[a];
    m.col_max[a] = lhi[a] + pad[a];
    m.col_inv[a] = (double)cd / (m.col_max[a] - m.col_origin[a]);
  }
  std::vector<uint32_t> cnt((size_t)cd * cd + 1, 0), start((size_t)cd * cd + 1, 0);
  auto span = [&](uint32_t f, int* c0, int* c1) {
    double mn[2] = {1e300, 1e300}, mx[2] = {-1e300, -1e300};
    for (int e = 0; e < 3; ++e) {
      const uint32_t vi = indices[3 * (size_t)f + e];
      for (int a = 0; a < 2; ++a) {
        mn[a] = std::min(mn[a], lv[3 * (size_t)vi + a]);
        mx[a] = std::max(mx[a], lv[3 * (size_t)vi + a]);
      }
    }
    for (int a = 0; a < 2; ++a) {
      c0[a] = std::max(0, std::min(cd - 1, (int)std::floor((mn[a] - pad[a] - m.col_origin[a]) * m.col_inv[a])));
      c1[a] = std::max(0, std::min(cd - 1, (int)std::floor((mx[a] + pad[a] - m.col_origin[a]) * m.col_inv[a])));
    }
  };
  for (uint32_t f = 0; f < triangle_count; ++f) {
    int c0[2], c1[2];
    span(f, c0, c1);
    for (int y = c0[1]; y <= c1[1]; ++y)
      for (int x = c0[0]; x <= c1[0]; ++x) ++cnt[(size_t)y * cd + x];
  }
  for (size_t c = 0; c < (size_t)cd * cd; ++c) start[c + 1] = start[c] + cnt[c];
  // columns hold triangles in index order, so the first nearest hit is the
  // one a scan over all triangles finds
  std::vector<uint32_t> col_tri(start[(size_t)cd * cd]), fill(start.begin(), start.end() - 1);
  for (uint32_t f = 0; f < triangle_count; ++f) {
    int c0[2], c1[2];
    span(f, c0, c1);
    for (int y = c0[1]; y <= c1[1]; ++y)
      for (int x = c0[0]; x <= c1[0]; ++x) col_tri[fill[(size_t)y * cd + x]++] = f;
  }
  std::memcpy(m.inv, inv, sizeof(inv));
  cudaError_t e = cudaMalloc(&P.dv, lv.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&P.dt, 3ull * triangle_count * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&P.ds, start.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&P.dc, std::max<size_t>(col_tri.size(), 1) * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P.dv, lv.data(), lv.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P.dt, indices, 3ull * triangle_count * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P.ds, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !col_tri.empty())
    e = cudaMemcpyAsync(P.dc, col_tri.data(), col_tri.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  // the host staging vectors end with this call
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return PBF_ECUDA;
  m.v = P.dv;
  m.tri = P.dt;
  m.col_start = P.ds;
  m.col_tri = P.dc;
  return PBF_OK;
}

// Flags of a lattice's kept points and their exclusive offsets; *kept gets
// their number.  flag/off hold lattice_size + 1 entries.
struct Compaction {
  uint32_t* flag = nullptr;
  uint32_t* off = nullptr;
  ~Compaction() {
    cudaFree(flag);
    cudaFree(off);
  }
  int alloc(uint64_t n, cudaStream_t st) {
    if (cudaMalloc(&flag, (n + 1) * sizeof(uint32_t)) != cudaSuccess) return PBF_ECUDA;
    if (cudaMalloc(&off, (n + 1) * sizeof(uint32_t)) != cudaSuccess) return PBF_ECUDA;
    return cudaMemsetAsync(flag + n, 0, sizeof(uint32_t), st) == cudaSuccess ? PBF_OK : PBF_ECUDA;
  }
  int count(uint64_t n, cudaStream_t st, uint32_t* kept) {
    if (cudaGetLastError() != cudaSuccess) return PBF_ECUDA;
    int rc = pbf_exclusive_scan_u32(flag, off, (size_t)n + 1, (void*)st);
    if (rc) return rc;
    if (cudaMemcpyAsync(kept, off + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess) return PBF_ECUDA;
    return cudaStreamSynchronize(st) == cudaSuccess ? PBF_OK : PBF_ECUDA;
  }
};

uint64_t lattice_count(const Lattice& L) { return (uint64_t)L.dim[0] * L.dim[1] * L.dim[2]; }

// Appends one seeding item's points at out[*base ..]; *base advances by the
// number of points even when they do not fit (then PBF_ECAPACITY).
int seed_item(const pbf_seed_item& it, double radius, float4* out, uint32_t capacity, uint64_t* base,
              cudaStream_t st) {
  const double diam = 2.0 * radius;
  Lattice L{};
  L.diam = diam;
  if (it.kind == PBF_SEED_CUBE) {
    // SPH.voxelizeCube (SPH.ts:99-121)
    uint64_t n = 1;
    for (int a = 0; a < 3; ++a) {
      if (!std::isfinite(it.a[a]) || !std::isfinite(it.b[a])) return PBF_EINVAL;
      const double d = std::floor(((double)it.b[a] - it.a[a]) / diam);
      L.dim[a] = d > 0.0 ? (uint32_t)std::min(d, 4096.0) : 0u;
      if (d > 4096.0) return PBF_EINVAL;
      L.org[a] = it.a[a];
      n *= L.dim[a];
    }
    if (n == 0) return PBF_OK;
    const uint64_t at = *base;
    *base += n;
    if (*base > capacity) return PBF_ECAPACITY;
    k_emit<<<blocks_for(n), 256, 0, st>>>(L, nullptr, nullptr, out + at);
    return cudaGetLastError() == cudaSuccess ? PBF_OK : PBF_ECUDA;
  }
  Compaction C;
  MeshPrep P;
  uint64_t n = 0;
  if (it.kind == PBF_SEED_SPHERE) {
    // SPH.voxelizeSphere (SPH.ts:123-149)
    const double r = it.b[0];
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(it.a[a])) return PBF_EINVAL;
    if (!std::isfinite(r)) return PBF_EINVAL;
    const double vd = std::floor(r / radius / 2.0);
    if (vd < 0.0) return PBF_OK;                  // a negative radius seeds nothing
    if (vd > 511.0) return PBF_EINVAL;            // lattice limit: 2^30 points per item
    for (int a = 0; a < 3; ++a) {
      L.dim[a] = 2 * (uint32_t)vd + 1;
      L.org[a] = it.a[a];
    }
    L.shift = (int64_t)vd;
    n = lattice_count(L);
    int rc = C.alloc(n, st);
    if (rc) return rc;
    k_sphere_flags<<<blocks_for(n), 256, 0, st>>>(L, r * r, C.flag);
  } else if (it.kind == PBF_SEED_MESH) {
    int rc = prepare_mesh(it.vertices, it.vertex_count, it.indices, it.triangle_count, it.world, radius, P, st);
    if (rc) return rc;
    L = P.lat;
    n = lattice_count(L);
    if (n == 0) return PBF_OK;
    rc = C.alloc(n, st);
    if (rc) return rc;
    k_mesh_flags<<<blocks_for(n), 256, 0, st>>>(L, P.m, C.flag);
  } else {
    return PBF_EINVAL;
  }
  uint32_t kept = 0;
  int rc = C.count(n, st, &kept);
  if (rc) return rc;
  const uint64_t at = *base;
  *base += kept;
  if (*base > capacity) return PBF_ECAPACITY;
  if (kept) k_emit<<<blocks_for(n), 256, 0, st>>>(L, C.flag, C.off, out + at);
  if (cudaGetLastError() != cudaSuccess) return PBF_ECUDA;
  // the temporaries are freed on return: finish with them first
  return cudaStreamSynchronize(st) == cudaSuccess ? PBF_OK : PBF_ECUDA;
}

}  // namespace

namespace pbf {

int seed_device(const pbf_seed_item* items, uint32_t count, double radius, float jitter, uint64_t seed, float4* out,
                uint32_t* ids, uint32_t capacity, uint32_t* total, cudaStream_t st) {
  *total = 0;
  if ((!items && count) || !(radius > 0.0) || !std::isfinite(jitter) || jitter < 0.0f) return PBF_EINVAL;
  uint64_t base = 0;
  int status = PBF_OK;
  for (uint32_t q = 0; q < count; ++q) {
    int rc = seed_item(items[q], radius, out, capacity, &base, st);
    if (rc == PBF_ECAPACITY) {
      status = PBF_ECAPACITY;  // keep counting what the scene would need
      continue;
    }
    if (rc) return rc;
  }
  *total = (uint32_t)std::min<uint64_t>(base, 0xffffffffull);
  if (status) return status;
  const uint32_t n = (uint32_t)base;
  if (n && jitter > 0.0f) k_jitter<<<blocks_for(n), 256, 0, st>>>(out, n, (double)jitter, seed);
  if (n && ids) k_iota<<<blocks_for(n), 256, 0, st>>>(ids, n);
  if (cudaGetLastError() != cudaSuccess) return PBF_ECUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? PBF_OK : PBF_ECUDA;
}

}  // namespace pbf

namespace pbf {

int voxelize_mesh_host(const float* vertices, uint32_t vertex_count, const uint32_t* indices, uint32_t triangle_count,
                       const double* world, double particle_radius, bool emit, std::vector<float>* pts,
                       uint32_t* kept) {
  *kept = 0;
  cudaStream_t st = 0;
  MeshPrep P;
  int rc = prepare_mesh(vertices, vertex_count, indices, triangle_count, world, particle_radius, P, st);
  if (rc) return rc;
  const uint64_t n = lattice_count(P.lat);
  if (n == 0) return PBF_OK;
  Compaction C;
  rc = C.alloc(n, st);
  if (rc) return rc;
  k_mesh_flags<<<blocks_for(n), 256, 0, st>>>(P.lat, P.m, C.flag);
  rc = C.count(n, st, kept);
  if (rc || !emit || *kept == 0) return rc;
  float4* d = nullptr;
  if (cudaMalloc(&d, (size_t)*kept * sizeof(float4)) != cudaSuccess) return PBF_ECUDA;
  k_emit<<<blocks_for(n), 256, 0, st>>>(P.lat, C.flag, C.off, d);
  pts->resize((size_t)*kept * 4);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(pts->data(), d, (size_t)*kept * sizeof(float4), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? PBF_OK : PBF_ECUDA;
}

}  // namespace pbf

extern "C" {

int pbf_voxelize_mesh_points(const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                             uint32_t triangle_count, const double world[16], double particle_radius, float* out_xyzw,
                             uint32_t capacity, uint32_t* count) {
  if (!count || (!out_xyzw && capacity)) return PBF_EINVAL;
  *count = 0;
  std::vector<float> pts;
  uint32_t kept = 0;
  int rc = pbf::voxelize_mesh_host(vertices, vertex_count, indices, triangle_count, world, particle_radius,
                                   capacity > 0, &pts, &kept);
  if (rc) return rc;
  *count = kept;
  const uint32_t copy = std::min(kept, capacity);
  if (copy) std::memcpy(out_xyzw, pts.data(), (size_t)copy * 4 * sizeof(float));
  return kept > capacity ? PBF_ECAPACITY : PBF_OK;
}

}  // extern "C"
