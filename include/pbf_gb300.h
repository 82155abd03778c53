/*
 * pbf_gb300.h — C ABI of the GB300-native Position Based Fluids substep.
 *
 * This is the drop-in boundary for the simulator of WebGPU-Fluid-Simulation
 * (TypeScript + WGSL).  Every entry point below names the reference member it
 * replaces (paths are relative to the reference project root).  A TypeScript
 * host binds these through the N-API addon in the package's napi/ folder; the
 * Python tests bind them through ctypes.
 *
 * Conventions
 *  - Every call returns a pbf_status (0 = ok).  The reference throws
 *    synchronous JS errors for the same conditions
 *    (src/simulator/PBF/PBFConfig.ts:50-55, src/simulator/boundary/volumeMap.ts:31-33,
 *    src/simulator/neighbor/exclusiveScan.ts:38-41); here the call fails and
 *    pbf_last_error() holds the message.
 *  - One handle owns one CUDA stream and all device buffers.  Device pointers
 *    handed out stay valid until pbf_reset / pbf_destroy.  Calls on one handle
 *    are not thread-safe.  Step calls are asynchronous until a copy or
 *    pbf_synchronize.
 *  - Particle arrays crossing the boundary are float4 per particle
 *    (x, y, z, w), indexed by particle id, exactly like the reference's
 *    `position` GPU buffer (src/simulator/SPH.ts:39, w = density written by
 *    src/simulator/PBF/shader/attributeUpdate.ts:56).
 */
#ifndef PBF_GB300_H
#define PBF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBF_ABI_VERSION 1

typedef enum pbf_status {
  PBF_OK = 0,
  PBF_EINVAL = 1,     /* bad argument or length */
  PBF_ECAPACITY = 2,  /* too many particles / neighbour list overflow */
  PBF_EFORMAT = 3,    /* malformed .cdm boundary text */
  PBF_ECUDA = 4,      /* CUDA runtime error */
  PBF_ETIMEOUT = 5,   /* a bounded device wait gave up (scan look-back) */
  PBF_EDIVERGED = 6,  /* NaN/Inf found in the particle state */
  PBF_ESTATE = 7      /* call not valid in the current state */
} pbf_status;

typedef enum pbf_jitter_mode {
  PBF_JITTER_HASH = 0, /* integer hash of the float bits: bit-identical on every platform */
  PBF_JITTER_SIN = 1   /* fract(sin(dot(p, (12.9898, 78.233))) * 43758.5453), common.ts:51-59 */
} pbf_jitter_mode;

typedef enum pbf_fp_mode {
  PBF_FP_FAST = 0,     /* FMA contraction allowed (production) */
  PBF_FP_EXACT = 1     /* no contraction: bit-identical with the CPU restatement */
} pbf_fp_mode;

typedef enum pbf_boundary_interp {
  PBF_INTERP_CUBIC = 0,     /* 32-node cubic serendipity cell, discreteFieldShader.ts:15-192 */
  PBF_INTERP_TRILINEAR = 1  /* trilinear over the corner nodes only (fast mode) */
} pbf_boundary_interp;

/* Runtime options: SimulationOptions (src/common/shader.ts:50-58) plus the
 * iteration count, set by PBFConfig.setConfig (src/simulator/PBF/PBFConfig.ts:31-46)
 * with the GUI defaults of src/common/config.ts:22-28. */
typedef struct pbf_options {
  uint32_t iterations;      /* constrainIterationCount (default 5) */
  float xsph;               /* XSPHCoef (0.01) */
  float vorticity;          /* vorticityCoef (0.1) */
  float surface_tension;    /* tensionCoef (0.5) */
  float gravity;            /* g; the step applies (0, -g, 0) (9.8) */
} pbf_options;

/* Static configuration.  The reference bakes these into WGSL constants and
 * pipeline override constants (src/simulator/SPH.ts:24-27,49-50,
 * src/simulator/PBF/PBFConfig.ts:8,21, src/simulator/neighbor/neighborSearch.ts:9-14).
 * pbf_config_default() fills the reference's values. */
typedef struct pbf_config {
  uint32_t struct_size;     /* sizeof(pbf_config) */
  uint32_t max_particles;   /* capacity (reference: 1 << 18 - 1 == 131072) */
  float particle_radius;    /* r (0.006) */
  float kernel_radius;      /* h (0.025) */
  float rest_density;       /* rho0 (1000) */
  float time_step;          /* dt of one substep (1/300) */
  uint32_t substeps;        /* stepCount: substeps per pbf_step frame (1) */
  float domain_min[3];      /* simulation box (0,0,0) */
  float domain_max[3];      /* (1,1,1) */
  uint32_t grid_dim[3];     /* hash-grid cells per axis; 0 = ceil(extent / h) (40) */
  float lambda_eps;         /* lambdaEPS (1e-6) */
  float wall_jitter;        /* EPS of boundary_rand (1e-4) */
  uint32_t jitter_mode;     /* pbf_jitter_mode */
  uint32_t volume_quirk;    /* 1 = read the volume-map nodes exactly as the reference
                               does (discreteFieldShader.ts:146-147,152-153) */
  uint32_t fp_mode;         /* pbf_fp_mode */
  uint32_t boundary_interp; /* pbf_boundary_interp */
  uint32_t max_neighbors;   /* neighbour-list capacity per particle (60; the reference
                               sizes its list as SPH.MAX_NEIGHBOR_COUNT x particles,
                               neighborSearch.ts:81).  Each particle has a fixed slice
                               of this many entries; a particle with more neighbours
                               fails its substep with PBF_ECAPACITY and grows the slice */
  pbf_options options;
  void* stream;             /* cudaStream_t to run on, or NULL for a library-owned stream */
} pbf_config;

/* Per-particle fields readable with pbf_copy_field (all indexed by particle id). */
typedef enum pbf_field {
  PBF_FIELD_POSITION = 0,     /* float4 (x, rho)   — SPH.position */
  PBF_FIELD_VELOCITY = 1,     /* float4 (v, 0)     — SPH.velocity */
  PBF_FIELD_ACCELERATION = 2, /* float4 (a, 0)     — SPH.acceleration */
  PBF_FIELD_PREDICTED = 3,    /* float4 (x*, 0)    — PBF.position2 before the non-pressure passes */
  PBF_FIELD_LAMBDA = 4,       /* float             — PBF.lambda (last iteration) */
  PBF_FIELD_BOUNDARY = 5,     /* float4 (x_b, V_b) — PBF.boundaryData (last iteration) */
  PBF_FIELD_OMEGA = 6,        /* float4 (w, |w|)   — PBF.angularVelocity */
  PBF_FIELD_NORMAL = 7,       /* float4 (n, 0)     — PBF.normal */
  PBF_FIELD_DELTA_P = 8,      /* float4 (dp, 0)    — PBF.deltaPosition of the last iteration
                                 (kept only when capture is enabled) */
  PBF_FIELD_NEIGHBOR_COUNT = 9/* uint32 per particle — NeighborSearch.neighborCount */
} pbf_field;

typedef struct pbf_metrics {
  uint32_t particles;
  uint32_t nonfinite;        /* particles with a NaN/Inf in x or v */
  uint32_t penetrations;     /* particles whose boundary SDF is < 0 */
  uint32_t error_flags;      /* device error word (see PBF_DEVERR_*) */
  float max_compression;     /* max_i max(0, rho_i/rho0 - 1) */
  float mean_abs_density_err;/* mean_i |rho_i/rho0 - 1| */
  float max_abs_density_err; /* max_i |rho_i/rho0 - 1| */
  float kinetic_energy;      /* 0.5 m sum |v|^2 */
  float mean_compression;    /* mean_i max(0, rho_i/rho0 - 1) */
  uint32_t neighbor_total;   /* neighbour-list entries of the last substep */
  uint32_t fallback_steps;   /* learned-start substeps that fell back to the plain solve */
} pbf_metrics;

#define PBF_DEVERR_NEIGHBOR_OVERFLOW 0x1u
#define PBF_DEVERR_SCAN_TIMEOUT 0x2u
#define PBF_DEVERR_CELL_OVERFLOW 0x4u
#define PBF_DEVERR_MMA_TIMEOUT 0x8u  /* a tensor-core completion wait gave up (network pass) */
#define PBF_DEVERR_STAGE_TIMEOUT 0x10u /* a cell-block pass's shared-memory staging wait gave up (the tile
                                          then read global memory; results are still complete) */

typedef struct pbf_handle pbf_handle;

/* ---- life cycle: PBF constructor + initResource (src/simulator/PBF/PBF.ts:67-69,262-279) */
int pbf_config_default(pbf_config* cfg);
int pbf_create(const pbf_config* cfg, pbf_handle** out);
int pbf_destroy(pbf_handle* h);
/* PBF.reset (PBF.ts:71-89): clears all particle buffers, the particle array and the boundary. */
int pbf_reset(pbf_handle* h);
const char* pbf_last_error(const pbf_handle* h);
int pbf_abi_version(void);

/* ---- options: PBFConfig.setConfig / optionsChange (PBFConfig.ts:31-46,64-66) */
int pbf_set_options(pbf_handle* h, const pbf_options* opt);
int pbf_get_options(const pbf_handle* h, pbf_options* opt);

/* ---- scene seeding: SPH.voxelizeCube / voxelizeSphere (src/simulator/SPH.ts:99-149).
 * They append lattice points (spacing 2r) to the host particle array and
 * return how many were added; pbf_set_particle_position uploads the array
 * (PBFConfig.setParticlePosition, PBFConfig.ts:48-62). */
int pbf_voxelize_cube(pbf_handle* h, const float mn[3], const float mx[3], uint32_t* added);
int pbf_voxelize_sphere(pbf_handle* h, const float center[3], float radius, uint32_t* added);
/* SPH.voxelizeMesh (SPH.ts:151-187) on the GPU: lattice points at spacing
 * 2r over the mesh's world bounding box (the local vertex box's corners
 * through the world matrix, Box3.expandByObject) that a +z ray in the mesh's
 * local space shows to be inside (its nearest hit, over both face
 * orientations, is a face pointing along the ray).  vertices: float3 in local
 * space; indices: 3 per triangle; world: 4x4 column-major doubles, affine
 * (three.js Matrix4.elements of mesh.matrixWorld).  Appends to the host
 * particle array like pbf_voxelize_cube. */
int pbf_voxelize_mesh(pbf_handle* h, const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                      uint32_t triangle_count, const double world[16], uint32_t* added);
/* The same without a handle: up to `capacity` points (x, y, z, 0) into
 * out_xyzw, their number in *count (PBF_ECAPACITY if it exceeds capacity;
 * out_xyzw may be NULL with capacity 0 to count only). */
int pbf_voxelize_mesh_points(const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                             uint32_t triangle_count, const double world[16], double particle_radius, float* out_xyzw,
                             uint32_t capacity, uint32_t* count);
/* Scene seeding on the device.  No single counterpart in the reference: the
 * result equals pbf_reset's particle array cleared, the items voxelised in
 * order (PBF_SEED_CUBE = voxelizeCube(a, b); PBF_SEED_SPHERE =
 * voxelizeSphere(a, b[0]); PBF_SEED_MESH = voxelizeMesh of the mesh fields),
 * pbf_jitter_particles(jitter_amplitude, jitter_seed) when the amplitude is
 * positive, then pbf_set_particle_position — bit for bit — but the lattices,
 * the compaction and the jitter run on the GPU and the points are written
 * straight into the particle buffers (no host array, no upload; the host
 * particle array is left empty).  *total gets the number of particles the
 * items make; above max_particles nothing is seeded and PBF_ECAPACITY is
 * returned.  Lattices are limited to 4096 points per axis and 2^30 points
 * per item. */
enum { PBF_SEED_CUBE = 0, PBF_SEED_SPHERE = 1, PBF_SEED_MESH = 2 };
typedef struct pbf_seed_item {
  uint32_t kind;            /* PBF_SEED_* */
  float a[3];               /* cube: minimum corner; sphere: centre */
  float b[3];               /* cube: maximum corner; sphere: b[0] = radius */
  const float* vertices;    /* mesh: float3 per vertex, local space */
  uint32_t vertex_count;
  const uint32_t* indices;  /* mesh: 3 per triangle */
  uint32_t triangle_count;
  double world[16];         /* mesh: column-major affine world matrix */
} pbf_seed_item;
int pbf_seed_device(pbf_handle* h, const pbf_seed_item* items, uint32_t count, float jitter_amplitude,
                    uint64_t jitter_seed, uint32_t* total);
/* Seeded uniform jitter in [-amplitude, amplitude] on the host array (splitmix64). */
int pbf_jitter_particles(pbf_handle* h, float amplitude, uint64_t seed);
int pbf_host_particle_count(const pbf_handle* h, uint32_t* count);
int pbf_copy_host_particles(const pbf_handle* h, float* xyzw, uint32_t n);
int pbf_set_particle_position(pbf_handle* h);
/* Direct upload of n float4 positions (w ignored); velocities/accelerations are zeroed. */
int pbf_set_particles(pbf_handle* h, const float* xyzw, uint32_t n);
/* Optional: overwrite velocities (float4 per particle, by id). */
int pbf_set_velocities(pbf_handle* h, const float* xyzw, uint32_t n);
/* Optional: overwrite the accelerations (SPH.acceleration, float4 per
 * particle, by id): the XSPH / vorticity / tension force the next substep's
 * TimeIntegration applies (timeIntegration.ts:25-28).  With
 * pbf_set_particles and pbf_set_velocities it restores a saved state. */
int pbf_set_accelerations(pbf_handle* h, const float* xyzw, uint32_t n);

/* ---- boundary: PBF.setBoundaryData -> BoundaryModel.setData (PBF.ts:91-94, volumeMap.ts:23-39).
 * `text` is the .cdm file: "nx ny nz\n<len>\n<sdf floats>\n<len>\n<volume floats>".
 * The field covers the simulation domain. */
int pbf_set_boundary_data(pbf_handle* h, const char* text, size_t len);
/* The same, from arrays in the .cdm node layout; origin/extent give the box the field covers. */
int pbf_set_boundary_field(pbf_handle* h, const uint32_t res[3], const float origin[3],
                           const float extent[3], const float* sdf, const float* volume,
                           size_t nodes);
int pbf_clear_boundary(pbf_handle* h);
/* Number of floats per field for a resolution (BoundaryModel.FIELD_LENGTH, volumeMap.ts:7-11). */
size_t pbf_field_length(const uint32_t res[3]);

/* ---- volume-map generation (Bender et al. 2019 volume maps in the .cdm node layout).
 * The reference ships precomputed maps (public/model/torus.cdm,
 * domain_boundary.cdm); this builds maps for analytic shapes on the GPU in
 * FP64.  The SDF is the minimum over the shapes (positive on the fluid side);
 * the volume at a node x is
 *   V(x) = 0.8 * integral over |y| <= h of gamma(x + y) dy,
 *   gamma = 1 where SDF <= 0, C(SDF/h) for 0 < SDF < h (C = cubic spline,
 *   C(0) = 1), 0 beyond,
 * integrated with an n^3 Gauss-Legendre rule over [-h, h]^3. */
typedef enum pbf_shape_kind {
  PBF_SHAPE_BOX_CONTAINER = 0, /* fluid inside the box center +- size; solid outside */
  PBF_SHAPE_SPHERE = 1,        /* solid sphere, radius size[0] */
  PBF_SHAPE_CYLINDER = 2,      /* solid cylinder along y: radius size[0], half height size[1] */
  PBF_SHAPE_TORUS = 3,         /* solid torus around the y axis: radii size[0] (major), size[1] (minor) */
  PBF_SHAPE_BOX_SOLID = 4      /* solid box, half extents size */
} pbf_shape_kind;
typedef struct pbf_shape {
  uint32_t kind;
  float center[3];
  float size[3];
} pbf_shape;
/* Treat points outside the field's box as empty when integrating the volume
 * (the convention the reference's domain_boundary.cdm was built with). */
#define PBF_VOLMAP_OUTSIDE_EMPTY 0x1u
/* Evaluate gamma through the map's own cubic interpolation of the node SDF
 * (instead of the analytic SDF), as the reference's assets were built. */
#define PBF_VOLMAP_DISCRETE_SDF 0x2u
/* sdf_out / vol_out are host arrays of pbf_field_length(res) floats. */
int pbf_generate_volume_map(const pbf_shape* shapes, uint32_t count, const uint32_t res[3],
                            const float origin[3], const float extent[3], float support_radius,
                            uint32_t quadrature, uint32_t flags, float* sdf_out, float* vol_out);

/* Volumes for a given node SDF (e.g. of a triangle mesh), integrated through
 * the map's own cubic interpolation; vol_out has pbf_field_length(res) floats. */
int pbf_volume_from_sdf(const uint32_t res[3], const float origin[3], const float extent[3],
                        float support_radius, uint32_t quadrature, uint32_t flags, const float* sdf,
                        float* vol_out);

/* ---- stepping: PBF.run (PBF.ts:398-448) is one substep; the controller
 * calls it stepCount times per frame (src/controller.ts:375-376). */
int pbf_run(pbf_handle* h);
int pbf_step(pbf_handle* h, uint32_t frames);
/* PBF.runTimestamp (PBF.ts:450-510): one substep split into the four
 * reference intervals [integrate | neighbour search | constraint loop | non-pressure],
 * returned in milliseconds (CUDA events on the handle's stream). */
int pbf_run_timestamp(pbf_handle* h, float ms[4]);
int pbf_synchronize(pbf_handle* h);
/* SPH.pause / switch / start / stop (SPH.ts:82-84): a paused handle's pbf_run is a no-op. */
int pbf_set_paused(pbf_handle* h, int paused);
int pbf_is_paused(const pbf_handle* h);

/* Capture the whole frame (substeps x passes) in a CUDA graph and replay it. */
int pbf_enable_graph(pbf_handle* h, int enable);

/* Per-kernel device timing: when enabled, every launch of pbf_run / pbf_step
 * is bracketed by CUDA events on the handle's stream (graphs are bypassed).
 * pbf_get_kernel_timing synchronises, sums the durations per pass name and
 * clears the record. */
typedef struct pbf_kernel_time {
  char name[32];
  uint32_t launches;
  float total_ms;
} pbf_kernel_time;
int pbf_set_kernel_timing(pbf_handle* h, int enable);
int pbf_get_kernel_timing(pbf_handle* h, pbf_kernel_time* out, uint32_t max, uint32_t* count);

/* ---- state access */
uint32_t pbf_particle_count(const pbf_handle* h);
/* Device float4 (x, rho) per particle id, valid after each run/step — the
 * buffer the renderer binds (paricleRasterizer.ts:74-77). */
const float* pbf_position_device(pbf_handle* h);
const float* pbf_velocity_device(pbf_handle* h);
int pbf_copy_field(pbf_handle* h, int field, void* host, size_t bytes);
/* The positions of the last frame (x, y, z, density by particle id, the
 * buffer pbf_position_device exposes) copied to host memory asynchronously:
 * a device-side copy after the frame, then the host copy on a second stream,
 * so the host read overlaps the next frames and the call returns at once.
 * host: n float4 (16 n bytes), ideally pinned; it is complete after
 * pbf_synchronize, and must stay valid until then. */
int pbf_copy_positions_async(pbf_handle* h, float* host, size_t bytes);
int pbf_get_metrics(pbf_handle* h, pbf_metrics* out);
/* The neighbour search of the last substep (NeighborSearch's buffers,
 * src/simulator/neighbor/neighborSearch.ts:25-29): the cell key of each
 * particle's predicted position (by id, ParticleInsert), cellParticleCount
 * (per cell), cellOffset (per cell + 1: the exclusive scan and the total) and
 * particleSortIndexCopy (the order, slot -> particle id, stable by id within
 * a cell).  `count` must be the array's length (n, n, cells, cells + 1).
 * Valid right after a substep, before the next one; single-scene handles. */
typedef enum pbf_search_array {
  PBF_SEARCH_CELL_KEY = 0,
  PBF_SEARCH_CELL_COUNT = 1,
  PBF_SEARCH_CELL_OFFSET = 2,
  PBF_SEARCH_ORDER = 3
} pbf_search_array;
int pbf_copy_search_state(pbf_handle* h, int which, uint32_t* host, size_t count);
/* Keep per-iteration debug fields (PBF_FIELD_DELTA_P); off by default. */
int pbf_set_capture(pbf_handle* h, int enable);
void* pbf_stream(pbf_handle* h);

/* ---- neighbour search alone: NeighborSearch.execute (src/simulator/neighbor/neighborSearch.ts:270-301).
 * All pointers are device pointers.  Inputs: n float4 positions.  Outputs
 * (each may be NULL to skip): per-particle cell key (ParticleInsert),
 * per-cell count (cellParticleCount), per-cell exclusive offset
 * (cellOffset, cells+1 entries), the sorted order slot -> particle id
 * (particleSortIndexCopy), per-particle rank within its cell
 * (particleSortIndex), stable by particle id. */
typedef struct pbf_grid {
  float origin[3];
  float inv_cell[3];        /* cells per unit length per axis */
  uint32_t dim[3];
} pbf_grid;
typedef struct pbf_ns pbf_ns;
int pbf_ns_create(const pbf_grid* grid, uint32_t max_particles, void* stream, pbf_ns** out);
int pbf_ns_destroy(pbf_ns* ns);
int pbf_ns_run(pbf_ns* ns, const float* d_pos4, uint32_t n, uint32_t* d_keys,
               uint32_t* d_cell_count, uint32_t* d_cell_offset, uint32_t* d_order,
               uint32_t* d_rank);
/* Neighbour lists in the reference layout (NeighborCount + particle scan +
 * NeighborList, neighborShader.ts:101-246): d_nbr_offset has n+1 entries and
 * d_nbr_list holds particle ids.  Call after pbf_ns_run with the same positions.
 * Fails with PBF_ECAPACITY (writing nothing past capacity) if the lists need
 * more than `capacity` entries; *total receives the needed size. */
int pbf_ns_lists(pbf_ns* ns, const float* d_pos4, uint32_t n, float radius,
                 uint32_t* d_nbr_offset, uint32_t* d_nbr_list, uint32_t capacity,
                 uint32_t* total);
int pbf_ns_sync(pbf_ns* ns);
const char* pbf_ns_last_error(const pbf_ns* ns);
/* Per-phase device times of pbf_ns_run (no counterpart in the reference):
 * when enabled, each run records CUDA events on the context's stream and
 * pbf_ns_timings returns the last run's phases in milliseconds after
 * synchronising: [0] cell keys (ParticleInsert), [1] the stable radix-sort
 * passes (CountingSort; the last one also counts the cells), [2] cell
 * offsets (ExclusiveScan of the counts), [3] outputs (ranks, copies of
 * counts, offsets and order).  PBF_ESTATE before a timed run. */
int pbf_ns_set_timing(pbf_ns* ns, int enable);
int pbf_ns_timings(pbf_ns* ns, float ms[4]);

/* ---- exclusive scan (ExclusiveScan.execute, exclusiveScan.ts:134-166):
 * single-pass decoupled look-back over any length (no 512-multiple or
 * 262144 limit).  Scratch is owned by the call's context. */
int pbf_exclusive_scan_u32(const uint32_t* d_in, uint32_t* d_out, size_t n, void* stream);
/* Self-test of the bounded device waits (no counterpart in the reference):
 * runs a scan tile whose look-back waits on a predecessor that never
 * publishes; the wait gives up after its poll limit and the kernel
 * completes.  Returns PBF_ETIMEOUT when the give-up was reported as it
 * should be (the expected result), another status otherwise.  Takes a few
 * hundred milliseconds. */
int pbf_selftest_bounded_wait(void);

/* ---- learned lambda warm start.  No counterpart in the reference (its solve
 * is a fixed number of plain iterations, PBF.ts:417-431): an MLP
 * 8 -> 64 -> 64 -> 1 (SiLU, BF16 weights/activations, FP32 accumulate)
 * predicts an effective multiplier per particle from features at the
 * predicted positions: density error, previous substep's multiplier,
 * neighbour count, |v'| dt/h, velocity divergence -div(v') dt (by the
 * continuity equation: (rho_prev - rho*) / rho*, rho_prev the particle's
 * density after the previous substep), boundary SDF/h, boundary volume/V,
 * substep index.  One projection with it (ConstrainSolve with lambda_hat)
 * is followed by `iterations` plain iterations; when the substep's density
 * error — the mean over particles of max(0, rho/rho0 - 1) after the solve,
 * the mean_compression of pbf_get_metrics — exceeds `fallback_bound`, the
 * substep is re-solved from its predicted positions with the plain solve
 * (options.iterations), on the device, without a host round trip.  Training targets are the sums of the plain solver's
 * per-iteration multipliers, captured by the trace below. */
#define PBF_MLP_PARAMS 4801  /* W1 8x64, b1 64, W2 64x64, b2 64, w3 64, b3 */
typedef struct pbf_mlp {
  float params[PBF_MLP_PARAMS];
  float feat_mean[8];
  float feat_inv_std[8];
  float lam_scale;          /* target scale: the network predicts lambda / lam_scale */
} pbf_mlp;
/* Gradient kernels of the training (no counterpart in the reference):
 * PBF_MLP_TRAIN_TCGEN05 (the default) runs forward and backward on tcgen05.mma
 * with the accumulators in tensor memory, the weight and bias gradients
 * accumulated there over each CTA's 128-row tiles; PBF_MLP_TRAIN_MMA_SYNC is
 * the warp-level mma.sync.m16n8k16 kernel.  Both use the same bf16 rounding
 * points. */
#define PBF_MLP_TRAIN_TCGEN05 0u
#define PBF_MLP_TRAIN_MMA_SYNC 1u
typedef struct pbf_train_config {
  uint32_t epochs;
  uint32_t batch;
  float learning_rate;      /* Adam, cosine-decayed over the epochs */
  uint32_t kernel;          /* PBF_MLP_TRAIN_*: the gradient kernel (0: tcgen05) */
  uint64_t seed;
} pbf_train_config;
int pbf_mlp_init(pbf_mlp* m, uint64_t seed);
int pbf_mlp_fit_normalization(pbf_mlp* m, const float* feat, const float* target, uint32_t rows);
/* Host arrays: feat rows x 8 (raw features), out rows (lambda_hat). */
int pbf_mlp_forward(const pbf_mlp* m, const float* feat, uint32_t rows, float* out);
/* The same with a choice of inference kernel: PBF_MLP_KERNEL_MMA_SYNC
 * (mma.sync.m16n8k16, one warp per 16-row tile) or PBF_MLP_KERNEL_TCGEN05
 * (tcgen05.mma, 128-row tiles, accumulators in tensor memory).  Both use the
 * same bf16 rounding points; PBF_ETIMEOUT if a tensor-core wait gave up. */
#define PBF_MLP_KERNEL_MMA_SYNC 0u
#define PBF_MLP_KERNEL_TCGEN05 1u
int pbf_mlp_forward_ex(const pbf_mlp* model, const float* feat, uint32_t rows, float* out, uint32_t kernel);
/* Gradient of mean((y - target/lam_scale)^2) w.r.t. params (PBF_MLP_PARAMS floats), one GPU pass. */
int pbf_mlp_gradient(const pbf_mlp* m, const float* feat, const float* target, uint32_t rows, float* grad,
                     float* loss);
/* The same with a choice of gradient kernel (PBF_MLP_TRAIN_*); PBF_ETIMEOUT if
 * a tensor-core completion wait gave up. */
int pbf_mlp_gradient_ex(const pbf_mlp* m, const float* feat, const float* target, uint32_t rows, float* grad,
                        float* loss, uint32_t kernel);
int pbf_mlp_train(pbf_mlp* m, const float* feat, const float* target, uint32_t rows,
                  const pbf_train_config* cfg, float* final_loss);
/* Trace capture during plain substeps: every `stride`-th particle (hashed
 * with `salt`) appends (features, target) rows until `capacity`; 0 = off. */
int pbf_set_trace(pbf_handle* h, uint32_t capacity, uint32_t stride, uint64_t salt);
int pbf_trace_rows(pbf_handle* h, uint32_t* rows);
int pbf_copy_trace(pbf_handle* h, float* feat, float* target, uint32_t rows);
/* The plain solve's own density error over the traced substeps: the largest
 * and the average per-substep mean compression after the solve (the measure
 * the learned start's fallback test uses; its largest value is the bound at
 * which the learned start matches the plain solve's worst error). */
int pbf_trace_error(pbf_handle* h, float* max_mean, float* avg_mean);
/* Learned start: each substep projects once with the network's multipliers,
 * then runs `iterations` plain iterations (0 allowed); a substep whose mean
 * compression after the solve exceeds fallback_bound is re-solved on the
 * device with the plain solve from the same predicted positions.
 * model = NULL switches the learned start off.  A negative bound makes every
 * substep fall back (the result is then the plain solve's). */
int pbf_set_learned(pbf_handle* h, const pbf_mlp* model, uint32_t iterations, float fallback_bound);
/* Inference kernel of the learned start's network pass (PBF_MLP_KERNEL_*;
 * default PBF_MLP_KERNEL_TCGEN05). */
int pbf_set_mlp_kernel(pbf_handle* h, uint32_t kernel);
/* Adaptive iterations of the learned start (no counterpart in the reference):
 * when enabled, each of the `iterations` plain iterations after the learned
 * projection first measures the density error at its starting positions in
 * its lambda pass (the mean compression AttributeUpdate reports, fluid
 * only), and runs its position update only if that error exceeds the
 * fallback bound; otherwise the positions pass through unchanged.  The
 * substep's final error test and fallback are unchanged.  Off by default.
 * pbf_adaptive_counts: tests made and position updates run since the last
 * pbf_set_adaptive_iterations (device counters, so graph replays count). */
int pbf_set_adaptive_iterations(pbf_handle* h, int enable);
/* Lagged iteration control of the learned start (no counterpart in the
 * reference): with fraction > 0, a substep runs its plain iterations
 * (boundary sampling, lambda, delta-p) only when the previous substep's final
 * mean compression exceeded fraction x the fallback bound; otherwise it keeps
 * the learned projection alone.  The decision uses the error AttributeUpdate
 * already measured (no extra neighbour pass); the final error test and
 * fallback are unchanged.  fraction <= 0 turns it off (default); it takes
 * precedence over pbf_set_adaptive_iterations.  pbf_adaptive_counts then
 * reports decisions made and substeps that iterated. */
int pbf_set_lagged_iterations(pbf_handle* h, float fraction);
int pbf_adaptive_counts(pbf_handle* h, uint32_t* tests, uint32_t* updates_run);

/* ---- allocation-free exclusive scan.  No counterpart in the reference: an
 * addition for callers that cannot allocate device memory when they scan —
 * hosts whose own pool owns all device memory, real-time loops that must not
 * enter the allocator.  Same result as pbf_exclusive_scan_u32, but the
 * look-back scratch is a fixed static device array of about 256 KB that
 * every GPU loading this library keeps until exit, and the call allocates
 * nothing (no cudaMalloc / cudaMallocAsync / cudaFree).  Sizes above
 * PBF_SCAN_NOALLOC_MAX elements return PBF_ECAPACITY without launching
 * anything.  The call is synchronous: it reads the device error word back to
 * the host and synchronises `stream` before returning (so it cannot be
 * recorded into a CUDA graph).  The first call on a device looks up the
 * array's device address and caches it for the process; the library must
 * not be used on a device after cudaDeviceReset there.  All calls on a
 * device share the array: calls that overlap on the GPU (e.g. on unordered
 * streams) race and give wrong results; serialise them. */
#define PBF_SCAN_NOALLOC_MAX (1u << 26)
int pbf_exclusive_scan_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, size_t n, void* stream);

/* ---- launch shape and autotuner.  No counterpart in the reference (its
 * passes use a fixed workgroup size of 256).  The step's passes are
 * grid-stride loops over tiles of `block` slots: ctas_per_sm = 0 launches one
 * tile per CTA; k > 0 launches at most k CTAs per SM that loop over the
 * tiles.  cell_ratio is the hash-grid cell height (z) over the kernel
 * radius: 1 is the reference's grid (h cells, 27-cell search, neighbour order
 * and results as the reference); 0.5 keeps h in x and y and halves the cells
 * in z, searched as 3 x 3 columns of 5 half cells (2.5 h instead of 3 h of
 * candidates per column; the same neighbour sets, summed in a different
 * order, so results differ in rounding). */
typedef struct pbf_launch {
  uint32_t block;        /* threads per CTA: 128 or 256 (default 256) */
  uint32_t ctas_per_sm;  /* 0 (default) or 1..16 */
  float cell_ratio;      /* 1 (default) or 0.5 */
  uint32_t build;        /* neighbour-build variant: PBF_BUILD_THREAD (default, one slot
                            per thread), PBF_BUILD_PAIR (two slots of one cell per thread,
                            sharing candidate loads), PBF_BUILD_WARP (warp-cooperative
                            per cell: coalesced candidate chunks, ballot-collected hits);
                            or one of the cell-block modes, which replace the neighbour
                            lists: each neighbour pass runs one CTA per 128 sorted slots,
                            stages the tile's 27-cell halo (the 3 x 3 neighbouring
                            columns' slot runs) into shared memory with bulk copies and
                            walks it in the reference's neighbour order.
                            PBF_BUILD_CELLBLOCK_MASK keeps 9 membership masks per particle
                            (one 32-bit mask per neighbour column, written by a cell-block
                            search); PBF_BUILD_CELLBLOCK_FREE keeps no neighbour structure
                            and tests every candidate at the search positions in every
                            pass.  Both give the list's neighbour sets and order (exact
                            mode stays bit-identical to the reference method); single-scene
                            handles with ctas_per_sm = 0 only. */
} pbf_launch;
#define PBF_BUILD_THREAD 0u
#define PBF_BUILD_PAIR 1u
#define PBF_BUILD_WARP 2u
#define PBF_BUILD_CELLBLOCK_MASK 3u
#define PBF_BUILD_CELLBLOCK_FREE 4u
int pbf_set_launch(pbf_handle* h, const pbf_launch* launch);
/* Shared-memory plan of the cell-block passes (no counterpart in the
 * reference): the records per staged field a CTA holds (a multiple of 16 in
 * [16, 3072]; default 2048).  A tile whose halo needs more (or spans more
 * than 8 cell columns) walks global memory instead, with the same results. */
int pbf_set_cellblock_capacity(pbf_handle* h, uint32_t records);
int pbf_get_launch(const pbf_handle* h, pbf_launch* launch);

typedef struct pbf_tune_trial {
  pbf_launch launch;
  float ms_per_substep;
} pbf_tune_trial;
#define PBF_TUNE_CELL_RATIO 0x1u /* also try cell_ratio 0.5 */
/* Times `substeps` substeps (after 2 warm-up substeps) for every candidate
 * launch shape — block {128, 256} x ctas_per_sm {0, 2048/block} x
 * build {THREAD, PAIR, WARP} (x cell_ratio {1, 0.5} with PBF_TUNE_CELL_RATIO) — on
 * the current state, restores the state (positions, velocities,
 * accelerations, ids), keeps the fastest
 * shape (also returned in *best).  trials (up to max_trials) receive every
 * candidate's time.  PBF_ESTATE while trace capture is on. */
int pbf_autotune(pbf_handle* h, uint32_t substeps, uint32_t flags, pbf_tune_trial* trials, uint32_t max_trials,
                 uint32_t* count, pbf_launch* best);

/* ---- batched scenes.  The reference runs one scene per simulator; a batch
 * runs many independent scenes of uneven sizes, each with its own domain,
 * volume map and iteration count, in ONE launch per pass: the scenes share
 * the particle arrays (scene s holds ids and slots [first_id, first_id + n))
 * and one cell-key space (scene s's grid keys follow scene s-1's), so one
 * counting sort orders them all, and the passes look up each slot's scene in
 * a device table.  The shared pbf_config gives the particle/kernel radius,
 * density, time step, substeps, options (the default iteration count),
 * jitter, fp mode, interpolation and list slice; its domain, grid_dim and
 * max_particles are ignored.  Each scene's grid has floor(extent / (ratio h))
 * cells per axis (cells no smaller than ratio x h).  The returned handle
 * works with pbf_step / pbf_run / pbf_enable_graph (one graph per substep
 * group) / pbf_set_launch / pbf_autotune / pbf_copy_field (all scenes, by
 * global id) / pbf_get_metrics (all scenes); the single-scene setup calls
 * (particles, boundary, reset, learned start, trace) return PBF_ESTATE.  In
 * PBF_FP_EXACT mode a scene's results are bit-identical to the same scene
 * run alone with the same grid. */
typedef struct pbf_scene {
  uint32_t struct_size;    /* sizeof(pbf_scene) */
  uint32_t particles;
  const float* positions;  /* host float4 [particles]: x, y, z, (ignored) */
  float domain_min[3], domain_max[3];
  uint32_t iterations;     /* solver iterations; 0 = the shared options' count */
  uint32_t field_res[3];   /* volume-map cells per axis; 0,0,0 = no map */
  float field_origin[3], field_extent[3];
  const float* sdf;        /* pbf_field_length(field_res) nodes each, .cdm layout */
  const float* volume;
} pbf_scene;
typedef struct pbf_scene_info {
  uint32_t first_id;
  uint32_t particles;
  uint32_t iterations;
  uint32_t grid_dim[3];
  uint32_t cells;
} pbf_scene_info;
int pbf_batch_create(const pbf_config* shared, const pbf_scene* scenes, uint32_t count, pbf_handle** out);
uint32_t pbf_scene_count(const pbf_handle* h); /* 1 for a single-scene handle */
int pbf_get_scene_info(const pbf_handle* h, uint32_t scene, pbf_scene_info* out);
int pbf_get_scene_metrics(pbf_handle* h, uint32_t scene, pbf_metrics* out);

/* ---- screen-space fluid buffers: FilteredParticleFluid
 * (src/renderer/filteredParticleFluid/fluid.ts:150-185) without the WebGPU
 * render pipelines.  ParicleRasterizer.execute (paricleRasterizer.ts:170-204)
 * splats every particle of `position` twice: a camera-facing sprite of side
 * particle_radius into the depth map (W x H, eye-space depth of the nearest
 * sphere surface, 0 where empty; depthPassShader.ts), tested against and
 * written to the scene depth (reverse-Z, 'greater'), and a sprite of side
 * 2 * particle_radius into the volume map ((W/2) x (H/2), sum of
 * exp(-2 |uv|^2); volumePassShader.ts).  TextureFilter.execute
 * (textureFilter.ts:129-160, filterPassShader.ts) then applies the
 * separable narrow-range filter to the depth map when filter_size >= 2.
 * Everything runs as CUDA kernels on device buffers; the results are
 * deterministic (ties go to the lower particle index, the volume sum is
 * exact in 64-bit fixed point before one rounding to float). */
typedef struct pbf_render_options {  /* RenderingOptions (src/common/shader.ts:40-47) */
  uint32_t mode;          /* shading mode (kept for the screen-space shading pass) */
  uint32_t filter_size;   /* 0..32; < 2 disables the filter */
  float particle_radius;  /* rendering radius (0.02) */
  float opacity;
  float tint_color[3];    /* 0..1 */
} pbf_render_options;
typedef struct pbf_camera {  /* Camera uniform (src/common/shader.ts:2-10), column-major float32 */
  float position[3];
  float view[16];           /* matrixWorldInverse: affine */
  float view_inverse[16];   /* matrixWorld */
  float projection[16];     /* perspective (reverse-Z) or orthographic: no x/y shear */
  float params[4];
} pbf_camera;
typedef struct pbf_renderer pbf_renderer;
enum { PBF_RENDER_DEPTH = 0, PBF_RENDER_VOLUME = 1 };
int pbf_renderer_create(uint32_t width, uint32_t height, pbf_renderer** out);
int pbf_renderer_destroy(pbf_renderer* r);
/* FilteredParticleFluid.setConfig (fluid.ts:114-133). */
int pbf_renderer_set_config(pbf_renderer* r, const pbf_render_options* options);
/* The camera uniform (GlobalResource.update, globalResource.ts:165-181). */
int pbf_renderer_set_camera(pbf_renderer* r, const pbf_camera* camera);
/* Rasterize + filter for n particles at d_positions (device float4, xyz
 * used).  d_scene_depth: NULL (a cleared depth buffer, all 0) or a device
 * float [W*H] reverse-Z depth buffer, read and updated in place. */
int pbf_render(pbf_renderer* r, const float* d_positions, uint32_t n, float* d_scene_depth, void* stream);
/* TextureFilter.execute (textureFilter.ts:129-160) on any device r32float
 * image of width x height, in place, with options->filter_size and
 * options->particle_radius (threshold 5 r, high bound r). */
int pbf_texture_filter(const pbf_render_options* options, float* d_texture, uint32_t width, uint32_t height,
                       void* stream);
/* The same for a simulator's current particles (pbf_position_device, its stream). */
int pbf_render_simulation(pbf_renderer* r, pbf_handle* h, float* d_scene_depth);
const float* pbf_renderer_map_device(const pbf_renderer* r, uint32_t which); /* PBF_RENDER_* */
int pbf_renderer_map_size(const pbf_renderer* r, uint32_t which, uint32_t* width, uint32_t* height);
int pbf_renderer_copy_map(const pbf_renderer* r, uint32_t which, float* host, size_t bytes);
/* Device times of the last pbf_render: rasterization and filter
 * (FilteredParticleFluid.renderTimestamp, fluid.ts:150-175, timestamps 6-7). */
int pbf_renderer_timings(const pbf_renderer* r, float ms[2]);

#ifdef __cplusplus
}
#endif
#endif /* PBF_GB300_H */
