// pbf_params.h — plain-old-data parameter blocks passed by value to the kernels.
// Host code (pbf_api.cu) fills them from pbf_config; every derived constant
// is computed in double from the float configuration and rounded once.
#pragma once
#include <cstdint>

namespace pbf {

struct GridParams {
  float origin[3];
  float inv_cell[3];  // cells per unit length
  int dim[3];
  uint32_t cells;     // dim[0] * dim[1] * dim[2]
  uint32_t key_base;  // first key of this grid in a shared key space (batched scenes; 0 otherwise)
  int reach;          // neighbourhood half-width in cells along x and y
  int reach_z;        // ... along z (1: the 27-cell search; 2 when z cells are h/2)
};

struct FieldParams {
  int res[3];
  float origin[3];
  float scale[3];     // res / extent
  float gscale[3];    // 2 * res / extent (gradient scale, discreteFieldShader.ts:174)
  int quirk;          // reference volume-node quirk
  int trilinear;      // 1 = trilinear corner interpolation
  int loaded;
  uint32_t node_off;  // first node of this map in the concatenated SDF/volume arrays (batched scenes)
  uint32_t flag_off;  // first cell flag of this map in the concatenated flag array
};

struct SimParams {
  // kernels (common.ts:1-40)
  float h, h2, half_h, poly6, spiky, coh, coh_bias;
  // particle (SPH.ts:49-50, PBF.ts:328,390)
  float r, V, V2, m, rho0, two_rho0;
  // time integration
  float dt, inv_dt;
  float lambda_eps;
  float jitter;
  int jitter_mode;
  float dmin[3], dmax[3];
  // SimulationOptions (shader.ts:50-58)
  float gy, xsph, vorticity, tension;
  uint32_t n;
};

// Compression statistics of a solver iteration (learned-start fallback test).
struct SolveStats {
  unsigned int max_bits;     // max_i max(0, rho_i - 1) as float bits (non-negative)
  unsigned int count;        // particles accumulated
  unsigned long long sum_fx; // sum_i min(max(0, rho_i - 1), 1) in 2^-20 fixed point
};

// One scene of a batch: its grid (with its key range), volume map, domain and
// solver iterations.  Its particles occupy slots (and ids) [first, first + n)
// for the whole run: its keys sort after every earlier scene's keys.
struct SceneDesc {
  GridParams grid;
  FieldParams field;
  float dmin[3], dmax[3];
  uint32_t iterations;
  uint32_t first, n;
};

// Boundary band of the next boundary sampling: the particles whose field
// cell can produce a sample.  Whoever computes a new x* (the band pass, or
// delta-p for the next iteration) tests the cell flag: outside the band it
// writes bData = 0 (and SDF feature = 2h) at once, inside it appends the slot
// to the list that the sampling kernel then works through.
struct BandArgs {
  FieldParams f;        // the map (a batch uses each scene's own)
  const uint8_t* flag;  // per field cell, concatenated for batches
  float4* bdata;
  float* bsdf;          // optional: the learned start's SDF feature
  uint32_t* list;       // null: no band is built
  uint32_t* count;
};

// Packed node blocks of a volume map: for each field cell whose boundary
// sample can be non-zero (the band flag), its 32 SDF node values and then
// its 32 volume node values, in the node order of the 32-node cell, 16
// float4 (256 B) contiguous.  cell[] maps a field cell (the flag's index,
// concatenated for batches) to its block, or to kNoBlock.  The volume
// values are stored without the reference's node quirk; the sampler applies
// it to the loaded values.
struct FieldBlocks {
  const uint32_t* cell;
  const float4* nodes;
};
constexpr uint32_t kNoBlock = 0xffffffffu;

// Per-slot scene lookup of a batch; scene == nullptr for a single scene
// (every parameter then comes by value).
struct SceneTab {
  const SceneDesc* scene;
  const uint16_t* slot_scene;
};

// The boundary terms of the learned start's features, added by the network
// pass instead of the neighbour build (so the boundary sampling at x*_0 can
// run beside the build): the build writes the fluid density in feature 0
// and the network pass adds V_b W(x*_0 - x_b), then writes feature 0 =
// rho - 1, feature 5 = min(SDF, 2h) / h and feature 6 = V_b / V, with the
// build's own arithmetic (fast mode).
struct LateBoundary {
  const float4* bdata;  // null: the features are complete
  const float* bsdf;
  float h, h2, poly6, V;
};

// Input normalisation of the learned start's network.
struct MLPNorm {
  float mean[8];
  float inv_std[8];
  float lam_scale;
};

// Optional inputs/outputs of the constraint passes used by the learned
// start and by trace capture.  All null/zero in the plain solve.
struct SolverAux {
  const int* guard;          // non-null: the kernel returns unless *guard != 0 (fallback path)
  float* bsdf;               // boundary pass: SDF at x* (features)
  float* lam_sum;            // lambda pass: multiplier accumulated over this substep
  int lam_first;             // lambda pass: 1 = this iteration starts lam_sum
  float4* feat;              // lambda pass: 8 raw features per particle (2 x float4)
  const float4* pos;         // lambda pass (features): x before the predict step
  const float* lam_prev;     // lambda pass (features): previous substep's multiplier
  SolveStats* stats;         // lambda pass: compression statistics
  int late_boundary;         // learned start's build: feature 0 = fluid density, 5 and 6 left to the network pass
  float substep_index;       // lambda pass (features)
  const float* mlp;          // lambda pass (network): flat FP32 parameters
  MLPNorm norm;              // lambda pass (network)
  SceneTab tab;              // batched scenes: per-scene iteration counts, domains, maps
  int iter;                  // solver iteration of this launch (scenes with fewer iterations skip it)
  const float4* xs_in;       // delta-p pass: x* of a scene that skips the iteration is copied through
  BandArgs band;             // delta-p pass: the band of the next iteration's boundary sampling
  const int* need;           // delta-p pass: *need == 0 skips the iteration (x* copied through from xs_in)
};

// Inputs of the cell-block neighbour passes (pbf_cellblock.cuh): the grid and
// its cell offsets, the search-time cell key and position of every slot, and
// the membership masks of the mask variant.
struct CbArgs {
  GridParams g;
  const uint32_t* cell_start;  // [cells + 1]
  const uint32_t* skey;        // [n] cell key of each slot at x*_0
  const float4* xs0;           // [n] x*_0 of each slot (the search positions)
  const uint32_t* mask;        // [9][n] window membership masks (mask variant)
  const uint16_t* ovf;         // [n] bit q: window q has more than 32 candidates (mask variant)
  uint32_t* err;               // device error word
  uint32_t cap;                // staged records per field (shared-memory plan)
  uint32_t n;
};

// The learned start's fallback: the plain solve of one substep from the saved
// predicted positions, run as one cooperative kernel when the device flag is
// set (a no-op launch otherwise).
struct FallbackArgs {
  SimParams p;
  FieldParams f;
  const int* guard;
  const float* sdf;
  const float* vol;
  const uint8_t* bflag;
  const float4* pos_old;    // the state before this substep's reorder: x at the start of the
  const uint32_t* perm;     // substep is pos_old[perm[t]] (the reorder's own gather)
  const float4* xs_save;    // (x*_0, lambda_hat) as the network pass wrote it
  float4* pos;
  float4* vel;
  float4* xs0;
  float4* xs1;
  float4* xl;
  float4* bdata;
  float* lam_sum;
  const uint32_t* nbr_cnt;
  const uint32_t* nbr_list;
  uint32_t max_nbr;
  int iters;
  int final_buf;            // xs buffer (0/1) the learned solve ended in: the result goes there
};

}  // namespace pbf
