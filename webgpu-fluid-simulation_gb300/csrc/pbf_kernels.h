// pbf_kernels.h — host-visible declarations of the device kernels and launch
// helpers.  The float passes exist twice (exact / fast) and are reached
// through a PassTable of kernel pointers.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "pbf_params.h"

namespace pbf {

// The step's passes of one variant: single scene or batch (scene table),
// one tile per CTA or persistent (grid-stride).
struct PassSet {
  void (*predict)(SimParams, GridParams, SceneTab, const float4*, const float4*, const float4*, float4*, uint32_t*,
                  uint32_t*, uint32_t*);
  void (*nbr_build)(SimParams, GridParams, SceneTab, const float4*, const uint32_t*, uint32_t, uint32_t*, uint32_t*,
                    uint32_t*, uint32_t*);
  void (*nbr_build2)(SimParams, GridParams, SceneTab, const float4*, const uint32_t*, uint32_t, uint32_t*,
                     uint32_t*, uint32_t*, uint32_t*);  // two slots per thread
  void (*nbr_build_warp)(SimParams, GridParams, SceneTab, const float4*, const uint32_t*, uint32_t, uint32_t*,
                         uint32_t*, uint32_t*, uint32_t*);  // warp-cooperative per cell
  void (*band)(SimParams, SceneTab, const float4*, BandArgs);
  void (*boundary_band)(SimParams, FieldParams, const float*, const float*, FieldBlocks, SceneTab, const float4*,
                        float4*, float*, const uint32_t*, const uint32_t*, uint32_t*, const int*);
  void (*lambda)(SimParams, int, const float4*, const float4*, uint32_t, const uint32_t*, const uint32_t*, float4*,
                 SolverAux);
  void (*lambda_feat)(SimParams, int, const float4*, const float4*, uint32_t, const uint32_t*, const uint32_t*,
                      float4*, SolverAux);
  void (*lambda_stats)(SimParams, int, const float4*, const float4*, uint32_t, const uint32_t*, const uint32_t*,
                      float4*, SolverAux);     // null in batch sets
  void (*nbr_build_feat)(SimParams, GridParams, const float4*, const uint32_t*, uint32_t, uint32_t*, uint32_t*,
                         uint32_t*, uint32_t*, int, const float4*, SolverAux);  // null in batch sets
  void (*deltap)(SimParams, SolverAux, int, const float4*, const float4*, uint32_t, const uint32_t*, const uint32_t*,
                 float4*, float4*);
  void (*density_velocity)(SimParams, SolverAux, const float4*, uint32_t, const uint32_t*, const uint32_t*, float4*,
                           float4*);
  void (*vorticity)(SimParams, const float4*, const float4*, uint32_t, const uint32_t*, const uint32_t*, float4*,
                    float4*);
  void (*xsph)(SimParams, const float4*, const float4*, const float4*, const float4*, uint32_t, const uint32_t*,
               const uint32_t*, float4*);
  // fast mode: XSPH's neighbour sum split over the vorticity and XSPH passes (null in exact mode)
  void (*vorticity_split)(SimParams, const float4*, const float4*, uint32_t, const uint32_t*, const uint32_t*,
                          float4*, float4*, float4*, float4*);
  void (*xsph_split)(SimParams, const float4*, const float4*, const float4*, const float4*, const float4*, uint32_t,
                     const uint32_t*, const uint32_t*, float4*);
};

// The cell-block passes of one membership variant (pbf_cellblock.cuh).
struct CbSet {
  void (*lambda)(SimParams, CbArgs, int, const float4*, const float4*, float4*, SolverAux);
  void (*lambda_feat)(SimParams, CbArgs, int, const float4*, const float4*, float4*, SolverAux);
  void (*lambda_stats)(SimParams, CbArgs, int, const float4*, const float4*, float4*, SolverAux);
  void (*deltap)(SimParams, CbArgs, SolverAux, int, const float4*, const float4*, float4*, float4*);
  void (*density_velocity)(SimParams, CbArgs, SolverAux, const float4*, float4*, float4*, uint32_t*);
  void (*vorticity)(SimParams, CbArgs, const float4*, const float4*, float4*, float4*);
  void (*xsph)(SimParams, CbArgs, const float4*, const float4*, const float4*, const float4*, float4*);
  void (*vorticity_split)(SimParams, CbArgs, const float4*, const float4*, float4*, float4*, float4*, float4*);
  void (*xsph_split)(SimParams, CbArgs, const float4*, const float4*, const float4*, const float4*, const float4*,
                     float4*);
  void (*fallback)(FallbackArgs, CbArgs);  // cooperative launch only
};

struct PassTable {
  // the stand-alone neighbour search (reference list layout)
  void (*nbr_count)(SimParams, GridParams, const float4*, const uint32_t*, uint32_t*);
  void (*nbr_list)(SimParams, GridParams, const float4*, const uint32_t*, const uint32_t*, uint32_t*, uint32_t,
                   uint32_t*);
  PassSet set[2][2];  // [batch][persistent]
  void (*fallback)(FallbackArgs);  // cooperative launch only
  // cell-block passes: the search (masks; with the learned start's features)
  // and the passes per membership variant [mask, test]
  void (*cb_build)(SimParams, CbArgs, uint32_t*, uint16_t*, uint32_t*, int, const float4*, SolverAux);
  void (*cb_build_feat)(SimParams, CbArgs, uint32_t*, uint16_t*, uint32_t*, int, const float4*, SolverAux);
  CbSet cb[2];
};

namespace exact {
void fill_pass_table(PassTable* tbl);
}
namespace fast {
void fill_pass_table(PassTable* tbl);
}

// ---- integer pipeline (pbf_sort.cu) ---------------------------------------------
// Elements per tile of the single-pass scan.
constexpr size_t kScanTileElements = 2048;
// Scratch of the single-pass scan for up to `n` elements, in bytes:
// 256 bytes (tile counter) + one 8-byte status word per tile.
size_t scan_scratch_bytes(size_t n);
// Exclusive scan of n u32 (out may alias nothing in in).  `scratch` holds
// scan_scratch_bytes(n) bytes; err receives PBF_DEVERR_SCAN_TIMEOUT when a
// bounded look-back wait gives up.
cudaError_t launch_exclusive_scan(const uint32_t* in, uint32_t* out, size_t n, void* scratch, uint32_t* err,
                                  cudaStream_t st);
// Self-test of the scan's bounded look-back wait (a predecessor status that
// nothing writes): *err receives PBF_DEVERR_SCAN_TIMEOUT.
cudaError_t launch_scan_timeout_selftest(uint32_t* err, cudaStream_t st);

// Counting-sort pipeline shared by the step and the stand-alone search.
struct SortBuffers {
  uint32_t* key;        // [n] cell key per input slot
  uint32_t* rank;       // [n] warp-aggregated (unordered) rank per input slot
  uint32_t* cell_count; // [cells + 1]
  uint32_t* cell_start; // [cells + 1] exclusive scan of cell_count
  uint32_t* perm_raw;   // [n] scattered slots (unordered within a cell)
  uint32_t* id_raw;     // [n] particle id of perm_raw entries
  uint32_t* perm;       // [n] output: sorted slot -> input slot, stable by id
  uint32_t* tmp_a;      // [n] radix scratch for very full cells
  uint32_t* tmp_b;      // [n]
  uint32_t* big_list;   // [cells] cells sorted by the block radix path
  uint32_t* big_count;  // [1]
  void* scan_scratch;
  uint32_t* err;
};

// Stable LSD radix sort of points in particle-id order by cell key (the
// stand-alone search): keys[n] (by id) receive the cell keys, skeys[n] the
// sorted keys and order[n] the ids in sorted order, stable by id.  tmp_k /
// tmp_v: two pairs of n-entry scratch arrays; scratch: radix_scratch_bytes(n)
// bytes.  after_keys (optional) is recorded after the keys.  cell_count
// (cells + 1 entries, zeroed by the caller) receives the cell counts from the
// last pass.
struct RadixPlan {
  int passes, width;
  size_t tiles;
};
RadixPlan radix_plan(uint32_t cells, size_t n);
size_t radix_scratch_bytes(size_t n);
cudaError_t launch_radix_sort_idorder(GridParams g, const float4* pos, uint32_t n, uint32_t* keys, uint32_t* skeys,
                                      uint32_t* order, uint32_t* const tmp_k[2], uint32_t* const tmp_v[2],
                                      void* scratch, uint32_t* err, cudaStream_t st, cudaEvent_t after_keys,
                                      uint32_t* cell_count);
// Exclusive offsets (cells + 1 entries) of the cell counts.
cudaError_t launch_cell_offsets(uint32_t cells, const uint32_t* cell_count, uint32_t* cell_start, void* scan_scratch,
                                uint32_t* err, cudaStream_t st);
// rank_out[order[q]] = q - cell_start[skeys[q]].
cudaError_t launch_rank_sorted(uint32_t n, const uint32_t* skeys, const uint32_t* order, const uint32_t* cell_start,
                               uint32_t* rank_out, cudaStream_t st);
// scatter + stable within-cell order + (optionally) gather of the particle state.
cudaError_t launch_sort_by_cell(GridParams g, uint32_t n, const uint32_t* ids, SortBuffers& b, uint32_t id_bits,
                                cudaStream_t st);
// f_in / f_out (optional): one scalar per particle gathered along (the
// learned start's previous multiplier sum).
cudaError_t launch_gather_state(uint32_t n, const uint32_t* perm, const float4* pos_in, const float4* xs_in,
                                const uint32_t* id_in, float4* pos_out, float4* xs_out, uint32_t* id_out,
                                cudaStream_t st, const float* f_in = nullptr, float* f_out = nullptr);
// The same gather that also writes, for the cell-block passes, the cell key
// of each sorted slot (skey_out[t] = key_in[perm[t]]) and a second copy of
// the predicted positions x*_0 (xs0_out) that the solve leaves untouched.
cudaError_t launch_gather_state_cb(uint32_t n, const uint32_t* perm, const float4* pos_in, const float4* xs_in,
                                   const uint32_t* id_in, const uint32_t* key_in, float4* pos_out, float4* xs_out,
                                   uint32_t* id_out, uint32_t* skey_out, float4* xs0_out, cudaStream_t st,
                                   const float* f_in = nullptr, float* f_out = nullptr);
cudaError_t launch_scatter_by_id(uint32_t n, const uint32_t* id, const float4* src, float4* dst, cudaStream_t st);
// dst[id[t]] = src[t].w (a scalar kept in the w lane of a packed float4 array)
cudaError_t launch_scatter_w_by_id(uint32_t n, const uint32_t* id, const float4* src, float* dst, cudaStream_t st);
cudaError_t launch_scatter_by_id_u32(uint32_t n, const uint32_t* id, const uint32_t* src, uint32_t* dst,
                                     cudaStream_t st);
cudaError_t launch_list_to_ids(uint32_t total, const uint32_t* list, const uint32_t* id, uint32_t* out,
                               cudaStream_t st);
// dst[id_off[ids[t]] + q] = src[slot_off[t] + q] for each slot t's run.
cudaError_t launch_copy_runs(uint32_t n, const uint32_t* slot_off, const uint32_t* id_off, const uint32_t* ids,
                             const uint32_t* src, uint32_t* dst, cudaStream_t st);

// Metrics (max / mean density error, kinetic energy, non-finite and penetration counts).
struct MetricsAccum {
  float max_compression;
  float max_abs_err;
  double sum_abs_err;
  double kinetic;
  uint32_t nonfinite;
  uint32_t penetrations;
};
cudaError_t launch_metrics(SimParams p, FieldParams f, const float* sdf, const float4* pos, const float4* vel,
                           const uint32_t* nbr_count, uint32_t n, float* accum_f, double* accum_d, uint32_t* accum_u,
                           cudaStream_t st);

// Learned start (pbf_learned.cu).
}  // namespace pbf
#include "../../include/pbf_gb300.h"
namespace pbf {
// lambda_hat per feature row into d_lambda, or, with d_xl, packed as
// d_xl[r] = (d_xs[r].xyz, lambda_hat); d_lam_sum (optional) starts the sum.
cudaError_t launch_mlp_infer(const float* d_params, const pbf_mlp& model, const float* d_feat, uint32_t rows,
                             float* d_lambda, float* d_lam_sum, cudaStream_t st, const float4* d_xs = nullptr,
                             float4* d_xl = nullptr);
// The same on the 5th-generation tensor cores (tcgen05.mma, TMEM
// accumulators; pbf_mlp_tc.cu); d_err receives PBF_DEVERR_MMA_TIMEOUT when a
// bounded completion wait gives up.
cudaError_t launch_mlp_infer_tc(const float* d_params, const pbf_mlp& model, const float* d_feat, uint32_t rows,
                                float* d_lambda, float* d_lam_sum, cudaStream_t st, const float4* d_xs,
                                float4* d_xl, uint32_t* d_err, LateBoundary lb = LateBoundary{});
// Forward + backward on tcgen05.mma (pbf_mlp_tc.cu): the gradient accumulates
// into d_grad (atomically), the summed squared error into d_loss; d_err
// receives PBF_DEVERR_MMA_TIMEOUT when a bounded completion wait gives up.
cudaError_t launch_mlp_grad_tc(const float* d_params, const pbf_mlp& model, const float* d_feat,
                               const float* d_target, uint32_t rows, float* d_grad, float* d_loss, uint32_t* d_err,
                               cudaStream_t st);
cudaError_t launch_mlp_grad(const float* d_params, const pbf_mlp& model, const float* d_feat, const float* d_target,
                            uint32_t rows, float* d_grad, float* d_loss, cudaStream_t st);
cudaError_t launch_fallback_decide(SolveStats* stats, float bound, int* flag, uint32_t* fallbacks, float* last_mean,
                                   cudaStream_t st);
// Lagged iteration control (counts[0] decisions, counts[1] substeps that iterated).
cudaError_t launch_lagged_decide(const float* last_mean, float threshold, int* flag, uint32_t* counts,
                                 cudaStream_t st);
// The adaptive iteration's test (counts[0] tests, counts[1] position updates run).
cudaError_t launch_iterate_decide(SolveStats* stats, float bound, int* flag, uint32_t* counts, float* last_mean,
                                  cudaStream_t st);
cudaError_t launch_stats_record(SolveStats* stats, float* rec, cudaStream_t st);
cudaError_t launch_trace_append(uint32_t n, const uint32_t* ids, const float4* feat, const float* lam_sum,
                                uint32_t stride, uint32_t salt, float* tf, float* tt, uint32_t* count, uint32_t cap,
                                cudaStream_t st);
// ---- scene seeding (pbf_seed.cu) -------------------------------------------------
// Writes the points of `items` (cube / sphere / mesh lattices, in order) to
// out[0 .. *total) as (x, y, z, 0), applies the host jitter's splitmix64
// draws when jitter > 0 and sets ids[i] = i.  *total gets the number of
// points the items make even on PBF_ECAPACITY (nothing beyond capacity is
// written).  Synchronises `st` before returning.
int seed_device(const pbf_seed_item* items, uint32_t count, double radius, float jitter, uint64_t seed, float4* out,
                uint32_t* ids, uint32_t capacity, uint32_t* total, cudaStream_t st);
// SPH.voxelizeMesh on the device with the kept points copied to *pts (when
// emit) and their number in *kept.
int voxelize_mesh_host(const float* vertices, uint32_t vertex_count, const uint32_t* indices, uint32_t triangle_count,
                       const double* world, double particle_radius, bool emit, std::vector<float>* pts,
                       uint32_t* kept);

}  // namespace pbf
