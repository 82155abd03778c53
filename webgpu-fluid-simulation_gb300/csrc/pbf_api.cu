// pbf_api.cu — the C ABI (include/pbf_gb300.h): handle life cycle, scene
// seeding, boundary upload, the substep driver and state access.
//
// One pbf_handle plays the role of the reference's PBF object
// (src/simulator/PBF/PBF.ts:27-576) together with its NeighborSearch
// (src/simulator/neighbor/neighborSearch.ts) and BoundaryModel
// (src/simulator/boundary/volumeMap.ts).  Device state is kept in
// cell-sorted slot order; the id-ordered `position` buffer the renderer reads
// is refreshed at the end of every pbf_run / pbf_step.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"
#include "pbf_device.cuh"
#include "pbf_kernels.h"

using namespace pbf;

namespace {

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    n = count;
    if (count == 0) count = 1;
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace

struct pbf_handle {
  pbf_config cfg;
  SimParams sp;
  GridParams gp;
  FieldParams fp;
  PassTable passes;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // asynchronous position reads: their stream, events and the staging copy
  cudaStream_t copy_stream = nullptr;
  // the learned start's boundary sampling at x*_0 beside the neighbour build
  // (fast mode, tcgen05 network): its stream and the fork / join events
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_frame = nullptr, ev_staged = nullptr;
  DBuf<float4> staging;
  std::string err;
  uint32_t n = 0;
  bool paused = false;
  bool capture = false;
  int cur = 0;  // which of pos[]/ids[] holds the current state
  std::vector<float> host_particles;  // SPH.particlePositionArray

  DBuf<float4> pos[2], xs[2], xl, vel, acc, bdata, omega, normal, dp, out_pos, out_tmp;
  DBuf<float4> visc, coh;  // fast mode: XSPH's viscosity and cohesion sums from the vorticity pass
  DBuf<uint32_t> ids[2], key, rank, perm_raw, id_raw, perm, tmp_a, tmp_b;
  DBuf<uint32_t> cell_count, cell_start, big_list, big_count;
  DBuf<uint32_t> nbr_count, nbr_max, nbr_list;
  DBuf<uint32_t> band_list[2], band_count;  // boundary band lists (ping-pong) and their lengths
  // cell-block passes (PBF_BUILD_CELLBLOCK_*): cell key and x*_0 per sorted
  // slot, the 9 window masks per slot and their overflow bits
  DBuf<uint32_t> skey, cb_mask;
  DBuf<uint16_t> cb_ovf;
  DBuf<float4> xs0;
  uint32_t cb_cap = 2048;   // staged records per field and CTA
  unsigned cb_fb_grid = 0;  // CTAs of the cell-block fallback kernel
  DBuf<float> sdf, vol;
  DBuf<uint8_t> bflag;  // per field cell: 1 when the boundary sample can be non-zero
  DBuf<uint32_t> bcell;  // per field cell: its packed node block, or kNoBlock (FieldBlocks)
  DBuf<float4> bnodes;   // 16 float4 per flagged field cell
  DBuf<uint32_t> err_word;
  DBuf<float> m_f;
  DBuf<double> m_d;
  DBuf<uint32_t> m_u;
  void* scan_scratch = nullptr;
  uint32_t nbr_slice = 0;  // list entries per particle (fixed slice)
  uint32_t id_bits = 1;

  cudaGraphExec_t graph_exec = nullptr;
  bool graph_enabled = false;
  bool graph_valid = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  uint32_t last_nbr_total = 0;
  // learned start and trace capture
  bool learned = false;
  uint32_t mlp_kernel = PBF_MLP_KERNEL_TCGEN05;  // network pass of the learned start
  uint32_t learned_iters = 2;
  float fallback_bound = 0.01f;
  // adaptive iterations (pbf_set_adaptive_iterations): each of the learned
  // start's iterations runs its position update only while the density error
  // at its start exceeds the fallback bound.  stats[1], fb_flag[1] and
  // fb_mean[1] hold the test's statistics, flag and last mean; fb_count[1..2]
  // count the tests and the updates run (on the device: graph replays count).
  bool adaptive = false;
  // lagged iteration control (pbf_set_lagged_iterations): a substep's
  // iterations run only when the previous substep's final mean compression
  // (fb_mean[0]) exceeded lagged_fraction x the bound; 0 = off.  Uses the same
  // flag and counters as the adaptive test.
  float lagged_fraction = 0.0f;
  pbf_mlp model;
  DBuf<float> mlp_params, lam_sum, lam_prev, bsdf, fb_mean;
  DBuf<float4> feat, xs_save;
  DBuf<SolveStats> stats;
  DBuf<int> fb_flag;
  DBuf<uint32_t> fb_count;
  uint32_t trace_cap = 0, trace_stride = 1;
  uint64_t trace_salt = 0;
  uint32_t substep_counter = 0;
  DBuf<float> trace_feat, trace_tgt, trace_err;  // trace_err: [max, sum, count] of the plain solve's error
  DBuf<uint32_t> trace_count;
  // launch shape of the step's passes (pbf_set_launch / pbf_autotune)
  int blk = 256;            // threads per CTA
  uint32_t grid_cap = 0;    // CTAs per launch at most (0: one tile of blk slots per CTA)
  uint32_t per_sm = 0;      // grid_cap / SM count as set by the caller
  float cell_ratio = 1.0f;  // grid cell edge / h
  uint32_t build = PBF_BUILD_THREAD;  // neighbour-build variant
  int sms = 152;            // SM count of the device
  unsigned fb_grid = 0;     // CTAs of the cooperative fallback kernel (resident wave)
  // batched scenes (pbf_batch_create)
  bool batch = false;
  std::vector<pbf_scene_info> scene_info;
  std::vector<SceneDesc> scenes;
  DBuf<SceneDesc> scenes_dev;
  DBuf<uint16_t> slot_scene;
  SceneTab tab{nullptr, nullptr};
  // per-kernel timing (pbf_set_kernel_timing)
  bool ktiming = false;
  std::vector<cudaEvent_t> kt_events;
  std::vector<std::pair<int, size_t>> kt_pairs;  // (pass id, index of the first event)
};

namespace {

enum PassId {
  K_PREDICT, K_SORT, K_GATHER, K_NBR_BUILD, K_BOUNDARY, K_LAMBDA, K_DELTAP, K_DENSITY, K_VORTICITY, K_XSPH,
  K_EXPORT, K_FEATURES, K_MLP, K_FALLBACK, K_NUM
};
const char* kPassNames[K_NUM] = {"predict",   "sort", "gather", "nbr_build", "boundary",     "lambda", "deltap_apply",
                                 "density_velocity", "vorticity", "xsph", "export", "nbr_build_feat", "mlp",
                                 "fallback_guarded"};

// Brackets one launch (or one group of launches) with events when timing is on.
struct KScope {
  pbf_handle* h;
  int id;
  size_t ev;
  KScope(pbf_handle* hh, int pass) : h(hh), id(pass), ev((size_t)-1) {
    if (!h->ktiming) return;
    ev = h->kt_pairs.size() * 2;
    while (h->kt_events.size() < ev + 2) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) {
        ev = (size_t)-1;
        return;
      }
      h->kt_events.push_back(e);
    }
    cudaEventRecord(h->kt_events[ev], h->stream);
  }
  ~KScope() {
    if (ev == (size_t)-1) return;
    cudaEventRecord(h->kt_events[ev + 1], h->stream);
    h->kt_pairs.emplace_back(id, ev);
  }
};

int fail(pbf_handle* h, int code, const char* fmt, ...) {
  if (h) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->err = buf;
  }
  return code;
}

#define CU(h, call)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return fail((h), PBF_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Hash grid over [dmin, dmax].  Cell ratio 1 keeps the reference's grid: the
// given dims, else ceil(extent / h) cells per axis, searched over 27 cells.
// Other ratios (and every batched scene: floor_dims) use floor(extent / h)
// cells in x and y and floor(extent / (ratio h)) in z, so no cell is smaller
// than h across and ratio h high; a search of +-1 cells in x and y and
// +-ceil(1/ratio) in z covers the kernel radius.  Keys are z-fastest, so the
// finer z only lengthens the 9 runs (5 half cells, 2.5 h, instead of 3 h).
GridParams make_grid(const float dmin[3], const float dmax[3], float hk, float ratio, const uint32_t fixed_dim[3],
                     bool floor_dims) {
  GridParams g{};
  uint64_t cells = 1;
  const bool ref = ratio == 1.0f && !floor_dims;
  for (int a = 0; a < 3; ++a) {
    double ext = (double)dmax[a] - (double)dmin[a];
    int d = fixed_dim ? (int)fixed_dim[a] : 0;
    if (d == 0) {
      if (ref) {
        d = (int)std::ceil(ext / (double)hk);
      } else {
        // x and y cells of at least h; z cells of at least ratio h
        d = (int)std::floor(ext / ((a == 2 ? (double)ratio : 1.0) * (double)hk));
        if (d < 1) d = 1;
      }
    }
    g.dim[a] = d;
    g.origin[a] = dmin[a];
    g.inv_cell[a] = (float)((double)d / ext);
    cells *= (uint64_t)d;
  }
  g.cells = cells > 0xfffffffeull ? 0u : (uint32_t)cells;
  g.key_base = 0;
  g.reach = 1;
  g.reach_z = ratio == 1.0f ? 1 : (int)std::ceil(1.0 / (double)ratio - 1e-9);
  return g;
}

void derive_params(pbf_handle* h) {
  const pbf_config& c = h->cfg;
  const double PI = 3.14159265358979323846;
  SimParams& p = h->sp;
  double hh = c.kernel_radius, r = c.particle_radius;
  p.h = (float)hh;
  p.h2 = (float)(hh * hh);
  p.half_h = (float)(0.5 * hh);
  p.poly6 = (float)(315.0 / (64.0 * PI * std::pow(hh, 9)));
  p.spiky = (float)(-45.0 / (PI * std::pow(hh, 6)));
  p.coh = (float)(32.0 / (PI * std::pow(hh, 9)));
  p.coh_bias = (float)(-std::pow(hh, 6) / 64.0);
  double diam = 2.0 * r;
  double V = 0.9 * diam * diam * diam;
  p.r = (float)r;
  p.V = (float)V;
  p.V2 = (float)(V * V);
  p.m = (float)(V * (double)c.rest_density);
  p.rho0 = c.rest_density;
  p.two_rho0 = (float)(2.0 * (double)c.rest_density);
  p.dt = c.time_step;
  p.inv_dt = (float)(1.0 / (double)c.time_step);
  p.lambda_eps = c.lambda_eps;
  p.jitter = c.wall_jitter;
  p.jitter_mode = (int)c.jitter_mode;
  for (int a = 0; a < 3; ++a) {
    p.dmin[a] = c.domain_min[a];
    p.dmax[a] = c.domain_max[a];
  }
  p.gy = (float)(-(double)c.options.gravity);
  p.xsph = c.options.xsph;
  p.vorticity = c.options.vorticity;
  p.tension = c.options.surface_tension;
  p.n = h->n;

  h->gp = make_grid(c.domain_min, c.domain_max, c.kernel_radius, h->cell_ratio, c.grid_dim, false);
}

FieldParams make_field(const pbf_config& c, const uint32_t res[3], const float origin[3], const float extent[3]) {
  FieldParams f{};
  for (int a = 0; a < 3; ++a) {
    f.res[a] = (int)res[a];
    f.origin[a] = origin[a];
    f.scale[a] = (float)((double)res[a] / (double)extent[a]);
    f.gscale[a] = (float)(2.0 * (double)res[a] / (double)extent[a]);
  }
  f.quirk = c.volume_quirk ? 1 : 0;
  f.trilinear = c.boundary_interp == PBF_INTERP_TRILINEAR ? 1 : 0;
  f.loaded = 1;
  return f;
}

void set_field_params(pbf_handle* h, const uint32_t res[3], const float origin[3], const float extent[3]) {
  FieldParams& f = h->fp;
  for (int a = 0; a < 3; ++a) {
    f.res[a] = (int)res[a];
    f.origin[a] = origin[a];
    f.scale[a] = (float)((double)res[a] / (double)extent[a]);
    f.gscale[a] = (float)(2.0 * (double)res[a] / (double)extent[a]);
  }
  f.quirk = h->cfg.volume_quirk ? 1 : 0;
  f.trilinear = h->cfg.boundary_interp == PBF_INTERP_TRILINEAR ? 1 : 0;
}

inline unsigned nblocks(uint32_t n, int t) { return (n + t - 1) / t; }

// Grid of a step pass over n slots: one tile of blk slots per CTA, capped
// at grid_cap CTAs (the kernels loop over the remaining tiles).
inline unsigned grid_of(const pbf_handle* h, uint32_t n) {
  unsigned g = nblocks(n, h->blk);
  if (h->grid_cap && g > h->grid_cap) g = h->grid_cap;
  return g ? g : 1u;
}

// Cell-block passes in use (PBF_BUILD_CELLBLOCK_*): single scene, one tile per CTA.
inline bool cb_active(const pbf_handle* h) {
  return (h->build == PBF_BUILD_CELLBLOCK_MASK || h->build == PBF_BUILD_CELLBLOCK_FREE) && !h->batch &&
         h->grid_cap == 0;
}
constexpr int kMemMaskHost = 0;  // CbSet index of the mask variant (1: the list-free variant)
inline int cb_memb(const pbf_handle* h) { return h->build == PBF_BUILD_CELLBLOCK_FREE ? 1 : kMemMaskHost; }
inline unsigned cb_grid(uint32_t n) { return (n + 127u) / 128u; }
// Dynamic shared memory of a cell-block pass staging kP fields (+ x*_0 when
// membership is tested).
inline size_t cb_smem(const pbf_handle* h, int kP) {
  return (size_t)(kP + cb_memb(h)) * h->cb_cap * sizeof(float4);
}
CbArgs cb_args(const pbf_handle* h) {
  CbArgs A{};
  A.g = h->gp;
  A.cell_start = h->cell_start.p;
  A.skey = h->skey.p;
  A.xs0 = h->xs0.p;
  A.mask = h->cb_mask.p;
  A.ovf = h->cb_ovf.p;
  A.err = h->err_word.p;
  A.cap = h->cb_cap;
  A.n = h->n;
  return A;
}

void invalidate_graph(pbf_handle* h) {
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  h->graph_exec = nullptr;
  h->graph_valid = false;
}

// Reads and clears the device error word.  A neighbour-list overflow (a
// particle with more neighbours than the per-particle slice) grows the slice
// to 1.25x the largest count seen; the results of that substep are invalid
// (its lists were truncated) and the overflow is reported once.
int check_device_errors(pbf_handle* h) {
  uint32_t e = 0;
  CU(h, cudaMemcpyAsync(&e, h->err_word.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  if (e) {
    CU(h, cudaMemsetAsync(h->err_word.p, 0, sizeof(uint32_t), h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    if (e & PBF_DEVERR_NEIGHBOR_OVERFLOW) {
      uint32_t need = 0;
      CU(h, cudaMemcpy(&need, h->nbr_max.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
      CU(h, cudaMemset(h->nbr_max.p, 0, sizeof(uint32_t)));
      const uint64_t rows = ((uint64_t)h->cfg.max_particles + 31) / 32 * 32;
      uint64_t grow = (uint64_t)need + need / 4 + 4;
      if (grow * rows > 0xffffffffull) grow = 0xffffffffull / rows;
      const uint32_t old = h->nbr_slice;
      if (grow > old) {
        invalidate_graph(h);
        h->nbr_list.release();
        CU(h, h->nbr_list.alloc(rows * grow));
        h->nbr_slice = (uint32_t)grow;
      }
      return fail(h, PBF_ECAPACITY,
                  "neighbour list overflow: a particle has %u neighbours, the per-particle capacity was %u; grown "
                  "to %u, the last substep's results are invalid",
                  need, old, h->nbr_slice);
    }
    if (e & PBF_DEVERR_SCAN_TIMEOUT) return fail(h, PBF_ETIMEOUT, "scan look-back wait gave up");
    if (e & PBF_DEVERR_MMA_TIMEOUT) return fail(h, PBF_ETIMEOUT, "tensor-core completion wait gave up");
    return fail(h, PBF_ECUDA, "device error word 0x%x", e);
  }
  return PBF_OK;
}

// One substep: the dispatch sequence of PBF.run (PBF.ts:398-448).  When
// `ev` is given, events are recorded at the reference's four interval
// boundaries (PBF.runTimestamp, PBF.ts:450-510).
int substep(pbf_handle* h, cudaEvent_t* ev) {
  const uint32_t n = h->n;
  cudaStream_t st = h->stream;
  SimParams p = h->sp;
  p.n = n;
  const GridParams g = h->gp;
  const int c = h->cur, nx = 1 - c;
  const PassSet& ps = h->passes.set[h->batch ? 1 : 0][h->grid_cap ? 1 : 0];
  // cell-block passes: one CTA per 128 sorted slots, the halo staged in
  // shared memory (pbf_cellblock.cuh)
  const bool cb = cb_active(h);
  const CbSet& cs = h->passes.cb[cb_memb(h)];
  CbArgs A = cb ? cb_args(h) : CbArgs{};
  const unsigned cbg = cb_grid(n);
  if (ev) CU(h, cudaEventRecord(ev[0], st));
  // neighborSearch.clearBuffer + TimeIntegration (+ ParticleInsert counts)
  CU(h, cudaMemsetAsync(h->cell_count.p, 0, ((size_t)g.cells + 1) * sizeof(uint32_t), st));
  {
  KScope ks(h, K_PREDICT);
  ps.predict<<<grid_of(h, n), h->blk, 0, st>>>(p, g, h->tab, h->pos[c].p, h->vel.p, h->acc.p, h->xs[1].p,
                                                       h->key.p, h->rank.p, h->cell_count.p);
  }
  CU(h, cudaGetLastError());
  if (ev) CU(h, cudaEventRecord(ev[1], st));
  // cell scan + counting sort (stable by id) + reorder of the state
  SortBuffers sb{h->key.p,     h->rank.p,  h->cell_count.p, h->cell_start.p, h->perm_raw.p, h->id_raw.p,
                 h->perm.p,    h->tmp_a.p, h->tmp_b.p,      h->big_list.p,   h->big_count.p, h->scan_scratch,
                 h->err_word.p};
  {
    KScope ks(h, K_SORT);
    CU(h, launch_sort_by_cell(g, n, h->ids[c].p, sb, h->id_bits, st));
  }
  // the learned start's and trace capture's features: the previous multiplier
  // sum is gathered with the state
  const bool need_feat = h->learned || h->trace_cap > 0;
  {
    KScope ks(h, K_GATHER);
    if (cb)
      CU(h, launch_gather_state_cb(n, h->perm.p, h->pos[c].p, h->xs[1].p, h->ids[c].p, h->key.p, h->pos[nx].p,
                                   h->xs[0].p, h->ids[nx].p, h->skey.p, h->xs0.p, st,
                                   need_feat ? h->lam_sum.p : nullptr, need_feat ? h->lam_prev.p : nullptr));
    else
      CU(h, launch_gather_state(n, h->perm.p, h->pos[c].p, h->xs[1].p, h->ids[c].p, h->pos[nx].p, h->xs[0].p,
                                h->ids[nx].p, st, need_feat ? h->lam_sum.p : nullptr,
                                need_feat ? h->lam_prev.p : nullptr));
  }
  h->cur = nx;
  const int cc = nx;
  const FieldParams f = h->fp;
  const uint32_t ms = h->nbr_slice;
  const float sub_index = (float)(h->substep_counter % h->cfg.substeps);
  // Boundary sampling works on a band list (BandArgs): the
  // band pass builds it at x*_0, each delta-p pass marks the band of the next
  // iteration at the positions it writes, and the sampling kernel interpolates
  // the volume map for the listed slots only.
  CU(h, cudaMemsetAsync(h->band_count.p, 0, 2 * sizeof(uint32_t), st));
  int band = -1;  // band list holding the current iteration's band (-1: not built)
  const unsigned band_grid = std::min(nblocks(n, 256), (unsigned)h->sms * 2u);  // one resident wave
  auto band_args = [&](int list, float* bsdf) {
    BandArgs B{};
    B.f = f;
    B.flag = h->bflag.p;
    B.bdata = h->bdata.p;
    B.bsdf = bsdf;
    B.list = h->band_list[list].p;
    B.count = h->band_count.p + list;
    return B;
  };
  // Boundary sampling at x*_a (bsdf: also the SDF feature); guard: the
  // lagged iteration control's flag (the sampling is skipped with it).
  auto sample_boundary = [&](int a, float* bsdf, const int* guard = nullptr,
                             cudaStream_t on = nullptr) -> cudaError_t {
    KScope ks(h, K_BOUNDARY);
    cudaStream_t sst = on ? on : st;
    if (band < 0) {
      ps.band<<<grid_of(h, n), h->blk, 0, sst>>>(p, h->tab, h->xs[a].p, band_args(0, bsdf));
      band = 0;
    }
    ps.boundary_band<<<band_grid, 256, 0, sst>>>(p, f, h->sdf.p, h->vol.p, FieldBlocks{h->bcell.p, h->bnodes.p},
                                                 h->tab, h->xs[a].p, h->bdata.p, bsdf,
                                                 h->band_list[band].p, h->band_count.p + band,
                                                 h->band_count.p + (1 - band), guard);
    return cudaGetLastError();
  };
  // NeighborCount + NeighborList in one pass (fixed per-particle slices: no
  // scan).  The learned start sums its features in the same traversal; their
  // boundary terms need the boundary sampling at x*_0, which runs before the
  // build, or (fast mode, tcgen05 network) on the side stream beside it, the
  // network pass then adding those terms (LateBoundary).
  const bool late = h->learned && f.loaded && !cb && !h->ktiming && h->side_stream &&
                    h->mlp_kernel == PBF_MLP_KERNEL_TCGEN05 && h->cfg.fp_mode == PBF_FP_FAST;
  // The plain solve's first boundary sampling (at x*_0) likewise runs on the
  // side stream beside the build; the first iteration waits for it.
  const bool pre_sampled = !h->learned && f.loaded && !cb && !h->ktiming && !h->batch && h->side_stream &&
                           h->cfg.options.iterations > 0;
  if (pre_sampled) {
    CU(h, cudaEventRecord(h->ev_fork, st));
    CU(h, cudaStreamWaitEvent(h->side_stream, h->ev_fork, 0));
    CU(h, sample_boundary(0, need_feat ? h->bsdf.p : nullptr, nullptr, h->side_stream));
    CU(h, cudaEventRecord(h->ev_join, h->side_stream));
  }
  if (h->learned) {
    if (late) {
      CU(h, cudaEventRecord(h->ev_fork, st));
      CU(h, cudaStreamWaitEvent(h->side_stream, h->ev_fork, 0));
      CU(h, sample_boundary(0, h->bsdf.p, nullptr, h->side_stream));
      CU(h, cudaEventRecord(h->ev_join, h->side_stream));
    } else if (f.loaded) {
      CU(h, sample_boundary(0, h->bsdf.p));
    }
    SolverAux al{};
    al.pos = h->pos[cc].p;
    al.lam_prev = h->lam_prev.p;
    al.bsdf = (f.loaded && !late) ? h->bsdf.p : nullptr;
    al.late_boundary = late ? 1 : 0;
    al.substep_index = sub_index;
    al.feat = h->feat.p;
    KScope ks(h, K_FEATURES);
    if (cb)
      h->passes.cb_build_feat<<<cbg, 128, (size_t)h->cb_cap * sizeof(float4), st>>>(
          p, A, h->cb_mask.p, h->cb_ovf.p, h->nbr_count.p, f.loaded, h->bdata.p, al);
    else
      ps.nbr_build_feat<<<grid_of(h, n), h->blk, 0, st>>>(p, g, h->xs[0].p, h->cell_start.p, ms, h->nbr_list.p,
                                                           h->nbr_count.p, h->nbr_max.p, h->err_word.p,
                                                           (f.loaded && !late) ? 1 : 0, h->bdata.p, al);
  } else if (cb) {
    // the mask variant's search; the list-free variant has none (the
    // density pass counts the neighbours)
    if (cb_memb(h) == kMemMaskHost) {
      KScope ks(h, K_NBR_BUILD);
      h->passes.cb_build<<<cbg, 128, (size_t)h->cb_cap * sizeof(float4), st>>>(
          p, A, h->cb_mask.p, h->cb_ovf.p, h->nbr_count.p, 0, nullptr, SolverAux{});
    }
  } else {
    KScope ks(h, K_NBR_BUILD);
    if (h->build == PBF_BUILD_PAIR)
      ps.nbr_build2<<<grid_of(h, (n + 1) / 2), h->blk, 0, st>>>(p, g, h->tab, h->xs[0].p, h->cell_start.p, ms,
                                                                  h->nbr_list.p, h->nbr_count.p, h->nbr_max.p,
                                                                  h->err_word.p);
    else if (h->build == PBF_BUILD_WARP)
      ps.nbr_build_warp<<<grid_of(h, n), h->blk, 0, st>>>(p, g, h->tab, h->xs[0].p, h->cell_start.p, ms,
                                                           h->nbr_list.p, h->nbr_count.p, h->nbr_max.p,
                                                           h->err_word.p);
    else
      ps.nbr_build<<<grid_of(h, n), h->blk, 0, st>>>(p, g, h->tab, h->xs[0].p, h->cell_start.p, ms, h->nbr_list.p,
                                                      h->nbr_count.p, h->nbr_max.p, h->err_word.p);
  }
  CU(h, cudaGetLastError());
  if (ev) CU(h, cudaEventRecord(ev[2], st));
  // constraint loop
  // `iters` plain iterations starting from xs[a]; returns the buffer holding
  // the result.  The first iteration's lambda pass records the features
  // (feat_first) and/or starts lam_sum; stats go with the last one.  Each
  // delta-p but the last marks the band of the next iteration.
  auto iterate = [&](int a, uint32_t iters, bool feat_first, bool lam_sum_on, bool first_starts_sum,
                     SolveStats* stats, int* rc, bool adaptive = false, bool lagged = false) -> int {
    const int* lag = nullptr;  // lagged control: every pass of the iterations is guarded by this flag
    if (lagged && iters > 0) {
      if (launch_lagged_decide(h->fb_mean.p, h->lagged_fraction * h->fallback_bound, h->fb_flag.p + 1,
                               h->fb_count.p + 1, st) != cudaSuccess) {
        *rc = PBF_ECUDA;
        return a;
      }
      lag = h->fb_flag.p + 1;
      adaptive = false;
    }
    for (uint32_t it = 0; it < iters; ++it) {
      float* bsdf_it = (need_feat && feat_first && it == 0) ? h->bsdf.p : nullptr;
      if (pre_sampled && it == 0 && !h->learned) {
        // sampled on the side stream beside the build
        if (cudaStreamWaitEvent(st, h->ev_join, 0) != cudaSuccess) {
          *rc = PBF_ECUDA;
          return a;
        }
      } else if (f.loaded && sample_boundary(a, bsdf_it, lag) != cudaSuccess) {
        *rc = PBF_ECUDA;
        return a;
      }
      SolverAux al{};
      al.tab = h->tab;
      al.iter = (int)it;
      al.guard = lag;
      if (lam_sum_on) {
        al.lam_sum = h->lam_sum.p;
        al.lam_first = (first_starts_sum && it == 0) ? 1 : 0;
      }
      if (stats && it + 1 == iters) al.stats = stats;
      if (adaptive) al.stats = h->stats.p + 1;  // the density error at this iteration's start
      const bool fe = feat_first && it == 0;
      if (fe) {
        al.feat = h->feat.p;
        al.pos = h->pos[cc].p;
        al.lam_prev = h->lam_prev.p;
        al.bsdf = f.loaded ? h->bsdf.p : nullptr;
        al.substep_index = sub_index;
      }
      {
        KScope ks(h, K_LAMBDA);
        if (cb) {
          auto kl = fe ? cs.lambda_feat : (al.stats && adaptive ? cs.lambda_stats : cs.lambda);
          kl<<<cbg, 128, cb_smem(h, 1), st>>>(p, A, f.loaded, h->bdata.p, h->xs[a].p, h->xl.p, al);
        } else {
          auto kl = fe ? ps.lambda_feat : (al.stats && adaptive ? ps.lambda_stats : ps.lambda);
          kl<<<grid_of(h, n), h->blk, 0, st>>>(p, f.loaded, h->bdata.p, h->xs[a].p, ms, h->nbr_count.p,
                                               h->nbr_list.p, h->xl.p, al);
        }
      }
      if (cudaGetLastError() != cudaSuccess) { *rc = PBF_ECUDA; return a; }
      SolverAux ad{};
      ad.tab = h->tab;
      ad.iter = (int)it;
      ad.xs_in = h->xs[a].p;
      ad.need = lag;
      if (adaptive) {
        // flag [1] = error above the bound: the position update runs (and is counted)
        if (launch_iterate_decide(h->stats.p + 1, h->fallback_bound, h->fb_flag.p + 1, h->fb_count.p + 1,
                                  h->fb_mean.p + 1, st) != cudaSuccess) {
          *rc = PBF_ECUDA;
          return a;
        }
        ad.need = h->fb_flag.p + 1;
      }
      if (f.loaded && it + 1 < iters) {  // the next iteration's band, at the positions written now
        ad.band = band_args(1 - band, nullptr);
        band = 1 - band;
      }
      {
        KScope ks(h, K_DELTAP);
        if (cb)
          cs.deltap<<<cbg, 128, cb_smem(h, 1), st>>>(p, A, ad, f.loaded, h->xl.p, h->bdata.p, h->xs[1 - a].p,
                                                     h->capture ? h->dp.p : nullptr);
        else
          ps.deltap<<<grid_of(h, n), h->blk, 0, st>>>(p, ad, f.loaded, h->xl.p, h->bdata.p, ms, h->nbr_count.p,
                                                       h->nbr_list.p, h->xs[1 - a].p, h->capture ? h->dp.p : nullptr);
      }
      if (cudaGetLastError() != cudaSuccess) { *rc = PBF_ECUDA; return a; }
      a = 1 - a;
    }
    *rc = PBF_OK;
    return a;
  };
  int a = 0, rc = PBF_OK;
  if (h->learned) {
    // learned start: (boundary and features at x*_0 from the neighbour
    // build) -> network -> (x*_0, lambda_hat) -> one projection ->
    // learned_iters plain iterations -> device-side fallback test.  The
    // network writes (x*_0, lambda_hat) into xs_save, which the projection
    // reads as its (x*, lambda) records and the fallback keeps as x*_0.
    {
      KScope ks(h, K_MLP);
      LateBoundary lb{};
      if (late) {
        CU(h, cudaStreamWaitEvent(st, h->ev_join, 0));  // the side stream's boundary sampling
        lb = LateBoundary{h->bdata.p, h->bsdf.p, p.h, p.h2, p.poly6, p.V};
      }
      if (h->mlp_kernel == PBF_MLP_KERNEL_TCGEN05)
        CU(h, launch_mlp_infer_tc(h->mlp_params.p, h->model, (const float*)h->feat.p, n, nullptr, h->lam_sum.p, st,
                                  h->xs[0].p, h->xs_save.p, h->err_word.p, lb));
      else
        CU(h, launch_mlp_infer(h->mlp_params.p, h->model, (const float*)h->feat.p, n, nullptr, h->lam_sum.p, st,
                               h->xs[0].p, h->xs_save.p));
    }
    {
      KScope ks(h, K_DELTAP);
      SolverAux ad{};
      if (f.loaded && h->learned_iters > 0) {
        ad.band = band_args(1 - band, nullptr);
        band = 1 - band;
      }
      if (cb)
        cs.deltap<<<cbg, 128, cb_smem(h, 1), st>>>(p, A, ad, f.loaded, h->xs_save.p, h->bdata.p, h->xs[1].p,
                                                   nullptr);
      else
        ps.deltap<<<grid_of(h, n), h->blk, 0, st>>>(p, ad, f.loaded, h->xs_save.p, h->bdata.p, ms, h->nbr_count.p,
                                                     h->nbr_list.p, h->xs[1].p, nullptr);
    }
    CU(h, cudaGetLastError());
    a = iterate(1, h->learned_iters, false, true, false, nullptr, &rc, h->adaptive, h->lagged_fraction > 0.0f);
    if (rc) return fail(h, rc, "learned solve launch failed");
  } else {
    a = iterate(0, h->cfg.options.iterations, need_feat, need_feat, true, nullptr, &rc);
    if (rc) return fail(h, rc, "solve launch failed");
    if (h->trace_cap > 0) {
      CU(h, launch_trace_append(n, h->ids[cc].p, h->feat.p, h->lam_sum.p, h->trace_stride,
                                (uint32_t)(h->trace_salt ^ (uint64_t)h->substep_counter * 0x9e3779b9ull),
                                h->trace_feat.p, h->trace_tgt.p, h->trace_count.p, h->trace_cap, st));
    }
  }
  h->substep_counter++;
  if (ev) CU(h, cudaEventRecord(ev[3], st));
  // non-pressure passes
  // AttributeUpdate.  Its density error (mean compression) is the learned
  // start's fallback test; while tracing it records the plain solve's error.
  const bool rec = !h->learned && h->trace_cap > 0 && h->stats.p && h->trace_err.p;
  {
    KScope ks(h, K_DENSITY);
    SolverAux ad{};
    if (h->learned || rec) ad.stats = h->stats.p;
    if (cb)
      cs.density_velocity<<<cbg, 128, cb_smem(h, 1), st>>>(p, A, ad, h->xs[a].p, h->pos[cc].p, h->vel.p,
                                                            cb_memb(h) == kMemMaskHost ? nullptr : h->nbr_count.p);
    else
      ps.density_velocity<<<grid_of(h, n), h->blk, 0, st>>>(p, ad, h->xs[a].p, ms, h->nbr_count.p,
                                                             h->nbr_list.p, h->pos[cc].p, h->vel.p);
  }
  CU(h, cudaGetLastError());
  if (rec) CU(h, launch_stats_record(h->stats.p, h->trace_err.p, st));
  if (h->learned) {
    CU(h, launch_fallback_decide(h->stats.p, h->fallback_bound, h->fb_flag.p, h->fb_count.p, h->fb_mean.p, st));
    // plain re-solve from x*_0 when the flag is set: one cooperative kernel
    // (returns at once otherwise)
    KScope ks(h, K_FALLBACK);
    FallbackArgs fa{};
    fa.p = p;
    fa.f = f;
    fa.guard = h->fb_flag.p;
    fa.sdf = h->sdf.p;
    fa.vol = h->vol.p;
    fa.bflag = h->bflag.p;
    fa.pos_old = h->pos[c].p;
    fa.perm = h->perm.p;
    fa.xs_save = h->xs_save.p;
    fa.pos = h->pos[cc].p;
    fa.vel = h->vel.p;
    fa.xs0 = h->xs[0].p;
    fa.xs1 = h->xs[1].p;
    fa.xl = h->xl.p;
    fa.bdata = h->bdata.p;
    fa.lam_sum = h->lam_sum.p;
    fa.nbr_cnt = h->nbr_count.p;
    fa.nbr_list = h->nbr_list.p;
    fa.max_nbr = ms;
    fa.iters = (int)h->cfg.options.iterations;
    fa.final_buf = a;
    if (cb) {
      if (h->cb_fb_grid == 0) {
        int per_sm = 0;
        CU(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cs.fallback, 256, 0));
        if (per_sm < 1) return fail(h, PBF_ECUDA, "fallback kernel does not fit on an SM");
        h->cb_fb_grid = (unsigned)per_sm * (unsigned)h->sms;
      }
      void* args[] = {&fa, &A};
      CU(h, cudaLaunchCooperativeKernel((const void*)cs.fallback, dim3(std::min(h->cb_fb_grid, nblocks(n, 256))),
                                        dim3(256), args, 0, st));
    } else {
      if (h->fb_grid == 0) {
        int per_sm = 0;
        CU(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->passes.fallback, 256, 0));
        if (per_sm < 1) return fail(h, PBF_ECUDA, "fallback kernel does not fit on an SM");
        h->fb_grid = (unsigned)per_sm * (unsigned)h->sms;
      }
      void* args[] = {&fa};
      CU(h, cudaLaunchCooperativeKernel((const void*)h->passes.fallback, dim3(std::min(h->fb_grid, nblocks(n, 256))),
                                        dim3(256), args, 0, st));
    }
  }
  if (a != 0) CU(h, cudaMemcpyAsync(h->xs[0].p, h->xs[1].p, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
  if (cb && cs.xsph_split) {  // fast mode: XSPH's sum split over the two passes
    {
      KScope ks(h, K_VORTICITY);
      cs.vorticity_split<<<cbg, 128, cb_smem(h, 2), st>>>(p, A, h->pos[cc].p, h->vel.p, h->omega.p, h->normal.p,
                                                          h->visc.p, h->coh.p);
    }
    CU(h, cudaGetLastError());
    {
      KScope ks(h, K_XSPH);
      cs.xsph_split<<<cbg, 128, cb_smem(h, 2), st>>>(p, A, h->pos[cc].p, h->omega.p, h->normal.p, h->visc.p,
                                                     h->coh.p, h->acc.p);
    }
    CU(h, cudaGetLastError());
  } else if (cb) {
    {
      KScope ks(h, K_VORTICITY);
      cs.vorticity<<<cbg, 128, cb_smem(h, 2), st>>>(p, A, h->pos[cc].p, h->vel.p, h->omega.p, h->normal.p);
    }
    CU(h, cudaGetLastError());
    {
      KScope ks(h, K_XSPH);
      cs.xsph<<<cbg, 128, cb_smem(h, 3), st>>>(p, A, h->pos[cc].p, h->vel.p, h->omega.p, h->normal.p, h->acc.p);
    }
    CU(h, cudaGetLastError());
  } else if (ps.xsph_split) {  // fast mode: XSPH's sum split over the two passes
    {
      KScope ks(h, K_VORTICITY);
      ps.vorticity_split<<<grid_of(h, n), h->blk, 0, st>>>(p, h->pos[cc].p, h->vel.p, ms, h->nbr_count.p,
                                                            h->nbr_list.p, h->omega.p, h->normal.p, h->visc.p,
                                                            h->coh.p);
    }
    CU(h, cudaGetLastError());
    {
      KScope ks(h, K_XSPH);
      ps.xsph_split<<<grid_of(h, n), h->blk, 0, st>>>(p, h->pos[cc].p, h->omega.p, h->normal.p, h->visc.p, h->coh.p,
                                                       ms, h->nbr_count.p, h->nbr_list.p, h->acc.p);
    }
    CU(h, cudaGetLastError());
  } else {
    {
      KScope ks(h, K_VORTICITY);
      ps.vorticity<<<grid_of(h, n), h->blk, 0, st>>>(p, h->pos[cc].p, h->vel.p, ms, h->nbr_count.p, h->nbr_list.p,
                                                      h->omega.p, h->normal.p);
    }
    CU(h, cudaGetLastError());
    {
      KScope ks(h, K_XSPH);
      ps.xsph<<<grid_of(h, n), h->blk, 0, st>>>(p, h->pos[cc].p, h->vel.p, h->omega.p, h->normal.p, ms,
                                                 h->nbr_count.p, h->nbr_list.p, h->acc.p);
    }
    CU(h, cudaGetLastError());
  }
  if (ev) CU(h, cudaEventRecord(ev[4], st));
  return PBF_OK;
}

int export_positions(pbf_handle* h) {
  KScope ks(h, K_EXPORT);
  CU(h, launch_scatter_by_id(h->n, h->ids[h->cur].p, h->pos[h->cur].p, h->out_pos.p, h->stream));
  return PBF_OK;
}

int frame(pbf_handle* h) {
  for (uint32_t s = 0; s < h->cfg.substeps; ++s) {
    int rc = substep(h, nullptr);
    if (rc) return rc;
  }
  return export_positions(h);
}

// The state after an upload of n particles whose positions (w = 0) and ids
// (0 .. n-1) are already in pos[0] / ids[0]: zero motion, exported positions.
int finish_upload(pbf_handle* h, uint32_t n) {
  invalidate_graph(h);
  h->n = n;
  h->cur = 0;
  h->sp.n = n;
  uint32_t bits = 1;
  while (bits < 32 && (1ull << bits) < (uint64_t)n) ++bits;
  h->id_bits = bits;
  cudaStream_t st = h->stream;
  if (n) {
    CU(h, cudaMemsetAsync(h->vel.p, 0, (size_t)n * sizeof(float4), st));
    CU(h, cudaMemsetAsync(h->acc.p, 0, (size_t)n * sizeof(float4), st));
    CU(h, cudaMemsetAsync(h->xl.p, 0, (size_t)n * sizeof(float4), st));
    CU(h, cudaMemsetAsync(h->bdata.p, 0, (size_t)n * sizeof(float4), st));
  }
  int rc = export_positions(h);
  if (rc) return rc;
  CU(h, cudaStreamSynchronize(st));
  return PBF_OK;
}

int upload_particles(pbf_handle* h, const float* xyzw, uint32_t n) {
  if (n > h->cfg.max_particles)
    return fail(h, PBF_ECAPACITY, "To Many Particles! (%u > max_particles %u)", n, h->cfg.max_particles);
  std::vector<float> tmp((size_t)n * 4);
  std::vector<uint32_t> iota(n);
  for (uint32_t i = 0; i < n; ++i) {
    tmp[4 * (size_t)i] = xyzw[4 * (size_t)i];
    tmp[4 * (size_t)i + 1] = xyzw[4 * (size_t)i + 1];
    tmp[4 * (size_t)i + 2] = xyzw[4 * (size_t)i + 2];
    tmp[4 * (size_t)i + 3] = 0.0f;
    iota[i] = i;
  }
  if (n) {
    invalidate_graph(h);
    CU(h, cudaMemcpyAsync(h->pos[0].p, tmp.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemcpyAsync(h->ids[0].p, iota.data(), (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice,
                          h->stream));
  }
  return finish_upload(h, n);
}

void release_all(pbf_handle* h) {
  invalidate_graph(h);
  DBuf<float4>* f4s[] = {&h->pos[0], &h->pos[1], &h->xs[0], &h->xs[1], &h->xl, &h->vel, &h->acc, &h->bdata,
                         &h->visc,   &h->coh,
                         &h->omega,  &h->normal, &h->dp,    &h->out_pos, &h->out_tmp, &h->xs0};
  for (auto* b : f4s) b->release();
  DBuf<uint32_t>* u32s[] = {&h->ids[0],   &h->ids[1],      &h->key,      &h->rank,      &h->perm_raw,
                            &h->id_raw,   &h->perm,        &h->tmp_a,    &h->tmp_b,     &h->cell_count,
                            &h->cell_start, &h->big_list,  &h->big_count, &h->nbr_count, &h->nbr_max,
                            &h->nbr_list, &h->err_word,    &h->m_u,      &h->skey,      &h->cb_mask};
  for (auto* b : u32s) b->release();
  h->cb_ovf.release();
  h->sdf.release();
  h->vol.release();
  h->bflag.release();
  h->bcell.release();
  h->bnodes.release();
  h->scenes_dev.release();
  h->slot_scene.release();
  h->band_list[0].release();
  h->band_list[1].release();
  h->band_count.release();
  h->mlp_params.release();
  h->lam_sum.release();
  h->lam_prev.release();
  h->bsdf.release();
  h->fb_mean.release();
  h->feat.release();
  h->xs_save.release();
  h->stats.release();
  h->fb_flag.release();
  h->fb_count.release();
  h->trace_feat.release();
  h->trace_tgt.release();
  h->trace_err.release();
  h->trace_count.release();
  h->m_f.release();
  h->m_d.release();
  if (h->scan_scratch) cudaFree(h->scan_scratch);
  h->scan_scratch = nullptr;
}

bool finite_positive(float v) { return std::isfinite(v) && v > 0.0f; }

// Per field cell, whether BoundaryVolume can return a non-zero bData there.
// It cannot when all 32 volume nodes are zero (the interpolated volume is
// exactly 0 and `volume > 0` fails) or when the interpolated SDF provably
// stays >= h (or <= 0) over the cell: the cubic serendipity weights sum to 1
// with at most 2.375 of negative weight, so the value lies within
// [m - 2.375 (M - m), M + 2.375 (M - m)] of the node range [m, M]; a margin
// covers the float rounding of the 32-term sum.
void boundary_flags(const uint32_t res[3], const float* sdf, const float* vol, float h, std::vector<uint8_t>& flag) {
  const size_t nx = res[0], ny = res[1], nz = res[2];
  const size_t nc = (nx + 1) * (ny + 1) * (nz + 1);
  const size_t nex = 2 * nx * (ny + 1) * (nz + 1);
  const size_t ney = (nx + 1) * 2 * ny * (nz + 1);
  flag.assign(nx * ny * nz, 1);
  for (size_t k = 0; k < nz; ++k)
    for (size_t j = 0; j < ny; ++j)
      for (size_t i = 0; i < nx; ++i) {
        size_t idx[32];
        int q = 0;
        for (int c = 0; c < 8; ++c)
          idx[q++] = ((k + (c >> 2 & 1)) * (ny + 1) + (j + (c >> 1 & 1))) * (nx + 1) + (i + (c & 1));
        for (int c = 0; c < 8; ++c)
          idx[q++] = nc + ((k + (c >> 1 & 1)) * (ny + 1) + (j + (c >> 2 & 1))) * (2 * nx) + 2 * i + (c & 1);
        for (int c = 0; c < 8; ++c)
          idx[q++] = nc + nex + ((i + (c >> 1 & 1)) * (nz + 1) + (k + (c >> 2 & 1))) * (2 * ny) + 2 * j + (c & 1);
        for (int c = 0; c < 8; ++c)
          idx[q++] = nc + nex + ney + ((j + (c >> 1 & 1)) * (nx + 1) + (i + (c >> 2 & 1))) * (2 * nz) + 2 * k + (c & 1);
        bool vzero = true;
        double m = 1e300, M = -1e300, amax = 0.0;
        for (int t = 0; t < 32; ++t) {
          if (vol[idx[t]] != 0.0f) vzero = false;
          double v = sdf[idx[t]];
          m = std::min(m, v);
          M = std::max(M, v);
          amax = std::max(amax, std::fabs(v));
        }
        double spread = 2.375 * (M - m) + 2e-5 * amax + 1e-30;
        bool far = (m - spread >= (double)h) || (M + spread <= 0.0);
        if (vzero || far) flag[(k * ny + j) * nx + i] = 0;
      }
}


// Packed node blocks (FieldBlocks) of one map's flagged cells, appended to
// blocks; cell[] gets each cell's block index (counted from the blocks
// already present) or kNoBlock.
void pack_field_blocks(const uint32_t res[3], const float* sdf, const float* vol, const std::vector<uint8_t>& flag,
                       std::vector<uint32_t>& cell, std::vector<float>& blocks) {
  FieldParams f{};
  for (int a = 0; a < 3; ++a) f.res[a] = (int)res[a];
  const size_t nx = res[0], ny = res[1], nz = res[2];
  cell.assign(nx * ny * nz, kNoBlock);
  for (size_t k = 0; k < nz; ++k)
    for (size_t j = 0; j < ny; ++j)
      for (size_t i = 0; i < nx; ++i) {
        const size_t c = (k * ny + j) * nx + i;
        if (!flag[c]) continue;
        uint32_t idx[32];
        cell_nodes(f, (int)i, (int)j, (int)k, false, idx);
        cell[c] = (uint32_t)(blocks.size() / 64);
        for (int q = 0; q < 32; ++q) blocks.push_back(sdf[idx[q]]);
        for (int q = 0; q < 32; ++q) blocks.push_back(vol[idx[q]]);
      }
}

// (Re)allocates the cell arrays for h->gp.cells cells.
cudaError_t alloc_cells(pbf_handle* h) {
  const size_t cells = h->gp.cells;
  if (h->cell_count.p && h->cell_count.n == cells + 1) return cudaSuccess;
  h->cell_count.release();
  h->cell_start.release();
  h->big_list.release();
  cudaError_t e = h->cell_count.alloc(cells + 1);
  if (e == cudaSuccess) e = h->cell_start.alloc(cells + 1);
  if (e == cudaSuccess) e = h->big_list.alloc(cells);
  if (h->scan_scratch) {
    cudaFree(h->scan_scratch);
    h->scan_scratch = nullptr;
  }
  if (e == cudaSuccess) e = cudaMalloc(&h->scan_scratch, scan_scratch_bytes(std::max(cells + 1, (size_t)h->cfg.max_particles + 1)));
  return e;
}

// Grids of the scenes of a batch at the handle's cell ratio, with consecutive
// key ranges; uploads the scene table.  Returns the total cell count (0 on
// overflow of the 32-bit key space).
uint64_t layout_scenes(pbf_handle* h) {
  uint64_t base = 0;
  for (auto& sd : h->scenes) {
    GridParams g = make_grid(sd.dmin, sd.dmax, h->cfg.kernel_radius, h->cell_ratio, nullptr, true);
    if (g.cells == 0) return 0;
    g.key_base = (uint32_t)base;
    sd.grid = g;
    base += g.cells;
    if (base > 0xfffffffeull) return 0;
  }
  return base;
}

// Applies a cell ratio: new grid(s), cell arrays, scene table.
int apply_cell_ratio(pbf_handle* h, float ratio) {
  if (ratio == h->cell_ratio) return PBF_OK;
  const float old = h->cell_ratio;
  h->cell_ratio = ratio;
  if (h->batch) {
    uint64_t cells = layout_scenes(h);
    if (cells == 0) {
      h->cell_ratio = old;
      layout_scenes(h);
      return fail(h, PBF_EINVAL, "cell ratio %g: too many cells", (double)ratio);
    }
    h->gp.cells = (uint32_t)cells;
    CU(h, cudaMemcpy(h->scenes_dev.p, h->scenes.data(), h->scenes.size() * sizeof(SceneDesc), cudaMemcpyHostToDevice));
  } else {
    GridParams g = make_grid(h->cfg.domain_min, h->cfg.domain_max, h->cfg.kernel_radius, ratio,
                             ratio == 1.0f ? h->cfg.grid_dim : nullptr, false);
    if (g.cells == 0) {
      h->cell_ratio = old;
      return fail(h, PBF_EINVAL, "cell ratio %g: too many cells", (double)ratio);
    }
    h->gp = g;
  }
  invalidate_graph(h);
  CU(h, alloc_cells(h));
  return PBF_OK;
}

// Buffers of the cell-block passes (allocated on first use) and the
// kernels' shared-memory limits: up to four staged fields of cb_cap records.
int ensure_cb(pbf_handle* h) {
  const size_t cap = std::max<size_t>(h->cfg.max_particles, 1);
  if (!h->skey.p) {
    CU(h, h->skey.alloc(cap));
    CU(h, h->xs0.alloc(cap));
    CU(h, h->cb_mask.alloc(9 * cap));
    CU(h, h->cb_ovf.alloc(cap));
    CU(h, cudaMemsetAsync(h->cb_ovf.p, 0, cap * sizeof(uint16_t), h->stream));
  }
  const int bytes = (int)(4 * (size_t)h->cb_cap * sizeof(float4));
  auto attr = [&](const void* k) -> cudaError_t {
    return k ? cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) : cudaSuccess;
  };
  const PassTable& T = h->passes;
  CU(h, attr((const void*)T.cb_build));
  CU(h, attr((const void*)T.cb_build_feat));
  for (const CbSet& c : T.cb) {
    for (const void* k : {(const void*)c.lambda, (const void*)c.lambda_feat, (const void*)c.lambda_stats,
                          (const void*)c.deltap, (const void*)c.density_velocity, (const void*)c.vorticity,
                          (const void*)c.xsph, (const void*)c.vorticity_split, (const void*)c.xsph_split})
      CU(h, attr(k));
  }
  return PBF_OK;
}

int apply_launch(pbf_handle* h, const pbf_launch& l) {
  if (l.block != 128 && l.block != 256) return fail(h, PBF_EINVAL, "block must be 128 or 256");
  if (l.ctas_per_sm > 16) return fail(h, PBF_EINVAL, "ctas_per_sm must be 0..16");
  if (l.cell_ratio != 1.0f && l.cell_ratio != 0.5f) return fail(h, PBF_EINVAL, "cell_ratio must be 1 or 0.5");
  if (l.build > PBF_BUILD_CELLBLOCK_FREE) return fail(h, PBF_EINVAL, "unknown neighbour-build variant %u", l.build);
  const bool cb = l.build == PBF_BUILD_CELLBLOCK_MASK || l.build == PBF_BUILD_CELLBLOCK_FREE;
  if (cb && (h->batch || l.ctas_per_sm != 0))
    return fail(h, PBF_EINVAL, "the cell-block passes need a single-scene handle and ctas_per_sm = 0");
  int rc = apply_cell_ratio(h, l.cell_ratio);
  if (rc) return rc;
  if (cb) {
    rc = ensure_cb(h);
    if (rc) return rc;
  }
  if ((int)l.block != h->blk || l.ctas_per_sm != h->per_sm || l.build != h->build) invalidate_graph(h);
  h->build = l.build;
  h->blk = (int)l.block;
  h->per_sm = l.ctas_per_sm;
  h->grid_cap = l.ctas_per_sm * (uint32_t)h->sms;
  return PBF_OK;
}

// Metrics of slots [first, first + n) with the given volume map.
int metrics_range(pbf_handle* h, uint32_t first, uint32_t n, const FieldParams& f, const float* sdf,
                  pbf_metrics* out) {
  std::memset(out, 0, sizeof(*out));
  out->particles = n;
  cudaStream_t st = h->stream;
  CU(h, cudaMemsetAsync(h->m_f.p, 0, 2 * sizeof(float), st));
  CU(h, cudaMemsetAsync(h->m_d.p, 0, 3 * sizeof(double), st));
  CU(h, cudaMemsetAsync(h->m_u.p, 0, 3 * sizeof(uint32_t), st));
  SimParams p = h->sp;
  p.n = n;
  if (n)
    CU(h, launch_metrics(p, f, f.loaded ? sdf : nullptr, h->pos[h->cur].p + first, h->vel.p + first,
                         h->nbr_count.p + first, n, h->m_f.p, h->m_d.p, h->m_u.p, st));
  float mf[2];
  double md[3];
  uint32_t mu[3], errw = 0;
  CU(h, cudaMemcpyAsync(mf, h->m_f.p, sizeof(mf), cudaMemcpyDeviceToHost, st));
  CU(h, cudaMemcpyAsync(md, h->m_d.p, sizeof(md), cudaMemcpyDeviceToHost, st));
  CU(h, cudaMemcpyAsync(mu, h->m_u.p, sizeof(mu), cudaMemcpyDeviceToHost, st));
  CU(h, cudaMemcpyAsync(&errw, h->err_word.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CU(h, cudaStreamSynchronize(st));
  out->max_compression = mf[0];
  out->max_abs_density_err = mf[1];
  out->mean_abs_density_err = n ? (float)(md[0] / n) : 0.0f;
  out->kinetic_energy = (float)md[1];
  out->mean_compression = n ? (float)(md[2] / n) : 0.0f;
  out->nonfinite = mu[0];
  out->penetrations = mu[1];
  out->error_flags = errw;
  out->neighbor_total = mu[2];
  return PBF_OK;
}

int not_for_batch(pbf_handle* h, const char* what) {
  return fail(h, PBF_ESTATE, "%s is not available on a batch handle", what);
}

}  // namespace

extern "C" {

int pbf_abi_version(void) { return PBF_ABI_VERSION; }

int pbf_config_default(pbf_config* c) {
  if (!c) return PBF_EINVAL;
  std::memset(c, 0, sizeof(*c));
  c->struct_size = sizeof(pbf_config);
  c->max_particles = 1u << 17;  // SPH.MAX_PARTICLE_NUM = 1 << 18 - 1 == 1 << 17 (SPH.ts:24)
  c->particle_radius = 0.006f;  // PBFConfig.ts:21
  c->kernel_radius = 0.025f;    // SPH.ts:26
  c->rest_density = 1000.0f;    // SPH.ts:33
  c->time_step = (float)(1.0 / 300.0);  // SPH.ts:27
  c->substeps = 1;              // PBFConfig.ts:21
  c->domain_min[0] = c->domain_min[1] = c->domain_min[2] = 0.0f;
  c->domain_max[0] = c->domain_max[1] = c->domain_max[2] = 1.0f;
  c->lambda_eps = 1e-6f;        // PBFConfig.ts:8
  c->wall_jitter = 1e-4f;       // common.ts:62
  c->jitter_mode = PBF_JITTER_HASH;
  c->volume_quirk = 1;
  c->fp_mode = PBF_FP_FAST;
  c->boundary_interp = PBF_INTERP_CUBIC;
  c->max_neighbors = 60;        // SPH.MAX_NEIGHBOR_COUNT (SPH.ts:25)
  c->options.iterations = 5;    // config.ts:22-28
  c->options.xsph = 0.01f;
  c->options.vorticity = 0.1f;
  c->options.surface_tension = 0.5f;
  c->options.gravity = 9.8f;
  c->stream = nullptr;
  return PBF_OK;
}

const char* pbf_last_error(const pbf_handle* h) { return h ? h->err.c_str() : "null handle"; }

int pbf_create(const pbf_config* cfg, pbf_handle** out) {
  if (!cfg || !out) return PBF_EINVAL;
  *out = nullptr;
  if (cfg->struct_size != sizeof(pbf_config)) return PBF_EINVAL;
  if (!finite_positive(cfg->particle_radius) || !finite_positive(cfg->kernel_radius) ||
      !finite_positive(cfg->rest_density) || !finite_positive(cfg->time_step) || cfg->max_particles == 0 ||
      cfg->substeps == 0 || cfg->max_neighbors == 0)
    return PBF_EINVAL;
  for (int a = 0; a < 3; ++a)
    if (!(cfg->domain_max[a] > cfg->domain_min[a])) return PBF_EINVAL;
  pbf_handle* h = new pbf_handle();
  h->cfg = *cfg;
  derive_params(h);
  if (h->gp.cells == 0 || (uint64_t)h->gp.dim[0] * h->gp.dim[1] * h->gp.dim[2] > 0xfffffffeull) {
    delete h;
    return PBF_EINVAL;
  }
  if (cfg->fp_mode == PBF_FP_EXACT)
    exact::fill_pass_table(&h->passes);
  else
    fast::fill_pass_table(&h->passes);
  h->fp = FieldParams{};
  h->fp.loaded = 0;
  cudaError_t e = cudaSuccess;
  if (cfg->stream) {
    h->stream = (cudaStream_t)cfg->stream;
  } else {
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    h->own_stream = true;
  }
  {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        sms > 0)
      h->sms = sms;
  }
  const size_t cap = cfg->max_particles, cells = h->gp.cells;
  const uint64_t rows = (uint64_t)(cap + 31) / 32 * 32;
  uint64_t slice = cfg->max_neighbors;
  if (slice * rows > 0xffffffffull) slice = 0xffffffffull / rows;
  h->nbr_slice = (uint32_t)slice;
  auto A = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  for (int i = 0; i < 2; ++i) {
    A(h->pos[i].alloc(cap));
    A(h->xs[i].alloc(cap));
    A(h->ids[i].alloc(cap));
  }
  A(h->vel.alloc(cap));
  A(h->acc.alloc(cap));
  A(h->bdata.alloc(cap));
  A(h->omega.alloc(cap));
  A(h->normal.alloc(cap));
  if (cfg->fp_mode != PBF_FP_EXACT) {
    A(h->visc.alloc(cap));
    A(h->coh.alloc(cap));
  }
  A(h->out_pos.alloc(cap));
  A(h->out_tmp.alloc(cap));
  A(h->key.alloc(cap));
  A(h->rank.alloc(cap));
  A(h->perm_raw.alloc(cap));
  A(h->id_raw.alloc(cap));
  A(h->perm.alloc(cap));
  A(h->tmp_a.alloc(cap));
  A(h->tmp_b.alloc(cap));
  A(h->cell_count.alloc(cells + 1));
  A(h->cell_start.alloc(cells + 1));
  A(h->big_list.alloc(cells));
  A(h->big_count.alloc(1));
  A(h->nbr_count.alloc(cap + 1));
  A(h->nbr_max.alloc(1));
  A(h->band_list[0].alloc(cap));
  A(h->band_list[1].alloc(cap));
  A(h->band_count.alloc(2));
  A(h->nbr_list.alloc(rows * h->nbr_slice));
  A(h->xl.alloc(cap));
  A(h->err_word.alloc(1));
  A(h->m_f.alloc(2));
  A(h->m_d.alloc(3));
  A(h->m_u.alloc(3));
  size_t sb = scan_scratch_bytes(cells + 1);
  size_t sb2 = scan_scratch_bytes(cap + 1);
  if (sb2 > sb) sb = sb2;
  A(cudaMalloc(&h->scan_scratch, sb));
  for (int i = 0; i < 5; ++i) A(cudaEventCreate(&h->ev[i]));
  A(cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking));
  A(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
  A(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
  if (e == cudaSuccess) {
    A(cudaMemsetAsync(h->nbr_max.p, 0, sizeof(uint32_t), h->stream));
    A(cudaMemsetAsync(h->err_word.p, 0, sizeof(uint32_t), h->stream));
    A(cudaMemsetAsync(h->vel.p, 0, cap * sizeof(float4), h->stream));
    A(cudaMemsetAsync(h->acc.p, 0, cap * sizeof(float4), h->stream));
    A(cudaStreamSynchronize(h->stream));
  }
  if (e != cudaSuccess) {
    release_all(h);
    if (h->side_stream) cudaStreamDestroy(h->side_stream);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    for (int i = 0; i < 5; ++i)
      if (h->ev[i]) cudaEventDestroy(h->ev[i]);
    delete h;
    return PBF_ECUDA;
  }
  *out = h;
  return PBF_OK;
}

int pbf_destroy(pbf_handle* h) {
  if (!h) return PBF_EINVAL;
  cudaStreamSynchronize(h->stream);
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamDestroy(h->copy_stream);
    cudaEventDestroy(h->ev_frame);
    cudaEventDestroy(h->ev_staged);
  }
  if (h->side_stream) {
    cudaStreamSynchronize(h->side_stream);
    cudaStreamDestroy(h->side_stream);
  }
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  h->staging.release();
  release_all(h);
  for (int i = 0; i < 5; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  for (auto e : h->kt_events) cudaEventDestroy(e);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PBF_OK;
}

int pbf_reset(pbf_handle* h) {
  if (!h) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_reset");
  invalidate_graph(h);
  h->host_particles.clear();
  h->n = 0;
  h->cur = 0;
  h->fp.loaded = 0;
  h->sdf.release();
  h->vol.release();
  const size_t cap = h->cfg.max_particles;
  cudaStream_t st = h->stream;
  for (int i = 0; i < 2; ++i) CU(h, cudaMemsetAsync(h->pos[i].p, 0, cap * sizeof(float4), st));
  CU(h, cudaMemsetAsync(h->vel.p, 0, cap * sizeof(float4), st));
  CU(h, cudaMemsetAsync(h->acc.p, 0, cap * sizeof(float4), st));
  CU(h, cudaMemsetAsync(h->out_pos.p, 0, cap * sizeof(float4), st));
  CU(h, cudaMemsetAsync(h->err_word.p, 0, sizeof(uint32_t), st));
  CU(h, cudaStreamSynchronize(st));
  return PBF_OK;
}

int pbf_set_options(pbf_handle* h, const pbf_options* o) {
  if (!h || !o) return PBF_EINVAL;
  if (!std::isfinite(o->xsph) || !std::isfinite(o->vorticity) || !std::isfinite(o->surface_tension) ||
      !std::isfinite(o->gravity))
    return fail(h, PBF_EINVAL, "non-finite option");
  if (std::memcmp(&h->cfg.options, o, sizeof(pbf_options)) == 0) return PBF_OK;
  h->cfg.options = *o;
  h->sp.gy = (float)(-(double)o->gravity);
  h->sp.xsph = o->xsph;
  h->sp.vorticity = o->vorticity;
  h->sp.tension = o->surface_tension;
  invalidate_graph(h);
  return PBF_OK;
}

int pbf_get_options(const pbf_handle* h, pbf_options* o) {
  if (!h || !o) return PBF_EINVAL;
  *o = h->cfg.options;
  return PBF_OK;
}

int pbf_voxelize_cube(pbf_handle* h, const float mn[3], const float mx[3], uint32_t* added) {
  if (!h || !mn || !mx) return PBF_EINVAL;
  const double diam = 2.0 * (double)h->cfg.particle_radius;
  long nx = (long)std::floor(((double)mx[0] - mn[0]) / diam);
  long ny = (long)std::floor(((double)mx[1] - mn[1]) / diam);
  long nz = (long)std::floor(((double)mx[2] - mn[2]) / diam);
  uint32_t count = 0;
  for (long i = 0; i < nx; ++i)
    for (long j = 0; j < ny; ++j)
      for (long k = 0; k < nz; ++k) {
        h->host_particles.push_back((float)(i * diam + mn[0]));
        h->host_particles.push_back((float)(j * diam + mn[1]));
        h->host_particles.push_back((float)(k * diam + mn[2]));
        h->host_particles.push_back(0.0f);
        ++count;
      }
  if (added) *added = count;
  return PBF_OK;
}

int pbf_voxelize_sphere(pbf_handle* h, const float c[3], float radius, uint32_t* added) {
  if (!h || !c) return PBF_EINVAL;
  const double diam = 2.0 * (double)h->cfg.particle_radius;
  long vd = (long)std::floor((double)radius / (double)h->cfg.particle_radius / 2.0);
  const double r2 = (double)radius * radius;
  uint32_t count = 0;
  for (long i = -vd; i <= vd; ++i)
    for (long j = -vd; j <= vd; ++j)
      for (long k = -vd; k <= vd; ++k) {
        double x = i * diam, y = j * diam, z = k * diam;
        if (x * x + y * y + z * z <= r2) {
          h->host_particles.push_back((float)(x + c[0]));
          h->host_particles.push_back((float)(y + c[1]));
          h->host_particles.push_back((float)(z + c[2]));
          h->host_particles.push_back(0.0f);
          ++count;
        }
      }
  if (added) *added = count;
  return PBF_OK;
}

int pbf_voxelize_mesh(pbf_handle* h, const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                      uint32_t triangle_count, const double world[16], uint32_t* added) {
  if (!h) return PBF_EINVAL;
  std::vector<float> pts;
  uint32_t count = 0;
  int rc = voxelize_mesh_host(vertices, vertex_count, indices, triangle_count, world,
                              (double)h->cfg.particle_radius, true, &pts, &count);
  if (rc) return fail(h, rc, "voxelizeMesh failed");
  h->host_particles.insert(h->host_particles.end(), pts.begin(), pts.end());
  if (added) *added = count;
  return PBF_OK;
}

int pbf_seed_device(pbf_handle* h, const pbf_seed_item* items, uint32_t count, float jitter_amplitude,
                    uint64_t jitter_seed, uint32_t* total) {
  if (!h || (!items && count)) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_seed_device");
  uint32_t made = 0;
  invalidate_graph(h);
  // the items are seeded into pos[1] / ids[1] first, so a failure leaves the
  // current particles as they were
  int rc = seed_device(items, count, (double)h->cfg.particle_radius, jitter_amplitude, jitter_seed, h->pos[1].p,
                       h->ids[1].p, h->cfg.max_particles, &made, h->stream);
  if (total) *total = made;
  if (rc == PBF_ECAPACITY)
    return fail(h, PBF_ECAPACITY, "To Many Particles! (%u > max_particles %u)", made, h->cfg.max_particles);
  if (rc) return fail(h, rc, "pbf_seed_device failed");
  if (made) {
    CU(h, cudaMemcpyAsync(h->pos[0].p, h->pos[1].p, (size_t)made * sizeof(float4), cudaMemcpyDeviceToDevice,
                          h->stream));
    CU(h, cudaMemcpyAsync(h->ids[0].p, h->ids[1].p, (size_t)made * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                          h->stream));
  }
  h->host_particles.clear();
  return finish_upload(h, made);
}

int pbf_jitter_particles(pbf_handle* h, float amplitude, uint64_t seed) {
  if (!h) return PBF_EINVAL;
  uint64_t s = seed;
  auto next = [&]() {  // splitmix64
    s += 0x9e3779b97f4a7c15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  };
  size_t n = h->host_particles.size() / 4;
  for (size_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      double u = (double)(next() >> 11) * (1.0 / 9007199254740992.0);
      h->host_particles[4 * i + a] = (float)((double)h->host_particles[4 * i + a] + (double)amplitude * (2.0 * u - 1.0));
    }
  return PBF_OK;
}

int pbf_host_particle_count(const pbf_handle* h, uint32_t* count) {
  if (!h || !count) return PBF_EINVAL;
  *count = (uint32_t)(h->host_particles.size() / 4);
  return PBF_OK;
}

int pbf_copy_host_particles(const pbf_handle* h, float* xyzw, uint32_t n) {
  if (!h || !xyzw) return PBF_EINVAL;
  if ((size_t)n * 4 != h->host_particles.size()) return PBF_EINVAL;
  std::memcpy(xyzw, h->host_particles.data(), h->host_particles.size() * sizeof(float));
  return PBF_OK;
}

int pbf_set_particle_position(pbf_handle* h) {
  if (!h) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_set_particle_position");
  if (h->host_particles.size() % 4 != 0) return fail(h, PBF_EINVAL, "Illegal length of Particle Position Buffer!");
  uint32_t n = (uint32_t)(h->host_particles.size() / 4);
  return upload_particles(h, h->host_particles.data(), n);
}

int pbf_set_particles(pbf_handle* h, const float* xyzw, uint32_t n) {
  if (!h || (!xyzw && n)) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_set_particles");
  for (size_t i = 0; i < (size_t)n * 4; ++i)
    if ((i & 3) != 3 && !std::isfinite(xyzw[i])) return fail(h, PBF_EINVAL, "non-finite particle position");
  h->host_particles.assign(xyzw, xyzw + (size_t)n * 4);
  return upload_particles(h, xyzw, n);
}

// Overwrites a per-particle float4 state array (slot order on the device)
// from a by-id host array: the host reorders through the current ids
// (slot -> id); w is cleared.
static int upload_by_id(pbf_handle* h, float4* dst, const float* xyzw, uint32_t n, const char* what) {
  if (!h || !xyzw) return PBF_EINVAL;
  if (n != h->n) return fail(h, PBF_EINVAL, "%s count %u != particle count %u", what, n, h->n);
  std::vector<uint32_t> ids(n);
  CU(h, cudaMemcpyAsync(ids.data(), h->ids[h->cur].p, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  std::vector<float> v((size_t)n * 4);
  for (uint32_t t = 0; t < n; ++t)
    for (int a = 0; a < 4; ++a) v[4 * (size_t)t + a] = (a == 3) ? 0.0f : xyzw[4 * (size_t)ids[t] + a];
  CU(h, cudaMemcpyAsync(dst, v.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  invalidate_graph(h);
  return PBF_OK;
}

int pbf_set_velocities(pbf_handle* h, const float* xyzw, uint32_t n) {
  return h ? upload_by_id(h, h->vel.p, xyzw, n, "velocity") : PBF_EINVAL;
}

int pbf_set_accelerations(pbf_handle* h, const float* xyzw, uint32_t n) {
  return h ? upload_by_id(h, h->acc.p, xyzw, n, "acceleration") : PBF_EINVAL;
}

size_t pbf_field_length(const uint32_t res[3]) {
  const size_t nx = res[0], ny = res[1], nz = res[2];
  return (nx + 1) * (ny + 1) * (nz + 1) + 2 * nx * (ny + 1) * (nz + 1) + (nx + 1) * 2 * ny * (nz + 1) +
         (nx + 1) * (ny + 1) * 2 * nz;
}

int pbf_set_boundary_field(pbf_handle* h, const uint32_t res[3], const float origin[3], const float extent[3],
                           const float* sdf, const float* volume, size_t nodes) {
  if (!h || !res || !origin || !extent || !sdf || !volume) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_set_boundary_field");
  for (int a = 0; a < 3; ++a) {
    if (res[a] == 0 || res[a] > 4096) return fail(h, PBF_EINVAL, "bad field resolution");
    if (!finite_positive(extent[a])) return fail(h, PBF_EINVAL, "bad field extent");
  }
  size_t len = pbf_field_length(res);
  if (nodes != len) return fail(h, PBF_EFORMAT, "Invalid Boundary Model File! (%zu values, expected %zu)", nodes, len);
  if (len > 0xffffffffull) return fail(h, PBF_ECAPACITY, "field of %zu nodes (32-bit node indices)", len);
  invalidate_graph(h);
  h->sdf.release();
  h->vol.release();
  CU(h, h->sdf.alloc(len));
  CU(h, h->vol.alloc(len));
  CU(h, cudaMemcpyAsync(h->sdf.p, sdf, len * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CU(h, cudaMemcpyAsync(h->vol.p, volume, len * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CU(h, cudaMemsetAsync(h->bdata.p, 0, (size_t)h->cfg.max_particles * sizeof(float4), h->stream));
  {
    std::vector<uint8_t> flag;
    boundary_flags(res, sdf, volume, h->cfg.kernel_radius, flag);
    std::vector<uint32_t> cell;
    std::vector<float> blocks;
    pack_field_blocks(res, sdf, volume, flag, cell, blocks);
    h->bflag.release();
    h->bcell.release();
    h->bnodes.release();
    CU(h, h->bflag.alloc(flag.size()));
    CU(h, h->bcell.alloc(cell.size()));
    CU(h, h->bnodes.alloc(blocks.size() / 4));
    CU(h, cudaMemcpyAsync(h->bflag.p, flag.data(), flag.size(), cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemcpyAsync(h->bcell.p, cell.data(), cell.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    if (!blocks.empty())
      CU(h, cudaMemcpyAsync(h->bnodes.p, blocks.data(), blocks.size() * sizeof(float), cudaMemcpyHostToDevice,
                            h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
  }
  CU(h, cudaStreamSynchronize(h->stream));
  set_field_params(h, res, origin, extent);
  h->fp.loaded = 1;
  return PBF_OK;
}

// BoundaryModel.setData (volumeMap.ts:23-39): line 0 resolution, line 2 the
// SDF values, line 4 the volume values.  The field spans the simulation domain.
int pbf_set_boundary_data(pbf_handle* h, const char* text, size_t len) {
  if (!h || !text) return PBF_EINVAL;
  std::vector<std::string> lines;
  {
    size_t s = 0;
    for (size_t i = 0; i <= len; ++i) {
      if (i == len || text[i] == '\n') {
        lines.emplace_back(text + s, i - s);
        s = i + 1;
      }
    }
  }
  if (lines.size() < 5) return fail(h, PBF_EFORMAT, "Invalid Boundary Model File! (%zu lines)", lines.size());
  uint32_t res[3];
  {
    double r[3];
    if (std::sscanf(lines[0].c_str(), "%lf %lf %lf", &r[0], &r[1], &r[2]) != 3)
      return fail(h, PBF_EFORMAT, "Invalid Boundary Model File! (resolution line)");
    for (int a = 0; a < 3; ++a) {
      if (!(r[a] >= 1.0 && r[a] <= 4096.0) || r[a] != std::floor(r[a]))
        return fail(h, PBF_EFORMAT, "Invalid Boundary Model File! (resolution)");
      res[a] = (uint32_t)r[a];
    }
  }
  const size_t expect = pbf_field_length(res);
  auto parse = [&](const std::string& line, std::vector<float>& out) -> bool {
    out.clear();
    out.reserve(expect);
    const char* p = line.c_str();
    const char* end = p + line.size();
    while (p < end) {
      while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
      if (p >= end) break;
      char* q = nullptr;
      float v = std::strtof(p, &q);
      if (q == p) return false;
      if (!std::isfinite(v)) return false;
      out.push_back(v);
      p = q;
    }
    return true;
  };
  std::vector<float> sdf, vol;
  if (!parse(lines[2], sdf) || !parse(lines[4], vol))
    return fail(h, PBF_EFORMAT, "Invalid Boundary Model File! (non-numeric value)");
  if (sdf.size() != expect || vol.size() != expect)
    return fail(h, PBF_EFORMAT, "Invalid Boundary Model File! (%zu / %zu values, expected %zu)", sdf.size(),
                vol.size(), expect);
  float origin[3], extent[3];
  for (int a = 0; a < 3; ++a) {
    origin[a] = h->cfg.domain_min[a];
    extent[a] = h->cfg.domain_max[a] - h->cfg.domain_min[a];
  }
  return pbf_set_boundary_field(h, res, origin, extent, sdf.data(), vol.data(), expect);
}

int pbf_clear_boundary(pbf_handle* h) {
  if (!h) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_clear_boundary");
  invalidate_graph(h);
  h->fp.loaded = 0;
  return PBF_OK;
}

int pbf_set_paused(pbf_handle* h, int paused) {
  if (!h) return PBF_EINVAL;
  h->paused = paused != 0;
  return PBF_OK;
}
int pbf_is_paused(const pbf_handle* h) { return h ? (h->paused ? 1 : 0) : -1; }

int pbf_set_capture(pbf_handle* h, int enable) {
  if (!h) return PBF_EINVAL;
  invalidate_graph(h);
  if (enable && !h->dp.p) CU(h, h->dp.alloc(h->cfg.max_particles));
  h->capture = enable != 0;
  return PBF_OK;
}

int pbf_run(pbf_handle* h) {
  if (!h) return PBF_EINVAL;
  if (h->paused || h->n == 0) return PBF_OK;
  int rc = substep(h, nullptr);
  if (rc) return rc;
  return export_positions(h);
}

int pbf_enable_graph(pbf_handle* h, int enable) {
  if (!h) return PBF_EINVAL;
  invalidate_graph(h);
  h->graph_enabled = enable != 0;
  return PBF_OK;
}

int pbf_step(pbf_handle* h, uint32_t frames) {
  if (!h) return PBF_EINVAL;
  if (h->paused || h->n == 0) return PBF_OK;
  // Trace capture samples a different particle subset every substep (its salt
  // and the substep counter are host values a graph would freeze), so it
  // runs eagerly, as per-kernel timing does.
  if (!h->graph_enabled || h->ktiming || h->trace_cap > 0) {
    for (uint32_t f = 0; f < frames; ++f) {
      int rc = frame(h);
      if (rc) return rc;
    }
    return PBF_OK;
  }
  // Each substep swaps the state buffers once, so a graph covers an even
  // number of substeps (one frame, or two frames when substeps is odd) and
  // every replay starts from the same buffers.
  const uint32_t per_graph = (h->cfg.substeps % 2 == 0) ? 1u : 2u;
  if (!h->graph_valid) {
    const int start_cur = h->cur;
    cudaGraph_t g = nullptr;
    CU(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = PBF_OK;
    for (uint32_t f = 0; f < per_graph && rc == PBF_OK; ++f) rc = frame(h);
    cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    h->cur = start_cur;  // capture only recorded the work
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(h, PBF_ECUDA, "graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&h->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fail(h, PBF_ECUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    h->graph_valid = true;
  }
  uint32_t full = frames / per_graph, rest = frames % per_graph;
  for (uint32_t f = 0; f < full; ++f) CU(h, cudaGraphLaunch(h->graph_exec, h->stream));
  for (uint32_t f = 0; f < rest; ++f) {
    // an odd remainder runs eagerly and leaves the buffers swapped: the graph
    // no longer matches them
    invalidate_graph(h);
    int rc = frame(h);
    if (rc) return rc;
  }
  return PBF_OK;
}

int pbf_run_timestamp(pbf_handle* h, float ms[4]) {
  if (!h || !ms) return PBF_EINVAL;
  for (int i = 0; i < 4; ++i) ms[i] = 0.0f;
  if (h->n == 0) return PBF_OK;
  int rc = substep(h, h->ev);
  if (rc) return rc;
  rc = export_positions(h);
  if (rc) return rc;
  CU(h, cudaEventSynchronize(h->ev[4]));
  for (int i = 0; i < 4; ++i) CU(h, cudaEventElapsedTime(&ms[i], h->ev[i], h->ev[i + 1]));
  return check_device_errors(h);
}

int pbf_synchronize(pbf_handle* h) {
  if (!h) return PBF_EINVAL;
  CU(h, cudaStreamSynchronize(h->stream));
  if (h->copy_stream) CU(h, cudaStreamSynchronize(h->copy_stream));
  return check_device_errors(h);
}

int pbf_set_kernel_timing(pbf_handle* h, int enable) {
  if (!h) return PBF_EINVAL;
  h->ktiming = enable != 0;
  return PBF_OK;
}

int pbf_get_kernel_timing(pbf_handle* h, pbf_kernel_time* out, uint32_t max, uint32_t* count) {
  if (!h || (!out && max)) return PBF_EINVAL;
  CU(h, cudaStreamSynchronize(h->stream));
  double total[K_NUM] = {0};
  uint32_t launches[K_NUM] = {0};
  for (auto& pr : h->kt_pairs) {
    float ms = 0.0f;
    CU(h, cudaEventElapsedTime(&ms, h->kt_events[pr.second], h->kt_events[pr.second + 1]));
    total[pr.first] += ms;
    launches[pr.first] += 1;
  }
  h->kt_pairs.clear();
  uint32_t c = 0;
  for (int k = 0; k < K_NUM; ++k) {
    if (!launches[k]) continue;
    if (c < max) {
      std::memset(out[c].name, 0, sizeof(out[c].name));
      std::strncpy(out[c].name, kPassNames[k], sizeof(out[c].name) - 1);
      out[c].launches = launches[k];
      out[c].total_ms = (float)total[k];
    }
    ++c;
  }
  if (count) *count = c;
  return PBF_OK;
}

// Buffers shared by trace capture and the learned start (allocated on first use).
static int ensure_feature_buffers(pbf_handle* h) {
  const size_t cap = h->cfg.max_particles;
  if (!h->feat.p) {
    CU(h, h->feat.alloc(2 * cap));
    CU(h, h->lam_sum.alloc(cap));
    CU(h, h->lam_prev.alloc(cap));
    CU(h, h->bsdf.alloc(cap));
    CU(h, cudaMemsetAsync(h->lam_sum.p, 0, cap * sizeof(float), h->stream));
    CU(h, cudaMemsetAsync(h->lam_prev.p, 0, cap * sizeof(float), h->stream));
    CU(h, cudaMemsetAsync(h->bsdf.p, 0, cap * sizeof(float), h->stream));
  }
  return PBF_OK;
}

int pbf_set_trace(pbf_handle* h, uint32_t capacity, uint32_t stride, uint64_t salt) {
  if (h && h->batch) return not_for_batch(h, "pbf_set_trace");
  if (!h || stride == 0) return PBF_EINVAL;
  invalidate_graph(h);
  h->trace_feat.release();
  h->trace_tgt.release();
  h->trace_cap = 0;
  if (capacity == 0) return PBF_OK;
  int rc = ensure_feature_buffers(h);
  if (rc) return rc;
  CU(h, h->trace_feat.alloc((size_t)capacity * 8));
  CU(h, h->trace_tgt.alloc(capacity));
  if (!h->stats.p) {
    CU(h, h->stats.alloc(1));
    CU(h, cudaMemsetAsync(h->stats.p, 0, sizeof(SolveStats), h->stream));
  }
  if (!h->trace_err.p) CU(h, h->trace_err.alloc(3));
  CU(h, cudaMemsetAsync(h->trace_err.p, 0, 3 * sizeof(float), h->stream));
  if (!h->trace_count.p) CU(h, h->trace_count.alloc(1));
  CU(h, cudaMemsetAsync(h->trace_count.p, 0, sizeof(uint32_t), h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  h->trace_cap = capacity;
  h->trace_stride = stride;
  h->trace_salt = salt;
  return PBF_OK;
}

int pbf_trace_rows(pbf_handle* h, uint32_t* rows) {
  if (!h || !rows) return PBF_EINVAL;
  *rows = 0;
  if (!h->trace_count.p) return PBF_OK;
  uint32_t c = 0;
  CU(h, cudaMemcpyAsync(&c, h->trace_count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  *rows = c < h->trace_cap ? c : h->trace_cap;
  return PBF_OK;
}

int pbf_copy_trace(pbf_handle* h, float* feat, float* target, uint32_t rows) {
  if (!h || !feat || !target) return PBF_EINVAL;
  uint32_t have = 0;
  int rc = pbf_trace_rows(h, &have);
  if (rc) return rc;
  if (rows > have) return fail(h, PBF_EINVAL, "trace holds %u rows, %u requested", have, rows);
  if (rows == 0) return PBF_OK;
  CU(h, cudaMemcpyAsync(feat, h->trace_feat.p, (size_t)rows * 8 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaMemcpyAsync(target, h->trace_tgt.p, (size_t)rows * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return PBF_OK;
}

int pbf_trace_error(pbf_handle* h, float* max_mean, float* avg_mean) {
  if (!h || !max_mean || !avg_mean) return PBF_EINVAL;
  *max_mean = *avg_mean = 0.0f;
  if (!h->trace_err.p) return PBF_OK;
  float r[3];
  CU(h, cudaMemcpyAsync(r, h->trace_err.p, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  *max_mean = r[0];
  *avg_mean = r[2] > 0 ? r[1] / r[2] : 0.0f;
  return PBF_OK;
}

int pbf_set_mlp_kernel(pbf_handle* h, uint32_t kernel) {
  if (!h) return PBF_EINVAL;
  if (kernel != PBF_MLP_KERNEL_MMA_SYNC && kernel != PBF_MLP_KERNEL_TCGEN05)
    return fail(h, PBF_EINVAL, "unknown network kernel %u", kernel);
  if (kernel != h->mlp_kernel) invalidate_graph(h);
  h->mlp_kernel = kernel;
  return PBF_OK;
}

int pbf_set_learned(pbf_handle* h, const pbf_mlp* model, uint32_t iterations, float fallback_bound) {
  if (h && h->batch) return not_for_batch(h, "pbf_set_learned");
  if (!h) return PBF_EINVAL;
  invalidate_graph(h);
  if (!model) {
    h->learned = false;
    return PBF_OK;
  }
  if (!std::isfinite(fallback_bound) || !(model->lam_scale > 0.0f))
    return fail(h, PBF_EINVAL, "learned start needs a finite bound and lam_scale > 0");
  int rc = ensure_feature_buffers(h);
  if (rc) return rc;
  const size_t cap = h->cfg.max_particles;
  if (!h->mlp_params.p) {
    CU(h, h->mlp_params.alloc(PBF_MLP_PARAMS));
    CU(h, h->xs_save.alloc(cap));
    if (h->stats.n < 2) {
      h->stats.release();
      CU(h, h->stats.alloc(2));
    }
    CU(h, h->fb_flag.alloc(2));
    CU(h, h->fb_count.alloc(3));
    CU(h, h->fb_mean.alloc(2));
    CU(h, cudaMemsetAsync(h->stats.p, 0, 2 * sizeof(SolveStats), h->stream));
    CU(h, cudaMemsetAsync(h->fb_flag.p, 0, 2 * sizeof(int), h->stream));
    CU(h, cudaMemsetAsync(h->fb_count.p, 0, 3 * sizeof(uint32_t), h->stream));
    CU(h, cudaMemsetAsync(h->fb_mean.p, 0, 2 * sizeof(float), h->stream));
  }
  if (!h->side_stream) {
    CU(h, cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking));
    CU(h, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    CU(h, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
  }
  h->model = *model;
  CU(h, cudaMemcpyAsync(h->mlp_params.p, model->params, sizeof(model->params), cudaMemcpyHostToDevice, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  h->learned_iters = iterations;
  h->fallback_bound = fallback_bound;
  h->learned = true;
  return PBF_OK;
}

int pbf_set_adaptive_iterations(pbf_handle* h, int enable) {
  if (!h) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_set_adaptive_iterations");
  if ((enable != 0) != h->adaptive) invalidate_graph(h);
  h->adaptive = enable != 0;
  if (h->fb_count.p) {  // restart the test counters
    CU(h, cudaMemsetAsync(h->fb_count.p + 1, 0, 2 * sizeof(uint32_t), h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
  }
  return PBF_OK;
}

int pbf_set_lagged_iterations(pbf_handle* h, float fraction) {
  if (!h) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_set_lagged_iterations");
  if (!std::isfinite(fraction)) return fail(h, PBF_EINVAL, "the lagged fraction must be finite");
  const float fr = fraction > 0.0f ? fraction : 0.0f;
  if (fr != h->lagged_fraction) invalidate_graph(h);
  h->lagged_fraction = fr;
  if (h->fb_count.p) {  // restart the decision counters
    CU(h, cudaMemsetAsync(h->fb_count.p + 1, 0, 2 * sizeof(uint32_t), h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
  }
  return PBF_OK;
}

int pbf_adaptive_counts(pbf_handle* h, uint32_t* tests, uint32_t* updates_run) {
  if (!h || !tests || !updates_run) return PBF_EINVAL;
  *tests = 0;
  *updates_run = 0;
  if (h->fb_count.p) {
    uint32_t c[3];
    CU(h, cudaStreamSynchronize(h->stream));
    CU(h, cudaMemcpy(c, h->fb_count.p, sizeof(c), cudaMemcpyDeviceToHost));
    *tests = c[1];
    *updates_run = c[2];
  }
  return PBF_OK;
}

uint32_t pbf_particle_count(const pbf_handle* h) { return h ? h->n : 0; }
const float* pbf_position_device(pbf_handle* h) { return h ? (const float*)h->out_pos.p : nullptr; }
const float* pbf_velocity_device(pbf_handle* h) {
  if (!h) return nullptr;
  if (launch_scatter_by_id(h->n, h->ids[h->cur].p, h->vel.p, h->out_tmp.p, h->stream) != cudaSuccess) return nullptr;
  return (const float*)h->out_tmp.p;
}
void* pbf_stream(pbf_handle* h) { return h ? (void*)h->stream : nullptr; }

// The frame's by-id positions are copied device to device into a staging
// buffer on a second stream, then from there to the host on that stream, so
// the host read overlaps the next frames.  The handle's stream waits only
// for the device-to-device copy (a few microseconds) before its next work,
// so the next frame's export cannot overwrite positions still being staged;
// the staging buffer itself is reused in order on the copy stream.
int pbf_copy_positions_async(pbf_handle* h, float* host, size_t bytes) {
  if (!h || (!host && bytes)) return PBF_EINVAL;
  if (bytes != (size_t)h->n * sizeof(float4))
    return fail(h, PBF_EINVAL, "positions need %zu bytes, got %zu", (size_t)h->n * sizeof(float4), bytes);
  if (bytes == 0) return PBF_OK;
  if (!h->copy_stream) {
    CU(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    CU(h, cudaEventCreateWithFlags(&h->ev_frame, cudaEventDisableTiming));
    CU(h, cudaEventCreateWithFlags(&h->ev_staged, cudaEventDisableTiming));
  }
  if (h->staging.n < h->n) {
    CU(h, cudaStreamSynchronize(h->copy_stream));
    h->staging.release();
    CU(h, h->staging.alloc(std::max<size_t>(h->cfg.max_particles, h->n)));
  }
  CU(h, cudaEventRecord(h->ev_frame, h->stream));
  CU(h, cudaStreamWaitEvent(h->copy_stream, h->ev_frame, 0));
  CU(h, cudaMemcpyAsync(h->staging.p, h->out_pos.p, bytes, cudaMemcpyDeviceToDevice, h->copy_stream));
  CU(h, cudaEventRecord(h->ev_staged, h->copy_stream));
  CU(h, cudaMemcpyAsync(host, h->staging.p, bytes, cudaMemcpyDeviceToHost, h->copy_stream));
  CU(h, cudaStreamWaitEvent(h->stream, h->ev_staged, 0));
  return PBF_OK;
}

int pbf_copy_field(pbf_handle* h, int field, void* host, size_t bytes) {
  if (!h || (!host && bytes)) return PBF_EINVAL;
  const uint32_t n = h->n;
  cudaStream_t st = h->stream;
  const uint32_t* id = h->ids[h->cur].p;
  size_t need4 = (size_t)n * sizeof(float4), need1 = (size_t)n * 4;
  const float4* src4 = nullptr;
  switch (field) {
    case PBF_FIELD_POSITION: src4 = h->pos[h->cur].p; break;
    case PBF_FIELD_VELOCITY: src4 = h->vel.p; break;
    case PBF_FIELD_ACCELERATION: src4 = h->acc.p; break;
    case PBF_FIELD_PREDICTED: src4 = h->xs[0].p; break;
    case PBF_FIELD_BOUNDARY: src4 = h->bdata.p; break;
    case PBF_FIELD_OMEGA: src4 = h->omega.p; break;
    case PBF_FIELD_NORMAL: src4 = h->normal.p; break;  // w (|omega|, internal) is cleared below
    case PBF_FIELD_DELTA_P:
      if (!h->capture || !h->dp.p) return fail(h, PBF_ESTATE, "delta_p needs pbf_set_capture(1) before the step");
      src4 = h->dp.p;
      break;
    case PBF_FIELD_LAMBDA:
    case PBF_FIELD_NEIGHBOR_COUNT: break;
    default: return fail(h, PBF_EINVAL, "unknown field %d", field);
  }
  if (src4) {
    if (bytes != need4) return fail(h, PBF_EINVAL, "field needs %zu bytes, got %zu", need4, bytes);
    if (n) {
      CU(h, launch_scatter_by_id(n, id, src4, h->out_tmp.p, st));
      if (field == PBF_FIELD_NORMAL) CU(h, cudaMemset2DAsync((char*)h->out_tmp.p + 12, 16, 0, 4, n, st));
      CU(h, cudaMemcpyAsync(host, h->out_tmp.p, need4, cudaMemcpyDeviceToHost, st));
    }
  } else {
    if (bytes != need1) return fail(h, PBF_EINVAL, "field needs %zu bytes, got %zu", need1, bytes);
    if (n) {
      if (field == PBF_FIELD_LAMBDA)
        CU(h, launch_scatter_w_by_id(n, id, h->xl.p, (float*)h->out_tmp.p, st));
      else
        CU(h, launch_scatter_by_id_u32(n, id, h->nbr_count.p, (uint32_t*)h->out_tmp.p, st));
      CU(h, cudaMemcpyAsync(host, h->out_tmp.p, need1, cudaMemcpyDeviceToHost, st));
    }
  }
  CU(h, cudaStreamSynchronize(st));
  return check_device_errors(h);
}

int pbf_copy_search_state(pbf_handle* h, int which, uint32_t* host, size_t count) {
  if (!h || (!host && count)) return PBF_EINVAL;
  if (h->batch) return not_for_batch(h, "pbf_copy_search_state");
  const uint32_t n = h->n;
  cudaStream_t st = h->stream;
  size_t need = 0;
  switch (which) {
    case PBF_SEARCH_CELL_KEY:
    case PBF_SEARCH_ORDER: need = n; break;
    case PBF_SEARCH_CELL_COUNT: need = h->gp.cells; break;
    case PBF_SEARCH_CELL_OFFSET: need = (size_t)h->gp.cells + 1; break;
    default: return fail(h, PBF_EINVAL, "unknown search array %d", which);
  }
  if (count != need) return fail(h, PBF_EINVAL, "search array %d has %zu entries, got %zu", which, need, count);
  if (need == 0) return PBF_OK;
  if (which == PBF_SEARCH_CELL_KEY) {
    // keys were computed in the slot order before the sort: slot s of the
    // previous order held particle ids[1 - cur][s]
    std::vector<uint32_t> key(n), old_ids(n);
    CU(h, cudaMemcpyAsync(key.data(), h->key.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    CU(h, cudaMemcpyAsync(old_ids.data(), h->ids[1 - h->cur].p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    CU(h, cudaStreamSynchronize(st));
    for (uint32_t s = 0; s < n; ++s) host[old_ids[s]] = key[s];
  } else {
    const uint32_t* src = which == PBF_SEARCH_ORDER        ? h->ids[h->cur].p
                          : which == PBF_SEARCH_CELL_COUNT ? h->cell_count.p
                                                           : h->cell_start.p;
    CU(h, cudaMemcpyAsync(host, src, need * 4, cudaMemcpyDeviceToHost, st));
    CU(h, cudaStreamSynchronize(st));
  }
  return check_device_errors(h);
}

int pbf_get_metrics(pbf_handle* h, pbf_metrics* out) {
  if (!h || !out) return PBF_EINVAL;
  if (!h->batch) {
    int rc = metrics_range(h, 0, h->n, h->fp, h->sdf.p, out);
    if (rc) return rc;
  } else {
    // all scenes: sums, maxima, particle-weighted means
    pbf_metrics acc;
    std::memset(&acc, 0, sizeof(acc));
    double mean_abs = 0.0, mean_c = 0.0;
    for (size_t s = 0; s < h->scenes.size(); ++s) {
      const SceneDesc& sd = h->scenes[s];
      pbf_metrics m;
      int rc = metrics_range(h, sd.first, sd.n, sd.field, h->sdf.p ? h->sdf.p + sd.field.node_off : nullptr, &m);
      if (rc) return rc;
      acc.particles += m.particles;
      acc.nonfinite += m.nonfinite;
      acc.penetrations += m.penetrations;
      acc.error_flags |= m.error_flags;
      acc.max_compression = std::max(acc.max_compression, m.max_compression);
      acc.max_abs_density_err = std::max(acc.max_abs_density_err, m.max_abs_density_err);
      acc.kinetic_energy += m.kinetic_energy;
      acc.neighbor_total += m.neighbor_total;
      mean_abs += (double)m.mean_abs_density_err * m.particles;
      mean_c += (double)m.mean_compression * m.particles;
    }
    if (acc.particles) {
      acc.mean_abs_density_err = (float)(mean_abs / acc.particles);
      acc.mean_compression = (float)(mean_c / acc.particles);
    }
    *out = acc;
  }
  if (h->fb_count.p) {
    uint32_t fb = 0;
    CU(h, cudaMemcpy(&fb, h->fb_count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    out->fallback_steps = fb;
  }
  return PBF_OK;
}

int pbf_set_launch(pbf_handle* h, const pbf_launch* l) {
  if (!h || !l) return PBF_EINVAL;
  return apply_launch(h, *l);
}

int pbf_set_cellblock_capacity(pbf_handle* h, uint32_t records) {
  if (!h) return PBF_EINVAL;
  if (records < 16 || records % 16 || records > 3072)
    return fail(h, PBF_EINVAL, "cell-block capacity must be a multiple of 16 in [16, 3072]");
  if (records != h->cb_cap) invalidate_graph(h);
  h->cb_cap = records;
  return cb_active(h) ? ensure_cb(h) : PBF_OK;
}

int pbf_get_launch(const pbf_handle* h, pbf_launch* l) {
  if (!h || !l) return PBF_EINVAL;
  l->block = (uint32_t)h->blk;
  l->ctas_per_sm = h->per_sm;
  l->cell_ratio = h->cell_ratio;
  l->build = h->build;
  return PBF_OK;
}

int pbf_autotune(pbf_handle* h, uint32_t substeps, uint32_t flags, pbf_tune_trial* trials, uint32_t max_trials,
                 uint32_t* count, pbf_launch* best) {
  if (!h || (!trials && max_trials)) return PBF_EINVAL;
  if (h->trace_cap > 0) return fail(h, PBF_ESTATE, "pbf_autotune while trace capture is on");
  if (h->n == 0) return fail(h, PBF_ESTATE, "pbf_autotune needs particles");
  if (substeps == 0) substeps = 4;
  const uint32_t n = h->n;
  cudaStream_t st = h->stream;
  CU(h, cudaStreamSynchronize(st));
  int rc = check_device_errors(h);
  if (rc) return rc;
  // the state the trials start from and that is restored afterwards
  const int cur0 = h->cur;
  const uint32_t ctr0 = h->substep_counter;
  DBuf<float4> s_pos, s_vel, s_acc;
  DBuf<uint32_t> s_ids;
  DBuf<float> s_lam;
  uint32_t fb0 = 0;
  struct Free {
    DBuf<float4>*a, *b, *c;
    DBuf<uint32_t>* d;
    DBuf<float>* e;
    ~Free() {
      a->release();
      b->release();
      c->release();
      d->release();
      e->release();
    }
  } fr{&s_pos, &s_vel, &s_acc, &s_ids, &s_lam};
  CU(h, s_pos.alloc(n));
  CU(h, s_vel.alloc(n));
  CU(h, s_acc.alloc(n));
  CU(h, s_ids.alloc(n));
  const size_t b4 = (size_t)n * sizeof(float4), b1 = (size_t)n * sizeof(uint32_t);
  CU(h, cudaMemcpyAsync(s_pos.p, h->pos[cur0].p, b4, cudaMemcpyDeviceToDevice, st));
  CU(h, cudaMemcpyAsync(s_vel.p, h->vel.p, b4, cudaMemcpyDeviceToDevice, st));
  CU(h, cudaMemcpyAsync(s_acc.p, h->acc.p, b4, cudaMemcpyDeviceToDevice, st));
  CU(h, cudaMemcpyAsync(s_ids.p, h->ids[cur0].p, b1, cudaMemcpyDeviceToDevice, st));
  if (h->lam_sum.p) {
    CU(h, s_lam.alloc(n));
    CU(h, cudaMemcpyAsync(s_lam.p, h->lam_sum.p, b1, cudaMemcpyDeviceToDevice, st));
  }
  if (h->fb_count.p) CU(h, cudaMemcpy(&fb0, h->fb_count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  auto restore = [&]() -> int {
    h->cur = cur0;
    h->substep_counter = ctr0;
    CU(h, cudaMemcpyAsync(h->pos[cur0].p, s_pos.p, b4, cudaMemcpyDeviceToDevice, st));
    CU(h, cudaMemcpyAsync(h->vel.p, s_vel.p, b4, cudaMemcpyDeviceToDevice, st));
    CU(h, cudaMemcpyAsync(h->acc.p, s_acc.p, b4, cudaMemcpyDeviceToDevice, st));
    CU(h, cudaMemcpyAsync(h->ids[cur0].p, s_ids.p, b1, cudaMemcpyDeviceToDevice, st));
    if (s_lam.p) CU(h, cudaMemcpyAsync(h->lam_sum.p, s_lam.p, b1, cudaMemcpyDeviceToDevice, st));
    if (h->fb_count.p) CU(h, cudaMemcpyAsync(h->fb_count.p, &fb0, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CU(h, cudaStreamSynchronize(st));
    return PBF_OK;
  };
  std::vector<pbf_launch> cand;
  const float ratios[2] = {1.0f, 0.5f};
  // one tile per CTA or a persistent grid holding all of an SM's 2048
  // threads; the three neighbour-build variants
  const uint32_t blocks[2] = {128, 256};
  for (int r = 0; r < ((flags & PBF_TUNE_CELL_RATIO) ? 2 : 1); ++r) {
    for (uint32_t b : blocks)
      for (uint32_t k : {0u, 2048u / b})
        for (uint32_t bv : {PBF_BUILD_THREAD, PBF_BUILD_PAIR, PBF_BUILD_WARP})
          cand.push_back(pbf_launch{b, k, ratios[r], bv});
    // the cell-block passes (single scenes): their own 128-slot tiles; the
    // other passes take either block size
    if (!h->batch)
      for (uint32_t b : blocks)
        for (uint32_t bv : {PBF_BUILD_CELLBLOCK_MASK, PBF_BUILD_CELLBLOCK_FREE})
          cand.push_back(pbf_launch{b, 0u, ratios[r], bv});
  }
  const pbf_launch orig{(uint32_t)h->blk, h->per_sm, h->cell_ratio, h->build};
  const bool kt = h->ktiming;
  h->ktiming = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CU(h, cudaEventCreate(&e0));
  CU(h, cudaEventCreate(&e1));
  float best_ms = 3.4e38f;
  pbf_launch best_l = orig;
  uint32_t c = 0;
  for (const pbf_launch& l : cand) {
    rc = apply_launch(h, l);
    for (int attempt = 0; rc == PBF_OK && attempt < 2; ++attempt) {
      rc = restore();
      for (int w = 0; rc == PBF_OK && w < 2; ++w) rc = substep(h, nullptr);
      if (rc == PBF_OK && cudaEventRecord(e0, st) != cudaSuccess) rc = PBF_ECUDA;
      for (uint32_t k = 0; rc == PBF_OK && k < substeps; ++k) rc = substep(h, nullptr);
      if (rc == PBF_OK && cudaEventRecord(e1, st) != cudaSuccess) rc = PBF_ECUDA;
      if (rc == PBF_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = PBF_ECUDA;
      if (rc == PBF_OK) rc = check_device_errors(h);
      if (rc != PBF_ECAPACITY) break;  // a grown neighbour list: time the candidate again
      rc = PBF_OK;
    }
    if (rc) break;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)substeps;
    if (c < max_trials) trials[c] = pbf_tune_trial{l, ms};
    ++c;
    if (ms < best_ms) {
      best_ms = ms;
      best_l = l;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->ktiming = kt;
  const std::string err = h->err;
  int rc2 = apply_launch(h, rc ? orig : best_l);
  if (rc2 == PBF_OK) rc2 = restore();
  if (rc2 == PBF_OK) rc2 = export_positions(h);
  invalidate_graph(h);
  if (count) *count = c;
  if (best) *best = rc ? orig : best_l;
  if (rc) {
    h->err = err;
    return rc;
  }
  return rc2;
}

int pbf_batch_create(const pbf_config* shared, const pbf_scene* scenes, uint32_t count, pbf_handle** out) {
  if (!shared || !scenes || !out || count == 0 || count > 65535) return PBF_EINVAL;
  *out = nullptr;
  uint64_t total = 0;
  uint32_t max_it = 0;
  for (uint32_t s = 0; s < count; ++s) {
    const pbf_scene& sc = scenes[s];
    if (sc.struct_size != sizeof(pbf_scene) || sc.particles == 0 || !sc.positions) return PBF_EINVAL;
    for (int a = 0; a < 3; ++a)
      if (!(sc.domain_max[a] > sc.domain_min[a])) return PBF_EINVAL;
    const bool fld = sc.field_res[0] || sc.field_res[1] || sc.field_res[2];
    if (fld) {
      if (!sc.sdf || !sc.volume) return PBF_EINVAL;
      for (int a = 0; a < 3; ++a)
        if (sc.field_res[a] == 0 || sc.field_res[a] > 4096 || !finite_positive(sc.field_extent[a])) return PBF_EINVAL;
    }
    for (size_t i = 0; i < (size_t)sc.particles * 4; ++i)
      if ((i & 3) != 3 && !std::isfinite(sc.positions[i])) return PBF_EINVAL;
    total += sc.particles;
    uint32_t it = sc.iterations ? sc.iterations : shared->options.iterations;
    max_it = std::max(max_it, it);
  }
  if (total > 0x7fffffffull) return PBF_ECAPACITY;
  pbf_config c = *shared;
  c.max_particles = (uint32_t)total;
  for (int a = 0; a < 3; ++a) {
    c.domain_min[a] = scenes[0].domain_min[a];
    c.domain_max[a] = scenes[0].domain_max[a];
    c.grid_dim[a] = 0;
  }
  c.options.iterations = max_it;
  pbf_handle* h = nullptr;
  int rc = pbf_create(&c, &h);
  if (rc) return rc;
  auto bail = [&](int code, const char* msg) {
    pbf_destroy(h);
    (void)msg;
    return code;
  };
  h->batch = true;
  h->scenes.resize(count);
  h->scene_info.resize(count);
  uint64_t nodes = 0, flags = 0;
  bool any_field = false;
  uint32_t first = 0;
  for (uint32_t s = 0; s < count; ++s) {
    const pbf_scene& sc = scenes[s];
    SceneDesc sd{};
    for (int a = 0; a < 3; ++a) {
      sd.dmin[a] = sc.domain_min[a];
      sd.dmax[a] = sc.domain_max[a];
    }
    sd.iterations = sc.iterations ? sc.iterations : shared->options.iterations;
    sd.first = first;
    sd.n = sc.particles;
    first += sc.particles;
    if (sc.field_res[0] || sc.field_res[1] || sc.field_res[2]) {
      sd.field = make_field(c, sc.field_res, sc.field_origin, sc.field_extent);
      sd.field.node_off = (uint32_t)nodes;
      sd.field.flag_off = (uint32_t)flags;
      nodes += pbf_field_length(sc.field_res);
      flags += (uint64_t)sc.field_res[0] * sc.field_res[1] * sc.field_res[2];
      if (nodes > 0xffffffffull || flags > 0xffffffffull) return bail(PBF_ECAPACITY, "fields");
      any_field = true;
    } else {
      sd.field.loaded = 0;
    }
    h->scenes[s] = sd;
  }
  const uint64_t cells = layout_scenes(h);
  if (cells == 0) return bail(PBF_EINVAL, "cells");
  h->gp.cells = (uint32_t)cells;
  if (alloc_cells(h) != cudaSuccess) return bail(PBF_ECUDA, "cells");
  if (any_field) {
    std::vector<float> sdf(nodes), vol(nodes), blocks;
    std::vector<uint8_t> flag(flags), f1;
    std::vector<uint32_t> cell(flags, kNoBlock), c1;
    for (uint32_t s = 0; s < count; ++s) {
      const pbf_scene& sc = scenes[s];
      const SceneDesc& sd = h->scenes[s];
      if (!sd.field.loaded) continue;
      const size_t len = pbf_field_length(sc.field_res);
      std::memcpy(sdf.data() + sd.field.node_off, sc.sdf, len * sizeof(float));
      std::memcpy(vol.data() + sd.field.node_off, sc.volume, len * sizeof(float));
      boundary_flags(sc.field_res, sc.sdf, sc.volume, c.kernel_radius, f1);
      std::memcpy(flag.data() + sd.field.flag_off, f1.data(), f1.size());
      pack_field_blocks(sc.field_res, sc.sdf, sc.volume, f1, c1, blocks);
      std::memcpy(cell.data() + sd.field.flag_off, c1.data(), c1.size() * sizeof(uint32_t));
    }
    if (blocks.size() / 64 >= (size_t)kNoBlock) return bail(PBF_ECAPACITY, "fields");
    if (h->sdf.alloc(nodes) != cudaSuccess || h->vol.alloc(nodes) != cudaSuccess ||
        h->bflag.alloc(flags) != cudaSuccess || h->bcell.alloc(flags) != cudaSuccess ||
        h->bnodes.alloc(blocks.size() / 4) != cudaSuccess)
      return bail(PBF_ECUDA, "fields");
    if (cudaMemcpy(h->sdf.p, sdf.data(), nodes * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->vol.p, vol.data(), nodes * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->bflag.p, flag.data(), flags, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->bcell.p, cell.data(), flags * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess ||
        (!blocks.empty() && cudaMemcpy(h->bnodes.p, blocks.data(), blocks.size() * sizeof(float),
                                       cudaMemcpyHostToDevice) != cudaSuccess))
      return bail(PBF_ECUDA, "fields");
    h->fp = FieldParams{};
    h->fp.loaded = 1;
  }
  std::vector<uint16_t> slot_scene((size_t)total);
  std::vector<float> xyzw((size_t)total * 4);
  for (uint32_t s = 0; s < count; ++s) {
    const SceneDesc& sd = h->scenes[s];
    std::fill(slot_scene.begin() + sd.first, slot_scene.begin() + sd.first + sd.n, (uint16_t)s);
    std::memcpy(xyzw.data() + (size_t)sd.first * 4, scenes[s].positions, (size_t)sd.n * 4 * sizeof(float));
  }
  if (h->scenes_dev.alloc(count) != cudaSuccess || h->slot_scene.alloc(total) != cudaSuccess)
    return bail(PBF_ECUDA, "table");
  if (cudaMemcpy(h->scenes_dev.p, h->scenes.data(), count * sizeof(SceneDesc), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->slot_scene.p, slot_scene.data(), total * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(PBF_ECUDA, "table");
  h->tab = SceneTab{h->scenes_dev.p, h->slot_scene.p};
  rc = upload_particles(h, xyzw.data(), (uint32_t)total);
  if (rc) {
    pbf_destroy(h);
    return rc;
  }
  for (uint32_t s = 0; s < count; ++s) {
    const SceneDesc& sd = h->scenes[s];
    pbf_scene_info& in = h->scene_info[s];
    in.first_id = sd.first;
    in.particles = sd.n;
    in.iterations = sd.iterations;
  }
  *out = h;
  return PBF_OK;
}

uint32_t pbf_scene_count(const pbf_handle* h) {
  if (!h) return 0;
  return h->batch ? (uint32_t)h->scenes.size() : 1u;
}

int pbf_get_scene_info(const pbf_handle* h, uint32_t scene, pbf_scene_info* out) {
  if (!h || !out || scene >= pbf_scene_count(h)) return PBF_EINVAL;
  std::memset(out, 0, sizeof(*out));
  const GridParams& g = h->batch ? h->scenes[scene].grid : h->gp;
  if (h->batch) {
    *out = h->scene_info[scene];
  } else {
    out->first_id = 0;
    out->particles = h->n;
    out->iterations = h->cfg.options.iterations;
  }
  for (int a = 0; a < 3; ++a) out->grid_dim[a] = (uint32_t)g.dim[a];
  out->cells = g.cells;
  return PBF_OK;
}

int pbf_get_scene_metrics(pbf_handle* h, uint32_t scene, pbf_metrics* out) {
  if (!h || !out || scene >= pbf_scene_count(h)) return PBF_EINVAL;
  if (!h->batch) return pbf_get_metrics(h, out);
  const SceneDesc& sd = h->scenes[scene];
  return metrics_range(h, sd.first, sd.n, sd.field, h->sdf.p ? h->sdf.p + sd.field.node_off : nullptr, out);
}

// ---- neighbour search alone -------------------------------------------------------
}  // extern "C"

struct pbf_ns {
  GridParams g;
  uint32_t max_n;
  cudaStream_t stream;
  bool own_stream;
  std::string err;
  DBuf<uint32_t> key, rank, cell_count, cell_start, perm_raw, id_raw, perm, tmp_a, tmp_b, big_list, big_count, err_word;
  DBuf<uint32_t> nbr_count;
  void* scan_scratch = nullptr;
  void* radix_scratch = nullptr;  // histograms and look-back words of the radix passes
  // pbf_ns_set_timing: events at the phase boundaries of pbf_ns_run
  bool timing = false, timed = false;
  cudaEvent_t ev[5] = {};
};

namespace {
int nsfail(pbf_ns* s, int code, const char* msg) {
  if (s) s->err = msg;
  return code;
}
#define NSCU(s, call)                                                    \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) return nsfail((s), PBF_ECUDA, cudaGetErrorString(e_)); \
  } while (0)

// NeighborCount / NeighborList over positions in id order: reuse the fast
// pass kernels with the stand-alone radius (distance test only, no float
// arithmetic beyond d.d, identical in both variants).
}  // namespace

extern "C" {

int pbf_ns_create(const pbf_grid* grid, uint32_t max_particles, void* stream, pbf_ns** out) {
  if (!grid || !out || max_particles == 0) return PBF_EINVAL;
  *out = nullptr;
  uint64_t cells = 1;
  for (int a = 0; a < 3; ++a) {
    if (grid->dim[a] == 0 || !(grid->inv_cell[a] > 0.0f)) return PBF_EINVAL;
    cells *= grid->dim[a];
  }
  if (cells > 0xfffffffeull) return PBF_EINVAL;
  pbf_ns* s = new pbf_ns();
  for (int a = 0; a < 3; ++a) {
    s->g.origin[a] = grid->origin[a];
    s->g.inv_cell[a] = grid->inv_cell[a];
    s->g.dim[a] = (int)grid->dim[a];
  }
  s->g.cells = (uint32_t)cells;
  s->g.key_base = 0;
  s->g.reach = 1;
  s->g.reach_z = 1;
  s->max_n = max_particles;
  cudaError_t e = cudaSuccess;
  if (stream) {
    s->stream = (cudaStream_t)stream;
    s->own_stream = false;
  } else {
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    s->own_stream = true;
  }
  auto A = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  size_t n = max_particles;
  A(s->key.alloc(n));
  A(s->rank.alloc(n));
  A(s->perm_raw.alloc(n));
  A(s->id_raw.alloc(n));
  A(s->perm.alloc(n));
  A(s->tmp_a.alloc(n));
  A(s->tmp_b.alloc(n));
  A(s->cell_count.alloc(cells + 1));
  A(s->cell_start.alloc(cells + 1));
  A(s->big_list.alloc(cells));
  A(s->big_count.alloc(1));
  A(s->err_word.alloc(1));
  A(s->nbr_count.alloc(n + 1));
  size_t sb = scan_scratch_bytes(cells + 1), sb2 = scan_scratch_bytes(n + 1);
  A(cudaMalloc(&s->scan_scratch, sb > sb2 ? sb : sb2));
  A(cudaMalloc(&s->radix_scratch, radix_scratch_bytes(n)));
  if (e == cudaSuccess) {
    A(cudaMemsetAsync(s->err_word.p, 0, 4, s->stream));
    A(cudaStreamSynchronize(s->stream));
  }
  if (e != cudaSuccess) {
    pbf_ns_destroy(s);
    return PBF_ECUDA;
  }
  *out = s;
  return PBF_OK;
}

int pbf_ns_destroy(pbf_ns* s) {
  if (!s) return PBF_EINVAL;
  if (s->stream) cudaStreamSynchronize(s->stream);
  DBuf<uint32_t>* bufs[] = {&s->key,   &s->rank,  &s->cell_count, &s->cell_start, &s->perm_raw, &s->id_raw, &s->perm,
                            &s->tmp_a, &s->tmp_b, &s->big_list,   &s->big_count,  &s->err_word, &s->nbr_count};
  for (auto* b : bufs) b->release();
  if (s->scan_scratch) cudaFree(s->scan_scratch);
  if (s->radix_scratch) cudaFree(s->radix_scratch);
  for (cudaEvent_t& e : s->ev)
    if (e) cudaEventDestroy(e);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return PBF_OK;
}

const char* pbf_ns_last_error(const pbf_ns* s) { return s ? s->err.c_str() : "null"; }

int pbf_ns_run(pbf_ns* s, const float* d_pos4, uint32_t n, uint32_t* d_keys, uint32_t* d_cell_count,
               uint32_t* d_cell_offset, uint32_t* d_order, uint32_t* d_rank) {
  if (!s || (!d_pos4 && n)) return PBF_EINVAL;
  if (n > s->max_n) return nsfail(s, PBF_ECAPACITY, "too many particles for this search context");
  cudaStream_t st = s->stream;
  const GridParams g = s->g;
  const bool tm = s->timing;
  s->timed = false;
  if (tm) NSCU(s, cudaEventRecord(s->ev[0], st));
  NSCU(s, cudaMemsetAsync(s->cell_count.p, 0, ((size_t)g.cells + 1) * 4, st));
  // The points come in particle-id order, so a stable radix sort of the ids
  // by cell key is the counting sort with each cell in id order.  Keys go
  // straight to the caller's array when it wants them.
  uint32_t* key = d_keys ? d_keys : s->key.p;
  uint32_t* const tk[2] = {s->tmp_a.p, s->perm_raw.p};
  uint32_t* const tv[2] = {s->tmp_b.p, s->id_raw.p};
  NSCU(s, launch_radix_sort_idorder(g, (const float4*)d_pos4, n, key, s->rank.p, s->perm.p, tk, tv, s->radix_scratch,
                                    s->err_word.p, st, tm ? s->ev[1] : nullptr, s->cell_count.p));
  if (tm) NSCU(s, cudaEventRecord(s->ev[2], st));
  // offsets from the counts the last pass made (s->rank holds the sorted
  // keys); the order and offsets stay in the context for pbf_ns_lists
  NSCU(s, launch_cell_offsets(g.cells, s->cell_count.p, s->cell_start.p, s->scan_scratch, s->err_word.p, st));
  if (tm) NSCU(s, cudaEventRecord(s->ev[3], st));
  if (d_rank) NSCU(s, launch_rank_sorted(n, s->rank.p, s->perm.p, s->cell_start.p, d_rank, st));
  if (d_cell_count)
    NSCU(s, cudaMemcpyAsync(d_cell_count, s->cell_count.p, (size_t)g.cells * 4, cudaMemcpyDeviceToDevice, st));
  if (d_cell_offset)
    NSCU(s, cudaMemcpyAsync(d_cell_offset, s->cell_start.p, ((size_t)g.cells + 1) * 4, cudaMemcpyDeviceToDevice, st));
  if (d_order && n) NSCU(s, cudaMemcpyAsync(d_order, s->perm.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  if (tm) {
    NSCU(s, cudaEventRecord(s->ev[4], st));
    s->timed = true;
  }
  return PBF_OK;
}

int pbf_ns_set_timing(pbf_ns* s, int enable) {
  if (!s) return PBF_EINVAL;
  if (enable)
    for (cudaEvent_t& e : s->ev)
      if (!e) NSCU(s, cudaEventCreate(&e));
  s->timing = enable != 0;
  s->timed = false;
  return PBF_OK;
}

int pbf_ns_timings(pbf_ns* s, float ms[4]) {
  if (!s || !ms) return PBF_EINVAL;
  if (!s->timed) return nsfail(s, PBF_ESTATE, "no timed pbf_ns_run since timing was enabled");
  NSCU(s, cudaEventSynchronize(s->ev[4]));
  for (int i = 0; i < 4; ++i) NSCU(s, cudaEventElapsedTime(&ms[i], s->ev[i], s->ev[i + 1]));
  return PBF_OK;
}

int pbf_ns_lists(pbf_ns* s, const float* d_pos4, uint32_t n, float radius, uint32_t* d_nbr_offset,
                 uint32_t* d_nbr_list, uint32_t capacity, uint32_t* total) {
  if (!s || !d_nbr_offset || (!d_pos4 && n)) return PBF_EINVAL;
  if (n > s->max_n) return nsfail(s, PBF_ECAPACITY, "too many particles for this search context");
  cudaStream_t st = s->stream;
  // The pass kernels traverse particles in cell-sorted order; gather the
  // positions into that order (tmp buffers reinterpreted as float4 need 4x
  // room, so use a temporary allocation).
  float4* sorted = nullptr;
  uint32_t* sorted_list = nullptr;
  uint32_t* ids = nullptr;
  NSCU(s, cudaMallocAsync((void**)&sorted, ((size_t)n + 1) * sizeof(float4), st));
  NSCU(s, cudaMallocAsync((void**)&ids, ((size_t)n + 1) * 4, st));
  SimParams p{};
  p.h = radius;
  p.h2 = (float)((double)radius * (double)radius);
  p.n = n;
  PassTable tbl;
  exact::fill_pass_table(&tbl);
  NSCU(s, launch_gather_state(n, s->perm.p, (const float4*)d_pos4, (const float4*)d_pos4, nullptr, sorted, sorted,
                              ids, st));
  tbl.nbr_count<<<nblocks(n + 1, 256), 256, 0, st>>>(p, s->g, sorted, s->cell_start.p, s->nbr_count.p);
  NSCU(s, cudaGetLastError());
  // counts are in slot order; the reference's offsets are by particle id
  uint32_t* cnt_by_id = nullptr;
  NSCU(s, cudaMallocAsync((void**)&cnt_by_id, ((size_t)n + 1) * 4, st));
  NSCU(s, cudaMemsetAsync(cnt_by_id, 0, ((size_t)n + 1) * 4, st));
  NSCU(s, launch_scatter_by_id_u32(n, ids, s->nbr_count.p, cnt_by_id, st));
  NSCU(s, launch_exclusive_scan(cnt_by_id, d_nbr_offset, (size_t)n + 1, s->scan_scratch, s->err_word.p, st));
  // slot-order offsets for the list kernel
  uint32_t* slot_off = nullptr;
  NSCU(s, cudaMallocAsync((void**)&slot_off, ((size_t)n + 1) * 4, st));
  NSCU(s, launch_exclusive_scan(s->nbr_count.p, slot_off, (size_t)n + 1, s->scan_scratch, s->err_word.p, st));
  uint32_t tot = 0;
  NSCU(s, cudaMemcpyAsync(&tot, slot_off + n, 4, cudaMemcpyDeviceToHost, st));
  NSCU(s, cudaStreamSynchronize(st));
  if (total) *total = tot;
  int rc = PBF_OK;
  if (tot > capacity) {
    rc = nsfail(s, PBF_ECAPACITY, "neighbour lists exceed capacity");
  } else if (tot && d_nbr_list) {
    NSCU(s, cudaMallocAsync((void**)&sorted_list, (size_t)tot * 4, st));
    tbl.nbr_list<<<nblocks(n, 256), 256, 0, st>>>(p, s->g, sorted, s->cell_start.p, slot_off, sorted_list, tot,
                                                   s->err_word.p);
    NSCU(s, cudaGetLastError());
    // translate slot ids to particle ids, then move each particle's run to its id-order offset
    NSCU(s, launch_list_to_ids(tot, sorted_list, ids, sorted_list, st));
    // move each particle's run from its slot-order offset to its id-order offset
    NSCU(s, launch_copy_runs(n, slot_off, d_nbr_offset, ids, sorted_list, d_nbr_list, st));
    NSCU(s, cudaFreeAsync(sorted_list, st));
  }
  NSCU(s, cudaFreeAsync(slot_off, st));
  NSCU(s, cudaFreeAsync(cnt_by_id, st));
  NSCU(s, cudaFreeAsync(sorted, st));
  NSCU(s, cudaFreeAsync(ids, st));
  NSCU(s, cudaStreamSynchronize(st));
  return rc;
}

int pbf_ns_sync(pbf_ns* s) {
  if (!s) return PBF_EINVAL;
  NSCU(s, cudaStreamSynchronize(s->stream));
  uint32_t e = 0;
  NSCU(s, cudaMemcpy(&e, s->err_word.p, 4, cudaMemcpyDeviceToHost));
  if (e & PBF_DEVERR_SCAN_TIMEOUT) {
    cudaMemset(s->err_word.p, 0, 4);
    return nsfail(s, PBF_ETIMEOUT, "scan look-back wait gave up");
  }
  return PBF_OK;
}

int pbf_selftest_bounded_wait(void) {
  uint32_t* err = nullptr;
  if (cudaMalloc(&err, sizeof(uint32_t)) != cudaSuccess) return PBF_ECUDA;
  uint32_t e = 0;
  cudaError_t ce = cudaMemset(err, 0, sizeof(uint32_t));
  if (ce == cudaSuccess) ce = launch_scan_timeout_selftest(err, 0);
  if (ce == cudaSuccess) ce = cudaMemcpy(&e, err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (ce != cudaSuccess) return PBF_ECUDA;
  return (e & PBF_DEVERR_SCAN_TIMEOUT) ? PBF_ETIMEOUT : PBF_EINVAL;
}

int pbf_exclusive_scan_u32(const uint32_t* d_in, uint32_t* d_out, size_t n, void* stream) {
  if ((!d_in || !d_out) && n) return PBF_EINVAL;
  if (n == 0) return PBF_OK;
  cudaStream_t st = (cudaStream_t)stream;
  void* scratch = nullptr;
  uint32_t* err = nullptr;
  size_t bytes = scan_scratch_bytes(n);
  if (cudaMallocAsync(&scratch, bytes + 16, st) != cudaSuccess) return PBF_ECUDA;
  err = (uint32_t*)((char*)scratch + bytes);
  uint32_t e = 0;
  // every path after the allocation releases the scratch
  cudaError_t ce = cudaMemsetAsync(err, 0, 4, st);
  if (ce == cudaSuccess) ce = launch_exclusive_scan(d_in, d_out, n, scratch, err, st);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, st);
  const cudaError_t fe = cudaFreeAsync(scratch, st);
  if (ce == cudaSuccess) ce = fe;
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) return PBF_ECUDA;
  return e ? PBF_ETIMEOUT : PBF_OK;
}

}  // extern "C"
