/* cube_drop.c - the reference controller's "Cube Drop" scene driven through
 * the C ABI from plain C (the calls a non-Python host makes; the TypeScript
 * host makes the same ones through the N-API addon):
 *   new PBF() + initResource         -> pbf_config_default + pbf_create
 *   voxelizeCube((0.15, 0.35, 0.15), (0.65, 0.85, 0.65))
 *                                     -> pbf_voxelize_cube
 *   setParticlePosition()             -> pbf_set_particle_position
 *   setConfig({iteration: 5, ...})    -> pbf_set_options
 *   run() x stepCount per frame       -> pbf_step
 *   the renderer's position buffer    -> pbf_copy_positions_async + pbf_synchronize
 * (src/controller.ts:202-208, 343-347, 375-376).  Prints one line and exits
 * 0 when the scene stepped without error and stayed finite. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "pbf_gb300.h"

static int check(pbf_handle* h, int rc, const char* what) {
  if (rc != PBF_OK) fprintf(stderr, "%s failed (%d): %s\n", what, rc, h ? pbf_last_error(h) : "");
  return rc;
}

int main(int argc, char** argv) {
  const unsigned frames = argc > 1 ? (unsigned)atoi(argv[1]) : 60u;
  pbf_config cfg;
  pbf_handle* h = NULL;
  if (check(NULL, pbf_config_default(&cfg), "pbf_config_default")) return 1;
  if (check(NULL, pbf_create(&cfg, &h), "pbf_create")) return 1;
  const float mn[3] = {0.15f, 0.35f, 0.15f}, mx[3] = {0.65f, 0.85f, 0.65f};
  uint32_t added = 0;
  if (check(h, pbf_voxelize_cube(h, mn, mx, &added), "pbf_voxelize_cube")) return 1;
  if (check(h, pbf_set_particle_position(h), "pbf_set_particle_position")) return 1;
  pbf_options opt;
  if (check(h, pbf_get_options(h, &opt), "pbf_get_options")) return 1;
  opt.iterations = 5; /* the reference's GUI defaults (src/common/config.ts:22-28) */
  opt.xsph = 0.01f;
  opt.vorticity = 0.1f;
  opt.surface_tension = 0.5f;
  opt.gravity = 9.8f;
  if (check(h, pbf_set_options(h, &opt), "pbf_set_options")) return 1;
  const uint32_t n = pbf_particle_count(h);
  float* pos = (float*)malloc((size_t)n * 4 * sizeof(float));
  if (!pos) return 1;
  for (unsigned f = 0; f < frames; ++f) {
    if (check(h, pbf_step(h, 1), "pbf_step")) return 1;
    if (check(h, pbf_copy_positions_async(h, pos, (size_t)n * 4 * sizeof(float)), "pbf_copy_positions_async"))
      return 1;
  }
  if (check(h, pbf_synchronize(h), "pbf_synchronize")) return 1;
  double ymin = 1e30, ymax = -1e30;
  unsigned bad = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const float y = pos[4 * (size_t)i + 1];
    if (!isfinite(y) || !isfinite(pos[4 * (size_t)i]) || !isfinite(pos[4 * (size_t)i + 2])) ++bad;
    if (y < ymin) ymin = y;
    if (y > ymax) ymax = y;
  }
  pbf_metrics m;
  if (check(h, pbf_get_metrics(h, &m), "pbf_get_metrics")) return 1;
  printf("cube_drop: %u particles (%u seeded), %u frames, y in [%.4f, %.4f], nonfinite %u, "
         "max compression %.4f, device errors 0x%x\n",
         n, added, frames, ymin, ymax, bad, (double)m.max_compression, m.error_flags);
  free(pos);
  pbf_destroy(h);
  return (bad == 0 && m.nonfinite == 0 && m.error_flags == 0 && added == 41u * 41u * 41u) ? 0 : 2;
}
