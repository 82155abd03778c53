"""Python mirror of the reference simulator interface over the C ABI.

The class `PBF` keeps the member names of the reference's TypeScript
classes so that host code and tests read alike:
  SPH        src/simulator/SPH.ts:7-208      (seeding, pause/start/stop, position buffer)
  PBFConfig  src/simulator/PBF/PBFConfig.ts  (setConfig, setParticlePosition)
  PBF        src/simulator/PBF/PBF.ts        (reset, setBoundaryData, run, runTimestamp, debug)
All work runs in libpbf_gb300.so on the GPU; this file only marshals arguments.
"""
import ctypes

import numpy as np

from . import _lib as L


def _f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


class PBF:
    """One simulator instance (one CUDA stream, device-resident state)."""

    MAX_NEIGHBOR_COUNT = 60       # SPH.ts:25
    KERNEL_RADIUS = 0.025         # SPH.ts:26
    TIME_STEP = 1.0 / 300.0       # SPH.ts:27
    MAX_PARTICLE_NUM = 1 << 17    # SPH.ts:24 (1 << 18 - 1 evaluates to 1 << 17)

    def __init__(self, config=None, **overrides):
        self._lib = L.load()
        cfg = config if config is not None else L.default_config()
        for k, v in overrides.items():
            if k in ("domain_min", "domain_max"):
                getattr(cfg, k)[:] = [float(x) for x in v]
            elif k == "grid_dim":
                cfg.grid_dim[:] = [int(x) for x in v]
            elif k == "options":
                for ok, ov in v.items():
                    setattr(cfg.options, ok, ov)
            else:
                setattr(cfg, k, v)
        cfg.struct_size = ctypes.sizeof(L.Config)
        self.config = cfg
        h = ctypes.c_void_p()
        rc = self._lib.pbf_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise L.PBFError(rc, "pbf_create failed")
        self._h = h

    # ---- life cycle -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.pbf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc:
            raise L.PBFError(rc, "%s: %s" % (what, self._lib.pbf_last_error(self._h).decode()))

    def initResource(self):
        """Buffers are allocated at construction (PBF.initResource, PBF.ts:262-279)."""
        return None

    def reset(self):
        self._check(self._lib.pbf_reset(self._h), "reset")

    # ---- config -----------------------------------------------------------
    def setConfig(self, conf):
        """PBFConfig.setConfig: {iteration, XSPH, vorticity, surfaceTension, gravity}."""
        o = L.Options()
        self._check(self._lib.pbf_get_options(self._h, ctypes.byref(o)), "get_options")
        if "iteration" in conf:
            o.iterations = int(conf["iteration"])
        if "XSPH" in conf:
            o.xsph = float(conf["XSPH"])
        if "vorticity" in conf:
            o.vorticity = float(conf["vorticity"])
        if "surfaceTension" in conf:
            o.surface_tension = float(conf["surfaceTension"])
        if "gravity" in conf:
            o.gravity = float(conf["gravity"])
        self._check(self._lib.pbf_set_options(self._h, ctypes.byref(o)), "setConfig")

    def optionsChange(self, e):
        self.setConfig(e["object"] if isinstance(e, dict) and "object" in e else e)

    # ---- seeding ------------------------------------------------------------
    def voxelizeCube(self, mn, mx):
        c = ctypes.c_uint32()
        self._check(self._lib.pbf_voxelize_cube(self._h, _f3(mn), _f3(mx), ctypes.byref(c)), "voxelizeCube")
        return c.value

    def voxelizeSphere(self, center, radius):
        c = ctypes.c_uint32()
        self._check(self._lib.pbf_voxelize_sphere(self._h, _f3(center), float(radius), ctypes.byref(c)),
                    "voxelizeSphere")
        return c.value

    def voxelizeMesh(self, vertices, triangles, world=None):
        """SPH.voxelizeMesh (SPH.ts:151-187) for a triangle mesh given as
        local-space vertices (V, 3), triangles (T, 3) and a 4x4 world matrix
        (row-major numpy array, float64 like three.js matrices; identity by
        default)."""
        v = np.ascontiguousarray(vertices, np.float32)
        t = np.ascontiguousarray(triangles, np.uint32)
        w = np.eye(4) if world is None else np.asarray(world, np.float64)
        wc = np.ascontiguousarray(w.T, np.float64)  # column-major, as three.js Matrix4.elements
        c = ctypes.c_uint32()
        self._check(self._lib.pbf_voxelize_mesh(self._h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), v.shape[0],
                                                t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), t.shape[0],
                                                wc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(c)),
                    "voxelizeMesh")
        return c.value

    def seed_device(self, items, jitter=0.0, seed=0):
        """Scene seeding on the GPU (pbf_seed_device): the same particles as
        reset + voxelizeCube / voxelizeSphere / voxelizeMesh over `items` in
        order + jitter(jitter, seed) + setParticlePosition, written straight
        into the device buffers.  items: ("cube", mn, mx), ("sphere", centre,
        radius) or ("mesh", vertices, triangles, world-or-None)."""
        arr = (L.SeedItem * max(len(items), 1))()
        keep = []
        for q, it in enumerate(items):
            d = arr[q]
            if it[0] == "cube":
                d.kind = L.SEED_CUBE
                d.a[:] = [float(x) for x in it[1]]
                d.b[:] = [float(x) for x in it[2]]
            elif it[0] == "sphere":
                d.kind = L.SEED_SPHERE
                d.a[:] = [float(x) for x in it[1]]
                d.b[:] = [float(it[2]), 0.0, 0.0]
            elif it[0] == "mesh":
                d.kind = L.SEED_MESH
                v = np.ascontiguousarray(it[1], np.float32)
                t = np.ascontiguousarray(it[2], np.uint32)
                w = np.eye(4) if len(it) < 4 or it[3] is None else np.asarray(it[3], np.float64)
                keep += [v, t]
                d.vertices = v.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
                d.vertex_count = v.shape[0]
                d.indices = t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
                d.triangle_count = t.shape[0]
                d.world[:] = [float(x) for x in w.T.ravel()]   # column-major
            else:
                raise ValueError("unknown seeding item %r" % (it[0],))
        total = ctypes.c_uint32()
        self._check(self._lib.pbf_seed_device(self._h, arr, len(items), float(jitter), int(seed), ctypes.byref(total)),
                    "seed_device")
        return total.value

    def jitter(self, amplitude, seed):
        self._check(self._lib.pbf_jitter_particles(self._h, float(amplitude), int(seed)), "jitter")

    def hostParticles(self):
        c = ctypes.c_uint32()
        self._check(self._lib.pbf_host_particle_count(self._h, ctypes.byref(c)), "host count")
        out = np.zeros((c.value, 4), dtype=np.float32)
        self._check(self._lib.pbf_copy_host_particles(
            self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), c.value), "host particles")
        return out

    def setParticlePosition(self):
        self._check(self._lib.pbf_set_particle_position(self._h), "setParticlePosition")

    def set_particles(self, xyzw):
        a = np.ascontiguousarray(xyzw, dtype=np.float32)
        if a.ndim != 2 or a.shape[1] != 4:
            raise ValueError("positions must be (n, 4) float32")
        self._check(self._lib.pbf_set_particles(
            self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.shape[0]), "set_particles")

    def set_velocities(self, xyzw):
        a = np.ascontiguousarray(xyzw, dtype=np.float32)
        self._check(self._lib.pbf_set_velocities(
            self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.shape[0]), "set_velocities")

    def set_accelerations(self, xyzw):
        a = np.ascontiguousarray(xyzw, dtype=np.float32)
        self._check(self._lib.pbf_set_accelerations(
            self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.shape[0]), "set_accelerations")

    def set_state(self, positions, velocities, accelerations):
        """Restores a saved state (by particle id): x, v and a."""
        self.set_particles(positions)
        self.set_velocities(velocities)
        self.set_accelerations(accelerations)

    def search_state(self, which, cells=None):
        """The last substep's neighbour search: 'keys' (per particle),
        'cell_count' / 'cell_offset' (per cell; `cells` = the grid's cell
        count) or 'order' (slot -> particle id)."""
        n = self.particleCount
        size = {"keys": n, "order": n, "cell_count": cells, "cell_offset": None if cells is None else cells + 1}[which]
        if size is None:
            raise ValueError("search_state(%r) needs the grid's cell count" % which)
        out = np.zeros(size, np.uint32)
        self._check(self._lib.pbf_copy_search_state(self._h, L.SEARCH_ARRAYS[which],
                                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), size),
                    "search_state")
        return out

    # ---- boundary -----------------------------------------------------------
    def setBoundaryData(self, text):
        b = text.encode() if isinstance(text, str) else bytes(text)
        self._check(self._lib.pbf_set_boundary_data(self._h, b, len(b)), "setBoundaryData")

    def set_boundary_field(self, res, origin, extent, sdf, vol):
        r = (ctypes.c_uint32 * 3)(*[int(x) for x in res])
        s = np.ascontiguousarray(sdf, dtype=np.float32)
        v = np.ascontiguousarray(vol, dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self._lib.pbf_set_boundary_field(self._h, r, _f3(origin), _f3(extent), s.ctypes.data_as(fp),
                                                      v.ctypes.data_as(fp), s.size), "set_boundary_field")

    def clear_boundary(self):
        self._check(self._lib.pbf_clear_boundary(self._h), "clear_boundary")

    # ---- stepping -----------------------------------------------------------
    def run(self):
        """One substep (PBF.run)."""
        self._check(self._lib.pbf_run(self._h), "run")

    def step(self, frames=1):
        """`frames` x stepCount substeps (the controller loop, controller.ts:375-376)."""
        self._check(self._lib.pbf_step(self._h, int(frames)), "step")

    def runTimestamp(self):
        ms = (ctypes.c_float * 4)()
        self._check(self._lib.pbf_run_timestamp(self._h, ms), "runTimestamp")
        return list(ms)

    def synchronize(self):
        self._check(self._lib.pbf_synchronize(self._h), "synchronize")

    def enable_graph(self, on=True):
        self._check(self._lib.pbf_enable_graph(self._h, 1 if on else 0), "enable_graph")

    def set_capture(self, on=True):
        self._check(self._lib.pbf_set_capture(self._h, 1 if on else 0), "set_capture")

    def set_kernel_timing(self, on=True):
        self._check(self._lib.pbf_set_kernel_timing(self._h, 1 if on else 0), "set_kernel_timing")

    def kernel_timing(self):
        """{pass name: (launches, total ms)} since the last call (synchronises)."""
        buf = (L.KernelTime * 32)()
        c = ctypes.c_uint32()
        self._check(self._lib.pbf_get_kernel_timing(self._h, buf, 32, ctypes.byref(c)), "kernel_timing")
        return {buf[i].name.decode(): (int(buf[i].launches), float(buf[i].total_ms)) for i in range(c.value)}

    # ---- learned start ------------------------------------------------------
    def set_trace(self, capacity, stride=1, salt=0):
        self._check(self._lib.pbf_set_trace(self._h, int(capacity), int(stride), int(salt)), "set_trace")

    def trace(self):
        """(features (rows, 8), targets (rows,)) captured so far."""
        c = ctypes.c_uint32()
        self._check(self._lib.pbf_trace_rows(self._h, ctypes.byref(c)), "trace_rows")
        f = np.zeros((c.value, 8), np.float32)
        t = np.zeros(c.value, np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self._lib.pbf_copy_trace(self._h, f.ctypes.data_as(fp), t.ctypes.data_as(fp), c.value),
                    "copy_trace")
        return f, t

    def trace_error(self):
        """(max, average) per-substep mean compression of the traced plain solve."""
        a, b = ctypes.c_float(), ctypes.c_float()
        self._check(self._lib.pbf_trace_error(self._h, ctypes.byref(a), ctypes.byref(b)), "trace_error")
        return a.value, b.value

    def set_mlp_kernel(self, kernel):
        """Inference kernel of the learned start's network pass (L.MLP_KERNEL_*)."""
        self._check(self._lib.pbf_set_mlp_kernel(self._h, int(kernel)), "set_mlp_kernel")

    def set_learned(self, model, iterations=2, fallback_bound=0.01):
        m = None if model is None else ctypes.byref(model)
        self._check(self._lib.pbf_set_learned(self._h, m, int(iterations), float(fallback_bound)), "set_learned")

    def set_adaptive_iterations(self, enable=True):
        """Run each learned-start iteration's position update only while the
        density error at its start exceeds the fallback bound."""
        self._check(self._lib.pbf_set_adaptive_iterations(self._h, 1 if enable else 0), "set_adaptive_iterations")

    def set_lagged_iterations(self, fraction):
        """Run a substep's iterations only when the previous substep's final
        mean compression exceeded fraction x the fallback bound (0: off)."""
        self._check(self._lib.pbf_set_lagged_iterations(self._h, float(fraction)), "set_lagged_iterations")

    def adaptive_counts(self):
        """(tests made, position updates run) since set_adaptive_iterations."""
        t, r = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self._lib.pbf_adaptive_counts(self._h, ctypes.byref(t), ctypes.byref(r)), "adaptive_counts")
        return t.value, r.value

    def update(self):
        return None

    # ---- pause (SPH.ts:82-84) ---------------------------------------------
    @property
    def pause(self):
        return self._lib.pbf_is_paused(self._h) == 1

    @pause.setter
    def pause(self, v):
        self._lib.pbf_set_paused(self._h, 1 if v else 0)

    def switch(self):
        self.pause = not self.pause

    def stop(self):
        self.pause = True

    def start(self):
        self.pause = False

    # ---- state --------------------------------------------------------------
    @property
    def particleCount(self):
        return int(self._lib.pbf_particle_count(self._h))

    @property
    def stepCount(self):
        return int(self.config.substeps)

    @property
    def position(self):
        """Device address of the float4 (x, rho) buffer, by particle id."""
        return int(self._lib.pbf_position_device(self._h) or 0)

    @property
    def stream(self):
        return int(self._lib.pbf_stream(self._h) or 0)

    def copy_field(self, field):
        n = self.particleCount
        if field in L.SCALAR_FIELDS:
            out = np.zeros(n, dtype=np.dtype(L.SCALAR_FIELDS[field]))
        else:
            out = np.zeros((n, 4), dtype=np.float32)
        self._check(self._lib.pbf_copy_field(self._h, int(field), out.ctypes.data_as(ctypes.c_void_p),
                                             out.nbytes), "copy_field")
        return out

    def positions(self):
        return self.copy_field(L.FIELD_POSITION)

    def velocities(self):
        return self.copy_field(L.FIELD_VELOCITY)

    def metrics(self):
        m = L.Metrics()
        self._check(self._lib.pbf_get_metrics(self._h, ctypes.byref(m)), "metrics")
        return {k: getattr(m, k) for k, _ in L.Metrics._fields_}

    def debug(self):
        """PBF.debug (PBF.ts:514-573) read back the acceleration buffer; here
        the same read-back plus the step metrics."""
        return {"acceleration": self.copy_field(L.FIELD_ACCELERATION), "metrics": self.metrics()}

    # ---- launch shape and autotuner (no reference counterpart) -------------
    def set_launch(self, block=256, ctas_per_sm=0, cell_ratio=1.0, build=0):
        lc = L.Launch(int(block), int(ctas_per_sm), float(cell_ratio), int(build))
        self._check(self._lib.pbf_set_launch(self._h, ctypes.byref(lc)), "set_launch")

    def set_cellblock_capacity(self, records):
        """Records per staged field of the cell-block passes' shared-memory plan."""
        self._check(self._lib.pbf_set_cellblock_capacity(self._h, int(records)), "set_cellblock_capacity")

    def launch(self):
        lc = L.Launch()
        self._check(self._lib.pbf_get_launch(self._h, ctypes.byref(lc)), "get_launch")
        return {"block": lc.block, "ctas_per_sm": lc.ctas_per_sm, "cell_ratio": lc.cell_ratio,
                "build": lc.build}

    def autotune(self, substeps=4, cell_ratio=False):
        """Times every candidate launch shape on the current state (restored
        afterwards) and keeps the fastest; returns (best, trials)."""
        trials = (L.TuneTrial * 64)()
        cnt = ctypes.c_uint32()
        best = L.Launch()
        flags = L.TUNE_CELL_RATIO if cell_ratio else 0
        self._check(self._lib.pbf_autotune(self._h, int(substeps), flags, trials, 64, ctypes.byref(cnt),
                                           ctypes.byref(best)), "autotune")
        as_dict = lambda lc: {"block": lc.block, "ctas_per_sm": lc.ctas_per_sm, "cell_ratio": lc.cell_ratio,
                              "build": lc.build}
        return as_dict(best), [dict(as_dict(t.launch), ms_per_substep=t.ms_per_substep)
                               for t in trials[:min(cnt.value, 64)]]

    # ---- scenes (a batch handle holds many; a single handle holds one) ---------
    def scene_count(self):
        return int(self._lib.pbf_scene_count(self._h))

    def scene_info(self, s):
        si = L.SceneInfo()
        self._check(self._lib.pbf_get_scene_info(self._h, int(s), ctypes.byref(si)), "scene_info")
        return {"first_id": si.first_id, "particles": si.particles, "iterations": si.iterations,
                "grid_dim": tuple(si.grid_dim), "cells": si.cells}

    def scene_metrics(self, s):
        m = L.Metrics()
        self._check(self._lib.pbf_get_scene_metrics(self._h, int(s), ctypes.byref(m)), "scene_metrics")
        return {k: getattr(m, k) for k, _ in L.Metrics._fields_}


class PBFBatch(PBF):
    """Many independent scenes stepped together, one launch per pass
    (pbf_batch_create).  `scenes` is a list of dicts with keys
    positions ((n, 3|4) float32), domain_min, domain_max, and optionally
    iterations and field (dict with res, origin, extent, sdf, vol)."""

    def __init__(self, config, scenes):
        self._lib = L.load()
        cfg = config
        cfg.struct_size = ctypes.sizeof(L.Config)
        self.config = cfg
        arr = (L.Scene * len(scenes))()
        self._keep = []
        for i, sc in enumerate(scenes):
            x = np.asarray(sc["positions"], dtype=np.float32)
            if x.shape[1] == 3:
                x = np.concatenate([x, np.zeros((x.shape[0], 1), np.float32)], axis=1)
            x = np.ascontiguousarray(x)
            self._keep.append(x)
            d = arr[i]
            d.struct_size = ctypes.sizeof(L.Scene)
            d.particles = x.shape[0]
            d.positions = x.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
            d.domain_min[:] = [float(v) for v in sc["domain_min"]]
            d.domain_max[:] = [float(v) for v in sc["domain_max"]]
            d.iterations = int(sc.get("iterations", 0))
            f = sc.get("field")
            if f is not None:
                sdf = np.ascontiguousarray(f["sdf"], dtype=np.float32)
                vol = np.ascontiguousarray(f["vol"], dtype=np.float32)
                self._keep += [sdf, vol]
                d.field_res[:] = [int(v) for v in f["res"]]
                d.field_origin[:] = [float(v) for v in f["origin"]]
                d.field_extent[:] = [float(v) for v in f["extent"]]
                d.sdf = sdf.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
                d.volume = vol.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        h = ctypes.c_void_p()
        rc = self._lib.pbf_batch_create(ctypes.byref(cfg), arr, len(scenes), ctypes.byref(h))
        self._keep = None
        if rc:
            raise L.PBFError(rc, "pbf_batch_create failed")
        self._h = h

    def scene_positions(self, s):
        info = self.scene_info(s)
        x = self.positions()
        return x[info["first_id"]:info["first_id"] + info["particles"]]


class NeighborSearch:
    """Stand-alone hash-grid search (NeighborSearch.execute, neighborSearch.ts:270-301)
    on device pointers; see pbf_ns_run in include/pbf_gb300.h."""

    def __init__(self, origin, inv_cell, dim, max_particles, stream=0):
        self._lib = L.load()
        g = L.Grid()
        g.origin[:] = [float(x) for x in origin]
        g.inv_cell[:] = [float(x) for x in inv_cell]
        g.dim[:] = [int(x) for x in dim]
        self.cells = int(dim[0]) * int(dim[1]) * int(dim[2])
        h = ctypes.c_void_p()
        rc = self._lib.pbf_ns_create(ctypes.byref(g), int(max_particles), ctypes.c_void_p(stream or None),
                                     ctypes.byref(h))
        if rc:
            raise L.PBFError(rc, "pbf_ns_create")
        self._h = h

    def _check(self, rc, what):
        if rc:
            raise L.PBFError(rc, "%s: %s" % (what, self._lib.pbf_ns_last_error(self._h).decode()))

    def run(self, d_pos4, n, d_keys=0, d_cell_count=0, d_cell_offset=0, d_order=0, d_rank=0):
        v = lambda p: ctypes.c_void_p(p or None)
        self._check(self._lib.pbf_ns_run(self._h, v(d_pos4), int(n), v(d_keys), v(d_cell_count),
                                         v(d_cell_offset), v(d_order), v(d_rank)), "pbf_ns_run")

    def lists(self, d_pos4, n, radius, d_offset, d_list, capacity):
        tot = ctypes.c_uint32()
        v = lambda p: ctypes.c_void_p(p or None)
        rc = self._lib.pbf_ns_lists(self._h, v(d_pos4), int(n), float(radius), v(d_offset), v(d_list),
                                    int(capacity), ctypes.byref(tot))
        return rc, tot.value

    def sync(self):
        self._check(self._lib.pbf_ns_sync(self._h), "pbf_ns_sync")

    def set_timing(self, enable=True):
        self._check(self._lib.pbf_ns_set_timing(self._h, 1 if enable else 0), "pbf_ns_set_timing")

    def timings(self):
        """The last timed run's phases in ms: [cell keys + counts, scan of the
        counts, counting-sort reorder, outputs]."""
        ms = (ctypes.c_float * 4)()
        self._check(self._lib.pbf_ns_timings(self._h, ms), "pbf_ns_timings")
        return [float(x) for x in ms]

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pbf_ns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def exclusive_scan(d_in, d_out, n, stream=0):
    lib = L.load()
    rc = lib.pbf_exclusive_scan_u32(ctypes.c_void_p(d_in), ctypes.c_void_p(d_out), int(n),
                                    ctypes.c_void_p(stream or None))
    if rc:
        raise L.PBFError(rc, "pbf_exclusive_scan_u32")


# ---- MLP helpers (the learned start's network) ------------------------------------------
def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def mlp_init(seed=0):
    m = L.MLP()
    L.load().pbf_mlp_init(ctypes.byref(m), int(seed))
    return m


def mlp_params(m):
    return np.ctypeslib.as_array(m.params).copy()


def mlp_fit_normalization(m, feat, target):
    f = np.ascontiguousarray(feat, np.float32)
    t = np.ascontiguousarray(target, np.float32)
    rc = L.load().pbf_mlp_fit_normalization(ctypes.byref(m), _fp(f), _fp(t), f.shape[0])
    if rc:
        raise L.PBFError(rc, "mlp_fit_normalization")


def mlp_forward(m, feat, kernel=L.MLP_KERNEL_MMA_SYNC):
    f = np.ascontiguousarray(feat, np.float32)
    out = np.zeros(f.shape[0], np.float32)
    rc = L.load().pbf_mlp_forward_ex(ctypes.byref(m), _fp(f), f.shape[0], _fp(out), int(kernel))
    if rc:
        raise L.PBFError(rc, "mlp_forward")
    return out


def mlp_gradient(m, feat, target, kernel=None):
    """Gradient and mean loss of the network on (feat, target); kernel:
    L.MLP_TRAIN_TCGEN05 (default) or L.MLP_TRAIN_MMA_SYNC."""
    f = np.ascontiguousarray(feat, np.float32)
    t = np.ascontiguousarray(target, np.float32)
    g = np.zeros(L.MLP_PARAMS, np.float32)
    loss = ctypes.c_float()
    k = L.MLP_TRAIN_TCGEN05 if kernel is None else int(kernel)
    rc = L.load().pbf_mlp_gradient_ex(ctypes.byref(m), _fp(f), _fp(t), f.shape[0], _fp(g), ctypes.byref(loss), k)
    if rc:
        raise L.PBFError(rc, "mlp_gradient")
    return g, loss.value


def mlp_train(m, feat, target, epochs=20, batch=8192, lr=2e-3, seed=0, kernel=None):
    f = np.ascontiguousarray(feat, np.float32)
    t = np.ascontiguousarray(target, np.float32)
    k = L.MLP_TRAIN_TCGEN05 if kernel is None else int(kernel)
    tc = L.TrainConfig(epochs=int(epochs), batch=int(batch), learning_rate=float(lr), kernel=k, seed=int(seed))
    loss = ctypes.c_float()
    rc = L.load().pbf_mlp_train(ctypes.byref(m), _fp(f), _fp(t), f.shape[0], ctypes.byref(tc), ctypes.byref(loss))
    if rc:
        raise L.PBFError(rc, "mlp_train")
    return loss.value


def voxelize_mesh_points(vertices, triangles, particle_radius, world=None):
    """Stand-alone mesh voxelisation on the GPU (pbf_voxelize_mesh_points):
    the kept lattice points as (n, 4) float32.  world: 4x4 row-major float64
    (identity by default)."""
    lib = L.load()
    v = np.ascontiguousarray(vertices, np.float32)
    t = np.ascontiguousarray(triangles, np.uint32)
    w = np.eye(4) if world is None else np.asarray(world, np.float64)
    wc = np.ascontiguousarray(w.T, np.float64)
    fp, up, dp = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_double)
    c = ctypes.c_uint32()
    rc = lib.pbf_voxelize_mesh_points(v.ctypes.data_as(fp), v.shape[0], t.ctypes.data_as(up), t.shape[0],
                                      wc.ctypes.data_as(dp), float(particle_radius), None, 0, ctypes.byref(c))
    if rc not in (L.PBF_OK, L.PBF_ECAPACITY):
        raise L.PBFError(rc, "voxelize_mesh_points")
    out = np.zeros((c.value, 4), np.float32)
    rc = lib.pbf_voxelize_mesh_points(v.ctypes.data_as(fp), v.shape[0], t.ctypes.data_as(up), t.shape[0],
                                      wc.ctypes.data_as(dp), float(particle_radius),
                                      out.ctypes.data_as(fp), c.value, ctypes.byref(c))
    if rc:
        raise L.PBFError(rc, "voxelize_mesh_points")
    return out
