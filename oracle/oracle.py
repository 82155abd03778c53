"""ctypes binding of the CPU restatement (oracle/_build/libpbf_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product library.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "webgpu-fluid-simulation_gb300"))
from pbf_gb300 import _lib as L  # noqa: E402  (structure layouts only)

LIB_PATH = os.path.join(HERE, "_build", "libpbf_oracle.so")
_lib = None
_P = ctypes.c_void_p
_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)
_UP = ctypes.POINTER(ctypes.c_uint32)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = ctypes.CDLL(LIB_PATH)
    sig = {
        "oracle_create": (_P, [ctypes.POINTER(L.Config), ctypes.c_int]),
        "oracle_destroy": (None, [_P]),
        "oracle_set_options": (None, [_P, ctypes.POINTER(L.Options)]),
        "oracle_set_particles": (None, [_P, _FP, ctypes.c_uint32]),
        "oracle_set_velocities": (None, [_P, _FP, ctypes.c_uint32]),
        "oracle_set_accelerations": (None, [_P, _FP, ctypes.c_uint32]),
        "oracle_search_state": (ctypes.c_long, [_P, ctypes.c_int, _UP, ctypes.c_size_t]),
        "oracle_set_field": (ctypes.c_int, [_P, _UP, _FP, _FP, _FP, _FP, ctypes.c_size_t]),
        "oracle_substep": (None, [_P, ctypes.c_uint32]),
        "oracle_get_field": (ctypes.c_int, [_P, ctypes.c_int, _DP]),
        "oracle_neighbor_search": (ctypes.c_int, [ctypes.POINTER(L.Config), _FP, ctypes.c_uint32, _UP, _UP, _UP,
                                                  _UP, _UP, _UP, _UP, ctypes.c_uint64,
                                                  ctypes.POINTER(ctypes.c_uint64)]),
        "oracle_grid_cells": (ctypes.c_int, [ctypes.POINTER(L.Config), _UP]),
        "oracle_exclusive_scan": (None, [_UP, _UP, ctypes.c_uint64]),
        "oracle_sample_field": (ctypes.c_int, [ctypes.POINTER(L.Config), _UP, _FP, _FP, _FP, _FP, ctypes.c_size_t,
                                               _FP, ctypes.c_uint32, ctypes.c_int, _DP]),
        "oracle_interpolate": (ctypes.c_int, [_UP, _FP, _FP, _FP, _FP, ctypes.c_size_t, _DP, ctypes.c_uint32,
                                              ctypes.c_int, _DP]),
        "oracle_bruteforce_density": (ctypes.c_double, [_FP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                                        ctypes.c_double]),
        "oracle_generate_volume_map": (ctypes.c_int, [ctypes.POINTER(L.Shape), ctypes.c_uint32, _UP, _FP, _FP,
                                                      ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32, _FP, _FP]),
        "oracle_volume_from_sdf": (ctypes.c_int, [_UP, _FP, _FP, ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32,
                                                  _FP, _FP]),
        "oracle_voxelize_mesh": (ctypes.c_int, [_FP, ctypes.c_uint32, _UP, ctypes.c_uint32, _DP, ctypes.c_double,
                                                _FP, ctypes.c_uint32, _UP]),
        "oracle_render": (ctypes.c_int, [_FP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _FP, _FP,
                                         ctypes.c_float, ctypes.c_uint32, _FP, _FP, _FP]),
        "oracle_splat_exp": (ctypes.c_float, [ctypes.c_float]),
        "oracle_narrow_range_filter": (ctypes.c_int, [_FP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                      ctypes.c_float]),
        "oracle_threads": (ctypes.c_int, []),
        "oracle_set_threads": (None, [ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _fp(a):
    return a.ctypes.data_as(_FP)


def _up(a):
    return a.ctypes.data_as(_UP)


def _dp(a):
    return a.ctypes.data_as(_DP)


class Oracle:
    """The reference substep on the CPU, in f32 (precision=32) or f64 (64)."""

    def __init__(self, config, precision=32):
        self._lib = load()
        self.config = config
        self._h = self._lib.oracle_create(ctypes.byref(config), precision)
        self.n = 0

    def close(self):
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_options(self, opts):
        self._lib.oracle_set_options(self._h, ctypes.byref(opts))

    def set_particles(self, xyzw):
        a = np.ascontiguousarray(xyzw, dtype=np.float32)
        self.n = a.shape[0]
        self._lib.oracle_set_particles(self._h, _fp(a), self.n)

    def set_velocities(self, xyzw):
        a = np.ascontiguousarray(xyzw, dtype=np.float32)
        self._lib.oracle_set_velocities(self._h, _fp(a), a.shape[0])

    def set_accelerations(self, xyzw):
        a = np.ascontiguousarray(xyzw, dtype=np.float32)
        self._lib.oracle_set_accelerations(self._h, _fp(a), a.shape[0])

    def set_state(self, positions, velocities, accelerations):
        """A saved simulation state (by particle id): x, v and a."""
        self.set_particles(positions)
        self.set_velocities(velocities)
        self.set_accelerations(accelerations)

    def search_state(self, which):
        """The last substep's neighbour search: 'keys' (per particle),
        'cell_count', 'cell_offset' or 'order'."""
        k = {"keys": 0, "cell_count": 1, "cell_offset": 2, "order": 3}[which]
        m = self._lib.oracle_search_state(self._h, k, None, 0)
        out = np.zeros(max(m, 0), np.uint32)
        self._lib.oracle_search_state(self._h, k, _up(out), out.size)
        return out

    def set_field(self, res, origin, extent, sdf, vol):
        r = np.asarray(res, dtype=np.uint32)
        o = np.asarray(origin, dtype=np.float32)
        e = np.asarray(extent, dtype=np.float32)
        s = np.ascontiguousarray(sdf, dtype=np.float32)
        v = np.ascontiguousarray(vol, dtype=np.float32)
        self._lib.oracle_set_field(self._h, _up(r), _fp(o), _fp(e), _fp(s), _fp(v), s.size)

    def substep(self, count=1):
        self._lib.oracle_substep(self._h, int(count))

    def field(self, field):
        if field in (L.FIELD_LAMBDA, L.FIELD_NEIGHBOR_COUNT):
            out = np.zeros(self.n, dtype=np.float64)
        else:
            out = np.zeros((self.n, 4), dtype=np.float64)
        rc = self._lib.oracle_get_field(self._h, int(field), _dp(out))
        if rc:
            raise ValueError("oracle field %d" % field)
        return out


def grid_dims(config):
    dims = np.zeros(3, dtype=np.uint32)
    cells = load().oracle_grid_cells(ctypes.byref(config), _up(dims))
    return dims, cells


def neighbor_search(config, xyzw, lists=False, capacity=None):
    """Reference neighbour search on f32 positions: returns a dict of arrays."""
    lib = load()
    a = np.ascontiguousarray(xyzw, dtype=np.float32)
    n = a.shape[0]
    dims, cells = grid_dims(config)
    keys = np.zeros(n, np.uint32)
    rank = np.zeros(n, np.uint32)
    cc = np.zeros(cells, np.uint32)
    co = np.zeros(cells + 1, np.uint32)
    order = np.zeros(n, np.uint32)
    out = dict(keys=keys, rank=rank, cell_count=cc, cell_offset=co, order=order, dims=dims)
    null = ctypes.POINTER(ctypes.c_uint32)()
    if lists:
        cap = capacity if capacity is not None else max(1, 80 * n)
        off = np.zeros(n + 1, np.uint32)
        lst = np.zeros(cap, np.uint32)
        tot = ctypes.c_uint64()
        rc = lib.oracle_neighbor_search(ctypes.byref(config), _fp(a), n, _up(keys), _up(cc), _up(co), _up(order),
                                        _up(rank), _up(off), _up(lst), cap, ctypes.byref(tot))
        if rc:
            raise ValueError("oracle neighbour lists exceed capacity")
        out.update(nbr_offset=off, nbr_list=lst[:tot.value].copy())
    else:
        lib.oracle_neighbor_search(ctypes.byref(config), _fp(a), n, _up(keys), _up(cc), _up(co), _up(order),
                                   _up(rank), null, null, 0, None)
    return out


def exclusive_scan(x):
    a = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros_like(a)
    load().oracle_exclusive_scan(_up(a), _up(out), a.size)
    return out


def interpolate(res, origin, extent, sdf, vol, pts, quirk=False):
    r = np.asarray(res, dtype=np.uint32)
    o = np.asarray(origin, dtype=np.float32)
    e = np.asarray(extent, dtype=np.float32)
    s = np.ascontiguousarray(sdf, dtype=np.float32)
    v = np.ascontiguousarray(vol, dtype=np.float32)
    p = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros((p.shape[0], 5), dtype=np.float64)
    load().oracle_interpolate(_up(r), _fp(o), _fp(e), _fp(s), _fp(v), s.size, _dp(p), p.shape[0], int(quirk),
                              _dp(out))
    return out


def sample_field(config, res, origin, extent, sdf, vol, pts4, precision=32):
    r = np.asarray(res, dtype=np.uint32)
    o = np.asarray(origin, dtype=np.float32)
    e = np.asarray(extent, dtype=np.float32)
    s = np.ascontiguousarray(sdf, dtype=np.float32)
    v = np.ascontiguousarray(vol, dtype=np.float32)
    p = np.ascontiguousarray(pts4, dtype=np.float32)
    out = np.zeros((p.shape[0], 4), dtype=np.float64)
    load().oracle_sample_field(ctypes.byref(config), _up(r), _fp(o), _fp(e), _fp(s), _fp(v), s.size, _fp(p),
                               p.shape[0], precision, _dp(out))
    return out


def bruteforce_density(xyzw, i, h, mass):
    a = np.ascontiguousarray(xyzw, dtype=np.float32)
    return load().oracle_bruteforce_density(_fp(a), a.shape[0], int(i), float(h), float(mass))


def set_threads(t):
    load().oracle_set_threads(int(t))


def threads():
    return load().oracle_threads()


def generate_volume_map_backend():
    """Callable with the argument list of pbf_generate_volume_map (CPU, FP64)."""
    return load().oracle_generate_volume_map


def volume_from_sdf(res, origin, extent, h, sdf, quadrature=16, flags=1):
    r = np.asarray(res, dtype=np.uint32)
    o = np.asarray(origin, dtype=np.float32)
    e = np.asarray(extent, dtype=np.float32)
    s = np.ascontiguousarray(sdf, dtype=np.float32)
    out = np.zeros_like(s)
    load().oracle_volume_from_sdf(_up(r), _fp(o), _fp(e), float(h), int(quadrature), int(flags), _fp(s), _fp(out))
    return out


def voxelize_mesh(vertices, triangles, particle_radius, world=None):
    """SPH.voxelizeMesh restated (brute force, double precision): the kept
    lattice points as (n, 4) float32 in lattice order.  world: 4x4 row-major
    float64 (identity by default)."""
    lib = load()
    v = np.ascontiguousarray(vertices, np.float32)
    t = np.ascontiguousarray(triangles, np.uint32)
    w = np.eye(4) if world is None else np.asarray(world, np.float64)
    wc = np.ascontiguousarray(w.T, np.float64)
    c = ctypes.c_uint32()
    rc = lib.oracle_voxelize_mesh(_fp(v), v.shape[0], _up(t), t.shape[0], _dp(wc), float(particle_radius), None, 0,
                                  ctypes.byref(c))
    if rc not in (0, 2):
        raise RuntimeError("oracle_voxelize_mesh failed (%d)" % rc)
    out = np.zeros((c.value, 4), np.float32)
    rc = lib.oracle_voxelize_mesh(_fp(v), v.shape[0], _up(t), t.shape[0], _dp(wc), float(particle_radius), _fp(out),
                                  c.value, ctypes.byref(c))
    if rc:
        raise RuntimeError("oracle_voxelize_mesh failed (%d)" % rc)
    return out


def render(positions, width, height, view, projection, radius, filter_size, scene_depth=None):
    """FilteredParticleFluid's rasterisation + narrow-range filter restated on
    the CPU: (depth map (H, W), volume map (H/2, W/2), updated scene depth or
    None).  view / projection: 4x4 row-major float32 arrays."""
    lib = load()
    p = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
    v = np.ascontiguousarray(np.asarray(view, np.float32).T)
    pr = np.ascontiguousarray(np.asarray(projection, np.float32).T)
    depth = np.zeros((height, width), np.float32)
    volume = np.zeros((height // 2, width // 2), np.float32)
    scene = None if scene_depth is None else np.ascontiguousarray(scene_depth, np.float32).copy()
    rc = lib.oracle_render(_fp(p), p.shape[0], width, height, _fp(v), _fp(pr), float(radius), int(filter_size),
                           None if scene is None else _fp(scene), _fp(depth), _fp(volume))
    if rc:
        raise RuntimeError("oracle_render failed (%d)" % rc)
    return depth, volume, scene


def splat_exp(x):
    return float(load().oracle_splat_exp(float(x)))


def narrow_range_filter(img, filter_size, radius):
    """TextureFilter.execute restated: the filtered copy of a float32 image."""
    out = np.ascontiguousarray(img, np.float32).copy()
    rc = load().oracle_narrow_range_filter(_fp(out), out.shape[1], out.shape[0], int(filter_size), float(radius))
    if rc:
        raise RuntimeError("oracle_narrow_range_filter failed (%d)" % rc)
    return out
