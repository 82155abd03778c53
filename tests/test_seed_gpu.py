"""Mesh voxelisation on the GPU (pbf_voxelize_mesh_points / PBF.voxelizeMesh,
the reference's SPH.voxelizeMesh, src/simulator/SPH.ts:151-187) against the
CPU restatement: the same kept lattice points, bit for bit, in the same order.
Both compute in double precision with the same operation order; the GPU tests
only the triangles binned to the ray's xy column, the restatement all of
them."""
import numpy as np
import pytest

from oracle import oracle as O
from pbf_gb300 import _lib as L
from pbf_gb300 import scenes
from pbf_gb300.simulator import PBF, voxelize_mesh_points

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("radius,world", [
    (0.02, None),
    (0.006, scenes.trs_matrix(translate=(0.5, 0.3, 0.5), scale=0.4)),   # the Bunny Drop placement
    (0.006, scenes.trs_matrix(translate=(0.45, 0.35, 0.5), rotate_deg=(15.0, -30.0, 60.0), scale=0.35)),
])
def test_torus_matches_oracle(radius, world):
    v, t = scenes.load_mesh_npz("torus")
    got = voxelize_mesh_points(v, t, radius, world)
    want = O.voxelize_mesh(v, t, radius, world)
    assert want.shape[0] > 1000
    _same(got, want)


def test_dense_sphere_matches_oracle():
    v, t = scenes.uv_sphere(0.5, (0.03, -0.02, 0.01), stacks=48, slices=96)   # 9,024 triangles
    W = scenes.trs_matrix(translate=(0.5, 0.5, 0.5), rotate_deg=(5.0, 10.0, 20.0), scale=0.6)
    got = voxelize_mesh_points(v, t, 0.006, W)
    want = O.voxelize_mesh(v, t, 0.006, W)
    assert want.shape[0] > 50000
    _same(got, want)


def test_open_and_inside_out_meshes_match_oracle():
    v, t = scenes.uv_sphere(0.4, stacks=20, slices=40)
    half = t[: len(t) // 2]                          # an open cap: rays that miss, rays that see one face
    _same(voxelize_mesh_points(v, half, 0.01), O.voxelize_mesh(v, half, 0.01))
    flipped = t[:, ::-1].copy()
    _same(voxelize_mesh_points(v, flipped, 0.01), O.voxelize_mesh(v, flipped, 0.01))


def test_pbf_voxelize_mesh_appends_to_host_particles():
    v, t = scenes.load_mesh_npz("torus")
    W = scenes.trs_matrix(translate=(0.5, 0.3, 0.5), scale=0.2)
    sim = PBF(scenes.base_config())
    try:
        n_cube = sim.voxelizeCube((0.1, 0.1, 0.1), (0.2, 0.2, 0.2))
        n_mesh = sim.voxelizeMesh(v, t, W)
        host = sim.hostParticles()
        assert host.shape[0] == n_cube + n_mesh and n_mesh > 1000
        r = float(sim.config.particle_radius)   # the float32 radius, widened
        _same(host[n_cube:], O.voxelize_mesh(v, t, r, W))
        sim.setParticlePosition()
        assert sim.particleCount == n_cube + n_mesh
        assert np.array_equal(sim.positions()[:, :3], host[:, :3])
    finally:
        sim.close()


def test_capacity_is_reported():
    import ctypes
    v, t = scenes.load_mesh_npz("torus")
    n = voxelize_mesh_points(v, t, 0.05).shape[0]
    lib = L.load()
    vv = np.ascontiguousarray(v, np.float32)
    tt = np.ascontiguousarray(t, np.uint32)
    W = np.ascontiguousarray(np.eye(4))
    out = np.zeros((n - 1, 4), np.float32)
    c = ctypes.c_uint32()
    rc = lib.pbf_voxelize_mesh_points(vv.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), vv.shape[0],
                                      tt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), tt.shape[0],
                                      W.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0.05,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n - 1, ctypes.byref(c))
    assert rc == L.PBF_ECAPACITY and c.value == n


def _host_seeded(cfg, items, jitter, seed):
    sim = PBF(cfg)
    for it in items:
        if it[0] == "cube":
            sim.voxelizeCube(it[1], it[2])
        elif it[0] == "sphere":
            sim.voxelizeSphere(it[1], it[2])
        else:
            sim.voxelizeMesh(it[1], it[2], it[3])
    if jitter > 0:
        sim.jitter(jitter, seed)
    sim.setParticlePosition()
    return sim


def _scene_items():
    v, t = scenes.load_mesh_npz("torus")
    return [("cube", (0.15, 0.35, 0.15), (0.65, 0.85, 0.65)),
            ("sphere", (0.5, 0.7, 0.5), 0.12),
            ("mesh", v, t, scenes.trs_matrix(translate=(0.5, 0.15, 0.5), rotate_deg=(0.0, 30.0, 0.0), scale=0.15)),
            ("cube", (0.3, 0.1, 0.3), (0.1, 0.2, 0.4))]          # empty: max below min on x


@pytest.mark.parametrize("jitter", [0.0, 0.0006])
def test_device_seeding_equals_host_seeding(jitter):
    items = _scene_items()
    host = _host_seeded(scenes.base_config(max_neighbors=96), items, jitter, 42)
    dev = PBF(scenes.base_config(max_neighbors=96))
    try:
        dev.voxelizeCube((0.1, 0.1, 0.1), (0.2, 0.2, 0.2))   # cleared by device seeding
        n = dev.seed_device(items, jitter, 42)
        assert n == host.particleCount > 41 ** 3
        assert dev.particleCount == n and dev.hostParticles().shape[0] == 0
        assert np.array_equal(dev.positions().view(np.uint32), host.positions().view(np.uint32))
        # identical state: one substep gives identical particles
        host.run()
        dev.run()
        assert np.array_equal(dev.positions().view(np.uint32), host.positions().view(np.uint32))
        assert np.array_equal(dev.velocities().view(np.uint32), host.velocities().view(np.uint32))
    finally:
        host.close()
        dev.close()


def test_device_seeding_capacity_keeps_current_particles():
    cfg = scenes.base_config()
    cfg.max_particles = 50000
    sim = PBF(cfg)
    try:
        n0 = sim.seed_device([("cube", (0.2, 0.2, 0.2), (0.5, 0.5, 0.5))])
        before = sim.positions()
        with pytest.raises(L.PBFError) as e:
            sim.seed_device(_scene_items())
        assert e.value.code == L.PBF_ECAPACITY
        assert sim.particleCount == n0
        assert np.array_equal(sim.positions(), before)
        assert sim.seed_device([]) == 0 and sim.particleCount == 0
    finally:
        sim.close()
