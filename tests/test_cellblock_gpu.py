"""The cell-block neighbour passes (pbf_cellblock.cuh) against the CPU
restatement and against the list passes.

Bars:
  - exact mode: every field bit-identical to the FP32 restatement after 1 and
    4 substeps on the three reference scenes (one on the torus map), for the
    mask and the list-free variant, with the halo staged in shared memory
    and with every tile walking global memory (a capacity of 16 records
    stages no tile): the walk order is the reference's;
  - the cell-block search's neighbour counts equal the list build's;
  - fast mode: the cell-block passes evaluate the same sums as the list
    passes, in the same order: positions within 1e-6 of scale, neighbour
    counts equal;
  - the learned start's fallback on the cell-block search equals the plain
    cell-block solve bit for bit; graph replay equals eager;
  - no staging wait gives up (device error word clear).
"""
import numpy as np
import pytest

from oracle import oracle as O
from pbf_gb300 import PBF, scenes
from pbf_gb300 import _lib as L

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = [(L.FIELD_POSITION, "position"), (L.FIELD_VELOCITY, "velocity"), (L.FIELD_ACCELERATION, "acceleration"),
          (L.FIELD_LAMBDA, "lambda"), (L.FIELD_BOUNDARY, "boundary"), (L.FIELD_OMEGA, "omega"),
          (L.FIELD_NORMAL, "normal"), (L.FIELD_DELTA_P, "delta_p"), (L.FIELD_NEIGHBOR_COUNT, "nbr_count")]
SCENES = ["cube_small", "boundary_small", "water_droplet"]
BUILDS = [L.BUILD_CELLBLOCK_MASK, L.BUILD_CELLBLOCK_FREE]


def _sim(sc, fp_mode, pts, build, ratio=1.0, cap=None, block=128):
    cfg = scenes.copy_config(sc.config)
    cfg.fp_mode = fp_mode
    sim = PBF(cfg)
    sim.set_capture(True)
    sim.set_particles(pts)
    if sc.field is not None:
        f = sc.field
        sim.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
    sim.set_launch(block=block, ctas_per_sm=0, cell_ratio=ratio, build=build)
    if cap is not None:
        sim.set_cellblock_capacity(cap)
    return sim


def _fields(sim):
    return {name: sim.copy_field(f) for f, name in FIELDS}


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("substeps", [1, 4])
@pytest.mark.parametrize("build", BUILDS)
@pytest.mark.parametrize("cap", [None, 16])
def test_cellblock_exact_mode_bitexact(name, substeps, build, cap):
    sc = scenes.reference_scene(name)
    pts = scenes.jitter(sc.particles, 0.001, seed=substeps)
    sim = _sim(sc, L.FP_EXACT, pts, build, cap=cap)
    orc = O.Oracle(scenes.copy_config(sc.config), 32)
    orc.set_particles(pts)
    if sc.field is not None:
        f = sc.field
        orc.set_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
    for _ in range(substeps):
        sim.run()
    orc.substep(substeps)
    a = _fields(sim)
    assert sim.metrics()["error_flags"] == 0
    sim.close()
    for f, k in FIELDS:
        v = orc.field(f)
        b = v.astype(np.uint32) if f == L.FIELD_NEIGHBOR_COUNT else v.astype(np.float32)
        assert np.array_equal(a[k], b), (name, build, k, float(np.abs(a[k].astype(np.float64) - b).max()))
    orc.close()


@pytest.mark.parametrize("build", BUILDS)
@pytest.mark.parametrize("ratio", [1.0, 0.5])
def test_cellblock_fast_mode_matches_list_passes(build, ratio):
    sc = scenes.reference_scene("water_droplet")
    pts = scenes.jitter(sc.particles, 0.001, seed=21)
    ref = _sim(sc, L.FP_FAST, pts, L.BUILD_THREAD, ratio=ratio)
    sim = _sim(sc, L.FP_FAST, pts, build, ratio=ratio)
    for _ in range(3):
        ref.run()
        sim.run()
    a, b = _fields(ref), _fields(sim)
    ref.close()
    sim.close()
    assert np.array_equal(a["nbr_count"], b["nbr_count"])
    for k in ("position", "velocity", "lambda", "acceleration", "omega", "normal"):
        scale = max(float(np.abs(a[k]).max()), 1e-30)
        assert float(np.abs(a[k] - b[k]).max()) <= 1e-6 * scale, (k, float(np.abs(a[k] - b[k]).max()) / scale)


def test_cellblock_learned_fallback_equals_plain_solve_bitexact():
    from test_learned_gpu import random_model
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=6)
    for build in BUILDS:
        a = _sim(sc, L.FP_EXACT, pts, build)
        b = _sim(sc, L.FP_EXACT, pts, build)
        m, _, _ = random_model(7)
        b.set_learned(m, iterations=2, fallback_bound=-1.0)
        for _ in range(3):
            a.run()
            b.run()
        assert np.array_equal(a.positions(), b.positions())
        assert np.array_equal(a.velocities(), b.velocities())
        assert b.metrics()["fallback_steps"] == 3
        a.close()
        b.close()


@pytest.mark.parametrize("build", BUILDS)
def test_cellblock_graph_replay_matches_eager(build):
    sc = scenes.reference_scene("cube_small")
    cfg = scenes.copy_config(sc.config)
    cfg.substeps = 2
    out = []
    for graph in (False, True):
        s = PBF(cfg)
        s.set_particles(sc.particles)
        s.set_launch(block=128, ctas_per_sm=0, cell_ratio=0.5, build=build)
        s.enable_graph(graph)
        s.step(4)
        out.append((s.positions(), s.velocities()))
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_cellblock_rejected_for_batches_and_persistent_grids():
    sc = scenes.reference_scene("cube_small")
    s = PBF(sc.config)
    s.set_particles(sc.particles)
    with pytest.raises(L.PBFError) as e:
        s.set_launch(block=128, ctas_per_sm=2, cell_ratio=1.0, build=L.BUILD_CELLBLOCK_MASK)
    assert e.value.code == L.PBF_EINVAL
    with pytest.raises(L.PBFError):
        s.set_cellblock_capacity(17)
    s.close()
