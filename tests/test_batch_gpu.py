"""Batched scenes, launch shapes and the autotuner on the GPU.

Bars:
  - a batch in PBF_FP_EXACT mode is bit-identical, scene by scene, to each
    scene run alone on the same grid (positions, velocities, neighbour
    counts), including scenes with fewer iterations and without a map;
  - the launch shape (threads per CTA, persistent CTAs per SM, CUDA graph)
    does not change a bit of the results;
  - cell ratio 0.5 finds the same neighbour sets and results within float
    rounding of the reference grid's;
  - the autotuner leaves the state as it found it.
"""
import numpy as np
import pytest

from pbf_gb300 import PBF, PBFBatch, scenes
from pbf_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def small_batch(count=4, seed=7, n_min=700, n_max=3000, res=(16, 16, 16)):
    cfg, sc, fa = scenes.batch_scenes_spec(count=count, n_min=n_min, n_max=n_max, seed=seed, field_res=res)
    cfg.fp_mode = L.FP_EXACT
    cfg, sc = scenes.build_batch((cfg, sc, fa), quadrature=4)
    return cfg, sc


def alone(cfg, sc, info):
    c = scenes.copy_config(cfg)
    c.max_particles = sc["positions"].shape[0]
    c.domain_min[:] = list(sc["domain_min"])
    c.domain_max[:] = list(sc["domain_max"])
    c.grid_dim[:] = list(info["grid_dim"])
    c.options.iterations = info["iterations"]
    sim = PBF(c)
    sim.set_particles(sc["positions"])
    f = sc.get("field")
    if f is not None:
        sim.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
    return sim


def test_batch_matches_each_scene_alone_bitexact():
    cfg, sc = small_batch()
    sc[1] = dict(sc[1], iterations=2)            # mixed iteration counts
    sc[2] = {k: v for k, v in sc[2].items() if k != "field"}  # a scene without a map
    b = PBFBatch(cfg, sc)
    assert b.scene_count() == len(sc)
    b.step(3)
    x, v = b.positions(), b.velocities()
    cnt = b.copy_field(L.FIELD_NEIGHBOR_COUNT)
    for s in range(len(sc)):
        info = b.scene_info(s)
        assert info["iterations"] == (sc[s]["iterations"] or cfg.options.iterations)
        sim = alone(cfg, sc[s], info)
        sim.step(3)
        lo, hi = info["first_id"], info["first_id"] + info["particles"]
        assert np.array_equal(x[lo:hi], sim.positions()), s
        assert np.array_equal(v[lo:hi], sim.velocities()), s
        assert np.array_equal(cnt[lo:hi], sim.copy_field(L.FIELD_NEIGHBOR_COUNT)), s
        ms, m1 = b.scene_metrics(s), sim.metrics()
        assert ms["max_compression"] == m1["max_compression"] and ms["penetrations"] == m1["penetrations"]
        sim.close()
    m = b.metrics()
    assert m["particles"] == sum(s["positions"].shape[0] for s in sc)
    b.close()


def test_batch_rejects_single_scene_setup():
    cfg, sc = small_batch(count=2)
    b = PBFBatch(cfg, sc)
    with pytest.raises(L.PBFError) as e:
        b.set_particles(sc[0]["positions"])
    assert e.value.code == L.PBF_ESTATE
    b.close()


@pytest.mark.parametrize("shape", [(128, 0, 0), (256, 2, 1), (128, 16, 2), (256, 0, 2), (256, 8, 1)])
def test_launch_shape_does_not_change_results(shape):
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=9)
    f = sc.field

    def run(launch, graph):
        sim = PBF(sc.config)
        sim.set_particles(pts)
        sim.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
        if launch:
            sim.set_launch(block=launch[0], ctas_per_sm=launch[1], build=launch[2])
        sim.enable_graph(graph)
        sim.step(4)
        out = sim.positions(), sim.velocities()
        sim.close()
        return out

    ref = run(None, False)
    for graph in (False, True):
        got = run(shape, graph)
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])


def test_batch_graph_and_persistent_launch_bitexact():
    cfg, sc = small_batch(count=5, seed=11)
    a = PBFBatch(cfg, sc)
    a.step(2)
    b = PBFBatch(cfg, sc)
    b.set_launch(block=128, ctas_per_sm=2, build=2)
    b.enable_graph(True)
    b.step(2)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())
    a.close()
    b.close()


def test_cell_ratio_half_same_neighbours():
    sc = scenes.reference_scene("cube_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=4)
    out = {}
    for ratio in (1.0, 0.5):
        sim = PBF(sc.config)
        sim.set_particles(pts)
        sim.set_launch(cell_ratio=ratio)
        assert sim.launch()["cell_ratio"] == ratio
        sim.run()
        out[ratio] = (sim.copy_field(L.FIELD_NEIGHBOR_COUNT), sim.positions(), sim.velocities(),
                      sim.scene_info(0)["grid_dim"])
        sim.close()
    assert np.array_equal(out[1.0][0], out[0.5][0])     # same neighbour sets
    assert tuple(out[0.5][3]) != tuple(out[1.0][3])
    xs = np.abs(out[1.0][1][:, :3]).max()
    assert np.abs(out[1.0][1][:, :3] - out[0.5][1][:, :3]).max() <= 1e-6 * xs
    dens = out[1.0][1][:, 3]
    assert np.abs(dens - out[0.5][1][:, 3]).max() <= 1e-5 * np.abs(dens).max()


def test_autotune_restores_state_and_keeps_results():
    sc = scenes.reference_scene("cube_drop", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=2)
    a, b = PBF(sc.config), PBF(sc.config)
    for s in (a, b):
        s.set_particles(pts)
        s.step(2)
    before = b.positions().copy(), b.velocities().copy()
    best, trials = b.autotune(substeps=2)
    # 12 list-build shapes and 4 cell-block ones (a single scene)
    assert len(trials) == 16 and best["block"] in (128, 256) and best["cell_ratio"] == 1.0
    assert sorted(t["build"] for t in trials if t["build"] >= L.BUILD_CELLBLOCK_MASK) == [3, 3, 4, 4]
    assert all(t["ms_per_substep"] > 0 for t in trials)
    assert b.launch() == best
    assert np.array_equal(b.positions(), before[0]) and np.array_equal(b.velocities(), before[1])
    a.step(2)
    b.step(2)
    assert np.array_equal(a.positions(), b.positions())
    a.close()
    b.close()


def test_batch_of_sixteen_scenes_runs_stably():
    cfg, sc, fa = scenes.batch_scenes_spec(count=16, n_min=4096, n_max=32768, seed=3, field_res=(32, 32, 32))
    cfg, sc = scenes.build_batch((cfg, sc, fa), quadrature=6)
    b = PBFBatch(cfg, sc)
    best, _ = b.autotune(substeps=2, cell_ratio=True)
    b.enable_graph(True)
    b.step(30)
    m = b.metrics()
    assert m["nonfinite"] == 0
    per = [b.scene_metrics(s) for s in range(16)]
    assert sum(p["particles"] for p in per) == m["particles"]
    assert max(p["max_compression"] for p in per) == m["max_compression"]
    assert m["penetrations"] <= 1e-3 * m["particles"]
    b.close()
