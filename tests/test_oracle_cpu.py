"""CPU checks of the oracle (the CPU restatement of the reference step).

The reference ships no golden vectors; these pin the restatement against
the reference's own CPU self-checks and assets:
  - exact exclusive scan              (ExclusiveScan.debug, exclusiveScan.ts:193-199)
  - brute-force neighbour sets, <= h  (NeighborSearch.debug, neighborSearch.ts:337-372)
  - brute-force density               (PBF.computeParticleDensity, PBF.ts:96-116)
  - the .cdm node layout              (domain_boundary.cdm SDF = distance to the unit-cube walls)
plus committed regression vectors of the restatement itself.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from pbf_gb300 import _lib as L
from pbf_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_scan_matches_sequential_sum():
    rng = np.random.default_rng(1)
    for n in (0, 1, 511, 512, 513, 262144, 262145, 1000003):
        x = rng.integers(0, 50, size=n, dtype=np.uint32)
        ref = np.concatenate([[0], np.cumsum(x, dtype=np.uint64)[:-1]]).astype(np.uint32) if n else x
        assert np.array_equal(O.exclusive_scan(x), ref)


@pytest.mark.parametrize("dist", ["uniform", "clumps"])
def test_neighbor_search_invariants(dist):
    cfg, pts = scenes.neighbor_case(20000, dist, seed=3, dim=32)
    ns = O.neighbor_search(cfg, pts)
    keys, cc, co, order, rank = ns["keys"], ns["cell_count"], ns["cell_offset"], ns["order"], ns["rank"]
    c = np.floor(pts[:, :3].astype(np.float32) * np.float32(32)).astype(np.int64).clip(0, 31)
    assert np.array_equal(keys, (c[:, 0] * 32 * 32 + c[:, 1] * 32 + c[:, 2]).astype(np.uint32))
    assert np.array_equal(cc, np.bincount(keys, minlength=32 ** 3).astype(np.uint32))
    assert np.array_equal(co[:-1], O.exclusive_scan(cc)) and co[-1] == len(pts)
    # stable counting sort: order == argsort(keys, stable)
    assert np.array_equal(order, np.argsort(keys, kind="stable").astype(np.uint32))
    assert np.array_equal(rank, (np.arange(len(pts)) - co[keys[order]])[np.argsort(order)].astype(np.uint32))


def test_neighbor_sets_match_bruteforce():
    sc = scenes.reference_scene("cube_small")
    pts = scenes.jitter(sc.particles, 0.002, seed=5)
    ns = O.neighbor_search(sc.config, pts, lists=True)
    h2 = np.float32(sc.config.kernel_radius) * np.float32(sc.config.kernel_radius)
    rng = np.random.default_rng(0)
    for i in rng.choice(len(pts), 40, replace=False):
        d = pts[:, :3] - pts[i, :3]
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        truth = np.nonzero(d2 <= h2)[0]
        got = np.sort(ns["nbr_list"][ns["nbr_offset"][i]:ns["nbr_offset"][i + 1]])
        assert np.array_equal(got, truth)


def test_density_matches_bruteforce_helper():
    # FP64 replica's attribute-update density vs the reference's CPU helper,
    # on a scene that is static over one step (g = 0, no motion).
    sc = scenes.reference_scene("cube_small", options=dict(gravity=0.0, iterations=0))
    pts = scenes.jitter(sc.particles, 0.0015, seed=2)
    o = O.Oracle(sc.config, 64)
    o.set_particles(pts)
    o.substep(1)
    rho = o.field(L.FIELD_POSITION)[:, 3]
    V = 0.9 * (2.0 * np.float64(np.float32(0.006))) ** 3
    m = V * 1000.0
    x = o.field(L.FIELD_POSITION)[:, :3].astype(np.float32)
    x4 = np.concatenate([x, np.zeros((len(x), 1), np.float32)], axis=1)
    for i in (0, 100, 1000, len(pts) - 1):
        bf = O.bruteforce_density(x4, i, float(np.float32(0.025)), m)
        assert abs(rho[i] - bf) <= 1e-9 * bf


def test_cdm_layout_against_analytic_box_sdf():
    f = scenes.load_cdm_npz("domain_boundary")
    rng = np.random.default_rng(4)
    pts = rng.uniform(0.12, 0.88, size=(500, 3))
    out = O.interpolate(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"], pts)
    dist = np.minimum.reduce([pts[:, 0], 1 - pts[:, 0], pts[:, 1], 1 - pts[:, 1], pts[:, 2], 1 - pts[:, 2]])
    # away from the kinks the cubic element reproduces the piecewise-linear SDF
    second = np.sort(np.stack([pts[:, 0], 1 - pts[:, 0], pts[:, 1], 1 - pts[:, 1], pts[:, 2], 1 - pts[:, 2]]), axis=0)
    smooth = (second[1] - second[0]) > 0.06
    assert smooth.sum() > 100
    assert np.abs(out[smooth, 0] - dist[smooth]).max() < 2e-6
    # gradient = inward normal of the nearest wall
    g = out[smooth, 1:4]
    assert np.allclose(np.linalg.norm(g, axis=1), 1.0, atol=1e-4)


def test_cdm_fixture_sizes():
    for name in ("torus", "domain_boundary"):
        f = scenes.load_cdm_npz(name)
        n = 21 ** 3 + 3 * 40 * 21 ** 2
        assert f["sdf"].size == n == f["vol"].size == 62181


def test_volume_quirk_changes_only_volume():
    f = scenes.load_cdm_npz("torus")
    rng = np.random.default_rng(9)
    pts = rng.uniform(0.05, 0.95, size=(400, 3))
    a = O.interpolate(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"], pts, quirk=False)
    b = O.interpolate(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"], pts, quirk=True)
    assert np.array_equal(a[:, :4], b[:, :4])
    assert not np.array_equal(a[:, 4], b[:, 4])


def test_regression_vectors():
    d = np.load(os.path.join(GOLDEN, "oracle_ns_clumps4096.npz"))
    cfg, pts = scenes.neighbor_case(4096, "clumps", seed=7, dim=128)
    assert np.array_equal(pts, d["pts"])
    ns = O.neighbor_search(cfg, pts)
    for k in ("keys", "cell_count", "cell_offset", "order", "rank"):
        assert np.array_equal(ns[k], d[k]), k
    s = np.load(os.path.join(GOLDEN, "oracle_step_cube2197.npz"))
    sc = scenes.reference_scene("cube_small")
    o = O.Oracle(sc.config, 32)
    o.set_particles(sc.particles)
    o.substep(1)
    assert np.array_equal(o.field(0).astype(np.float32), s["position"])
    assert np.array_equal(o.field(2).astype(np.float32), s["acceleration"])
    assert np.array_equal(o.field(4).astype(np.float32), s["lam"])


def test_fp32_mirror_close_to_fp64_replica():
    """The FP32 mirror tracks the FP64 replica to float precision on the
    well-conditioned fields.  lambda, dp, omega and v are differences of
    nearly equal f32 numbers in the reference formulas (max(0, rho - 1),
    (x* - x)/dt, v_j - v_i), so their f32 error is bounded by the position
    quantisation instead: |dv| <= 8 ulp(|x|max)/dt."""
    sc = scenes.reference_scene("cube_small")
    pts = scenes.jitter(sc.particles, 0.002, seed=1)
    a = O.Oracle(sc.config, 32)
    b = O.Oracle(sc.config, 64)
    for o in (a, b):
        o.set_particles(pts)
        o.substep(1)
    pa, pb = a.field(L.FIELD_POSITION), b.field(L.FIELD_POSITION)
    assert np.abs(pa[:, 3] - pb[:, 3]).max() <= 1e-5 * np.abs(pb[:, 3]).max()      # rho
    assert np.abs(pa[:, :3] - pb[:, :3]).max() <= 4 * np.spacing(np.float32(1.0))   # x
    ulp = np.spacing(np.float32(np.abs(pb[:, :3]).max()))
    dv = np.abs(a.field(L.FIELD_VELOCITY) - b.field(L.FIELD_VELOCITY)).max()
    assert dv <= 8 * ulp / sc.config.time_step
    na, nb = a.field(L.FIELD_NORMAL), b.field(L.FIELD_NORMAL)
    assert np.abs(na - nb).max() <= 1e-4 * np.abs(nb).max()


def test_volume_generator_pinned_to_domain_asset():
    """The generator's definition reproduces the reference's domain_boundary.cdm:
    16-point Gauss-Legendre, 0.8 factor, cubic fall-off on the fluid side,
    the integrand read through the map's own cubic interpolation, points
    outside the map empty.  SDF to float precision, volumes to 0.2 % of the
    map's maximum (mean 1e-5)."""
    f = scenes.load_cdm_npz("domain_boundary")
    shapes = [(L.SHAPE_BOX_CONTAINER, (0.5, 0.5, 0.5), (0.5, 0.5, 0.5))]
    g = scenes.generate_field(shapes, (20, 20, 20), (0, 0, 0), (1, 1, 1), 0.025, quadrature=16,
                              flags=L.VOLMAP_OUTSIDE_EMPTY | L.VOLMAP_DISCRETE_SDF,
                              backend=O.generate_volume_map_backend())
    assert np.abs(g["sdf"] - f["sdf"]).max() < 1e-6
    vmax = f["vol"].max()
    assert np.abs(g["vol"] - f["vol"]).max() < 2e-3 * vmax
    assert np.abs(g["vol"] - f["vol"]).mean() < 1e-5 * vmax


def test_volume_from_sdf_pinned_to_torus_asset():
    """Volumes recomputed from the torus asset's own node SDF match its stored volumes."""
    f = scenes.load_cdm_npz("torus")
    v = O.volume_from_sdf(f["res"], (0, 0, 0), (1, 1, 1), 0.025, f["sdf"], quadrature=16,
                          flags=L.VOLMAP_OUTSIDE_EMPTY)
    vmax = f["vol"].max()
    err = np.abs(v - f["vol"])
    assert err.max() < 1e-2 * vmax, err.max() / vmax
    assert err.mean() < 1e-4 * vmax
