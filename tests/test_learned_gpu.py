"""The learned lambda warm start: BF16 mma MLP kernels against an FP64 CPU
reference, training, the device-side fallback, and the gain over the method
without the network."""
import ctypes

import numpy as np
import pytest

from oracle import mlp_ref
from pbf_gb300 import PBF, scenes
from pbf_gb300 import _lib as L
from pbf_gb300 import mlp_fit_normalization, mlp_forward, mlp_gradient, mlp_init, mlp_params, mlp_train

pytestmark = pytest.mark.gpu


def random_model(seed, rows=1024):
    rng = np.random.default_rng(seed)
    m = mlp_init(seed)
    feat = rng.normal(size=(rows, 8)).astype(np.float32) * np.array([0.02, 1e-5, 30, 0.2, 0.01, 1.5, 0.3, 1],
                                                                     np.float32)
    feat += np.array([0.0, -2e-5, 35, 0.1, 0.0, 1.0, 0.1, 0.5], np.float32)
    target = (feat[:, 0] * -3e-4 + feat[:, 1] * 0.7).astype(np.float32)
    mlp_fit_normalization(m, feat, target)
    # non-trivial biases
    p = np.ctypeslib.as_array(m.params)
    p[mlp_ref.OFF_B1:mlp_ref.OFF_W2] = rng.normal(size=64).astype(np.float32) * 0.1
    p[mlp_ref.OFF_B2:mlp_ref.OFF_W3] = rng.normal(size=64).astype(np.float32) * 0.1
    p[mlp_ref.OFF_B3] = 0.05
    return m, feat, target


def norm_of(m):
    return (np.ctypeslib.as_array(m.feat_mean).copy(), np.ctypeslib.as_array(m.feat_inv_std).copy(),
            float(m.lam_scale))


def test_mlp_forward_matches_fp64_reference():
    m, feat, _ = random_model(1, rows=1000)  # not a multiple of 16: ragged last tile
    got = mlp_forward(m, feat)
    mean, istd, scale = norm_of(m)
    ref = mlp_ref.forward(mlp_params(m), mean, istd, scale, feat, emulate=True)["lam"]
    exact = mlp_ref.forward(mlp_params(m), mean, istd, scale, feat, emulate=False)["lam"]
    scl = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 2e-3 * scl          # same bf16 rounding points, FP32 accumulation
    assert np.abs(got - exact).max() <= 3e-2 * scl        # against full FP64 (bf16 quantisation)


@pytest.mark.parametrize("rows", [1, 127, 128, 129, 5000])
def test_mlp_forward_tcgen05_matches_mma_sync_and_fp64(rows):
    """The tensor-core (tcgen05.mma, TMEM) inference kernel against the
    mma.sync kernel and the FP64 reference with the same bf16 rounding
    points; ragged last tiles included."""
    m, feat, _ = random_model(11, rows=max(rows, 2))
    feat = feat[:rows]
    tc = mlp_forward(m, feat, kernel=L.MLP_KERNEL_TCGEN05)
    ms = mlp_forward(m, feat, kernel=L.MLP_KERNEL_MMA_SYNC)
    mean, istd, scale = norm_of(m)
    ref = mlp_ref.forward(mlp_params(m), mean, istd, scale, feat, emulate=True)["lam"]
    scl = max(np.abs(ref).max(), 1e-30)
    assert np.abs(tc - ref).max() <= 2e-3 * scl
    assert np.abs(tc - ms).max() <= 2e-3 * scl


def test_mlp_forward_tcgen05_many_tiles():
    """300,001 rows (2,344 tiles over 152 x 8 pipelines, so every pipeline
    walks several tiles, and a ragged last tile): each row's result depends
    on its own features only, so the rows of a slice evaluated in a separate
    launch (other tiles, other lanes) are bit-identical to the full run's.
    Against the FP64 reference with the same bf16 rounding points: 99.99 % of
    the rows within 2e-3 of scale and the maximum within 1e-2 (over this many
    rows, a few land where the FP32 accumulation and FP64 round one
    activation to different bf16 neighbours)."""
    rows = 300001
    m, feat, _ = random_model(11, rows=rows)
    tc = mlp_forward(m, feat, kernel=L.MLP_KERNEL_TCGEN05)
    for lo, hi in ((0, 5000), (250000, 255000), (299000, rows)):
        part = mlp_forward(m, np.ascontiguousarray(feat[lo:hi]), kernel=L.MLP_KERNEL_TCGEN05)
        assert np.array_equal(part, tc[lo:hi]), (lo, hi)
    mean, istd, scale = norm_of(m)
    ref = mlp_ref.forward(mlp_params(m), mean, istd, scale, feat, emulate=True)["lam"]
    scl = max(np.abs(ref).max(), 1e-30)
    err = np.abs(tc - ref) / scl
    assert np.quantile(err, 0.9999) <= 2e-3
    assert err.max() <= 1e-2


def test_learned_step_tcgen05_network_matches_mma_sync():
    """The learned substep with the tcgen05 network pass stays within bf16
    rounding of the mma.sync pass after a few substeps."""
    sc = scenes.reference_scene("boundary_small")
    pts = scenes.jitter(sc.particles, 0.001, seed=14)
    f = sc.field
    m, _, _ = random_model(15)
    out = []
    for kernel in (L.MLP_KERNEL_MMA_SYNC, L.MLP_KERNEL_TCGEN05):
        s = PBF(sc.config)
        s.set_particles(pts)
        s.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
        s.set_mlp_kernel(kernel)
        s.set_learned(m, iterations=1, fallback_bound=1e9)
        s.step(3)
        out.append(s.positions()[:, :3])
        s.close()
    span = np.abs(out[0]).max()
    assert np.abs(out[0] - out[1]).max() <= 1e-4 * span


@pytest.mark.parametrize("kernel", [L.MLP_TRAIN_TCGEN05, L.MLP_TRAIN_MMA_SYNC])
@pytest.mark.parametrize("rows", [777, 20000])
def test_mlp_gradient_matches_fp64_reference(kernel, rows):
    """Both gradient kernels (tcgen05 with TMEM accumulators across a CTA's
    tiles, and mma.sync) against the FP64 reference with the same bf16
    rounding points; 20,000 rows make each tcgen05 CTA accumulate several
    128-row tiles."""
    m, feat, target = random_model(2, rows=rows)
    g, loss = mlp_gradient(m, feat, target, kernel=kernel)
    mean, istd, scale = norm_of(m)
    ge, le = mlp_ref.gradient(mlp_params(m), mean, istd, scale, feat, target, emulate=True)
    gx, _ = mlp_ref.gradient(mlp_params(m), mean, istd, scale, feat, target, emulate=False)
    assert abs(loss - le) <= 1e-3 * max(le, 1e-12)
    blocks = [(mlp_ref.OFF_W1, mlp_ref.OFF_B1), (mlp_ref.OFF_B1, mlp_ref.OFF_W2), (mlp_ref.OFF_W2, mlp_ref.OFF_B2),
              (mlp_ref.OFF_B2, mlp_ref.OFF_W3), (mlp_ref.OFF_W3, mlp_ref.OFF_B3), (mlp_ref.OFF_B3, 4801)]
    for a, b in blocks:
        ref = ge[a:b]
        err = np.linalg.norm(g[a:b] - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= 2e-2, (a, b, err)
        cos = float(np.dot(g[a:b], gx[a:b]) / max(np.linalg.norm(g[a:b]) * np.linalg.norm(gx[a:b]), 1e-30))
        assert cos >= 0.99, (a, b, cos)


@pytest.mark.parametrize("kernel", [L.MLP_TRAIN_TCGEN05, L.MLP_TRAIN_MMA_SYNC])
def test_training_reduces_loss(kernel):
    rng = np.random.default_rng(3)
    feat = rng.normal(size=(50000, 8)).astype(np.float32)
    target = (np.tanh(feat[:, 0]) - 0.5 * feat[:, 1] * feat[:, 2] + 0.1 * feat[:, 3]).astype(np.float32) * 1e-5
    m = mlp_init(3)
    mlp_fit_normalization(m, feat, target)
    _, l0 = mlp_gradient(m, feat, target, kernel=kernel)
    loss = mlp_train(m, feat, target, epochs=30, batch=2048, lr=3e-3, seed=3, kernel=kernel)
    _, l1 = mlp_gradient(m, feat, target, kernel=kernel)
    assert l1 < 0.05 * l0 and loss < 0.05 * l0, (l0, l1, loss)


def test_gradient_kernels_agree():
    """The tcgen05 and mma.sync gradient kernels on the same rows: every
    parameter block within 2 % (relative L2) of each other, equal losses
    within 1e-3."""
    m, feat, target = random_model(5, rows=5000)
    g_tc, l_tc = mlp_gradient(m, feat, target, kernel=L.MLP_TRAIN_TCGEN05)
    g_ms, l_ms = mlp_gradient(m, feat, target, kernel=L.MLP_TRAIN_MMA_SYNC)
    assert abs(l_tc - l_ms) <= 1e-3 * max(l_ms, 1e-12)
    blocks = [(mlp_ref.OFF_W1, mlp_ref.OFF_B1), (mlp_ref.OFF_B1, mlp_ref.OFF_W2), (mlp_ref.OFF_W2, mlp_ref.OFF_B2),
              (mlp_ref.OFF_B2, mlp_ref.OFF_W3), (mlp_ref.OFF_W3, mlp_ref.OFF_B3), (mlp_ref.OFF_B3, 4801)]
    for a, b in blocks:
        err = np.linalg.norm(g_tc[a:b] - g_ms[a:b]) / max(np.linalg.norm(g_ms[a:b]), 1e-30)
        assert err <= 2e-2, (a, b, err)


def test_trace_target_is_sum_of_iteration_multipliers():
    sc = scenes.reference_scene("cube_small", options=dict(iterations=1))
    sim = PBF(sc.config)
    sim.set_particles(scenes.jitter(sc.particles, 0.001, seed=4))
    sim.set_trace(10 * sc.n, stride=1)
    sim.run()
    feat, tgt = sim.trace()
    lam = sim.copy_field(L.FIELD_LAMBDA)
    assert len(tgt) == sc.n
    assert np.array_equal(np.sort(tgt), np.sort(lam))  # one iteration: target == its lambda
    nb = sim.copy_field(L.FIELD_NEIGHBOR_COUNT)
    assert np.array_equal(np.sort(feat[:, 2].astype(np.uint32)), np.sort(nb))
    sim.close()


def test_always_fallback_equals_plain_solve_bitexact():
    """With a negative bound every substep falls back to the plain solve from
    its predicted positions: the learned path then reproduces the plain path
    bit for bit (exact mode), including the network and feature passes that
    ran before the fallback."""
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=6)
    f = sc.field
    a, b = PBF(sc.config), PBF(sc.config)
    for s in (a, b):
        s.set_particles(pts)
        s.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
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


def _state(sim):
    return sim.positions(), sim.velocities()


def _run_mean_compression(cfg, field, state, frames, model=None, iters=None, learned_iters=2):
    c = scenes.copy_config(cfg)
    if iters is not None:
        c.options.iterations = iters
    sim = PBF(c)
    x, v = state
    sim.set_particles(x)
    sim.set_velocities(v)
    sim.set_boundary_field(field["res"], field["origin"], field["extent"], field["sdf"], field["vol"])
    if model is not None:
        sim.set_learned(model, iterations=learned_iters, fallback_bound=1e9)
    errs = []
    for _ in range(frames):
        sim.step(1)
        errs.append(sim.metrics()["mean_compression"])
    m = sim.metrics()
    sim.close()
    return float(np.mean(errs)), m


def test_learned_start_gain_over_plain_two_iterations():
    """Train on plain 4-iteration traces of a dam break, then compare from the
    same state: learned start + 2 iterations against plain 2 and plain 4."""
    cfg, pts, fa = scenes.dam_break_16k_spec()
    field = scenes.generate_field(fa["shapes"], (32, 32, 32), fa["origin"], fa["extent"], fa["h"], quadrature=8)
    sim = PBF(cfg)
    sim.set_particles(pts)
    sim.set_boundary_field(field["res"], field["origin"], field["extent"], field["sdf"], field["vol"])
    sim.step(40)  # the column collapses and hits the far wall
    sim.set_trace(400000, stride=2, salt=11)
    sim.step(40)
    feat, tgt = sim.trace()
    state = _state(sim)
    sim.close()
    assert len(tgt) > 100000
    m = mlp_init(5)
    mlp_fit_normalization(m, feat, tgt)
    loss = mlp_train(m, feat, tgt, epochs=20, batch=4096, lr=3e-3, seed=5)
    assert loss < 0.5  # normalised MSE well below the target variance (1.0)
    e2, _ = _run_mean_compression(cfg, field, state, 20, iters=2)
    e4, _ = _run_mean_compression(cfg, field, state, 20, iters=4)
    el, ml = _run_mean_compression(cfg, field, state, 20, model=m)
    print("mean compression: plain-2 %.5f  plain-4 %.5f  learned+2 %.5f" % (e2, e4, el))
    assert ml["nonfinite"] == 0
    assert e4 < e2
    assert el < e2  # the network's start beats the method without it at equal iterations


@pytest.mark.parametrize("bound", [-1.0, 1e9])
def test_learned_graph_replay_matches_eager(bound):
    """The learned substep (network pass, projection, iterations, the
    cooperative fallback kernel) replayed from a CUDA graph gives the eager
    results bit for bit, with the fallback taken every substep and never."""
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=12)
    f = sc.field
    m, _, _ = random_model(9)
    out = []
    for graph in (False, True):
        s = PBF(sc.config)
        s.set_particles(pts)
        s.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
        s.set_learned(m, iterations=1, fallback_bound=bound)
        s.enable_graph(graph)
        s.step(4)
        out.append((s.positions(), s.velocities(), s.metrics()["fallback_steps"]))
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] == (4 * sc.config.substeps if bound < 0 else 0)


def _learned_sim(sc, pts, model, iterations, bound, adaptive, graph=False, vel=None):
    f = sc.field
    s = PBF(sc.config)
    s.set_particles(pts)
    if vel is not None:
        s.set_velocities(vel)
    s.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
    s.set_learned(model, iterations=iterations, fallback_bound=bound)
    if adaptive:
        s.set_adaptive_iterations(True)
    s.enable_graph(graph)
    return s


def test_adaptive_iterations_skip_to_the_projection():
    """With a bound no error reaches, every adaptive test skips its position
    update: one substep ends exactly where the learned start with no plain
    iteration ends (exact mode), and the counters show the tests and no
    updates."""
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=14)
    m, _, _ = random_model(11)
    a = _learned_sim(sc, pts, m, 2, 1e9, adaptive=True)
    b = _learned_sim(sc, pts, m, 0, 1e9, adaptive=False)
    a.run()
    b.run()
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())
    assert a.adaptive_counts() == (2, 0)
    a.close()
    b.close()


def test_adaptive_iterations_run_while_needed():
    """With a bound below the error after the projection, the first update
    runs and the test is repeated per iteration; the results are the same
    eagerly and from a CUDA graph, and at the end the final error test of
    each substep either passes or falls back."""
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    settle = PBF(sc.config)  # a compressed state: the block after falling onto the floor
    f = sc.field
    settle.set_particles(scenes.jitter(sc.particles, 0.001, seed=15))
    settle.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
    settle.step(60)
    pts, vel = settle.positions(), settle.velocities()
    settle.close()
    m, _, _ = random_model(13)
    probe = _learned_sim(sc, pts, m, 0, 1e9, adaptive=False, vel=vel)
    probe.run()
    e0 = probe.metrics()["mean_compression"]  # the error after the projection alone
    probe.close()
    assert e0 > 0.0
    bound = 0.5 * e0
    out = []
    for graph in (False, True):
        s = _learned_sim(sc, pts, m, 2, bound, adaptive=True, graph=graph, vel=vel)
        s.step(3)
        tests, runs = s.adaptive_counts()
        out.append((s.positions(), s.velocities(), tests, runs, s.metrics()["fallback_steps"]))
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2:] == out[1][2:]
    tests, runs = out[0][2], out[0][3]
    assert tests == 2 * 3 * sc.config.substeps and 1 <= runs <= tests


def test_lagged_iterations_never_and_always():
    """Lagged iteration control: with a threshold no error reaches, every
    substep keeps the projection alone (bit for bit the learned start with no
    iteration, over several substeps); with a tiny threshold every substep
    after the first iterates, identically eager and from a CUDA graph."""
    sc = scenes.reference_scene("boundary_small", fp_mode=L.FP_EXACT)
    pts = scenes.jitter(sc.particles, 0.001, seed=16)
    m, _, _ = random_model(17)
    a = _learned_sim(sc, pts, m, 1, 1e9, adaptive=False)
    a.set_lagged_iterations(1.0)  # threshold 1e9: never iterates
    b = _learned_sim(sc, pts, m, 0, 1e9, adaptive=False)
    for _ in range(4):
        a.run()
        b.run()
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())
    assert a.adaptive_counts() == (4, 0)
    a.close()
    b.close()
    settle = PBF(sc.config)  # a compressed state: the block after falling onto the floor
    f = sc.field
    settle.set_particles(pts)
    settle.set_boundary_field(f["res"], f["origin"], f["extent"], f["sdf"], f["vol"])
    settle.step(60)
    x, v = settle.positions(), settle.velocities()
    settle.close()
    out = []
    for graph in (False, True):
        s = _learned_sim(sc, x, m, 1, 1e9, adaptive=False, graph=graph, vel=v)
        s.set_lagged_iterations(1e-15)  # threshold 1e-15 x 1e9 = 1e-6: iterates once any compression was seen
        s.step(3)
        out.append((s.positions(), s.velocities(), s.adaptive_counts()))
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    n_sub = 3 * sc.config.substeps
    # the first substep has no previous error (it keeps the projection); the others iterate
    assert out[0][2] == out[1][2] == (n_sub, n_sub - 1)
