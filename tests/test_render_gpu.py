"""Screen-space fluid buffers on the GPU (pbf_renderer / pbf_texture_filter)
against the CPU restatement: the depth map, the volume map and the updated
depth buffer bit for bit.  The sprites, the 64-bit depth/index keys, the
fixed-point volume sum and the filter are deterministic, so equality is
exact whatever the thread order."""
import numpy as np
import pytest

from oracle import oracle as O
from pbf_gb300 import render as Rd
from pbf_gb300 import scenes
from pbf_gb300.simulator import PBF

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _particles(seed, n=60000):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 4), np.float32)
    k = n // 2
    p[:k, :3] = rng.uniform(0.0, 1.0, (k, 3)) * [0.5, 0.4, 0.5] + [0.1, 0.0, 0.1]   # a block of fluid
    p[k:, :3] = rng.uniform(-3.0, 3.0, (n - k, 3))                                   # spray, some behind the camera
    p[:, 3] = rng.uniform(900, 1100, n)                                              # density (ignored)
    return p


def _render_gpu(p, W, H, fs, R=0.02, scene=None, cam=None):
    r = Rd.FilteredParticleFluid(W, H)
    try:
        r.setConfig(filterSize=fs, particleRadius=R)
        r.set_camera(cam or Rd.reference_camera(W, H))
        dp = torch.from_numpy(p).cuda()
        ds = None if scene is None else torch.from_numpy(scene).cuda()
        r.render(dp.data_ptr(), p.shape[0], 0 if ds is None else ds.data_ptr())
        torch.cuda.synchronize()
        t = r.timings()
        assert t[0] > 0.0 and t[1] >= 0.0
        return r.depth(), r.volume(), None if ds is None else ds.cpu().numpy()
    finally:
        r.close()


def _same(a, b):
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("fs", [32, 16, 7, 0])
def test_render_matches_oracle(fs):
    W, H = 640, 360
    p = _particles(fs)
    cam = Rd.reference_camera(W, H)
    got = _render_gpu(p, W, H, fs, cam=cam)
    want = O.render(p, W, H, cam["view"], cam["projection"], 0.02, fs)
    assert np.count_nonzero(want[0]) > 10000
    _same(got[0], want[0])
    _same(got[1], want[1])


def test_render_with_depth_buffer_and_odd_size():
    W, H = 333, 211
    rng = np.random.default_rng(9)
    scene = rng.uniform(0.0, 0.08, (H, W)).astype(np.float32)     # scene geometry behind / in front of the fluid
    scene[:, : W // 4] = 1.0
    p = _particles(5, 20000)
    cam = Rd.reference_camera(W, H, eye=(1.5, 1.2, 1.4), target=(0.35, 0.2, 0.35))
    got = _render_gpu(p, W, H, 32, R=0.03, scene=scene, cam=cam)
    want = O.render(p, W, H, cam["view"], cam["projection"], 0.03, 32, scene)
    for a, b in zip(got, want):
        _same(a, b)
    assert not np.any(got[0][:, : W // 4 - 16])


def test_ties_and_duplicates():
    W, H = 256, 160
    p = _particles(11, 4000)
    p = np.concatenate([p, p, p[::-1]])                   # every position three times
    cam = Rd.reference_camera(W, H)
    got = _render_gpu(p, W, H, 32, cam=cam)
    want = O.render(p, W, H, cam["view"], cam["projection"], 0.02, 32)
    _same(got[0], want[0])
    _same(got[1], want[1])


def test_render_simulation_frame():
    sc = scenes.reference_scene("cube_small")
    sim = PBF(sc.config)
    r = Rd.FilteredParticleFluid(480, 270)
    try:
        sim.set_particles(sc.particles)
        sim.step(3)
        cam = Rd.reference_camera(480, 270, eye=(1.6, 1.4, 1.2), target=(0.4, 0.4, 0.4))
        r.set_camera(cam)
        r.render_simulation(sim)
        torch.cuda.synchronize()
        want = O.render(sim.positions(), 480, 270, cam["view"], cam["projection"], 0.02, 32)
        _same(r.depth(), want[0])
        _same(r.volume(), want[1])
        assert np.count_nonzero(want[0]) > 1000
    finally:
        r.close()
        sim.close()


@pytest.mark.parametrize("fs,size", [(32, (97, 131)), (12, (64, 300)), (3, (40, 40))])
def test_texture_filter_matches_oracle(fs, size):
    rng = np.random.default_rng(fs)
    H, W = size
    img = (2.0 + 0.3 * rng.uniform(size=(H, W))).astype(np.float32)
    img[rng.uniform(size=(H, W)) < 0.3] = 0.0
    d = torch.from_numpy(img).cuda()
    Rd.texture_filter(d.data_ptr(), W, H, filterSize=fs, particleRadius=0.02)
    torch.cuda.synchronize()
    _same(d.cpu().numpy(), O.narrow_range_filter(img, fs, 0.02))


def test_empty_and_errors():
    r = Rd.FilteredParticleFluid(64, 48)
    try:
        with pytest.raises(Exception):
            r.render(0, 0)                                 # no camera yet
        r.set_camera(Rd.reference_camera(64, 48))
        r.render(0, 0)
        torch.cuda.synchronize()
        assert not r.depth().any() and not r.volume().any()
        with pytest.raises(Exception):
            r.setConfig(filterSize=40)
        bad = Rd.reference_camera(64, 48)
        bad["projection"] = bad["projection"].copy()
        bad["projection"][0, 1] = 0.1                      # x/y shear
        with pytest.raises(Exception):
            r.set_camera(bad)
    finally:
        r.close()


@pytest.mark.parametrize("R", [0.2, 0.6])
def test_large_sprites_match_oracle(R):
    """Sprites wider and taller than 32 pixels (the column-stepped walk, the
    per-fragment row factor) and particles close to the camera."""
    W, H = 400, 300
    rng = np.random.default_rng(21)
    p = np.zeros((1500, 4), np.float32)
    p[:, :3] = rng.uniform(-0.6, 0.6, (1500, 3))
    p[:40, :3] = np.array([1.6, 1.6, 0.0]) + rng.uniform(-0.1, 0.1, (40, 3))   # near the eye at (2, 2, 0)
    cam = Rd.reference_camera(W, H)
    got = _render_gpu(p, W, H, 32, R=R, cam=cam)
    want = O.render(p, W, H, cam["view"], cam["projection"], R, 32)
    assert np.count_nonzero(want[0]) > 5000
    _same(got[0], want[0])
    _same(got[1], want[1])
