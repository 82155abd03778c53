"""Screen-space fluid buffers without a GPU: the CPU restatement of the
reference's particle sprites (src/renderer/filteredParticleFluid/
shader/depthPassShader.ts, volumePassShader.ts) and narrow-range filter
(filterPassShader.ts) against analytic answers and against a second,
independent restatement of the filter written here in plain Python."""
import numpy as np
import pytest

from oracle import oracle as O
from pbf_gb300 import render as Rd

F = np.float32


def test_reference_camera_geometry():
    cam = Rd.reference_camera(640, 360)
    v, p = cam["view"].astype(np.float64), cam["projection"].astype(np.float64)
    c = v @ np.array([0.0, 0.0, 0.0, 1.0])
    assert np.allclose(c[:3], [0.0, 0.0, -np.sqrt(8.0)], atol=1e-6)
    # reverse-Z: the near plane maps to depth 1, the far plane to 0
    for z, want in ((-0.1, 1.0), (-30.0, 0.0)):
        clip = p @ np.array([0.0, 0.0, z, 1.0])
        assert abs(clip[2] / clip[3] - want) < 1e-6
    # 50 degree vertical field of view
    clip = p @ np.array([0.0, np.tan(np.radians(25.0)), -1.0, 1.0])
    assert abs(clip[1] / clip[3] - 1.0) < 1e-6


def test_splat_exp_is_accurate():
    xs = np.linspace(-2.0, 0.0, 20001).astype(np.float32)
    got = np.array([O.splat_exp(x) for x in xs], np.float32)
    want = np.exp(xs.astype(np.float64))
    ulp = np.spacing(want.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(got - want) / ulp) <= 2.0


def test_single_sprite_depth_profile():
    """One particle on the view axis: covered pixels form the disc of radius
    R/2 (the sprite's side is R) and each holds the eye depth of the sphere
    point d - R sqrt(1 - (2 rho / R)^2), rho the camera-space offset."""
    W = H = 256
    cam = Rd.reference_camera(W, H)
    R = 0.2
    d, vol, _ = O.render(np.zeros((1, 4), F), W, H, cam["view"], cam["projection"], R, 0)
    ys, xs = np.nonzero(d)
    assert len(xs) > 100
    dist = np.sqrt(8.0)
    # camera-space offset of a pixel centre at the particle's depth
    scale = 2.0 * dist * np.tan(np.radians(25.0)) / H
    rho = np.hypot(xs + 0.5 - W / 2, ys + 0.5 - H / 2) * scale
    assert rho.max() <= R / 2 * 1.001
    want = dist - R * np.sqrt(np.clip(1.0 - (2.0 * rho / R) ** 2, 0.0, 1.0))
    assert np.max(np.abs(d[ys, xs] - want)) < 2e-5
    # area of the disc
    assert abs(len(xs) - np.pi * (R / 2 / scale) ** 2) < 0.05 * len(xs)
    # volume sprite: side 2R on the half-resolution map, exp(-2 |n|^2) peaks near 1 at the centre
    assert 0.95 < vol.max() <= 1.0 and np.count_nonzero(vol) > 100


def test_occlusion_ties_and_scene_depth():
    W, H = 96, 64
    cam = Rd.reference_camera(W, H)
    near = np.array([[0.3, 0.3, 0.0, 0.0]], F)      # on the line to the camera at (2, 2, 0)
    far = np.zeros((1, 4), F)
    both, _, _ = O.render(np.concatenate([far, near]), W, H, cam["view"], cam["projection"], 0.05, 0)
    only_near, _, _ = O.render(near, W, H, cam["view"], cam["projection"], 0.05, 0)
    hit = only_near > 0
    assert np.array_equal(both[hit], only_near[hit])
    # duplicates: the same result as one particle
    one, vol1, _ = O.render(far, W, H, cam["view"], cam["projection"], 0.05, 0)
    two, vol2, _ = O.render(np.concatenate([far, far]), W, H, cam["view"], cam["projection"], 0.05, 0)
    assert np.array_equal(one, two)
    assert np.array_equal(vol2, (vol1.astype(np.float64) * 2).astype(np.float32))
    # a depth buffer at the near plane hides everything and stays as it was
    scene = np.ones((H, W), F)
    d, _, s = O.render(far, W, H, cam["view"], cam["projection"], 0.05, 0, scene)
    assert not d.any() and np.array_equal(s, scene)
    # a cleared buffer receives the fluid's depth where the fluid is
    d, _, s = O.render(far, W, H, cam["view"], cam["projection"], 0.05, 0, np.zeros((H, W), F))
    assert np.array_equal(s > 0, d > 0) and np.all(s[d > 0] < 1.0)


def test_order_independence():
    rng = np.random.default_rng(3)
    p = np.zeros((2000, 4), F)
    p[:, :3] = rng.uniform(-0.3, 0.3, (2000, 3))
    W, H = 128, 96
    cam = Rd.reference_camera(W, H)
    a = O.render(p, W, H, cam["view"], cam["projection"], 0.02, 32)
    b = O.render(p[rng.permutation(len(p))], W, H, cam["view"], cam["projection"], 0.02, 32)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _py_filter(img, fs, R):
    """filterPassShader.ts in float32 Python scalars, texel by texel."""
    H, W = img.shape
    half = fs >> 1
    sigma = F(half) * F(0.5)
    k = F(0.5) / (sigma * sigma)
    g = [F(np.exp(np.float64(F(-(i * i)) * k))) for i in range(half + 1)]
    thr, mu = F(R) * F(5.0), F(R)

    def texel(line, pos):
        n = len(line)
        at = lambda q: line[min(max(q, 0), n - 1)]
        c = pos - (16 - half)
        center = at(c)
        if not center > 0:
            return None
        vs, ws, lo, hi, bh = center, F(1.0), center - thr, center + thr, center + mu
        for i in range(1, half + 1):
            a, b = at(c - i), at(c + i)
            if a < lo or b < lo:
                continue
            a = bh if a > hi else a
            b = bh if b > hi else b
            lo = min(lo, min(a, b) - thr)
            hi = max(hi, max(a, b) + thr)
            ws = ws + g[i] * F(2.0)
            vs = vs + (a + b) * g[i]
        return vs / ws

    tmp = np.zeros_like(img)
    for y in range(H):
        row = [F(x) for x in img[y]]
        for x in range(W):
            t = texel(row, x)
            tmp[y, x] = F(0.0) if t is None else t
    out = img.copy()
    for x in range(W):
        col = [F(v) for v in tmp[:, x]]
        for y in range(H):
            t = texel(col, y)
            if t is not None:
                out[y, x] = t
    return out


@pytest.mark.parametrize("fs", [32, 16, 7, 2])
def test_filter_matches_independent_restatement(fs):
    rng = np.random.default_rng(fs)
    H, W = 30, 44
    img = (2.8 + 0.05 * rng.standard_normal((H, W))).astype(F)
    img[rng.uniform(size=(H, W)) < 0.2] = 0.0          # holes
    img[:, 30:] += 0.3                                  # a step above the 5 R threshold
    got = O.narrow_range_filter(img, fs, 0.02)
    want = _py_filter(img, fs, 0.02)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_filter_properties():
    # a constant image stays constant; the step between two plateaus survives
    img = np.full((24, 40), 2.5, F)
    out = O.narrow_range_filter(img, 32, 0.02)
    assert np.allclose(out, 2.5, rtol=0, atol=1e-6)
    img[:, 20:] = 3.0
    out = O.narrow_range_filter(img, 32, 0.02)
    assert np.all(out[:, :18] < 2.6) and np.all(out[:, 22:] > 2.9)
