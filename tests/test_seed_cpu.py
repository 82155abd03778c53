"""Mesh voxelisation (SPH.voxelizeMesh, src/simulator/SPH.ts:151-187) without
a GPU: the CPU restatement checked against closed meshes whose insides are
known analytically (the reference's torus.obj and a UV sphere), and the C
ABI's argument checks, which return before any CUDA call."""
import ctypes

import numpy as np

from oracle import oracle as O
from pbf_gb300 import _lib as L
from pbf_gb300 import scenes


def _lattice(vertices, world, radius):
    """The lattice SPH.voxelizeMesh walks: world box of the local box's
    corners, spacing 2r from its minimum, floor(extent / 2r) per axis."""
    lo_l, hi_l = vertices.min(0).astype(np.float64), vertices.max(0).astype(np.float64)
    corners = np.array([[hi_l[0] if c & 4 else lo_l[0], hi_l[1] if c & 2 else lo_l[1], hi_l[2] if c & 1 else lo_l[2], 1.0]
                        for c in range(8)])
    wc = corners @ world.T
    lo, hi = wc[:, :3].min(0), wc[:, :3].max(0)
    d = 2.0 * radius
    dims = np.floor((hi - lo) / d).astype(np.int64)
    ii, jj, kk = np.meshgrid(*[np.arange(n) for n in dims], indexing="ij")
    pts = np.stack([ii * d + lo[0], jj * d + lo[1], kk * d + lo[2]], -1).reshape(-1, 3)
    return pts, dims, (ii.ravel(), jj.ravel(), kk.ravel())


def _kept_mask(lattice, kept):
    key = lambda a: [tuple(r) for r in np.asarray(a, np.float32).view(np.uint32).reshape(-1, 3)]
    s = set(key(kept[:, :3]))
    return np.array([k in s for k in key(lattice)])


def test_torus_mesh_fixture_is_the_reference_torus():
    v, t = scenes.load_mesh_npz("torus")
    assert v.shape == (400, 3) and t.shape == (800, 3)
    assert t.max() == 399
    # outward-facing winding: positive signed volume close to 2 pi^2 R r^2 (R = 1, r = 0.5)
    a, b, c = (v[t[:, q]].astype(np.float64) for q in range(3))
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    assert 0.95 * 2 * np.pi ** 2 * 0.25 < vol < 2 * np.pi ** 2 * 0.25


def test_parse_obj_fans_polygons_and_handles_slashes():
    text = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nf 1/1/1 2/1/1 3/1/1 4/1/1\nf -1 -2 -3\n"
    v, t = scenes.parse_obj(text)
    assert v.shape == (4, 3)
    assert t.tolist() == [[0, 1, 2], [0, 2, 3], [3, 2, 1]]


def test_oracle_torus_matches_analytic_inside():
    """Every lattice point clearly inside the polygonal torus is kept, none
    clearly outside is.  The layer j = 0 lies in the plane of the mesh's
    lowest vertex ring (the lattice starts at the box minimum), where +z rays
    graze the ring's edges and the answer is a tie between the faces on either
    side; it is left out of the analytic check."""
    v, t = scenes.load_mesh_npz("torus")
    r = 0.02
    kept = O.voxelize_mesh(v, t, r)
    lat, dims, (i, j, k) = _lattice(v, np.eye(4), r)
    assert kept.shape[0] > 0 and np.all(kept[:, 3] == 0.0)
    m = _kept_mask(lat, kept)
    assert m.sum() == kept.shape[0]
    rho = np.sqrt(lat[:, 0] ** 2 + lat[:, 2] ** 2)
    dist = np.sqrt((rho - 1.0) ** 2 + lat[:, 1] ** 2)
    # faceting of the 20-segment rings: at most 1.5 (1 - cos(pi/20)) + 0.5 (1 - cos(pi/20)) < 0.025 inward
    inner = dist < 0.5 - 0.025 - 0.005
    outer = dist > 0.5 + 0.005
    body = j > 0
    assert (inner & body).sum() > 60000
    assert np.all(m[inner & body])
    assert not np.any(m[outer & body])
    # lattice order: x slowest, z fastest
    order = np.lexsort((kept[:, 2], kept[:, 1], kept[:, 0]))
    assert np.all(order == np.arange(kept.shape[0]))


def test_oracle_sphere_under_world_transform():
    """A UV sphere under scale + rotation + translation: the ray runs along
    the LOCAL z axis (the reference transforms the origin only), and inside
    is decided in local space, so a point is kept iff its local image lies in
    the local sphere."""
    v, t = scenes.uv_sphere(0.5, (0.1, -0.05, 0.02), stacks=32, slices=64)
    W = scenes.trs_matrix(translate=(0.5, 0.3, 0.5), rotate_deg=(10.0, 25.0, -40.0), scale=0.4)
    r = 0.006
    kept = O.voxelize_mesh(v, t, r, W)
    lat, dims, _ = _lattice(v, W, r)
    m = _kept_mask(lat, kept)
    assert m.sum() == kept.shape[0] > 1000
    local = (np.c_[lat, np.ones(len(lat))] @ np.linalg.inv(W).T)[:, :3]
    d = np.linalg.norm(local - np.array([0.1, -0.05, 0.02]), axis=1)
    inner = d < 0.5 * np.cos(np.pi / 32) ** 2 - 1e-3
    outer = d > 0.5 + 1e-3
    assert np.all(m[inner]) and not np.any(m[outer])


def test_oracle_inside_out_mesh_keeps_nothing_inside():
    """Flipped winding turns every inside point's exit face into an entry
    face: nothing strictly inside is kept (the reference's rule tests the
    face orientation, not a parity count)."""
    v, t = scenes.uv_sphere(0.5, stacks=16, slices=32)
    kept = O.voxelize_mesh(v, t[:, ::-1].copy(), 0.02)
    if kept.shape[0]:
        assert np.all(np.linalg.norm(kept[:, :3], axis=1) > 0.5 * np.cos(np.pi / 16) ** 2 - 1e-3)


def test_voxelize_points_rejects_bad_arguments_without_gpu():
    lib = L.load()
    v, t = scenes.uv_sphere(0.5, stacks=8, slices=8)
    v = np.ascontiguousarray(v, np.float32)
    fp, up, dp = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_double)
    c = ctypes.c_uint32()

    def call(vv, tt, W, r):
        tt = np.ascontiguousarray(tt, np.uint32)
        Wc = np.ascontiguousarray(np.asarray(W, np.float64).T)
        return lib.pbf_voxelize_mesh_points(vv.ctypes.data_as(fp), vv.shape[0], tt.ctypes.data_as(up), tt.shape[0],
                                            Wc.ctypes.data_as(dp), r, None, 0, ctypes.byref(c))

    bad_index = t.copy()
    bad_index[3, 1] = v.shape[0]
    assert call(v, bad_index, np.eye(4), 0.01) == L.PBF_EINVAL
    assert call(v, t, np.zeros((4, 4)), 0.01) == L.PBF_EINVAL       # singular
    proj = np.eye(4)
    proj[3, 2] = -1.0
    assert call(v, t, proj, 0.01) == L.PBF_EINVAL                   # not affine
    assert call(v, t, np.eye(4), 0.0) == L.PBF_EINVAL               # radius
    assert call(v, t, np.eye(4), 1e-6) == L.PBF_EINVAL              # > 4096 points per axis
    nan = v.copy()
    nan[0, 0] = np.nan
    assert call(nan, t, np.eye(4), 0.01) == L.PBF_EINVAL
