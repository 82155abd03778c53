"""Scene builders: the reference's scene presets and the benchmark workloads.

Reference presets (src/controller.ts:195-249) run at the reference's own
constants (unit cube, r = 0.006, h = 0.025, dt = 1/300, GUI options of
src/common/config.ts:22-28).  The benchmark workloads are seeded synthetic
scenes; their geometry is resolved where the stated sizes do not fit:

  dam_break_16k   16,384 particles, 32x16x32 lattice at spacing 2r (r = 0.025,
                  h = 4r), jitter +-0.1r, box 3.2 x 1.0 x 1.6 with the block
                  at x < 1.6 (a 1.6-wide lattice cannot sit in the x < 0.5 part
                  of a 1.6 x 1.0 x 0.8 box), 64^3 box volume map,
                  dt = 1/60 in 2 substeps, 4 iterations, no surface tension.
  sphere_drop_1m  1,048,576 particles as a 128x64x128 lattice at spacing 2r
                  (r = 0.0125, h = 4r), jitter +-0.1r, dropped onto a sphere
                  (R = 0.4) resting on the floor of a 3.3 x 2.6 x 3.3 box
                  (a 128^3 block at this spacing would be 2,097,152 particles
                  and 3.2 high), 128^3 volume map of box + sphere,
                  gamma = 0.1, XSPH 0.01, vorticity 5e-4, 2 substeps of 1/300 s (the
                  reference's TIME_STEP; the workload states none), 4 iterations.
  neighbor_case   N particles in the unit cube on a 128^3-cell grid, uniform
                  or 64 Gaussian clumps (sigma = 2 cells) clipped to the cube.
"""
import ctypes
import os

import numpy as np

from . import _lib as L


class Scene:
    def __init__(self, name, config, particles, field=None, frames=1, note=""):
        self.name = name
        self.config = config
        self.particles = particles
        self.field = field  # dict(res, origin, extent, sdf, vol) or None
        self.frames = frames
        self.note = note

    @property
    def n(self):
        return int(self.particles.shape[0])


# ---- seeding (SPH.voxelizeCube / voxelizeSphere, SPH.ts:99-149) ---------------------
def lattice_cube(r, mn, mx):
    diam = 2.0 * float(np.float32(r))
    mn = [float(np.float32(v)) for v in mn]
    mx = [float(np.float32(v)) for v in mx]
    nx, ny, nz = (int(np.floor((mx[a] - mn[a]) / diam)) for a in range(3))
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pts = np.zeros((nx * ny * nz, 4), dtype=np.float32)
    pts[:, 0] = (i.ravel() * diam + mn[0]).astype(np.float32)
    pts[:, 1] = (j.ravel() * diam + mn[1]).astype(np.float32)
    pts[:, 2] = (k.ravel() * diam + mn[2]).astype(np.float32)
    return pts


def lattice_sphere(r, center, radius):
    diam = 2.0 * float(np.float32(r))
    c = [float(np.float32(v)) for v in center]
    R = float(np.float32(radius))
    vd = int(np.floor(R / float(np.float32(r)) / 2.0))
    rng = np.arange(-vd, vd + 1)
    i, j, k = np.meshgrid(rng, rng, rng, indexing="ij")
    x, y, z = i.ravel() * diam, j.ravel() * diam, k.ravel() * diam
    keep = x * x + y * y + z * z <= R * R
    pts = np.zeros((int(keep.sum()), 4), dtype=np.float32)
    pts[:, 0] = (x[keep] + c[0]).astype(np.float32)
    pts[:, 1] = (y[keep] + c[1]).astype(np.float32)
    pts[:, 2] = (z[keep] + c[2]).astype(np.float32)
    return pts


def _splitmix_stream(seed, count):
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def jitter(pts, amplitude, seed):
    """Seeded uniform jitter in [-a, a] (same stream as pbf_jitter_particles)."""
    out = pts.copy()
    u = _splitmix_stream(seed, pts.shape[0] * 3).reshape(-1, 3)
    a = float(np.float32(amplitude))
    out[:, :3] = (pts[:, :3].astype(np.float64) + a * (2.0 * u - 1.0)).astype(np.float32)
    return out


# ---- triangle meshes (SPH.voxelizeMesh inputs) ----------------------------------------
def parse_obj(text):
    """Vertices (V, 3) float32 and triangles (T, 3) uint32 of a Wavefront OBJ
    text (v and f records; polygons fanned into triangles, 1-based indices)."""
    verts, tris = [], []
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            verts.append([float(t[1]), float(t[2]), float(t[3])])
        elif t[0] == "f":
            idx = [int(f.split("/")[0]) for f in t[1:]]
            idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
            for q in range(1, len(idx) - 1):
                tris.append([idx[0], idx[q], idx[q + 1]])
    return np.array(verts, np.float32), np.array(tris, np.uint32)


def uv_sphere(radius, center=(0.0, 0.0, 0.0), stacks=24, slices=48):
    """Closed UV sphere with outward-facing triangles (counter-clockwise seen
    from outside)."""
    v = [[0.0, radius, 0.0]]
    for i in range(1, stacks):
        th = np.pi * i / stacks
        for j in range(slices):
            ph = 2.0 * np.pi * j / slices
            v.append([radius * np.sin(th) * np.cos(ph), radius * np.cos(th), radius * np.sin(th) * np.sin(ph)])
    v.append([0.0, -radius, 0.0])
    v = np.array(v, np.float64) + np.array(center, np.float64)
    t = []
    ring = lambda i, j: 1 + (i - 1) * slices + (j % slices)
    for j in range(slices):
        t.append([0, ring(1, j + 1), ring(1, j)])
    for i in range(1, stacks - 1):
        for j in range(slices):
            a, b, c, d = ring(i, j), ring(i, j + 1), ring(i + 1, j), ring(i + 1, j + 1)
            t.append([a, b, d])
            t.append([a, d, c])
    last = len(v) - 1
    for j in range(slices):
        t.append([last, ring(stacks - 1, j), ring(stacks - 1, j + 1)])
    return v.astype(np.float32), np.array(t, np.uint32)


def trs_matrix(translate=(0.0, 0.0, 0.0), rotate_deg=(0.0, 0.0, 0.0), scale=1.0):
    """4x4 row-major world matrix T * Rz * Ry * Rx * S (three.js Object3D
    order for the default XYZ Euler rotation)."""
    rx, ry, rz = np.radians(rotate_deg)
    cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    m = np.eye(4)
    m[:3, :3] = Rz @ Ry @ Rx * float(scale)
    m[:3, 3] = translate
    return m


def load_mesh_npz(name, folder=None):
    """A mesh fixture of tests/golden (vertices, triangles)."""
    folder = folder or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                    "tests", "golden")
    d = np.load(os.path.join(folder, "mesh_%s.npz" % name))
    return d["vertices"], d["triangles"]


# ---- configs ---------------------------------------------------------------------------
def base_config(**kw):
    c = L.Config()
    c.struct_size = ctypes.sizeof(L.Config)
    c.max_particles = 1 << 17
    c.particle_radius = 0.006
    c.kernel_radius = 0.025
    c.rest_density = 1000.0
    c.time_step = np.float32(1.0 / 300.0)
    c.substeps = 1
    c.domain_min[:] = [0.0, 0.0, 0.0]
    c.domain_max[:] = [1.0, 1.0, 1.0]
    c.grid_dim[:] = [0, 0, 0]
    c.lambda_eps = 1e-6
    c.wall_jitter = 1e-4
    c.jitter_mode = L.JITTER_HASH
    c.volume_quirk = 1
    c.fp_mode = L.FP_FAST
    c.boundary_interp = L.INTERP_CUBIC
    c.max_neighbors = 60
    c.options.iterations = 5
    c.options.xsph = 0.01
    c.options.vorticity = 0.1
    c.options.surface_tension = 0.5
    c.options.gravity = 9.8
    c.stream = None
    for k, v in kw.items():
        if k in ("domain_min", "domain_max"):
            getattr(c, k)[:] = list(v)
        elif k == "grid_dim":
            c.grid_dim[:] = list(v)
        elif k == "options":
            for ok, ov in v.items():
                setattr(c.options, ok, ov)
        else:
            setattr(c, k, v)
    return c


def copy_config(c):
    d = L.Config()
    ctypes.memmove(ctypes.byref(d), ctypes.byref(c), ctypes.sizeof(L.Config))
    return d


GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "tests",
                      "golden")


def load_cdm_npz(name, folder=None):
    d = np.load(os.path.join(folder or GOLDEN, "cdm_%s.npz" % name))
    return dict(res=d["res"].astype(np.uint32), origin=np.zeros(3, np.float32), extent=np.ones(3, np.float32),
                sdf=d["sdf"], vol=d["vol"])


def cdm_text(field):
    """Serialise a field as .cdm text (volumeMap.ts:23-39 reads it back)."""
    r = field["res"]
    fmt = lambda a: " ".join(repr(float(x)) for x in a) + " "
    return "%d %d %d\n%d\n%s\n%d\n%s\n" % (r[0], r[1], r[2], field["sdf"].size, fmt(field["sdf"]),
                                          field["vol"].size, fmt(field["vol"]))


def reference_scene(name, **kw):
    """Scene presets of Controller.setSceneConfig (controller.ts:195-249)."""
    cfg = base_config(**kw)
    r = cfg.particle_radius
    field = None
    if name == "cube_drop":
        pts = lattice_cube(r, (0.15, 0.35, 0.15), (0.65, 0.85, 0.65))
    elif name == "cube_small":  # a 13^3 version of Cube Drop for fast parity runs
        pts = lattice_cube(r, (0.35, 0.35, 0.35), (0.51, 0.51, 0.51))
    elif name == "water_droplet":
        pts = np.concatenate([lattice_cube(r, (0.005, 0.005, 0.005), (0.995, 0.08, 0.995)),
                              lattice_sphere(r, (0.5, 0.7, 0.5), 0.12)])
    elif name == "double_dam_break":
        pts = np.concatenate([lattice_cube(r, (0.005, 0.005, 0.005), (0.3, 0.6, 0.3)),
                              lattice_cube(r, (0.7, 0.005, 0.7), (0.995, 0.6, 0.995))])
    elif name == "boundary":
        pts = lattice_cube(r, (0.15, 0.35, 0.15), (0.65, 0.85, 0.65))
        field = load_cdm_npz("torus")
    elif name == "boundary_small":  # a slab resting on the torus tube: 235 of 845 particles in the band
        pts = lattice_cube(r, (0.42, 0.305, 0.22), (0.58, 0.37, 0.38))
        field = load_cdm_npz("torus")
    else:
        raise ValueError(name)
    if pts.shape[0] > cfg.max_particles:
        cfg.max_particles = int(pts.shape[0])
    return Scene(name, cfg, pts, field, frames=1)


def field_length(res):
    """Floats per field of a volume map of res = (nx, ny, nz) cells
    (BoundaryModel.FIELD_LENGTH, src/simulator/boundary/volumeMap.ts:7-11):
    the corner nodes, then two nodes on every x-, y- and z-edge."""
    nx, ny, nz = (int(v) for v in res)
    return ((nx + 1) * (ny + 1) * (nz + 1) + 2 * nx * (ny + 1) * (nz + 1) + (nx + 1) * 2 * ny * (nz + 1)
            + (nx + 1) * (ny + 1) * 2 * nz)


def generate_field(shapes, res, origin, extent, h, quadrature=12, flags=0, backend="gpu"):
    """Volume map for analytic shapes: list of (kind, center, size).
    backend "gpu" runs pbf_generate_volume_map; otherwise a callable with the
    same arguments (the CPU restatement's generator) is used and the CUDA
    library is not loaded."""
    arr = (L.Shape * len(shapes))()
    for i, (kind, c, s) in enumerate(shapes):
        arr[i].kind = kind
        arr[i].center[:] = list(c)
        arr[i].size[:] = list(s)
    r = (ctypes.c_uint32 * 3)(*[int(x) for x in res])
    o = (ctypes.c_float * 3)(*[float(x) for x in origin])
    e = (ctypes.c_float * 3)(*[float(x) for x in extent])
    n = field_length(res)
    sdf = np.zeros(n, np.float32)
    vol = np.zeros(n, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    if backend == "gpu":
        lib = L.load()
        rc = lib.pbf_generate_volume_map(arr, len(shapes), r, o, e, float(h), int(quadrature), int(flags),
                                         sdf.ctypes.data_as(fp), vol.ctypes.data_as(fp))
    else:
        rc = backend(arr, len(shapes), r, o, e, float(h), int(quadrature), int(flags), sdf.ctypes.data_as(fp),
                     vol.ctypes.data_as(fp))
    if rc:
        raise L.PBFError(rc, "volume map generation")
    return dict(res=np.array(res, np.uint32), origin=np.array(origin, np.float32),
                extent=np.array(extent, np.float32), sdf=sdf, vol=vol)


def dam_break_16k_spec(seed=0):
    r = 0.025
    cfg = base_config(particle_radius=r, kernel_radius=4 * r, time_step=np.float32(1.0 / 120.0), substeps=2,
                      domain_min=(0.0, 0.0, 0.0), domain_max=(3.2, 1.0, 1.6), max_particles=16384,
                      options=dict(iterations=4, xsph=0.01, vorticity=5e-4, surface_tension=0.0, gravity=9.8))
    cfg.max_neighbors = 96  # per-particle list slice: headroom for the wall impact
    d = 2 * r
    mn = (r, r, r)
    mx = (r + 32.5 * d, r + 16.5 * d, r + 32.5 * d)  # half a spacing of slack against float rounding
    pts = lattice_cube(r, mn, mx)
    assert pts.shape[0] == 32 * 16 * 32
    pts = jitter(pts, 0.1 * r, seed=seed)
    shapes = [(L.SHAPE_BOX_CONTAINER, (1.6, 0.5, 0.8), (1.6, 0.5, 0.8))]
    field_args = dict(shapes=shapes, res=(64, 64, 64), origin=(0.0, 0.0, 0.0), extent=(3.2, 1.0, 1.6),
                      h=4 * r)
    return cfg, pts, field_args


def sphere_drop_spec(nx=128, ny=64, nz=128, field_res=(128, 128, 128), seed=1):
    r = 0.0125
    box = (3.3, 2.6, 3.3)
    # The workload states no time step: use the reference's TIME_STEP (SPH.ts:27),
    # 1/300 s per substep, which keeps the ~4 m/s impact at ~0.27 h per substep
    # (1/120 s moves particles 0.68 h per substep and the 4-iteration solve
    # cannot hold the impact).
    cfg = base_config(particle_radius=r, kernel_radius=4 * r, time_step=np.float32(1.0 / 300.0), substeps=2,
                      domain_min=(0.0, 0.0, 0.0), domain_max=box, max_particles=nx * ny * nz,
                      options=dict(iterations=4, xsph=0.01, vorticity=5e-4, surface_tension=0.1, gravity=9.8))
    # per-particle list slice with headroom for the impact (a few particles
    # reach ~100 neighbours in long runs of the learned start); the passes
    # only touch the entries up to each warp's largest neighbour count
    cfg.max_neighbors = 128
    sphere_c = (box[0] / 2, 0.4, box[2] / 2)
    d = 2 * r
    x0 = (box[0] - nx * d) / 2 + r
    z0 = (box[2] - nz * d) / 2 + r
    y0 = 0.85 + r
    mn = (x0, y0, z0)
    mx = (x0 + (nx + 0.5) * d, y0 + (ny + 0.5) * d, z0 + (nz + 0.5) * d)  # slack against float rounding
    pts = lattice_cube(r, mn, mx)
    assert pts.shape[0] == nx * ny * nz
    pts = jitter(pts, 0.1 * r, seed=seed)
    shapes = [(L.SHAPE_BOX_CONTAINER, (box[0] / 2, box[1] / 2, box[2] / 2), (box[0] / 2, box[1] / 2, box[2] / 2)),
              (L.SHAPE_SPHERE, sphere_c, (0.4, 0.0, 0.0))]
    field_args = dict(shapes=shapes, res=field_res, origin=(0.0, 0.0, 0.0), extent=box, h=4 * r)
    return cfg, pts, field_args


BATCH_BOUNDARIES = ("box", "box+sphere", "box+cylinder")


def batch_scenes_spec(count=64, n_min=4096, n_max=262144, seed=3, field_res=(64, 64, 64)):
    """Independent scenes for one batch: particle counts log-uniform in
    [n_min, n_max] (seeded), each a jittered block (spacing 2r, r = 0.0125,
    h = 4r) in the corner of its own box (a dam break), the box with nothing
    inside, a sphere resting on the floor, or a vertical cylinder (pillar),
    each boundary a volume map of `field_res` cells over the box, and 3 or 4
    solver iterations.  Returns (shared config, scene dicts without fields,
    field arguments per scene)."""
    rng = np.random.default_rng(seed)
    r = 0.0125
    d = 2 * r
    cfg = base_config(particle_radius=r, kernel_radius=4 * r, time_step=np.float32(1.0 / 300.0), substeps=2,
                      max_particles=1,
                      options=dict(iterations=4, xsph=0.01, vorticity=5e-4, surface_tension=0.1, gravity=9.8))
    cfg.max_neighbors = 96
    counts = np.rint(np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count))).astype(np.int64)
    kinds = rng.integers(0, len(BATCH_BOUNDARIES), size=count)
    iters = rng.integers(3, 5, size=count)
    scenes, fields = [], []
    for i in range(count):
        n = int(counts[i])
        m = int(np.ceil(n ** (1.0 / 3.0)))
        ny = int(np.ceil(n / (m * m)))
        # block [d/2 + d/4, ...) so that the lattice keeps off the walls
        ext = np.array([2.0 * m * d + 4 * d, 1.6 * ny * d + 4 * d, 1.25 * m * d + 4 * d])
        ext = np.maximum(ext, 8 * 4 * r)
        idx = np.arange(m * m * ny)[:n]
        # x fastest within a layer, layers bottom-up, so a partial top layer stays on top
        ix, iz, iy = idx % m, (idx // m) % m, idx // (m * m)
        pts = np.stack([r + d * ix + d, r + d * iy + d, r + d * iz + d], axis=1).astype(np.float32)
        pts = jitter(np.concatenate([pts, np.zeros((n, 1), np.float32)], axis=1), 0.1 * r, seed=seed * 1000 + i)
        box = (L.SHAPE_BOX_CONTAINER, tuple(ext / 2), tuple(ext / 2))
        shapes = [box]
        kind = BATCH_BOUNDARIES[int(kinds[i])]
        if kind == "box+sphere":
            rad = 0.2 * min(ext[0], ext[2])
            shapes.append((L.SHAPE_SPHERE, (0.75 * ext[0], 0.0, 0.5 * ext[2]), (rad, 0.0, 0.0)))
        elif kind == "box+cylinder":
            rad = 0.1 * min(ext[0], ext[2])
            shapes.append((L.SHAPE_CYLINDER, (0.75 * ext[0], 0.5 * ext[1], 0.5 * ext[2]), (rad, ext[1], 0.0)))
        scenes.append(dict(positions=pts, domain_min=(0.0, 0.0, 0.0), domain_max=tuple(float(v) for v in ext),
                           iterations=int(iters[i]), boundary=kind))
        fields.append(dict(shapes=shapes, res=field_res, origin=(0.0, 0.0, 0.0), extent=tuple(float(v) for v in ext),
                           h=4 * r))
    return cfg, scenes, fields


def build_batch(spec, quadrature=8, backend="gpu"):
    """Scene dicts of a batch spec with their volume maps generated."""
    cfg, scenes, fields = spec
    out = []
    for sc, fa in zip(scenes, fields):
        f = generate_field(fa["shapes"], fa["res"], fa["origin"], fa["extent"], fa["h"], quadrature=quadrature,
                           backend=backend)
        out.append(dict(sc, field=f))
    return cfg, out


def build_scene(spec, quadrature=12, backend="gpu", name="scene", frames=1):
    cfg, pts, fa = spec
    field = generate_field(fa["shapes"], fa["res"], fa["origin"], fa["extent"], fa["h"], quadrature=quadrature,
                           backend=backend)
    return Scene(name, cfg, pts, field, frames=frames)


def neighbor_case(n, dist, seed=0, dim=128):
    """Stand-alone neighbour-search input: n float4 points in the unit cube."""
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        xyz = rng.random((n, 3), dtype=np.float64)
    elif dist == "clumps":
        centres = rng.random((64, 3))
        which = rng.integers(0, 64, size=n)
        sigma = 2.0 / dim
        xyz = centres[which] + rng.normal(0.0, sigma, size=(n, 3))
        xyz = np.clip(xyz, 0.0, np.nextafter(1.0, 0.0))
    else:
        raise ValueError(dist)
    pts = np.zeros((n, 4), np.float32)
    pts[:, :3] = xyz.astype(np.float32)
    pts[:, :3] = np.minimum(pts[:, :3], np.float32(np.nextafter(np.float32(1.0), np.float32(0.0))))
    cfg = base_config(kernel_radius=1.0 / dim, grid_dim=(dim, dim, dim), max_particles=max(n, 1))
    return cfg, pts
