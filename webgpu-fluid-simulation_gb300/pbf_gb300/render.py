"""Screen-space fluid buffers on the GPU: FilteredParticleFluid
(src/renderer/filteredParticleFluid/fluid.ts) without the WebGPU pipelines.

`FilteredParticleFluid(width, height)` owns the depth map (eye depth of the
nearest particle sphere, 0 where empty), the half-resolution volume
(thickness) map and the narrow-range filter; `render()` fills them from a
device float4 position buffer or from a `PBF` simulator.  The camera helpers
build the reference's camera: three.js PerspectiveCamera with the reverse-Z
`makePerspective` override of src/controller.ts:15-35, placed by `lookAt`."""
import ctypes

import numpy as np

from . import _lib as L


def perspective_reverse_z(fov_deg, aspect, near, far, zoom=1.0):
    """PerspectiveCamera.updateProjectionMatrix with the reverse-Z
    makePerspective (src/controller.ts:15-35): row-major float64 4x4."""
    top = near * np.tan(np.pi / 180.0 * 0.5 * fov_deg) / zoom
    height = 2.0 * top
    width = aspect * height
    left = -0.5 * width
    right, bottom = left + width, top - height
    m = np.zeros((4, 4))
    m[0, 0] = 2.0 * near / (right - left)
    m[1, 1] = 2.0 * near / (top - bottom)
    m[0, 2] = (right + left) / (right - left)
    m[1, 2] = (top + bottom) / (top - bottom)
    m[2, 2] = near / (far - near)
    m[2, 3] = far * near / (far - near)
    m[3, 2] = -1.0
    return m


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    """Camera placed at `eye` looking at `target` (Object3D.lookAt for a
    camera: its -z axis points at the target): (matrixWorld,
    matrixWorldInverse), row-major float64."""
    eye, target, up = (np.asarray(a, np.float64) for a in (eye, target, up))
    z = eye - target
    z = z / np.linalg.norm(z)
    x = np.cross(up, z)
    x = x / np.linalg.norm(x)
    y = np.cross(z, x)
    world = np.eye(4)
    world[:3, 0], world[:3, 1], world[:3, 2], world[:3, 3] = x, y, z, eye
    return world, np.linalg.inv(world)


def reference_camera(width, height, eye=(2.0, 2.0, 0.0), target=(0.0, 0.0, 0.0)):
    """The reference's camera (src/main.ts:66-68): fov 50, near 0.1, far 30,
    at (2, 2, 0) looking at the origin.  Returns a dict of row-major float32
    matrices and the uniform's params (globalResource.ts:94-109)."""
    fov, near, far = 50.0, 0.1, 30.0
    aspect = width / height
    world, view = look_at(eye, target)
    proj = perspective_reverse_z(fov, aspect, near, far)
    h = 2.0 * near * np.tan(np.pi / 180.0 * 0.5 * fov)
    params = [aspect * h / near, -h / near, (far - near) / (near * far), 1.0 / far]
    return {"position": np.asarray(eye, np.float32), "view": view.astype(np.float32),
            "view_inverse": world.astype(np.float32), "projection": proj.astype(np.float32),
            "params": np.asarray(params, np.float32)}


class FilteredParticleFluid:
    """pbf_renderer: FilteredParticleFluid's depth / volume maps and filter."""

    def __init__(self, width, height):
        self._lib = L.load()
        r = ctypes.c_void_p()
        rc = self._lib.pbf_renderer_create(int(width), int(height), ctypes.byref(r))
        if rc:
            raise L.PBFError(rc, "pbf_renderer_create")
        self._r = r
        self.width, self.height = int(width), int(height)

    def close(self):
        if getattr(self, "_r", None):
            self._lib.pbf_renderer_destroy(self._r)
            self._r = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            raise L.PBFError(rc, what)

    def setConfig(self, mode=0, filterSize=32, particleRadius=0.02, opacity=0.25, tintColor=(6, 105, 217)):
        """FilteredParticleFluid.setConfig (fluid.ts:114-133); tintColor in 0..255."""
        o = L.RenderOptions()
        o.mode, o.filter_size, o.particle_radius, o.opacity = int(mode), int(filterSize), float(particleRadius), \
            float(opacity)
        o.tint_color[:] = [c / 255.0 for c in tintColor]
        self._check(self._lib.pbf_renderer_set_config(self._r, ctypes.byref(o)), "setConfig")

    def set_camera(self, cam):
        """cam: a dict as `reference_camera` returns (row-major matrices)."""
        c = L.Camera()
        c.position[:] = [float(x) for x in cam["position"]]
        for name in ("view", "view_inverse", "projection"):
            getattr(c, name)[:] = [float(x) for x in np.asarray(cam[name], np.float32).T.ravel()]
        c.params[:] = [float(x) for x in cam.get("params", np.zeros(4))]
        self._check(self._lib.pbf_renderer_set_camera(self._r, ctypes.byref(c)), "set_camera")

    def render(self, positions_ptr, n, scene_depth_ptr=0, stream=0):
        """Rasterize + filter n particles from a device float4 buffer."""
        self._check(self._lib.pbf_render(self._r, ctypes.c_void_p(int(positions_ptr)), int(n),
                                         ctypes.c_void_p(int(scene_depth_ptr)), ctypes.c_void_p(int(stream))),
                    "render")

    def render_simulation(self, sim, scene_depth_ptr=0):
        self._check(self._lib.pbf_render_simulation(self._r, sim._h, ctypes.c_void_p(int(scene_depth_ptr))),
                    "render_simulation")

    def _map(self, which):
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self._lib.pbf_renderer_map_size(self._r, which, ctypes.byref(w), ctypes.byref(h)), "map size")
        out = np.zeros((h.value, w.value), np.float32)
        self._check(self._lib.pbf_renderer_copy_map(self._r, which, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                    out.nbytes), "copy map")
        return out

    def depth(self):
        """fluidDepthMap: (H, W) eye depth, 0 where no particle."""
        return self._map(L.RENDER_DEPTH)

    def volume(self):
        """fluidVolumeMap: (H/2, W/2) summed exp(-2 |uv|^2)."""
        return self._map(L.RENDER_VOLUME)

    def device_map(self, which):
        return self._lib.pbf_renderer_map_device(self._r, which)

    def timings(self):
        ms = (ctypes.c_float * 2)()
        self._check(self._lib.pbf_renderer_timings(self._r, ms), "timings")
        return float(ms[0]), float(ms[1])


def texture_filter(d_texture_ptr, width, height, filterSize=32, particleRadius=0.02, stream=0):
    """TextureFilter.execute on a device float32 image (pbf_texture_filter), in place."""
    lib = L.load()
    o = L.RenderOptions()
    o.filter_size, o.particle_radius = int(filterSize), float(particleRadius)
    rc = lib.pbf_texture_filter(ctypes.byref(o), ctypes.c_void_p(int(d_texture_ptr)), int(width), int(height),
                                ctypes.c_void_p(int(stream)))
    if rc:
        raise L.PBFError(rc, "texture_filter")
