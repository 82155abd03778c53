"""The C-ABI library loads without a GPU and exports every entry point the
public headers declare (no compute calls here)."""
import ctypes
import glob
import os
import re

from pbf_gb300 import _lib as L

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for hdr in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(pbf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = L.load()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    names = declared_functions()
    assert names <= set(L.SIGNATURES), sorted(names - set(L.SIGNATURES))


def test_struct_sizes_match_header_layout():
    # pbf_config: 11 u32/f32 scalars + 3 float[3] ... + options (20 B) + pointer, 8-byte aligned
    assert ctypes.sizeof(L.Options) == 20
    assert ctypes.sizeof(L.Config) % 8 == 0
    assert ctypes.sizeof(L.Shape) == 28
    assert ctypes.sizeof(L.SeedItem) == 192   # 28 B of kinds/corners, 3 pointers + counts, double[16]
    assert ctypes.sizeof(L.Grid) == 36


def test_config_default_is_reference_constants():
    c = L.default_config()  # host-only call
    assert c.struct_size == ctypes.sizeof(L.Config)
    assert c.max_particles == 1 << 17
    assert abs(c.particle_radius - 0.006) < 1e-9 and abs(c.kernel_radius - 0.025) < 1e-9
    assert abs(c.time_step - 1 / 300) < 1e-9 and c.substeps == 1
    o = c.options
    assert (o.iterations, round(o.xsph, 6), round(o.vorticity, 6), round(o.surface_tension, 6),
            round(o.gravity, 6)) == (5, 0.01, 0.1, 0.5, 9.8)


def test_field_length_matches_reference_formula():
    lib = L.load()
    r = (ctypes.c_uint32 * 3)(20, 20, 20)
    assert lib.pbf_field_length(r) == 62181  # BoundaryModel.FIELD_LENGTH (volumeMap.ts:7-11)
    r = (ctypes.c_uint32 * 3)(3, 4, 5)
    nx, ny, nz = 3, 4, 5
    assert lib.pbf_field_length(r) == ((nx + 1) * (ny + 1) * (nz + 1) + 2 * nx * (ny + 1) * (nz + 1) +
                                       (nx + 1) * 2 * ny * (nz + 1) + (nx + 1) * (ny + 1) * 2 * nz)
    from pbf_gb300 import scenes  # the host-side count the CPU-only paths use
    for res in ((20, 20, 20), (3, 4, 5), (128, 128, 128)):
        assert scenes.field_length(res) == lib.pbf_field_length((ctypes.c_uint32 * 3)(*res))


def test_host_argument_validation_without_gpu():
    lib = L.load()
    c = L.default_config()
    c.struct_size = 3  # wrong ABI size is rejected before any CUDA call
    h = ctypes.c_void_p()
    assert lib.pbf_create(ctypes.byref(c), ctypes.byref(h)) == L.PBF_EINVAL
    c = L.default_config()
    c.kernel_radius = -1.0
    assert lib.pbf_create(ctypes.byref(c), ctypes.byref(h)) == L.PBF_EINVAL
    assert lib.pbf_exclusive_scan_u32(None, None, 0, None) == L.PBF_OK
