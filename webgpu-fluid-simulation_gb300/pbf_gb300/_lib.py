"""ctypes binding of libpbf_gb300.so (include/pbf_gb300.h).

The structures below mirror the C declarations field by field.  Loading
fails loudly when the library has not been built: there is no CPU fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libpbf_gb300.so")

PBF_OK, PBF_EINVAL, PBF_ECAPACITY, PBF_EFORMAT, PBF_ECUDA, PBF_ETIMEOUT, PBF_EDIVERGED, PBF_ESTATE = range(8)
STATUS_NAMES = {0: "PBF_OK", 1: "PBF_EINVAL", 2: "PBF_ECAPACITY", 3: "PBF_EFORMAT", 4: "PBF_ECUDA",
                5: "PBF_ETIMEOUT", 6: "PBF_EDIVERGED", 7: "PBF_ESTATE"}
JITTER_HASH, JITTER_SIN = 0, 1
FP_FAST, FP_EXACT = 0, 1
INTERP_CUBIC, INTERP_TRILINEAR = 0, 1
(FIELD_POSITION, FIELD_VELOCITY, FIELD_ACCELERATION, FIELD_PREDICTED, FIELD_LAMBDA, FIELD_BOUNDARY,
 FIELD_OMEGA, FIELD_NORMAL, FIELD_DELTA_P, FIELD_NEIGHBOR_COUNT) = range(10)
SCAN_NOALLOC_MAX = 1 << 26
SEARCH_ARRAYS = {"keys": 0, "cell_count": 1, "cell_offset": 2, "order": 3}  # pbf_search_array
SCALAR_FIELDS = {FIELD_LAMBDA: "f4", FIELD_NEIGHBOR_COUNT: "u4"}

u32, f32 = ctypes.c_uint32, ctypes.c_float


class Options(ctypes.Structure):
    _fields_ = [("iterations", u32), ("xsph", f32), ("vorticity", f32), ("surface_tension", f32),
                ("gravity", f32)]


class Config(ctypes.Structure):
    _fields_ = [("struct_size", u32), ("max_particles", u32), ("particle_radius", f32),
                ("kernel_radius", f32), ("rest_density", f32), ("time_step", f32), ("substeps", u32),
                ("domain_min", f32 * 3), ("domain_max", f32 * 3), ("grid_dim", u32 * 3),
                ("lambda_eps", f32), ("wall_jitter", f32), ("jitter_mode", u32), ("volume_quirk", u32),
                ("fp_mode", u32), ("boundary_interp", u32), ("max_neighbors", u32), ("options", Options),
                ("stream", ctypes.c_void_p)]


class Metrics(ctypes.Structure):
    _fields_ = [("particles", u32), ("nonfinite", u32), ("penetrations", u32), ("error_flags", u32),
                ("max_compression", f32), ("mean_abs_density_err", f32), ("max_abs_density_err", f32),
                ("kinetic_energy", f32), ("mean_compression", f32), ("neighbor_total", u32),
                ("fallback_steps", u32)]


SHAPE_BOX_CONTAINER, SHAPE_SPHERE, SHAPE_CYLINDER, SHAPE_TORUS, SHAPE_BOX_SOLID = range(5)
VOLMAP_OUTSIDE_EMPTY = 0x1
VOLMAP_DISCRETE_SDF = 0x2


class Shape(ctypes.Structure):
    _fields_ = [("kind", u32), ("center", f32 * 3), ("size", f32 * 3)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", u32), ("total_ms", f32)]


MLP_PARAMS = 4801
MLP_KERNEL_MMA_SYNC, MLP_KERNEL_TCGEN05 = 0, 1
MLP_TRAIN_TCGEN05, MLP_TRAIN_MMA_SYNC = 0, 1  # pbf_train_config.kernel


class MLP(ctypes.Structure):
    _fields_ = [("params", f32 * MLP_PARAMS), ("feat_mean", f32 * 8), ("feat_inv_std", f32 * 8),
                ("lam_scale", f32)]


class TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", u32), ("batch", u32), ("learning_rate", f32), ("kernel", u32),
                ("seed", ctypes.c_uint64)]


class Grid(ctypes.Structure):
    _fields_ = [("origin", f32 * 3), ("inv_cell", f32 * 3), ("dim", u32 * 3)]


class Launch(ctypes.Structure):
    _fields_ = [("block", u32), ("ctas_per_sm", u32), ("cell_ratio", f32), ("build", u32)]

BUILD_THREAD, BUILD_PAIR, BUILD_WARP, BUILD_CELLBLOCK_MASK, BUILD_CELLBLOCK_FREE = 0, 1, 2, 3, 4
DEVERR_STAGE_TIMEOUT = 0x10


class TuneTrial(ctypes.Structure):
    _fields_ = [("launch", Launch), ("ms_per_substep", f32)]


TUNE_CELL_RATIO = 0x1


class Scene(ctypes.Structure):
    _fields_ = [("struct_size", u32), ("particles", u32), ("positions", ctypes.POINTER(f32)),
                ("domain_min", f32 * 3), ("domain_max", f32 * 3), ("iterations", u32), ("field_res", u32 * 3),
                ("field_origin", f32 * 3), ("field_extent", f32 * 3), ("sdf", ctypes.POINTER(f32)),
                ("volume", ctypes.POINTER(f32))]


class SceneInfo(ctypes.Structure):
    _fields_ = [("first_id", u32), ("particles", u32), ("iterations", u32), ("grid_dim", u32 * 3), ("cells", u32)]


SEED_CUBE, SEED_SPHERE, SEED_MESH = 0, 1, 2


class SeedItem(ctypes.Structure):
    _fields_ = [("kind", u32), ("a", f32 * 3), ("b", f32 * 3), ("vertices", ctypes.POINTER(f32)),
                ("vertex_count", u32), ("indices", ctypes.POINTER(u32)), ("triangle_count", u32),
                ("world", ctypes.c_double * 16)]


RENDER_DEPTH, RENDER_VOLUME = 0, 1


class RenderOptions(ctypes.Structure):
    _fields_ = [("mode", u32), ("filter_size", u32), ("particle_radius", f32), ("opacity", f32),
                ("tint_color", f32 * 3)]


class Camera(ctypes.Structure):
    _fields_ = [("position", f32 * 3), ("view", f32 * 16), ("view_inverse", f32 * 16), ("projection", f32 * 16),
                ("params", f32 * 4)]


# Every symbol the header declares, with (restype, argtypes).
_P = ctypes.c_void_p
_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)
_UP = ctypes.POINTER(ctypes.c_uint32)
SIGNATURES = {
    "pbf_abi_version": (ctypes.c_int, []),
    "pbf_config_default": (ctypes.c_int, [ctypes.POINTER(Config)]),
    "pbf_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    "pbf_destroy": (ctypes.c_int, [_P]),
    "pbf_reset": (ctypes.c_int, [_P]),
    "pbf_last_error": (ctypes.c_char_p, [_P]),
    "pbf_set_options": (ctypes.c_int, [_P, ctypes.POINTER(Options)]),
    "pbf_get_options": (ctypes.c_int, [_P, ctypes.POINTER(Options)]),
    "pbf_voxelize_cube": (ctypes.c_int, [_P, _FP, _FP, _UP]),
    "pbf_voxelize_sphere": (ctypes.c_int, [_P, _FP, ctypes.c_float, _UP]),
    "pbf_jitter_particles": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_uint64]),
    "pbf_voxelize_mesh": (ctypes.c_int, [_P, _FP, u32, _UP, u32, _DP, _UP]),
    "pbf_voxelize_mesh_points": (ctypes.c_int, [_FP, u32, _UP, u32, _DP, ctypes.c_double, _FP, u32, _UP]),
    "pbf_seed_device": (ctypes.c_int, [_P, ctypes.POINTER(SeedItem), u32, f32, ctypes.c_uint64, _UP]),
    "pbf_selftest_bounded_wait": (ctypes.c_int, []),
    "pbf_copy_positions_async": (ctypes.c_int, [_P, _FP, ctypes.c_size_t]),
    "pbf_renderer_create": (ctypes.c_int, [u32, u32, ctypes.POINTER(_P)]),
    "pbf_renderer_destroy": (ctypes.c_int, [_P]),
    "pbf_renderer_set_config": (ctypes.c_int, [_P, ctypes.POINTER(RenderOptions)]),
    "pbf_renderer_set_camera": (ctypes.c_int, [_P, ctypes.POINTER(Camera)]),
    "pbf_render": (ctypes.c_int, [_P, _P, u32, _P, _P]),
    "pbf_render_simulation": (ctypes.c_int, [_P, _P, _P]),
    "pbf_texture_filter": (ctypes.c_int, [ctypes.POINTER(RenderOptions), _P, u32, u32, _P]),
    "pbf_renderer_map_device": (_P, [_P, u32]),
    "pbf_renderer_map_size": (ctypes.c_int, [_P, u32, _UP, _UP]),
    "pbf_renderer_copy_map": (ctypes.c_int, [_P, u32, _FP, ctypes.c_size_t]),
    "pbf_renderer_timings": (ctypes.c_int, [_P, _FP]),
    "pbf_host_particle_count": (ctypes.c_int, [_P, _UP]),
    "pbf_copy_host_particles": (ctypes.c_int, [_P, _FP, u32]),
    "pbf_set_particle_position": (ctypes.c_int, [_P]),
    "pbf_set_particles": (ctypes.c_int, [_P, _FP, u32]),
    "pbf_set_velocities": (ctypes.c_int, [_P, _FP, u32]),
    "pbf_set_accelerations": (ctypes.c_int, [_P, _FP, u32]),
    "pbf_copy_search_state": (ctypes.c_int, [_P, ctypes.c_int, _UP, ctypes.c_size_t]),
    "pbf_set_boundary_data": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "pbf_set_boundary_field": (ctypes.c_int, [_P, _UP, _FP, _FP, _FP, _FP, ctypes.c_size_t]),
    "pbf_clear_boundary": (ctypes.c_int, [_P]),
    "pbf_field_length": (ctypes.c_size_t, [_UP]),
    "pbf_run": (ctypes.c_int, [_P]),
    "pbf_step": (ctypes.c_int, [_P, u32]),
    "pbf_run_timestamp": (ctypes.c_int, [_P, _FP]),
    "pbf_synchronize": (ctypes.c_int, [_P]),
    "pbf_set_paused": (ctypes.c_int, [_P, ctypes.c_int]),
    "pbf_is_paused": (ctypes.c_int, [_P]),
    "pbf_enable_graph": (ctypes.c_int, [_P, ctypes.c_int]),
    "pbf_particle_count": (u32, [_P]),
    "pbf_position_device": (_P, [_P]),
    "pbf_velocity_device": (_P, [_P]),
    "pbf_copy_field": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t]),
    "pbf_get_metrics": (ctypes.c_int, [_P, ctypes.POINTER(Metrics)]),
    "pbf_set_capture": (ctypes.c_int, [_P, ctypes.c_int]),
    "pbf_stream": (_P, [_P]),
    "pbf_set_kernel_timing": (ctypes.c_int, [_P, ctypes.c_int]),
    "pbf_get_kernel_timing": (ctypes.c_int, [_P, ctypes.POINTER(KernelTime), u32, _UP]),
    "pbf_ns_create": (ctypes.c_int, [ctypes.POINTER(Grid), u32, _P, ctypes.POINTER(_P)]),
    "pbf_ns_destroy": (ctypes.c_int, [_P]),
    "pbf_ns_run": (ctypes.c_int, [_P, _P, u32, _P, _P, _P, _P, _P]),
    "pbf_ns_lists": (ctypes.c_int, [_P, _P, u32, ctypes.c_float, _P, _P, u32, _UP]),
    "pbf_ns_sync": (ctypes.c_int, [_P]),
    "pbf_ns_set_timing": (ctypes.c_int, [_P, ctypes.c_int]),
    "pbf_ns_timings": (ctypes.c_int, [_P, _P]),
    "pbf_ns_last_error": (ctypes.c_char_p, [_P]),
    "pbf_exclusive_scan_u32": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "pbf_generate_volume_map": (ctypes.c_int, [ctypes.POINTER(Shape), u32, _UP, _FP, _FP, ctypes.c_float, u32, u32,
                                               _FP, _FP]),
    "pbf_volume_from_sdf": (ctypes.c_int, [_UP, _FP, _FP, ctypes.c_float, u32, u32, _FP, _FP]),
    "pbf_exclusive_scan_u32_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "pbf_mlp_init": (ctypes.c_int, [ctypes.POINTER(MLP), ctypes.c_uint64]),
    "pbf_mlp_fit_normalization": (ctypes.c_int, [ctypes.POINTER(MLP), _FP, _FP, u32]),
    "pbf_mlp_forward": (ctypes.c_int, [ctypes.POINTER(MLP), _FP, u32, _FP]),
    "pbf_mlp_gradient": (ctypes.c_int, [ctypes.POINTER(MLP), _FP, _FP, u32, _FP, _FP]),
    "pbf_mlp_gradient_ex": (ctypes.c_int, [ctypes.POINTER(MLP), _FP, _FP, u32, _FP, _FP, u32]),
    "pbf_mlp_train": (ctypes.c_int, [ctypes.POINTER(MLP), _FP, _FP, u32, ctypes.POINTER(TrainConfig), _FP]),
    "pbf_set_trace": (ctypes.c_int, [_P, u32, u32, ctypes.c_uint64]),
    "pbf_trace_rows": (ctypes.c_int, [_P, _UP]),
    "pbf_copy_trace": (ctypes.c_int, [_P, _FP, _FP, u32]),
    "pbf_trace_error": (ctypes.c_int, [_P, _FP, _FP]),
    "pbf_set_learned": (ctypes.c_int, [_P, ctypes.POINTER(MLP), u32, ctypes.c_float]),
    "pbf_mlp_forward_ex": (ctypes.c_int, [ctypes.POINTER(MLP), _FP, u32, _FP, u32]),
    "pbf_set_mlp_kernel": (ctypes.c_int, [_P, u32]),
    "pbf_set_adaptive_iterations": (ctypes.c_int, [_P, ctypes.c_int]),
    "pbf_set_lagged_iterations": (ctypes.c_int, [_P, ctypes.c_float]),
    "pbf_adaptive_counts": (ctypes.c_int, [_P, _UP, _UP]),
    "pbf_set_launch": (ctypes.c_int, [_P, ctypes.POINTER(Launch)]),
    "pbf_set_cellblock_capacity": (ctypes.c_int, [_P, u32]),
    "pbf_get_launch": (ctypes.c_int, [_P, ctypes.POINTER(Launch)]),
    "pbf_autotune": (ctypes.c_int, [_P, u32, u32, ctypes.POINTER(TuneTrial), u32, _UP, ctypes.POINTER(Launch)]),
    "pbf_batch_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(Scene), u32, ctypes.POINTER(_P)]),
    "pbf_scene_count": (u32, [_P]),
    "pbf_get_scene_info": (ctypes.c_int, [_P, u32, ctypes.POINTER(SceneInfo)]),
    "pbf_get_scene_metrics": (ctypes.c_int, [_P, u32, ctypes.POINTER(Metrics)]),
}

_lib = None


def load(path=None):
    """Load the library (once) and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError("libpbf_gb300.so not built (%s); run webgpu-fluid-simulation_gb300/build_lib.py" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PBFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, code), msg))
        self.code = code


def default_config():
    lib = load()
    c = Config()
    rc = lib.pbf_config_default(ctypes.byref(c))
    if rc:
        raise PBFError(rc, "pbf_config_default")
    return c
