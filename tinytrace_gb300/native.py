"""ctypes binding of libtinytrace_cuda.so (include/tinytrace_cuda.h) and the numpy dtypes of
the reference's GPU-side byte layouts.

The library is loaded from the in-tree build directory (tinytrace_gb300/_build).  There is no
CPU fallback: if the library is missing or no CUDA device is present, the calls fail with
TinytraceError.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libtinytrace_cuda.so"

# ---------------------------------------------------------------- status codes
TT_OK = 0
TT_ERR_INVALID_ARGUMENT = 1
TT_ERR_OOM = 2
TT_ERR_BAD_HANDLE = 3
TT_ERR_DEVICE = 4
TT_ERR_TIMEOUT = 5
TT_ERR_OVERFLOW = 6
TT_ERR_UNSUPPORTED = 7
TT_ERR_NO_DEVICE = 8

TT_LIFETIME_STATIC = 0
TT_LIFETIME_SURFACE = 1
TT_LIFETIME_SCENE = 2
TT_LIFETIME_FRAME = 3
TT_LIFETIME_RENDERER = 4

TT_FORMAT_RGBA32F = 0
TT_FORMAT_RGBA8_UNORM = 1
TT_OPTION_LIGHT_VISIBILITY = 9
TT_LIGHT_VISIBILITY_HASH = 0
TT_LIGHT_VISIBILITY_TRIANGLE = 1
TT_OPTION_LIGHT_SELECTION = 10
TT_LIGHT_SELECTION_UNIFORM = 0
TT_LIGHT_SELECTION_POWER = 1
TT_OPTION_PRIMARY_VISIBILITY = 11
TT_PRIMARY_TRAVERSE = 0
TT_PRIMARY_RASTER = 1
TT_TEXTURE_BC1_SRGB = 1
TT_TEXTURE_BC5_UNORM = 2
TT_TEXTURE_R8_UNORM = 3
TT_TEXTURE_R16_FLOAT = 4
TT_TEXTURE_MAX_LEVELS = 16
TT_TRACE_CULL_BACK_FACES = 1
TT_TRACE_NOALLOC_MAX_RAYS = 65536
TT_INTEGRATOR_WAVEFRONT = 0
TT_INTEGRATOR_MEGAKERNEL = 1
TT_OPTION_INTEGRATOR = 1
TT_OPTION_WAVEFRONT_SLOTS = 2
TT_OPTION_ACCEL = 3
TT_ACCEL_AUTO = 0
TT_ACCEL_FLAT = 1
TT_ACCEL_TWO_LEVEL = 2
TT_ACCEL_FLAT_WIDE = 3
TT_OPTION_STAGE_TIMING = 4
TT_OPTION_GRAPHS = 5
TT_SERVER_POLICY_FAIR = 0
TT_SERVER_POLICY_SMALLEST_FIRST = 1
TT_REQUEST_QUEUED = 0
TT_REQUEST_RUNNING = 1
TT_REQUEST_DONE = 2
TT_REQUEST_FAILED = 3
TT_OPTION_RADIANCE_CACHE = 8
TT_STAGE_CACHE = 6
TT_CACHE_WEIGHTS = 16896
TT_CACHE_GRID_FLOATS = 16777216
TT_OPTION_REFILL_LANES = 6
TT_OPTION_TRACE_BLOCKS_PER_SM = 7
TT_STAGE_REGEN = 0
TT_STAGE_EXTEND = 1
TT_STAGE_SHADE = 2
TT_STAGE_SHADOW = 3
TT_STAGE_REDUCE = 4
TT_STAGE_MEGAKERNEL = 5
TT_STAGE_RESTIR_GBUFFER = 8
TT_STAGE_RESTIR_INITIAL = 9
TT_STAGE_RESTIR_TEMPORAL = 10
TT_STAGE_RESTIR_SPATIAL = 11
TT_STAGE_RESTIR_SHADE = 12
TT_STAGE_PRIMARY = 13
TT_STAGE_COUNT = 16
TT_STAGE_CACHE_TRAIN = 7
STAGE_NAMES = ("regen", "extend", "shade", "shadow", "reduce", "megakernel", "cache", "cache_train",
               "restir_gbuffer", "restir_initial", "restir_temporal", "restir_spatial", "restir_shade", "primary")

# ---------------------------------------------------------------- byte layouts (numpy)
MATERIAL_CONSTANT_FIELDS = [
    ("base_color", "<f4", (4,)),
    ("specular_color", "<f4", (4,)),
    ("transmission_color", "<f4", (4,)),
    ("coat_color", "<f4", (4,)),
    ("fuzz_color", "<f4", (4,)),
    ("emission_color", "<f4", (4,)),
    ("geometry_normal", "<f4", (4,)),
    ("base_weight", "<f4"),
    ("base_metalness", "<f4"),
    ("base_diffuse_roughness", "<f4"),
    ("specular_weight", "<f4"),
    ("specular_roughness", "<f4"),
    ("specular_roughness_anisotropy", "<f4"),
    ("specular_ior", "<f4"),
    ("specular_rotation", "<f4"),
    ("transmission_weight", "<f4"),
    ("transmission_depth", "<f4"),
    ("coat_weight", "<f4"),
    ("coat_roughness", "<f4"),
    ("coat_roughness_anisotropy", "<f4"),
    ("coat_ior", "<f4"),
    ("coat_darkening", "<f4"),
    ("coat_rotation", "<f4"),
    ("fuzz_weight", "<f4"),
    ("fuzz_roughness", "<f4"),
    ("emission_luminance", "<f4"),
    ("geometry_opacity", "<f4"),
]
MATERIAL_CONSTANTS_DTYPE = np.dtype(MATERIAL_CONSTANT_FIELDS)  # 192 B
MATERIAL_DTYPE = np.dtype([("constants", MATERIAL_CONSTANTS_DTYPE), ("textures", "<u4", (27,)), ("padding", "<u4")])
VERTEX_DTYPE = np.dtype([("texture_coordinates", "<f2", (2,)), ("tangent_frame", "<u4")])
MESH_DTYPE = np.dtype([("center", "<f4", (3,)), ("radius", "<f4"), ("vertex_offset", "<u4"),
                       ("vertex_count", "<u4"), ("index_offset", "<u4"), ("index_count", "<u4")])
INSTANCE_DTYPE = np.dtype([("transform", "<f4", (16,)), ("inverse_transform", "<f4", (16,)),
                           ("normal_transform", "<f4", (16,)), ("vertex_offset", "<u4"),
                           ("index_offset", "<u4"), ("material_index", "<u4"), ("mesh_index", "<u4")])
EMISSIVE_DTYPE = np.dtype([("positions", "<i2", (3, 3)), ("hash", "<u2"),
                           ("texture_coordinates", "<f2", (3, 2)), ("instance_index", "<u4")])
CONSTANTS_DTYPE = np.dtype([("view", "<f4", (16,)), ("proj", "<f4", (16,)), ("proj_view", "<f4", (16,)),
                            ("inverse_view", "<f4", (16,)), ("inverse_proj", "<f4", (16,)),
                            ("camera_position", "<f4", (4,)), ("frame_index", "<u4"),
                            ("accumulated_frame_count", "<u4"), ("sample_count", "<u4"),
                            ("bounce_count", "<u4"), ("screen_size", "<u4", (2,)), ("tonemap", "<u4"),
                            ("light_sampling", "<u4")])
NODE4_DTYPE = np.dtype([("box", "<f4", (6, 4)), ("child", "<u4", (4,)), ("count", "<u4"), ("pad", "<u4", (3,))])
TRI_RECORD_DTYPE = np.dtype([("v0", "<f4", (3,)), ("prim", "<u4"), ("v1", "<f4", (3,)), ("mesh", "<u4"),
                             ("v2", "<f4", (3,)), ("pad", "<u4")])
# compressed 8-wide node of the flat structure (TT_ACCEL_FLAT_WIDE), 80 bytes
NODE8_DTYPE = np.dtype([("origin", "<f4", (3,)), ("exponent", "u1", (3,)), ("imask", "u1"), ("child_base", "<u4"),
                        ("tri_base", "<u4"), ("meta", "u1", (8,)), ("qlo_x", "u1", (8,)), ("qhi_x", "u1", (8,)),
                        ("qlo_y", "u1", (8,)), ("qhi_y", "u1", (8,)), ("qlo_z", "u1", (8,)), ("qhi_z", "u1", (8,))])
assert NODE8_DTYPE.itemsize == 80

assert MATERIAL_CONSTANTS_DTYPE.itemsize == 192
assert MATERIAL_DTYPE.itemsize == 304
assert VERTEX_DTYPE.itemsize == 8
assert MESH_DTYPE.itemsize == 32
assert INSTANCE_DTYPE.itemsize == 208
assert EMISSIVE_DTYPE.itemsize == 36
assert CONSTANTS_DTYPE.itemsize == 368
assert NODE4_DTYPE.itemsize == 128
assert TRI_RECORD_DTYPE.itemsize == 48


class MeshData(ctypes.Structure):
    """tt_mesh_data"""

    _fields_ = [("positions", ctypes.c_void_p), ("texture_coordinates", ctypes.c_void_p),
                ("indices", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("tangents", ctypes.c_void_p),
                ("vertex_count", ctypes.c_uint32), ("index_count", ctypes.c_uint32)]


class EmissiveSource(ctypes.Structure):
    """tt_emissive_source"""

    _fields_ = [("positions", ctypes.c_void_p), ("vertices", ctypes.c_void_p), ("vertex_count", ctypes.c_uint64),
                ("indices", ctypes.c_void_p), ("index_count", ctypes.c_uint64), ("meshes", ctypes.c_void_p),
                ("mesh_count", ctypes.c_uint32), ("model_count", ctypes.c_uint32),
                ("model_mesh", ctypes.c_void_p), ("model_instance", ctypes.c_void_p)]


class TextureDesc(ctypes.Structure):
    """tt_texture"""

    _fields_ = [("format", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("level_count", ctypes.c_uint32), ("data", ctypes.c_void_p), ("bytes", ctypes.c_uint64)]


class SceneDesc(ctypes.Structure):
    """tt_scene_desc"""

    _fields_ = [
        ("positions", ctypes.c_void_p),
        ("position_count", ctypes.c_uint64),
        ("indices", ctypes.c_void_p),
        ("index_count", ctypes.c_uint64),
        ("vertices", ctypes.c_void_p),
        ("vertex_count", ctypes.c_uint64),
        ("materials", ctypes.c_void_p),
        ("material_count", ctypes.c_uint32),
        ("mesh_count", ctypes.c_uint32),
        ("meshes", ctypes.c_void_p),
        ("instances", ctypes.c_void_p),
        ("instance_count", ctypes.c_uint32),
        ("emissive_triangle_count", ctypes.c_uint32),
        ("emissive_triangles", ctypes.c_void_p),
        ("textures", ctypes.c_void_p),
        ("texture_count", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class Timings(ctypes.Structure):
    _fields_ = [("integrate_ns", ctypes.c_uint64), ("post_process_ns", ctypes.c_uint64),
                ("scene_build_ns", ctypes.c_uint64)]


class SceneStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("triangle_count", "instance_count", "emissive_count", "blas_nodes",
                                               "tlas_nodes", "blas_levels", "tlas_levels", "device_bytes",
                                               "max_stack", "accel")]


class StageTimings(ctypes.Structure):
    _fields_ = [("ns", ctypes.c_uint64 * TT_STAGE_COUNT), ("launches", ctypes.c_uint64 * TT_STAGE_COUNT),
                ("overflow", ctypes.c_uint64)]


class RestirConfig(ctypes.Structure):
    _fields_ = [("candidates", ctypes.c_uint32), ("temporal_m_cap", ctypes.c_float),
                ("spatial_neighbours", ctypes.c_uint32), ("spatial_radius", ctypes.c_float)]


class CacheConfig(ctypes.Structure):
    _fields_ = [("learning_rate", ctypes.c_float), ("train_paths_per_frame", ctypes.c_uint32),
                ("terminate_depth", ctypes.c_uint32), ("seed", ctypes.c_uint32), ("spread_threshold", ctypes.c_float)]


class CacheStatus(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("pairs", ctypes.c_uint64), ("last_loss", ctypes.c_float),
                ("pad", ctypes.c_float)]


class TuneResult(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("refill_lanes", ctypes.c_uint32), ("trace_blocks_per_sm", ctypes.c_uint32),
                ("renders", ctypes.c_uint32), ("default_ms", ctypes.c_float), ("best_ms", ctypes.c_float)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("pool_paths", ctypes.c_uint32), ("round_items", ctypes.c_uint64), ("policy", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "queued", "inflight",
                                               "bytes_in_flight", "peak_bytes_in_flight", "peak_inflight",
                                               "rounds", "round_items", "gpu_busy_ns", "admit_ns", "launch_ns",
                                               "copy_out_ns", "wait_ns")]


class TraversalCounters(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("rays", "blas_nodes", "tlas_nodes", "triangles", "instances", "hits",
                                               "warp_steps", "lane_steps")]


# Every symbol declared in include/tinytrace_cuda.h: (name, restype, argtypes)
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_I32 = ctypes.c_int32
SIGNATURES = {
    "tt_abi_version": (_I32, []),
    "tt_last_error": (ctypes.c_char_p, []),
    "tt_context_create": (_I32, [_I32, ctypes.POINTER(_P)]),
    "tt_context_destroy": (_I32, [_P]),
    "tt_frame_index": (_I32, [_P, ctypes.POINTER(_U64)]),
    "tt_advance_frame": (_I32, [_P]),
    "tt_clear_lifetime": (_I32, [_P, _U32]),
    "tt_synchronize": (_I32, [_P]),
    "tt_image_create": (_I32, [_P, _U32, _U32, _U32, ctypes.POINTER(_U64)]),
    "tt_image_write": (_I32, [_P, _U64, _P, _U64]),
    "tt_image_download": (_I32, [_P, _U64, _P, _U64]),
    "tt_scene_create": (_I32, [_P, ctypes.POINTER(SceneDesc), ctypes.POINTER(_U64)]),
    "tt_scene_stats_get": (_I32, [_P, _U64, ctypes.POINTER(SceneStats)]),
    "tt_scene_bvh_download": (_I32, [_P, _U64, _P, _U64, _P, _U64, _P, _U64]),
    "tt_render": (_I32, [_P, _U64, _P, _U64]),
    "tt_render_counted": (_I32, [_P, _U64, _P, _U64, ctypes.POINTER(TraversalCounters)]),
    "tt_tonemap": (_I32, [_P, _U64, _P, _U32, _P, _U64]),
    "tt_set_option": (_I32, [_P, _U32, _U64]),
    "tt_timings_get": (_I32, [_P, ctypes.POINTER(Timings)]),
    "tt_stage_timings_get": (_I32, [_P, ctypes.POINTER(StageTimings)]),
    "tt_autotune": (_I32, [_P, _U64, _P, _U64, ctypes.POINTER(TuneResult)]),
    "tt_scene_update_instances": (_I32, [_P, _U64, _P, _U32]),
    "tt_mesh_ingest": (_I32, [_P, ctypes.POINTER(MeshData), _U32, _U32, _P, _P, _P]),
    "tt_emissive_extract": (_I32, [_P, ctypes.POINTER(EmissiveSource), _P, _U64, ctypes.POINTER(_U64)]),
    "tt_cache_configure": (_I32, [_P, ctypes.POINTER(CacheConfig)]),
    "tt_cache_query": (_I32, [_P, _P, _U32, _P]),
    "tt_cache_train": (_I32, [_P, _P, _P, _U32, _P]),
    "tt_cache_parameters": (_I32, [_P, _P, _P]),
    "tt_cache_gradients": (_I32, [_P, _P, _P, ctypes.c_uint32, _P, _P, _P]),
    "tt_cache_status_get": (_I32, [_P, ctypes.POINTER(CacheStatus)]),
    "tt_restir_configure": (_I32, [_P, ctypes.POINTER(RestirConfig)]),
    "tt_restir_reset": (_I32, [_P]),
    "tt_render_restir": (_I32, [_P, _U64, _P, _U64]),
    "tt_restir_download": (_I32, [_P, _P, _U64]),
    "tt_server_create": (_I32, [_P, ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "tt_server_destroy": (_I32, [_P]),
    "tt_server_submit": (_I32, [_P, _U64, _P, _P, _U64, ctypes.POINTER(ctypes.c_uint64)]),
    "tt_server_status": (_I32, [_P, _U64, ctypes.POINTER(_I32), ctypes.POINTER(ctypes.c_double)]),
    "tt_server_wait": (_I32, [_P, _U64, _U32, ctypes.POINTER(_I32)]),
    "tt_server_stats_get": (_I32, [_P, ctypes.POINTER(ServerStats)]),
    "tt_bsdf_eval_batch": (_I32, [_P, _P, _P, _U32, _P]),
    "tt_bsdf_sample_batch": (_I32, [_P, _P, _P, _U32, _P]),
    "tt_trace_batch": (_I32, [_P, _U64, _P, _U32, _U32, _P]),
    "tt_trace_batch_noalloc": (_I32, [_P, _U64, _P, _U32, _U32, _P]),
    "tt_math_batch": (_I32, [_P, _I32, _P, _U64, _P]),
    "tt_texture_sample_batch": (_I32, [_P, _U64, _U32, _P, _U32, _P]),
    "tt_flush_l2": (_I32, [_P]),
    "tt_event_record": (_I32, [_P, _U32]),
    "tt_event_elapsed_ms": (_I32, [_P, _U32, _U32, ctypes.POINTER(ctypes.c_float)]),
    "tt_host_alloc": (_I32, [_U64, ctypes.POINTER(_P)]),
    "tt_host_free": (_I32, [_P]),
}


class TinytraceError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"tinytrace error {code}: {message}")
        self.code = code
        self.message = message


_lib = None


def library_path() -> Path:
    return Path(os.environ.get("TINYTRACE_CUDA_LIB", LIB_PATH))


def load() -> ctypes.CDLL:
    """Loads libtinytrace_cuda.so (raising if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise TinytraceError(TT_ERR_NO_DEVICE, f"{path} is missing: run __graft_entry__.build() (no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != TT_OK:
        msg = load().tt_last_error()
        raise TinytraceError(status, msg.decode() if msg else "")


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be contiguous"
    return a.ctypes.data
