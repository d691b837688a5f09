"""ctypes mirror of include/pgx.h and the loader for libpgx.so.

The structures below are numpy dtypes with the exact byte layout of the C
structs, so arrays of them can be handed to the C ABI without copies.
Loading fails loudly when the library has not been built: there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libpgx.so"

# ---- status codes (pgx.h) ------------------------------------------------------
PGX_OK = 0
PGX_ERR_INVALID_ARG = 1
PGX_ERR_OOM = 2
PGX_ERR_CUDA = 3
PGX_ERR_OVERFLOW = 4
PGX_ERR_TIMEOUT = 5
PGX_ERR_STATE = 6
NOALLOC_MAX_RAYS = 65536  # PGX_NOALLOC_MAX_RAYS

MLP_PARAMS = 24424   # PGX_MLP_PARAMS
MLP_OUTPUTS = 40     # PGX_MLP_OUTPUTS
RENDER_TRAIN_GUIDE = 4
# pgx_radiance_sample: position, normal, wo, wi, weight
RADIANCE_SAMPLE = np.dtype([("position", "<f4", 3), ("normal", "<f4", 3), ("wo", "<f4", 3), ("wi", "<f4", 3),
                            ("weight", "<f4")])

# BSDF kinds
BSDF_DIFFUSE, BSDF_MIRROR, BSDF_CONDUCTOR, BSDF_GLASS, BSDF_DIELECTRIC, BSDF_ORENNAYAR, BSDF_PLASTIC = range(7)
# render modes
MODE_PLAIN, MODE_GUIDED_LI, MODE_GUIDED_QUADTREE, MODE_GUIDED_MLP, MODE_GUIDED_PSS = 0, 1, 2, 3, 4

# ---- numpy layouts of the C structs ---------------------------------------------
VERTEX = np.dtype([("p", "<f4", 3), ("n", "<f4", 3), ("u", "<f4"), ("v", "<f4")])
TRIANGLE = np.dtype([("v", VERTEX, 3), ("material", "<u4")])
MATERIAL = np.dtype([
    ("kind", "<i4"), ("albedo_texture", "<i4"), ("albedo", "<f4", 3), ("eta", "<f4", 3), ("k", "<f4", 3),
    ("int_ior", "<f4"), ("ext_ior", "<f4"), ("roughness", "<f4"), ("sigma", "<f4"), ("emission", "<f4", 3),
    ("layered", "<i4"),
])
RAY = np.dtype([("o", "<f4", 3), ("tmax", "<f4"), ("d", "<f4", 3), ("pad", "<f4")])
HIT = np.dtype([("id", "<i4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
BVH_NODE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left_first", "<i4"), ("used", "<i4")])
PATH_VERTEX = np.dtype([("position", "<f4", 3), ("normal", "<f4", 3), ("wi", "<f4", 3), ("Li", "<f4", 3)])
CACHE_NODE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left", "<i4"), ("right", "<i4"),
                       ("offset", "<i4"), ("used", "<i4")])
GUIDE_REGION = np.dtype([("first", "<i4"), ("count", "<i4"), ("node", "<i4"), ("qroot", "<i4")])
QUAD_NODE = np.dtype([("flux", "<f4", 4), ("child", "<i4", 4)])
GUIDE_MAX_QUAD_NODES = 256

assert VERTEX.itemsize == 32 and TRIANGLE.itemsize == 100 and MATERIAL.itemsize == 76
assert RAY.itemsize == 32 and HIT.itemsize == 16 and BVH_NODE.itemsize == 32
assert PATH_VERTEX.itemsize == 48 and CACHE_NODE.itemsize == 40


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.c_void_p)]


class Camera(C.Structure):
    _fields_ = [("from_", C.c_float * 3), ("to", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_degrees", C.c_float), ("width", C.c_int32), ("height", C.c_int32), ("flip_x", C.c_int32)]


class SceneData(C.Structure):
    """pgx_scene_data (include/pgx.h)."""
    _fields_ = [("triangles", C.c_void_p), ("ntris", C.c_int64), ("materials", C.c_void_p), ("nmats", C.c_int32),
                ("textures", C.c_void_p), ("ntextures", C.c_int32), ("has_env", C.c_int32), ("env", Texture),
                ("camera", Camera), ("internal", C.c_void_p)]


class BvhStats(C.Structure):
    _fields_ = [("nodes", C.c_int64), ("leaves", C.c_int64), ("max_depth", C.c_int32),
                ("max_leaf_size", C.c_int32), ("sah_cost", C.c_double), ("build_ms", C.c_double)]


RENDER_PROFILE = 1
RENDER_TIMING = 8
RENDER_FILTER_MITCHELL = 2


class RenderConfig(C.Structure):
    _fields_ = [("mode", C.c_int32), ("max_depth", C.c_int32), ("seed", C.c_uint64),
                ("guide_fraction", C.c_float), ("record_paths", C.c_int32), ("flags", C.c_int32),
                ("guide_depth", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("extension_rays", C.c_int64), ("shadow_rays", C.c_int64),
                ("path_vertices", C.c_int64), ("kernel_launches", C.c_int64), ("extend_launches", C.c_int64),
                ("extend_interior_visits", C.c_int64), ("extend_tri_tests", C.c_int64),
                ("shadow_interior_visits", C.c_int64), ("shadow_tri_tests", C.c_int64),
                ("ms_total", C.c_double), ("ms_extend", C.c_double), ("ms_shadow", C.c_double),
                ("ms_shade", C.c_double), ("guide_fallbacks", C.c_int64)]


class CacheStats(C.Structure):
    _fields_ = [("records", C.c_int64), ("nodes", C.c_int64), ("leaves", C.c_int64),
                ("min_leaf_depth", C.c_int32), ("max_leaf_depth", C.c_int32),
                ("mean_leaf_depth", C.c_double), ("build_ms", C.c_double)]


class GuideParams(C.Structure):
    _fields_ = [("region_records", C.c_int32), ("refine_fraction", C.c_float), ("clamp_median", C.c_float),
                ("uniform_share", C.c_float), ("compensate", C.c_float), ("glossy_alpha", C.c_float)]


class BatchTuning(C.Structure):
    _fields_ = [("wave_paths", C.c_int64), ("trace_blocks_per_sm", C.c_int32), ("shade_blocks_per_sm", C.c_int32),
                ("stack_shared", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("ms", C.c_double), ("graph_replayed", C.c_int32)]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32

# name -> (restype, argtypes); every function declared in include/pgx.h.
SIGNATURES = {
    "pgx_create": (C.c_int, [_I32, C.POINTER(_P)]),
    "pgx_destroy": (C.c_int, [_P]),
    "pgx_last_error": (C.c_char_p, [_P]),
    "pgx_version": (C.c_char_p, []),
    "pgx_scene_upload": (C.c_int, [_P, _P, _I64, _P, _I32, _P, _I32, _P, _P]),
    "pgx_bvh_build": (C.c_int, [_P]),
    "pgx_bvh_import": (C.c_int, [_P, _P, _I64, _P]),
    "pgx_bvh_export": (C.c_int, [_P, _P, C.POINTER(_I64), _P, C.POINTER(_I64)]),
    "pgx_bvh_get_stats": (C.c_int, [_P, C.POINTER(BvhStats)]),
    "pgx_trace_closest": (C.c_int, [_P, _P, _I64, _P]),
    "pgx_trace_any": (C.c_int, [_P, _P, _I64, _P]),
    "pgx_trace_closest_noalloc": (C.c_int, [_P, _P, _I64, _P]),
    "pgx_trace_closest_device": (C.c_int, [_P, _P, _I64, _P, _P]),
    "pgx_trace_any_device": (C.c_int, [_P, _P, _I64, _P, _P]),
    "pgx_trace_counters": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    "pgx_camera_rays": (C.c_int, [_P, _P, _P, _I64, _P]),
    "pgx_set_camera": (C.c_int, [_P, C.POINTER(Camera)]),
    "pgx_render": (C.c_int, [_P, C.POINTER(RenderConfig), _I32]),
    "pgx_clear": (C.c_int, [_P]),
    "pgx_get_spp": (C.c_int, [_P, C.POINTER(_I32)]),
    "pgx_film_read": (C.c_int, [_P, _P, _P, C.POINTER(_I32)]),
    "pgx_render_get_stats": (C.c_int, [_P, C.POINTER(RenderStats)]),
    "pgx_film_tonemap": (C.c_int, [_P, C.c_float, C.c_float, _P]),
    "pgx_bsdf_sample_batch": (C.c_int, [_P, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "pgx_bsdf_invert_batch": (C.c_int, [_P, _P, _P, _P, _P, _I64, _P]),
    "pgx_cache_build": (C.c_int, [_P, _P, _I64]),
    "pgx_cache_build_from_render": (C.c_int, [_P]),
    "pgx_cache_get_stats": (C.c_int, [_P, C.POINTER(CacheStats)]),
    "pgx_cache_export": (C.c_int, [_P, _P, C.POINTER(_I64), _P, C.POINTER(_I64)]),
    "pgx_cache_export_weights": (C.c_int, [_P, _P, C.POINTER(_I64)]),
    "pgx_cache_knn": (C.c_int, [_P, _P, _I64, _I32, _P, _P]),
    "pgx_guide_pdf": (C.c_int, [_P, _P, _P, _I64, _P]),
    "pgx_guide_sample": (C.c_int, [_P, _P, _P, _I64, _P, _P]),
    "pgx_guide_export": (C.c_int, [_P, _P, C.POINTER(_I32), _P, C.POINTER(_I32)]),
    "pgx_guide_configure": (C.c_int, [_P, C.POINTER(GuideParams)]),
    "pgx_guide_get_params": (C.c_int, [_P, C.POINTER(GuideParams)]),
    "pgx_mlp_init": (C.c_int, [_P, C.c_uint64, _P, _P]),
    "pgx_mlp_get_params": (C.c_int, [_P, _P]),
    "pgx_mlp_set_params": (C.c_int, [_P, _P]),
    "pgx_mlp_forward": (C.c_int, [_P, _P, _I64, _P]),
    "pgx_mlp_pdf": (C.c_int, [_P, _P, _P, _I64, _P]),
    "pgx_mlp_sample": (C.c_int, [_P, _P, _P, _I64, _P, _P]),
    "pgx_mlp_gradient": (C.c_int, [_P, _P, _I64, _P, C.POINTER(C.c_double)]),
    "pgx_mlp_train_step": (C.c_int, [_P, _P, _I64, C.c_float, C.POINTER(C.c_double)]),
    "pgx_mlp_configure": (C.c_int, [_P, C.c_float, C.c_float, _I64, _I32, _I32]),
    "pgx_mlp_set_fallback": (C.c_int, [_P, _I32]),
    "pgx_diff_set_params": (C.c_int, [_P, _P, _P, _P]),
    "pgx_diff_render": (C.c_int, [_P, _I32, C.c_uint64, _I32, _P]),
    "pgx_diff_adjoint": (C.c_int, [_P, _I32, C.c_uint64, _I32, _P, _P, _P, _P]),
    "pgx_batch_create": (C.c_int, [_P, _I32, C.POINTER(_P)]),
    "pgx_batch_destroy": (C.c_int, [_P]),
    "pgx_batch_render": (C.c_int, [_P, _I32, C.c_uint64, _I32]),
    "pgx_batch_autotune": (C.c_int, [_P, _I32, _I32, C.POINTER(BatchTuning)]),
    "pgx_batch_set_tuning": (C.c_int, [_P, C.POINTER(BatchTuning)]),
    "pgx_batch_get_stats": (C.c_int, [_P, C.POINTER(BatchStats)]),
    "pgx_batch_last_error": (C.c_char_p, [_P]),
    "pgx_image_decode_jpeg": (C.c_int, [_P, _I64, _P, _P, _P, _P, _I64, _P, _I32]),
    "pgx_scene_read": (C.c_int, [C.c_char_p, C.POINTER(C.POINTER(SceneData)), _P, _I32]),
    "pgx_scene_data_free": (None, [C.POINTER(SceneData)]),
    "pgx_scene_load": (C.c_int, [_P, C.c_char_p]),
}

_lib: C.CDLL | None = None


def load(path: str | Path | None = None) -> C.CDLL:
    """Load libpgx.so (built by ``pathguidingdissertation_gb300.build``).

    Raises if the library is missing — the package has no CPU path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"libpgx not built ({p} missing): run pathguidingdissertation_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class PgxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pgx error {code}: {msg}")
        self.code = code


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data
