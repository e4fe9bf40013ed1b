"""ctypes binding of libcraystal_gb300.so (declarations in include/craystal_c.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared library has not been built.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libcraystal_gb300.so")

CR_OK = 0
CR_ERR_INVALID_ARGUMENT = 1
CR_ERR_CUDA = 2
CR_ERR_OUT_OF_MEMORY = 3
CR_ERR_DEVICE = 4
CR_ERR_UNSUPPORTED = 5
CR_DEVICE_ERROR_STACK_OVERFLOW = 1
CR_MISS = 0xFFFFFFFF
CR_NOALLOC_MAX_RAYS = 65536
CR_NO_TEXTURE = 0xFFFFFFFF
CR_TRAVERSAL_ONE_LEVEL = 0
CR_TRAVERSAL_TWO_LEVEL = 1

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
MATERIAL_DTYPE = np.dtype([("diffuse", "<f4", 3), ("specular", "<f4", 3), ("emission", "<f4", 3),
                           ("shininess", "<f4"), ("type", "<u4"), ("flags", "<u4")])
MESH_DTYPE = np.dtype([("index_offset", "<u4"), ("index_count", "<u4"), ("vertex_offset", "<u4"),
                       ("material_id", "<u4")])
SPHERE_DTYPE = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("material", "<u4"), ("pad", "<u4", 3)])
CR_SPHERE_BIT = 0x80000000
SPHERE_LIGHT_DTYPE = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("emission", "<f4", 3), ("pad", "<f4")])
BVH_NODE_DTYPE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("is_leaf", "<u4"), ("a", "<u4"), ("b", "<u4")])


class CrCamera(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_float * 3), ("target", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov_y", ctypes.c_float), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class CrTexture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("texels", ctypes.POINTER(ctypes.c_float))]


class CrMeshDescC(ctypes.Structure):
    _fields_ = [("index_offset", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("vertex_offset", ctypes.c_uint32), ("material_id", ctypes.c_uint32)]


class CrImportView(ctypes.Structure):
    _fields_ = [("pos", ctypes.POINTER(ctypes.c_float)), ("nrm", ctypes.POINTER(ctypes.c_float)),
                ("uv", ctypes.POINTER(ctypes.c_float)), ("n_vertices", ctypes.c_uint64),
                ("idx", ctypes.POINTER(ctypes.c_uint32)), ("n_tris", ctypes.c_uint64),
                ("meshes", ctypes.c_void_p), ("n_meshes", ctypes.c_uint32),
                ("mats", ctypes.c_void_p), ("material_texture", ctypes.POINTER(ctypes.c_uint32)),
                ("n_mats", ctypes.c_uint32), ("emissive", ctypes.POINTER(ctypes.c_uint32)),
                ("n_emissive", ctypes.c_uint32), ("textures", ctypes.POINTER(CrTexture)),
                ("n_textures", ctypes.c_uint32), ("camera", CrCamera)]


class CrImage(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("channels", ctypes.c_uint32),
                ("pixels", ctypes.POINTER(ctypes.c_float))]


class CrIntegratorConfig(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_uint32), ("rr_threshold", ctypes.c_float), ("use_mis", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class CrBvhStats(ctypes.Structure):
    _fields_ = [("node_count", ctypes.c_uint32), ("leaf_count", ctypes.c_uint32), ("max_depth", ctypes.c_uint32),
                ("max_leaf_size", ctypes.c_uint32), ("max_leaf_depth", ctypes.c_uint32),
                ("levels", ctypes.c_uint32), ("root_min", ctypes.c_float * 3), ("root_max", ctypes.c_float * 3),
                ("build_ms", ctypes.c_double), ("device_bytes", ctypes.c_uint64)]


class CrMlpConfig(ctypes.Structure):
    _fields_ = [("lr", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float), ("eps", ctypes.c_float),
                ("seed", ctypes.c_uint32)]


class CrCacheConfig(ctypes.Structure):
    _fields_ = [("query_vertex", ctypes.c_uint32), ("train_every", ctypes.c_uint32),
                ("train_samples", ctypes.c_uint32), ("train_steps", ctypes.c_uint32), ("freeze", ctypes.c_uint32),
                ("scene_min", ctypes.c_float * 3), ("scene_max", ctypes.c_float * 3)]


class CrCacheStats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_uint64), ("queries", ctypes.c_uint64), ("train_records", ctypes.c_uint64),
                ("last_loss", ctypes.c_float), ("last_train_every", ctypes.c_uint32)]


class CrBatchItem(ctypes.Structure):
    _fields_ = [("config", CrIntegratorConfig), ("spp", ctypes.c_uint32), ("first_sample", ctypes.c_uint32)]


class CrBatchTuning(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_uint32), ("spp_per_item", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("wave_log2", ctypes.c_uint32)]


class CrBatchTuningResult(ctypes.Structure):
    _fields_ = [("tuning", CrBatchTuning), ("ms", ctypes.c_float)]


class CrayError(RuntimeError):
    """Raised for a non-zero status of the C ABI (the reference throws
    RuntimeError from CRAYSTAL_CHECK / CRAYSTAL_CUDA_CHECK)."""

    def __init__(self, code, msg):
        super().__init__(f"craystal_gb300 error {code}: {msg}")
        self.code = code


# (name, restype, argtypes)
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
SIGNATURES = [
    ("cr_last_error", ctypes.c_char_p, []),
    ("cr_version", ctypes.c_char_p, []),
    ("cr_set_device", ctypes.c_int, [ctypes.c_int]),
    ("cr_scene_create", ctypes.c_int, [_P, _P, _P, _U64, _P, _U64, _P, _U32, _P, _U32, _P, _U32,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    ("cr_scene_destroy", ctypes.c_int, [_P]),
    ("cr_scene_bvh_stats", ctypes.c_int, [_P, ctypes.POINTER(CrBvhStats)]),
    ("cr_scene_bvh_export", ctypes.c_int, [_P, _P, _P]),
    ("cr_scene_bvh_import", ctypes.c_int, [_P, _P, _U32, _P]),
    ("cr_scene_check_errors", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    ("cr_scene_set_error_flags", ctypes.c_int, [_P, _U32]),
    ("cr_scene_set_traversal", ctypes.c_int, [_P, _U32]),
    ("cr_scene_set_camera", ctypes.c_int, [_P, ctypes.POINTER(CrCamera)]),
    ("cr_scene_set_environment", ctypes.c_int, [_P, _P]),
    ("cr_scene_set_sphere_lights", ctypes.c_int, [_P, _P, _U32]),
    ("cr_scene_set_spheres", ctypes.c_int, [_P, _P, _U32]),
    ("cr_scene_set_diffuse_textures", ctypes.c_int, [_P, ctypes.POINTER(CrTexture), _U32, _P, _U32]),
    ("cr_texture_sample", ctypes.c_int, [_P, _U32, _P, _U64, _P]),
    ("cr_film_clear", ctypes.c_int, [_P]),
    ("cr_film_read", ctypes.c_int, [_P, _P, _P]),
    ("cr_film_resolve", ctypes.c_int, [_P, _P]),
    ("cr_render", ctypes.c_int, [_P, ctypes.POINTER(CrIntegratorConfig), _U32, _U32, _P]),
    ("cr_render_ray_count", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    ("cr_trace_closest", ctypes.c_int, [_P, _P, _U64, _P]),
    ("cr_trace_closest_device", ctypes.c_int, [_P, _P, _U64, _P, _P]),
    ("cr_trace_occluded", ctypes.c_int, [_P, _P, _U64, _P]),
    ("cr_trace_occluded_device", ctypes.c_int, [_P, _P, _U64, _P, _P]),
    ("cr_camera_generate_rays", ctypes.c_int, [ctypes.POINTER(CrCamera), _P, _U64, _P]),
    ("cr_bsdf_evaluate", ctypes.c_int, [_P, _P, _P, _P, _U64, _P, _P]),
    ("cr_bsdf_sample", ctypes.c_int, [_P, _P, _P, _P, _U64, _P, _P, _P]),
    ("cr_trace_closest_noalloc", ctypes.c_int, [_P, _P, _U64, _P, _P]),
    ("cr_mlp_param_count", ctypes.c_uint64, []),
    ("cr_mlp_create", ctypes.c_int, [ctypes.POINTER(CrMlpConfig), ctypes.POINTER(ctypes.c_void_p)]),
    ("cr_mlp_destroy", ctypes.c_int, [_P]),
    ("cr_mlp_get_params", ctypes.c_int, [_P, _P]),
    ("cr_mlp_set_params", ctypes.c_int, [_P, _P]),
    ("cr_mlp_infer", ctypes.c_int, [_P, _P, _U64, _P]),
    ("cr_mlp_gradients", ctypes.c_int, [_P, _P, _P, _U64, _P, _P]),
    ("cr_mlp_train_step", ctypes.c_int, [_P, _P, _P, _U64, _P]),
    ("cr_mlp_infer_device", ctypes.c_int, [_P, _P, _U64, _P, _P]),
    ("cr_mlp_train_step_device", ctypes.c_int, [_P, _P, _P, _U64, _P]),
    ("cr_render_cached", ctypes.c_int, [_P, ctypes.POINTER(CrIntegratorConfig), ctypes.POINTER(CrCacheConfig), _P,
                                        _U32, _U32, _P, ctypes.POINTER(CrCacheStats)]),
    ("cr_batch_create", ctypes.c_int, [_P, _P, _U32, ctypes.POINTER(ctypes.c_void_p)]),
    ("cr_batch_destroy", ctypes.c_int, [_P]),
    ("cr_batch_set_tuning", ctypes.c_int, [_P, ctypes.POINTER(CrBatchTuning)]),
    ("cr_batch_get_tuning", ctypes.c_int, [_P, ctypes.POINTER(CrBatchTuning)]),
    ("cr_batch_render", ctypes.c_int, [_P, _P]),
    ("cr_batch_render_cached", ctypes.c_int, [_P, _P, ctypes.POINTER(CrCacheConfig), _P]),
    ("cr_batch_autotune", ctypes.c_int, [_P, ctypes.POINTER(CrBatchTuning), _P, _U32,
                                         ctypes.POINTER(ctypes.c_uint32)]),
    ("cr_kernel_launch_count", ctypes.c_uint64, []),
    ("cr_device_read_bandwidth", ctypes.c_int, [_U64, _U32, ctypes.POINTER(ctypes.c_double)]),
    ("cr_import_xml", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("cr_import_get", ctypes.c_int, [_P, ctypes.POINTER(CrImportView)]),
    ("cr_import_material_name", ctypes.c_char_p, [_P, _U32]),
    ("cr_import_create_scene", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_void_p)]),
    ("cr_import_destroy", ctypes.c_int, [_P]),
    ("cr_image_load", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(CrImage)]),
    ("cr_image_free", ctypes.c_int, [ctypes.POINTER(CrImage)]),
    ("cr_image_write_exr", ctypes.c_int, [ctypes.c_char_p, _U32, _U32, _U32, _P]),
    ("cr_image_write_png", ctypes.c_int, [ctypes.c_char_p, _U32, _U32, _U32, _P, ctypes.c_int]),
]

_lib = None


def load(path: str = LIB_PATH):
    """Loads the shared library (once) and declares every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(craystal_gb300 has no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int):
    if code != CR_OK:
        raise CrayError(code, load().cr_last_error().decode())


def ptr(a) -> int:
    """Address of a numpy array (or None -> NULL)."""
    if a is None:
        return None
    return a.ctypes.data
