"""ctypes binding of libpmdas_gb300.so (the C ABI declared in include/mdas.h).

The library is the only compute path: if it cannot be loaded this module
raises, there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpmdas_gb300.so")

MDAS_OK = 0
MDAS_ERR_INVALID = 1
MDAS_ERR_CUDA = 2
MDAS_ERR_CAPACITY = 3
MDAS_ERR_TIMEOUT = 4
MDAS_ERR_ALLOC = 5
MDAS_ERR_STATE = 6

ARITH_REFERENCE = 0
ARITH_IEEE = 1

SCENE_DISCS_MB = 0
SCENE_DISCS_DOF = 1
SCENE_DISCS_MBDOF = 2
SCENE_DIRECT_LIGHT = 3

IMAGE_FLOAT4 = 0
IMAGE_UCHAR4 = 1

PRIM_STRIDE = 12


class MdasError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} (status {status})")


MLP_PARAMS = 5313


class LearnedConfig(C.Structure):
    _fields_ = [("tolerance", C.c_float), ("seed", C.c_uint64), ("params", C.c_void_p)]


class RenderStats(C.Structure):
    _fields_ = [("numberOfSamples", C.c_int), ("numberOfNodes", C.c_int), ("passes", C.c_int),
                ("reserved", C.c_int), ("stageMs", C.c_double * 5)]


class Config(C.Structure):
    _fields_ = [("mdas", C.c_int), ("samples", C.c_float), ("scaleFactor", C.c_float), ("alpha", C.c_float),
                ("bitsPerDim", C.c_int), ("extraImgBits", C.c_int), ("candidatesNum", C.c_int),
                ("width", C.c_int), ("height", C.c_int), ("focalDistance", C.c_float),
                ("lensRadius", C.c_float), ("fovy", C.c_float), ("sceneKind", C.c_int), ("sceneCount", C.c_int),
                ("sceneSeed", C.c_int64), ("filmFilename", C.c_char * 256)]


_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_FP = C.POINTER(C.c_float)

# name -> (restype, argtypes)
SIGNATURES = {
    "mdas_create": (_I, [C.POINTER(_P), _I, _I, _I, _I, _I, _F, _F, _F, C.c_char_p]),
    "mdas_create_ex": (_I, [C.POINTER(_P), _I, _I, _I, _I, _I, _F, _F, _F, C.c_char_p, _I, _P]),
    "mdas_destroy": (_I, [_P]),
    "mdas_set_stream": (_I, [_P, _P]),
    "mdas_initial_sampling": (_I, [_P]),
    "mdas_compute_errors": (_I, [_P]),
    "mdas_adaptive_sampling": (_I, [_P]),
    "mdas_sampling_pass": (_I, [_P]),
    "mdas_integrate": (_I, [_P, _P, _I, _I]),
    "mdas_convert_to_bytes": (_I, [_P, _P, _P, _I, _I]),
    "mdas_sampling_density": (_I, [_P, _P, _I, _I]),
    "mdas_sampling_density_device": (_I, [_P, _P, _I, _I]),
    "mdas_validate": (_I, [_P, C.POINTER(_I)]),
    "mdas_sample_coordinates": (_P, [_P]),
    "mdas_sample_values": (_P, [_P]),
    "mdas_get_counts": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "mdas_get_info": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), _FP, _FP,
                           C.POINTER(_I)]),
    "mdas_get_gerror": (_I, [_P, _FP]),
    "mdas_dump_state": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "mdas_load_state": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P]),
    "mdas_adaptive_sampling_static": (_I, [_I, _I, _I, _I, _F, _F, _I, _I, _P, _P, _P, _P, _P, C.POINTER(_I),
                                           C.POINTER(_I), _P]),
    "mdas_set_timing": (_I, [_P, _I]),
    "mdas_get_stage_times": (_I, [_P, C.POINTER(C.c_double), _I]),
    "mdas_get_stage_times_ex": (_I, [_P, C.POINTER(C.c_double), _I, _I]),
    "mdas_test_set_wait_limit": (_I, [_I]),
    "mdas_get_launch_count": (_I, [_P, C.POINTER(C.c_uint64)]),
    "mdas_get_pass_stats": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_int64)]),
    "mdas_save_image": (_I, [C.c_char_p, _P, _I, _I, _I]),
    "mdas_status_string": (C.c_char_p, [_I]),
    "mdas_scene_create": (_I, [C.POINTER(_P), _I, C.c_uint64, _I, _F, _F, _I, _I]),
    "mdas_scene_destroy": (_I, [_P]),
    "mdas_scene_desc_size": (_I, []),
    "mdas_scene_export": (_I, [_P, _P, _I, _P, _I, C.POINTER(_I), C.POINTER(_I)]),
    "mdas_evaluate": (_I, [_P, _P, _I, _I]),
    "mdas_scene_evaluate": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "mdas_scene_reference_image": (_I, [_P, _I, _I, _I, C.c_uint64, _P, _P]),
    "mdas_render": (_I, [_P, _P, _I, _P, _I, _I, C.POINTER(RenderStats)]),
    "mdas_render_host": (_I, [_P, _P, _P, _I, _P, _I, _I, C.POINTER(RenderStats)]),
    "mdas_render_graph": (_I, [_P, _P, _I, _P, _I, _I, C.POINTER(RenderStats)]),
    "mdas_batch_create": (_I, [C.POINTER(_P), _I, C.POINTER(_P), C.POINTER(_P), C.POINTER(_I), C.POINTER(_P),
                               C.POINTER(_I), C.POINTER(_I)]),
    "mdas_batch_destroy": (_I, [_P]),
    "mdas_batch_render": (_I, [_P, C.POINTER(RenderStats)]),
    "mdas_batch_render_stepped": (_I, [_P, C.POINTER(RenderStats)]),
    "mdas_batch_set_tuning": (_I, [_P, C.POINTER(_I)]),
    "mdas_batch_autotune": (_I, [_P, _I, C.POINTER(_I), C.POINTER(C.c_double)]),
    "mdas_batch_set_tiling": (_I, [_P, C.POINTER(_I), _I]),
    "mdas_batch_autotune_ex": (_I, [_P, _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_double), C.POINTER(_I)]),
    "mdas_morton_key_bits": (_I, [_I, _I, _I, _I]),
    "mdas_morton_encode": (_I, [_I, _I, _I, _I, _F, _F, _P, _I, _P, _P]),
    "mdas_morton_decode": (_I, [_I, _I, _I, _F, _F, _P, _I, _P, _P]),
    "mdas_radix_sort_pairs": (_I, [_P, C.POINTER(C.c_size_t), _P, _P, _P, _P, _I, _I, _I, _P]),
    "mdas_leaf_order": (_I, [_P, _I, _P, _P]),
    "mdas_build_hierarchy": (_I, [_P, _I]),
    "mdas_get_hierarchy": (_I, [_P, C.POINTER(_I), _P, _P, _P, _P, _P]),
    "mdas_locate": (_I, [_P, _P, _I, _P]),
    "mdas_learned_defaults": (_I, [C.POINTER(LearnedConfig)]),
    "mdas_learned_enable": (_I, [_P, C.POINTER(LearnedConfig)]),
    "mdas_learned_update": (_I, [_P]),
    "mdas_learned_predict": (_I, [_P]),
    "mdas_learned_stats": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_double),
                                C.POINTER(C.c_double)]),
    "mdas_leaf_true_errors": (_I, [_P, _P, _I, C.c_uint64, _P, _I, _P]),
    "mdas_mlp_adam": (_I, [_P, _P, _P, _P, _I, _F, _P]),
    "mdas_learned_get_params": (_I, [_P, _P]),
    "mdas_learned_set_params": (_I, [_P, _P]),
    "mdas_learned_pred_max": (_I, [_P, C.POINTER(C.c_float)]),
    "mdas_learned_predictions": (_I, [_P, _P]),
    "mdas_leaf_features": (_I, [_P, _P]),
    "mdas_mlp_forward": (_I, [_P, _P, _I, _P, _P]),
    "mdas_mlp_gradients": (_I, [_P, _P, _P, _I, _P, C.POINTER(_F), _P]),
    "mdas_config_defaults": (_I, [C.POINTER(Config)]),
    "mdas_config_read": (_I, [C.c_char_p, C.POINTER(Config), C.c_char_p, _I]),
}

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load the native library (once).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libpmdas_gb300 is not built ({p} missing); run `python -m pmdas_gb300.build`")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().mdas_status_string(status).decode()
    except Exception:  # pragma: no cover - only for error messages
        return "unknown"


def check(status: int, what: str) -> None:
    if status != MDAS_OK:
        raise MdasError(status, what)
