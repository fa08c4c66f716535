"""ctypes view of include/akua_pbf.h and the loader of the in-tree CUDA library."""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libakua_pbf.so")

AKUA_OK = 0
AKUA_ERR_INVALID_ARGUMENT = -1
AKUA_ERR_CUDA = -2
AKUA_ERR_OUT_OF_MEMORY = -3
AKUA_ERR_NOT_ATTACHED = -4
AKUA_ERR_DEVICE_CHECK = -5
AKUA_ERR_TOO_LARGE = -6
AKUA_ERR_CORRUPT = -7

OPT_EXACT_MATH = 0x1
OPT_RESIDENT = 0x2
OPT_NO_GRAPH = 0x4

MLP_INPUTS = 8
MLP_HIDDEN = 64
MLP_PARAMS = 8961
MLP_NORM = 18

STATE_LAMBDA_SUMS = 0x1

DEBUG_HASHES = 1
DEBUG_ORDER = 2
DEBUG_NEIGHBOUR_COUNTS = 3
DEBUG_NEIGHBOURS = 4
DEBUG_PARTICLES = 5
DEBUG_LAMBDA_SUMS = 6

FLAG_CAP_REACHED = 1
FLAG_BAD_TABLE = 2


class CConfig(ctypes.Structure):
    """akua_pbf_config == AkuaEngine::PBFConfig (PBFConfig.h:18-29)."""

    _fields_ = [
        ("restDensity", ctypes.c_float),
        ("particle_spacing", ctypes.c_float),
        ("smoothRadius", ctypes.c_float),
        ("spatialHashCellSize", ctypes.c_float),
        ("relaxation", ctypes.c_float),
        ("vorticityEpsilon", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("maxNeighbours", ctypes.c_int32),
        ("solverIterations", ctypes.c_int32),
        ("gravity", ctypes.c_float * 3),
    ]


class CCorr(ctypes.Structure):
    """akua_lambda_corr_params == AkuaEngine::LambdaCorrParams (PBFConfig.h:10-15)."""

    _fields_ = [
        ("enabled", ctypes.c_int32),
        ("k", ctypes.c_float),
        ("n", ctypes.c_float),
        ("delta_q", ctypes.c_float),
    ]


class CSceneDesc(ctypes.Structure):
    _fields_ = [("numParticles", ctypes.c_int32), ("gravity", ctypes.c_float * 3),
                ("boxMin", ctypes.c_float * 3), ("boxMax", ctypes.c_float * 3)]


class CStateHeader(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_char * 8), ("version", ctypes.c_uint32),
                ("recordBytes", ctypes.c_uint32), ("numParticles", ctypes.c_int64),
                ("step", ctypes.c_int64), ("config", CConfig), ("corr", CCorr),
                ("boxMin", ctypes.c_float * 3), ("boxMax", ctypes.c_float * 3),
                ("deltaTime", ctypes.c_float), ("tableSize", ctypes.c_uint32),
                ("sections", ctypes.c_uint32), ("numScenes", ctypes.c_int32),
                ("crc32", ctypes.c_uint32), ("options", ctypes.c_uint32),
                ("reserved", ctypes.c_uint8 * 112)]


class CCamera(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("gaze", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("fovDegrees", ctypes.c_float),
                ("nearZ", ctypes.c_float), ("farZ", ctypes.c_float)]


class CSdfShape(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("a", ctypes.c_float * 3), ("b", ctypes.c_float * 3),
                ("radius", ctypes.c_float)]


SDF_SPHERE, SDF_BOX, SDF_CAPSULE, SDF_PLANE = 1, 2, 3, 4


class CStats(ctypes.Structure):
    _fields_ = [
        ("numParticles", ctypes.c_int32),
        ("tableSize", ctypes.c_int32),
        ("maxNeighbours", ctypes.c_int32),
        ("solverIterations", ctypes.c_int32),
        ("steps", ctypes.c_int64),
        ("deviceFlags", ctypes.c_uint32),
        ("graphCaptures", ctypes.c_int32),
        ("deviceBytes", ctypes.c_uint64),
    ]


class CKernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 40), ("launches", ctypes.c_int32), ("total_ms", ctypes.c_double)]


# AkuaEngine::Particle (Particle.h:8-31): 108 bytes, 4-byte aligned.
PARTICLE_DTYPE = np.dtype(
    [
        ("position", "<f4", (3,)),
        ("velocity", "<f4", (3,)),
        ("new_position", "<f4", (3,)),
        ("new_velocity", "<f4", (3,)),
        ("position_delta", "<f4", (3,)),
        ("vorticity", "<f4", (3,)),
        ("mass", "<f4"),
        ("density", "<f4"),
        ("lambda", "<f4"),
        ("hash", "<u4"),
        ("color", "<f4", (4,)),
        ("size", "<f4"),
    ]
)
assert PARTICLE_DTYPE.itemsize == 108

# Every symbol include/akua_pbf.h declares, with (restype, argtypes).
_P = ctypes.c_void_p
_SIGS = {
    "akua_pbf_default_config": (None, [ctypes.POINTER(CConfig), ctypes.POINTER(CCorr)]),
    "akua_pbf_create": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(CConfig),
                                       ctypes.POINTER(CCorr), ctypes.POINTER(_P)]),
    "akua_pbf_destroy": (ctypes.c_int, [_P]),
    "akua_pbf_attach_particles": (ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    "akua_pbf_step": (ctypes.c_int, [_P, ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(ctypes.c_float)]),
    "akua_pbf_step_host": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.c_float,
                                          ctypes.POINTER(ctypes.c_float),
                                          ctypes.POINTER(ctypes.c_float)]),
    "akua_pbf_set_gravity": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float)]),
    "akua_pbf_set_boundary_damping": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float]),
    "akua_pbf_set_table_size": (ctypes.c_int, [_P, ctypes.c_int32]),
    "akua_pbf_set_stream": (ctypes.c_int, [_P, _P]),
    "akua_pbf_set_options": (ctypes.c_int, [_P, ctypes.c_uint32]),
    "akua_pbf_synchronize": (ctypes.c_int, [_P]),
    "akua_pbf_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(CStats)]),
    "akua_pbf_read_debug": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_size_t]),
    "akua_pbf_kernels_per_step": (ctypes.c_int, [_P]),
    "akua_pbf_profile_begin": (ctypes.c_int, [_P, ctypes.c_int32]),
    "akua_pbf_profile_end": (ctypes.c_int, [_P, ctypes.POINTER(CKernelTime), ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_int32)]),
    "akua_sort_pairs_noalloc": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int32, ctypes.c_int32, _P]),
    "akua_pbf_set_solver_iterations": (ctypes.c_int, [_P, ctypes.c_int32]),
    "akua_pbf_set_pair_blocks": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
    "akua_pbf_get_pair_blocks": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
    "akua_pbf_set_search_shape": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "akua_pbf_get_search_shape": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32),
                                                 ctypes.POINTER(ctypes.c_int32)]),
    "akua_pbf_autotune": (ctypes.c_int, [_P, ctypes.c_float, _P, _P, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32)]),
    "akua_pbf_set_sdf_shapes": (ctypes.c_int, [_P, ctypes.POINTER(CSdfShape), ctypes.c_int32,
                                               ctypes.c_float, ctypes.c_float]),
    "akua_camera_default": (None, [ctypes.POINTER(CCamera)]),
    "akua_camera_matrices": (ctypes.c_int, [ctypes.POINTER(CCamera), ctypes.c_float, _P, _P, _P]),
    "akua_splat_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_P)]),
    "akua_splat_destroy": (ctypes.c_int, [_P]),
    "akua_splat_render": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.c_int32,
                                         ctypes.POINTER(CCamera), _P, _P]),
    "akua_state_init_header": (None, [ctypes.POINTER(CStateHeader)]),
    "akua_state_save": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CStateHeader), _P, _P, _P]),
    "akua_state_read_header": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CStateHeader)]),
    "akua_state_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CStateHeader), _P,
                                       ctypes.c_int64, _P, _P, ctypes.c_int32]),
    "akua_pbf_set_lambda_sums": (ctypes.c_int, [_P, _P, ctypes.c_int64]),
    "akua_pbf_create_batch": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(CSceneDesc),
                                             ctypes.POINTER(CConfig), ctypes.POINTER(CCorr),
                                             ctypes.POINTER(_P)]),
    "akua_pbf_step_batch": (ctypes.c_int, [_P, ctypes.c_float]),
    "akua_pbf_set_scene": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(CSceneDesc)]),
    "akua_mlp_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "akua_mlp_destroy": (ctypes.c_int, [_P]),
    "akua_mlp_set_params": (ctypes.c_int, [_P, _P, ctypes.c_int32]),
    "akua_mlp_get_params": (ctypes.c_int, [_P, _P, ctypes.c_int32]),
    "akua_mlp_set_normalization": (ctypes.c_int, [_P, _P, ctypes.c_int32]),
    "akua_mlp_forward": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P]),
    "akua_mlp_gradient": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P,
                                         ctypes.POINTER(ctypes.c_float), _P]),
    "akua_mlp_adam_step": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_float, _P]),
    "akua_mlp_synchronize": (ctypes.c_int, [_P, _P]),
    "akua_pbf_set_warm_start": (ctypes.c_int, [_P, _P]),
    "akua_pbf_capture_training": (ctypes.c_int, [_P, _P, _P]),
    "akua_pbf_set_lambda_tracking": (ctypes.c_int, [_P, ctypes.c_int32]),
    "akua_pbf_density_error": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float),
                                              ctypes.POINTER(ctypes.c_float)]),
    "akua_pbf_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "akua_pbf_abi_version": (ctypes.c_int, []),
}

_lib = None
_lock = threading.Lock()


class AkuaError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        super().__init__("%s failed: %s (%d)" % (what or "akua_pbf call", msg, status))


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Loads libakua_pbf.so.  Raises if it is missing: there is no fallback implementation."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                "libakua_pbf.so is not built (%s); run __graft_entry__.build() or "
                "python akuaengine_gb300/build.py" % p)
        lib = ctypes.CDLL(p)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def status_string(status: int) -> str:
    return load_library().akua_pbf_status_string(int(status)).decode()


def check(status: int, what: str = "") -> int:
    if status < 0:
        raise AkuaError(status, what)
    return status


def vec3(v) -> ctypes.Array:
    a = (ctypes.c_float * 3)()
    for i in range(3):
        a[i] = float(v[i])
    return a
