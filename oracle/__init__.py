"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracle (oracle/pbf_oracle.cpp).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm as the checker
and baseline.  The product path (akuaengine_gb300) never imports this package.

Parity pin: see tests/golden/ — the oracle is checked against known-answer values of the
reference's own smoothing kernels compiled from its header (oracle/_ref, built by
oracle/ref_kat.py where the reference tree exists) and committed as fixtures.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")

FMA = 1
FP64 = 2

_lock = threading.Lock()
_lib = None


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("rest_density", ctypes.c_float),
        ("smooth_radius", ctypes.c_float),
        ("cell_size", ctypes.c_float),
        ("relaxation", ctypes.c_float),
        ("vorticity_epsilon", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("max_neighbours", ctypes.c_int32),
        ("solver_iterations", ctypes.c_int32),
        ("gravity", ctypes.c_float * 3),
        ("corr_k", ctypes.c_float),
        ("corr_n", ctypes.c_float),
        ("corr_delta_q", ctypes.c_float),
        ("table_size", ctypes.c_int32),
        ("dt", ctypes.c_float),
        ("box_min", ctypes.c_float * 3),
        ("box_max", ctypes.c_float * 3),
        ("restitution", ctypes.c_float),
        ("friction", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("num_threads", ctypes.c_int32),
        ("num_shapes", ctypes.c_int32),
        ("sdf_min_dist", ctypes.c_float),
        ("sdf_stiffness", ctypes.c_float),
        ("pad_", ctypes.c_int32),
        ("shapes", ctypes.c_void_p),
    ]


class OracleShape(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("a", ctypes.c_float * 3), ("b", ctypes.c_float * 3),
                ("radius", ctypes.c_float)]


def set_shapes(P: "OracleParams", shapes, min_dist: float = 0.025, stiffness: float = 0.5):
    """Attaches SDF obstacles (dicts with type, a, b, radius) to oracle parameters; the array is
    kept alive on P."""
    arr = (OracleShape * max(len(shapes), 1))()
    for k, d in enumerate(shapes):
        arr[k].type = int(d["type"])
        for q in range(3):
            arr[k].a[q] = float(d.get("a", (0, 0, 0))[q])
            arr[k].b[q] = float(d.get("b", (0, 0, 0))[q])
        arr[k].radius = float(d.get("radius", 0.0))
    P.num_shapes = len(shapes)
    P.sdf_min_dist = float(min_dist)
    P.sdf_stiffness = float(stiffness)
    P.shapes = ctypes.cast(arr, ctypes.c_void_p)
    P._shape_array = arr
    return P


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "pbf_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB


def load() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(LIB)
            lib.oracle_step.restype = ctypes.c_int
            lib.oracle_step.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]
            lib.oracle_poly6.restype = ctypes.c_float
            lib.oracle_poly6.argtypes = [ctypes.c_float, ctypes.c_float]
            lib.oracle_spiky.restype = None
            lib.oracle_spiky.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_float,
                                         ctypes.POINTER(ctypes.c_float)]
            lib.oracle_hash.restype = ctypes.c_uint32
            lib.oracle_hash.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int32]
            lib.oracle_cell.restype = ctypes.c_int
            lib.oracle_cell.argtypes = [ctypes.c_float, ctypes.c_float]
            lib.oracle_max_threads.restype = ctypes.c_int
            lib.oracle_particle_size.restype = ctypes.c_int
            _lib = lib
        return _lib


def make_params(config, corr, dt, box_min, box_max, *, n=None, table_size=None, flags=FMA,
                restitution=0.0, friction=0.95, num_threads=0) -> OracleParams:
    p = OracleParams()
    p.rest_density = config.restDensity
    p.smooth_radius = config.smoothRadius
    p.cell_size = config.spatialHashCellSize
    p.relaxation = config.relaxation
    p.vorticity_epsilon = config.vorticityEpsilon
    p.viscosity = config.viscosity
    p.max_neighbours = config.maxNeighbours
    p.solver_iterations = config.solverIterations
    for i in range(3):
        p.gravity[i] = config.gravity[i]
        p.box_min[i] = box_min[i]
        p.box_max[i] = box_max[i]
    p.corr_k, p.corr_n, p.corr_delta_q = corr.k, corr.n, corr.delta_q
    if table_size is None:
        table_size = config.maxNeighbours * int(n)
    p.table_size = int(table_size)
    p.dt = dt
    p.restitution = restitution
    p.friction = friction
    p.flags = flags
    p.num_threads = num_threads
    return p


def step(particles: np.ndarray, params: OracleParams, *, want_lists: bool = False):
    """One step in place over PARTICLE_DTYPE records.  Returns (perm, nbr, cnt); nbr and cnt are
    None unless `want_lists`."""
    lib = load()
    n = particles.shape[0]
    assert particles.dtype.itemsize == 108 and particles.flags.c_contiguous
    perm = np.zeros(n, dtype=np.uint32)
    nbr = cnt = None
    if want_lists:
        nbr = np.zeros((n, params.max_neighbours), dtype=np.uint32)
        cnt = np.zeros(n, dtype=np.uint32)
    rc = lib.oracle_step(ctypes.byref(params), n, particles.ctypes.data_as(ctypes.c_void_p),
                         perm.ctypes.data_as(ctypes.c_void_p),
                         nbr.ctypes.data_as(ctypes.c_void_p) if want_lists else None,
                         cnt.ctypes.data_as(ctypes.c_void_p) if want_lists else None)
    if rc != 0:
        raise RuntimeError("oracle_step failed: %d" % rc)
    return perm, nbr, cnt


def poly6(r2: float, h: float) -> float:
    return float(load().oracle_poly6(r2, h))


def spiky(rv, h: float):
    a = (ctypes.c_float * 3)(*[float(x) for x in rv])
    o = (ctypes.c_float * 3)()
    load().oracle_spiky(a, h, o)
    return np.array([o[0], o[1], o[2]], dtype=np.float32)


def cell_hash(cx: int, cy: int, cz: int, table: int) -> int:
    return int(load().oracle_hash(cx, cy, cz, table))


def cell(x: float, size: float) -> int:
    return int(load().oracle_cell(x, size))


def max_threads() -> int:
    return int(load().oracle_max_threads())
