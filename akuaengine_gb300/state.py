"""State files (C ABI akua_state_*): the particle records of a run plus what resuming it needs.

    save_state(path, particles, config, corr, box_min, box_max, dt, step=..., lambda_sums=...)
    st = load_state(path)      # State(particles, config, corr, box_min, box_max, dt, step, ...)

The records and the solver parameters determine every later step, so a run resumed from a file
continues bit for bit (with the lambda sums too when a warm start is in use).  For a batch of
scenes, `scenes` holds their descriptors (numParticles, gravity, box_min, box_max).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import PARTICLE_DTYPE, check, load_library
from .solver import LambdaCorrParams, PBFConfig


@dataclass
class State:
    particles: np.ndarray
    config: PBFConfig
    corr: LambdaCorrParams
    box_min: tuple
    box_max: tuple
    dt: float
    step: int = 0
    table_size: int = 0
    options: int = 0
    lambda_sums: np.ndarray | None = None
    scenes: list = field(default_factory=list)


def _config_from_c(c) -> PBFConfig:
    kw = {name: getattr(c, name) for name, _ in _abi.CConfig._fields_ if name != "gravity"}
    kw["gravity"] = tuple(float(c.gravity[i]) for i in range(3))
    return PBFConfig(**kw)


def save_state(path: str, particles: np.ndarray, config: PBFConfig, corr: LambdaCorrParams,
               box_min=(0.0, 0.0, 0.0), box_max=(0.0, 0.0, 0.0), dt: float = 0.0, step: int = 0,
               table_size: int | None = None, options: int = 0, lambda_sums=None,
               scenes=None) -> None:
    lib = load_library()
    p = np.ascontiguousarray(particles)
    if p.dtype != PARTICLE_DTYPE:
        raise ValueError("particles must be PARTICLE_DTYPE records")
    h = _abi.CStateHeader()
    lib.akua_state_init_header(ctypes.byref(h))
    h.numParticles = p.shape[0]
    h.step = int(step)
    h.config = config.to_c()
    h.corr = corr.to_c()
    for a in range(3):
        h.boxMin[a] = float(box_min[a])
        h.boxMax[a] = float(box_max[a])
    h.deltaTime = float(dt)
    h.tableSize = int(table_size if table_size is not None else config.maxNeighbours * p.shape[0])
    h.options = int(options)
    sums = None
    if lambda_sums is not None:
        sums = np.ascontiguousarray(lambda_sums, dtype=np.float32)
        if sums.shape != (p.shape[0],):
            raise ValueError("one lambda sum per particle")
        h.sections |= _abi.STATE_LAMBDA_SUMS
    descs = None
    if scenes:
        from .solver import _scene_desc

        descs = (_abi.CSceneDesc * len(scenes))()
        for k, d in enumerate(scenes):
            descs[k] = _scene_desc(d)
        h.numScenes = len(scenes)
    check(lib.akua_state_save(str(path).encode(), ctypes.byref(h),
                              p.ctypes.data_as(ctypes.c_void_p),
                              None if sums is None else sums.ctypes.data_as(ctypes.c_void_p),
                              descs), "akua_state_save")


def load_state(path: str) -> State:
    lib = load_library()
    h = _abi.CStateHeader()
    check(lib.akua_state_read_header(str(path).encode(), ctypes.byref(h)), "akua_state_read_header")
    n = int(h.numParticles)
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    sums = np.zeros(n, dtype=np.float32) if h.sections & _abi.STATE_LAMBDA_SUMS else None
    descs = (_abi.CSceneDesc * max(h.numScenes, 1))()
    check(lib.akua_state_load(str(path).encode(), ctypes.byref(h),
                              p.ctypes.data_as(ctypes.c_void_p), n,
                              None if sums is None else sums.ctypes.data_as(ctypes.c_void_p),
                              descs, max(h.numScenes, 1)), "akua_state_load")
    scenes = [{"numParticles": int(descs[k].numParticles),
               "gravity": tuple(float(x) for x in descs[k].gravity),
               "box_min": tuple(float(x) for x in descs[k].boxMin),
               "box_max": tuple(float(x) for x in descs[k].boxMax)} for k in range(h.numScenes)]
    c = h.corr
    return State(p, _config_from_c(h.config),
                 LambdaCorrParams(bool(c.enabled), float(c.k), float(c.n), float(c.delta_q)),
                 tuple(float(x) for x in h.boxMin), tuple(float(x) for x in h.boxMax),
                 float(h.deltaTime), int(h.step), int(h.tableSize), int(h.options), sums, scenes)


def save_solver_state(path: str, solver, box_min=(0.0, 0.0, 0.0), box_max=(0.0, 0.0, 0.0),
                      dt: float = 0.0, with_lambda_sums: bool = False) -> None:
    """The solver's current records (its last step's output) and parameters."""
    st = solver.stats()
    save_state(path, solver.read_debug(_abi.DEBUG_PARTICLES), solver.config, solver.corrParams,
               box_min, box_max, dt, st["steps"], st["tableSize"],
               lambda_sums=solver.read_debug(_abi.DEBUG_LAMBDA_SUMS) if with_lambda_sums else None,
               scenes=getattr(solver, "scenes", None))
