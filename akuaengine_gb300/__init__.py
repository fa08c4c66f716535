"""GB300-native Position-Based Fluids step: a drop-in for AkuaEngine's PBFSolver::step.

The compute path is the in-tree CUDA library libakua_pbf.so (hand-written sm_103a kernels behind
the C ABI of include/akua_pbf.h).  This package is its Python binding; it has no fallback: using
the solver without the built library raises.
"""
from ._abi import (  # noqa: F401
    AKUA_ERR_CUDA, AKUA_ERR_DEVICE_CHECK, AKUA_ERR_INVALID_ARGUMENT, AKUA_ERR_NOT_ATTACHED,
    AKUA_ERR_OUT_OF_MEMORY, AKUA_ERR_TOO_LARGE, AKUA_OK, DEBUG_HASHES, DEBUG_NEIGHBOUR_COUNTS,
    DEBUG_NEIGHBOURS, DEBUG_ORDER, DEBUG_PARTICLES, FLAG_BAD_TABLE, FLAG_CAP_REACHED, LIB_PATH,
    OPT_EXACT_MATH, OPT_NO_GRAPH, OPT_RESIDENT, PARTICLE_DTYPE, AkuaError, exported_symbols,
    load_library,
)
from .scene import (Scene, SceneBatch, batched_dam_breaks, benchmark_params, dam_break,  # noqa: F401
                    double_dam_break, reference_dam_break, workload)
from .solver import BatchSolver, LambdaCorrParams, ParticleBuffer, PBFConfig, PBFSolver  # noqa: F401

__all__ = [
    "PBFSolver", "PBFConfig", "LambdaCorrParams", "ParticleBuffer", "PARTICLE_DTYPE", "AkuaError",
    "load_library", "Scene", "dam_break", "double_dam_break", "reference_dam_break", "workload",
    "benchmark_params",
]
