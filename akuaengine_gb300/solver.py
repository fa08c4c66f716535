"""Python mirror of AkuaEngine's solver interface over the C ABI (include/akua_pbf.h).

Same names and argument meaning as the reference:
  PBFConfig, LambdaCorrParams      include/AkuaEngine/Simulation/PBFConfig.h:10-29
  PBFSolver(numParticles, config, corrParams)               PBFSolver.cpp:13-20
  PBFSolver.step(particles, deltaTime, boxMin, boxMax)      PBFSolver.cpp:22-78
  PBFSolver.setGravity(gravity)                             PBFSolver.h:29-31
`particles` takes the place of the reference's InteropResource (a GL buffer mapped to a device
pointer): a ParticleBuffer (device pointer + stride), a CUDA torch tensor holding the records, or
a host numpy array of PARTICLE_DTYPE records (copied to the device and back around the step).
The reference reports no errors; every failing call here raises AkuaError.
"""
from __future__ import annotations

import ctypes
import dataclasses
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import PARTICLE_DTYPE, AkuaError, check, load_library, vec3


@dataclass
class PBFConfig:
    restDensity: float = 7600.0
    particle_spacing: float = 0.05
    smoothRadius: float = 0.1
    spatialHashCellSize: float = 0.1
    relaxation: float = 600.0
    vorticityEpsilon: float = 0.00001
    viscosity: float = 0.01
    maxNeighbours: int = 128
    solverIterations: int = 4
    gravity: tuple = (0.0, -9.8, 0.0)

    def to_c(self) -> _abi.CConfig:
        c = _abi.CConfig()
        for name, _ in _abi.CConfig._fields_:
            if name == "gravity":
                for i in range(3):
                    c.gravity[i] = float(self.gravity[i])
            else:
                setattr(c, name, getattr(self, name))
        return c


@dataclass
class LambdaCorrParams:
    enabled: bool = True
    k: float = 0.0001
    n: float = 4.0
    delta_q: float = 0.03

    def to_c(self) -> _abi.CCorr:
        return _abi.CCorr(int(bool(self.enabled)), self.k, self.n, self.delta_q)


@dataclass
class ParticleBuffer:
    """A device array of particle records: what cudaGraphicsResourceGetMappedPointer returns for
    the reference's registered VBO (InteropResource.cpp:9-14)."""
    device_ptr: int
    stride: int = PARTICLE_DTYPE.itemsize
    owner: object = field(default=None, repr=False)


def as_particle_buffer(obj) -> ParticleBuffer:
    if isinstance(obj, ParticleBuffer):
        return obj
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(obj, torch.Tensor):
        if not obj.is_cuda or not obj.is_contiguous():
            raise ValueError("particle tensor must be a contiguous CUDA tensor")
        return ParticleBuffer(obj.data_ptr(), PARTICLE_DTYPE.itemsize, obj)
    raise TypeError("expected ParticleBuffer, CUDA tensor or numpy PARTICLE_DTYPE array")


class PBFSolver:
    def __init__(self, numParticles: int, config: PBFConfig | None = None,
                 corrParams: LambdaCorrParams | None = None, *, options: int = 0,
                 table_size: int | None = None, stream=None):
        self._lib = load_library()
        self.numParticles = int(numParticles)
        # own copies: setters below update them
        self.config = dataclasses.replace(config) if config is not None else PBFConfig()
        self.corrParams = (dataclasses.replace(corrParams) if corrParams is not None
                           else LambdaCorrParams())
        self._cfg = self.config.to_c()
        self._corr = self.corrParams.to_c()
        h = ctypes.c_void_p()
        check(self._lib.akua_pbf_create(self.numParticles, ctypes.byref(self._cfg),
                                        ctypes.byref(self._corr), ctypes.byref(h)),
              "akua_pbf_create")
        self._h = h
        self._attached = None
        if options:
            self.set_options(options)
        if table_size is not None:
            self.set_table_size(table_size)
        if stream is not None:
            self.set_stream(stream)

    # -- reference interface -------------------------------------------------------------------
    def step(self, particles, deltaTime: float, boxMin, boxMax) -> None:
        if isinstance(particles, np.ndarray):
            self.step_host(particles, deltaTime, boxMin, boxMax)
            return
        buf = as_particle_buffer(particles)
        self.attach(buf)
        check(self._lib.akua_pbf_step(self._h, float(deltaTime), vec3(boxMin), vec3(boxMax)),
              "akua_pbf_step")

    def setGravity(self, gravity) -> None:
        check(self._lib.akua_pbf_set_gravity(self._h, vec3(gravity)), "akua_pbf_set_gravity")
        self.config.gravity = tuple(float(g) for g in gravity)

    # -- additions -----------------------------------------------------------------------------
    def attach(self, buf: ParticleBuffer | None) -> None:
        if buf is None:
            check(self._lib.akua_pbf_attach_particles(self._h, None, 0), "attach")
            self._attached = None
            return
        key = (buf.device_ptr, buf.stride)
        if self._attached != key:
            check(self._lib.akua_pbf_attach_particles(self._h, ctypes.c_void_p(buf.device_ptr),
                                                      buf.stride), "akua_pbf_attach_particles")
            self._attached = key
        self._owner = buf.owner

    def step_host(self, particles: np.ndarray, deltaTime: float, boxMin, boxMax) -> None:
        if particles.dtype != PARTICLE_DTYPE or not particles.flags.c_contiguous:
            raise ValueError("host particles must be a contiguous PARTICLE_DTYPE array")
        if particles.shape[0] != self.numParticles:
            raise ValueError("expected %d particles" % self.numParticles)
        check(self._lib.akua_pbf_step_host(self._h, particles.ctypes.data_as(ctypes.c_void_p),
                                           PARTICLE_DTYPE.itemsize, float(deltaTime),
                                           vec3(boxMin), vec3(boxMax)), "akua_pbf_step_host")

    def set_solver_iterations(self, iterations: int) -> None:
        check(self._lib.akua_pbf_set_solver_iterations(self._h, int(iterations)),
              "akua_pbf_set_solver_iterations")
        self.config.solverIterations = int(iterations)

    def set_warm_start(self, net) -> None:
        """Attaches a LambdaNet (None: the plain solver)."""
        check(self._lib.akua_pbf_set_warm_start(self._h, net.handle if net is not None else None),
              "akua_pbf_set_warm_start")
        self._warm = net

    def capture_training(self, features, targets) -> None:
        """The next step writes features (CUDA float32 [N, 8]) and accumulated lambda (CUDA
        float32 [N]) in one particle order."""
        if features is None:
            check(self._lib.akua_pbf_capture_training(self._h, None, None), "capture_training")
            return
        n = self.numParticles
        if tuple(features.shape) != (n, 8) or tuple(targets.shape) != (n,):
            raise ValueError("expected features [%d, 8] and targets [%d]" % (n, n))
        for t in (features, targets):
            if not t.is_cuda or not t.is_contiguous() or str(t.dtype) != "torch.float32":
                raise ValueError("capture buffers must be contiguous CUDA float32 tensors")
        check(self._lib.akua_pbf_capture_training(self._h, ctypes.c_void_p(features.data_ptr()),
                                                  ctypes.c_void_p(targets.data_ptr())),
              "akua_pbf_capture_training")
        self._capture = (features, targets)

    PAIR_KERNELS = ("k_density_lambda", "k_delta_correct", "k_delta_final", "k_vorticity",
                    "k_confine", "k_xsph")

    def pair_blocks(self) -> dict:
        b = (ctypes.c_int32 * 6)()
        check(self._lib.akua_pbf_get_pair_blocks(self._h, b), "akua_pbf_get_pair_blocks")
        return dict(zip(self.PAIR_KERNELS, list(b)))

    def set_pair_blocks(self, blocks) -> None:
        """`blocks`: six block sizes (64, 128 or 256) or a dict by kernel name."""
        if isinstance(blocks, dict):
            blocks = [blocks[k] for k in self.PAIR_KERNELS]
        b = (ctypes.c_int32 * 6)(*[int(x) for x in blocks])
        check(self._lib.akua_pbf_set_pair_blocks(self._h, b), "akua_pbf_set_pair_blocks")

    def search_shape(self) -> tuple[int, int]:
        """The neighbour walk's tile shape: (block size, staged list entries per particle)."""
        b, g = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.akua_pbf_get_search_shape(self._h, ctypes.byref(b), ctypes.byref(g)),
              "akua_pbf_get_search_shape")
        return b.value, g.value

    def set_search_shape(self, block: int, staged: int) -> None:
        check(self._lib.akua_pbf_set_search_shape(self._h, int(block), int(staged)),
              "akua_pbf_set_search_shape")

    def autotune(self, deltaTime: float, boxMin=None, boxMax=None, steps: int = 3) -> dict:
        """Chooses each pair kernel's block size, then the walk's tile shape, by timing, on a copy
        of the attached records (attach a buffer first); returns the pair kernels' choice by
        kernel name (the walk's: `search_shape()`)."""
        b = (ctypes.c_int32 * 6)()
        check(self._lib.akua_pbf_autotune(self._h, float(deltaTime),
                                          None if boxMin is None else vec3(boxMin),
                                          None if boxMax is None else vec3(boxMax), int(steps), b),
              "akua_pbf_autotune")
        return dict(zip(self.PAIR_KERNELS, list(b)))

    def set_sdf_shapes(self, shapes, min_dist: float = 0.025, stiffness: float = 0.5) -> None:
        """Solid obstacles: dicts with type ("sphere", "box", "capsule", "plane" or the
        AKUA_SDF_* number), a, b, radius (see include/akua_pbf.h).  [] removes them."""
        arr = (_abi.CSdfShape * max(len(shapes), 1))()
        for k, d in enumerate(shapes):
            arr[k] = sdf_shape(d)
        check(self._lib.akua_pbf_set_sdf_shapes(self._h, arr, len(shapes), float(min_dist),
                                                float(stiffness)), "akua_pbf_set_sdf_shapes")

    def set_lambda_tracking(self, enabled: bool) -> None:
        check(self._lib.akua_pbf_set_lambda_tracking(self._h, int(bool(enabled))),
              "akua_pbf_set_lambda_tracking")

    def set_lambda_sums(self, sums) -> None:
        """The per-particle lambda sums the next step reads as the previous step's (record
        order), e.g. from a state file."""
        a = np.ascontiguousarray(sums, dtype=np.float32)
        check(self._lib.akua_pbf_set_lambda_sums(self._h, a.ctypes.data_as(ctypes.c_void_p),
                                                 a.size), "akua_pbf_set_lambda_sums")

    def density_error(self) -> tuple[float, float]:
        """(max_i max(rho_i/rho0 - 1, 0), mean_i |rho_i/rho0 - 1|) at the last step's end."""
        mx, mean = ctypes.c_float(), ctypes.c_float()
        check(self._lib.akua_pbf_density_error(self._h, ctypes.byref(mx), ctypes.byref(mean)),
              "akua_pbf_density_error")
        return float(mx.value), float(mean.value)

    def set_options(self, options: int) -> None:
        check(self._lib.akua_pbf_set_options(self._h, int(options)), "akua_pbf_set_options")

    def set_table_size(self, table_size: int) -> None:
        check(self._lib.akua_pbf_set_table_size(self._h, int(table_size)), "akua_pbf_set_table_size")

    def set_boundary_damping(self, restitution: float, friction: float) -> None:
        check(self._lib.akua_pbf_set_boundary_damping(self._h, restitution, friction),
              "akua_pbf_set_boundary_damping")

    def set_stream(self, stream) -> None:
        """`stream`: a torch.cuda.Stream, or an integer cudaStream_t handle."""
        handle = getattr(stream, "cuda_stream", stream)
        check(self._lib.akua_pbf_set_stream(self._h, ctypes.c_void_p(int(handle))),
              "akua_pbf_set_stream")

    def synchronize(self) -> None:
        check(self._lib.akua_pbf_synchronize(self._h), "akua_pbf_synchronize")

    def stats(self) -> dict:
        st = _abi.CStats()
        check(self._lib.akua_pbf_get_stats(self._h, ctypes.byref(st)), "akua_pbf_get_stats")
        return {name: getattr(st, name) for name, _ in _abi.CStats._fields_}

    def kernels_per_step(self) -> int:
        return check(self._lib.akua_pbf_kernels_per_step(self._h), "akua_pbf_kernels_per_step")

    def profile_begin(self, max_steps: int) -> None:
        """Times every kernel of the next `max_steps` steps with CUDA events (no graph)."""
        check(self._lib.akua_pbf_profile_begin(self._h, int(max_steps)), "akua_pbf_profile_begin")

    def profile_end(self) -> dict:
        """{kernel name: (launches, total milliseconds)}; synchronises."""
        cap = 64
        arr = (_abi.CKernelTime * cap)()
        cnt = ctypes.c_int32()
        check(self._lib.akua_pbf_profile_end(self._h, arr, cap, ctypes.byref(cnt)),
              "akua_pbf_profile_end")
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms)
                for i in range(min(cnt.value, cap))}

    def read_debug(self, what: int) -> np.ndarray:
        n = self.numParticles
        if what == _abi.DEBUG_PARTICLES:
            out = np.zeros(n, dtype=PARTICLE_DTYPE)
        elif what == _abi.DEBUG_LAMBDA_SUMS:
            out = np.zeros(n, dtype=np.float32)
        elif what == _abi.DEBUG_NEIGHBOURS:
            out = np.zeros((n, self.config.maxNeighbours), dtype=np.uint32)
        else:
            out = np.zeros(n, dtype=np.uint32)
        check(self._lib.akua_pbf_read_debug(self._h, what, out.ctypes.data_as(ctypes.c_void_p),
                                            out.nbytes), "akua_pbf_read_debug")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            rc = self._lib.akua_pbf_destroy(self._h)
            self._h = ctypes.c_void_p()
            check(rc, "akua_pbf_destroy")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver(PBFSolver):
    """Many independent scenes in one solver (C ABI akua_pbf_create_batch): every kernel of a step
    covers all scenes, and each scene's records come out as if it were stepped alone.  `scenes`:
    dicts (or objects) with numParticles, gravity, box_min, box_max."""

    def __init__(self, scenes, config: PBFConfig | None = None,
                 corrParams: LambdaCorrParams | None = None, *, options: int = 0, stream=None):
        self._lib = load_library()
        self.config = dataclasses.replace(config) if config is not None else PBFConfig()
        self.corrParams = (dataclasses.replace(corrParams) if corrParams is not None
                           else LambdaCorrParams())
        self._cfg = self.config.to_c()
        self._corr = self.corrParams.to_c()
        descs = (_abi.CSceneDesc * len(scenes))()
        for k, d in enumerate(scenes):
            descs[k] = _scene_desc(d)
        self.scenes = list(scenes)
        self.numParticles = int(sum(_get(d, "numParticles") for d in scenes))
        h = ctypes.c_void_p()
        check(self._lib.akua_pbf_create_batch(len(scenes), descs, ctypes.byref(self._cfg),
                                              ctypes.byref(self._corr), ctypes.byref(h)),
              "akua_pbf_create_batch")
        self._h = h
        self._attached = None
        if options:
            self.set_options(options)
        if stream is not None:
            self.set_stream(stream)

    def step(self, particles, deltaTime: float) -> None:
        self.attach(as_particle_buffer(particles))
        check(self._lib.akua_pbf_step_batch(self._h, float(deltaTime)), "akua_pbf_step_batch")

    def set_scene(self, k: int, scene) -> None:
        d = _scene_desc(scene)
        check(self._lib.akua_pbf_set_scene(self._h, int(k), ctypes.byref(d)), "akua_pbf_set_scene")
        self.scenes[k] = scene


def _get(d, name):
    return d[name] if isinstance(d, dict) else getattr(d, name)


def _scene_desc(d) -> "_abi.CSceneDesc":
    c = _abi.CSceneDesc()
    c.numParticles = int(_get(d, "numParticles"))
    for a in range(3):
        c.gravity[a] = float(_get(d, "gravity")[a])
        c.boxMin[a] = float(_get(d, "box_min")[a])
        c.boxMax[a] = float(_get(d, "box_max")[a])
    return c


SDF_TYPES = {"sphere": _abi.SDF_SPHERE, "box": _abi.SDF_BOX, "capsule": _abi.SDF_CAPSULE,
             "plane": _abi.SDF_PLANE}


def sdf_shape(d) -> "_abi.CSdfShape":
    c = _abi.CSdfShape()
    t = d["type"]
    c.type = SDF_TYPES[t] if isinstance(t, str) else int(t)
    for q in range(3):
        c.a[q] = float(d.get("a", (0.0, 0.0, 0.0))[q])
        c.b[q] = float(d.get("b", (0.0, 0.0, 0.0))[q])
    c.radius = float(d.get("radius", 0.0))
    return c
