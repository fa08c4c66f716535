"""Headless point-splat rendering of particle records (C ABI akua_splat_*): the reference's GL
particle pass as CUDA kernels writing an RGBA8 image, plus a PPM writer for the image."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import PARTICLE_DTYPE, check, load_library


@dataclass
class Camera:
    position: tuple = (3.0, 2.0, 6.0)
    gaze: tuple = (0.0, 0.0, -1.0)
    up: tuple = (0.0, 1.0, 0.0)
    fovDegrees: float = 45.0
    nearZ: float = 0.1
    farZ: float = 160.0

    def to_c(self) -> _abi.CCamera:
        c = _abi.CCamera()
        for a in range(3):
            c.position[a] = float(self.position[a])
            c.gaze[a] = float(self.gaze[a])
            c.up[a] = float(self.up[a])
        c.fovDegrees, c.nearZ, c.farZ = float(self.fovDegrees), float(self.nearZ), float(self.farZ)
        return c

    def matrices(self, aspect: float):
        """(view, projection, projection @ view) as float32 4x4 arrays (row-major indexing
        m[row, col])."""
        lib = load_library()
        out = [np.zeros(16, np.float32) for _ in range(3)]
        c = self.to_c()
        check(lib.akua_camera_matrices(ctypes.byref(c), float(aspect),
                                       *[o.ctypes.data_as(ctypes.c_void_p) for o in out]),
              "akua_camera_matrices")
        return [o.reshape(4, 4).T.copy() for o in out]  # column-major storage -> m[row, col]


class SplatRenderer:
    def __init__(self, width: int, height: int):
        self._lib = load_library()
        self.width, self.height = int(width), int(height)
        h = ctypes.c_void_p()
        check(self._lib.akua_splat_create(self.width, self.height, ctypes.byref(h)),
              "akua_splat_create")
        self._h = h

    def render(self, particles, camera: Camera | None = None, stream=None):
        """`particles`: a CUDA uint8 tensor of records (or an object with data_ptr()); returns a
        CUDA uint8 tensor [height, width, 4], row 0 at the top."""
        import torch

        cam = (camera or Camera()).to_c()
        n = particles.numel() // PARTICLE_DTYPE.itemsize
        out = torch.empty((self.height, self.width, 4), dtype=torch.uint8, device="cuda")
        sh = None if stream is None else ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))
        check(self._lib.akua_splat_render(self._h, ctypes.c_void_p(particles.data_ptr()),
                                          PARTICLE_DTYPE.itemsize, n, ctypes.byref(cam),
                                          ctypes.c_void_p(out.data_ptr()), sh), "akua_splat_render")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            rc = self._lib.akua_splat_destroy(self._h)
            self._h = ctypes.c_void_p()
            check(rc, "akua_splat_destroy")


def write_ppm(path: str, rgba: np.ndarray) -> None:
    """Binary PPM (P6) of an [height, width, 4] uint8 image (alpha dropped)."""
    img = np.ascontiguousarray(rgba[..., :3], dtype=np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (img.shape[1], img.shape[0]))
        f.write(img.tobytes())
