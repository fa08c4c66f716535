"""TEST INFRASTRUCTURE ONLY: host restatement of the point-splat renderer (numpy, float32).

Restates the reference's particle pass (assets/shaders/fluidParticle.vert:13-21,
fluidParticle.frag:7-18; GL state Application.cpp:72,112-113) with the operations in the order the
CUDA kernels use, so coverage decisions agree exactly and colours to the last unit (the fragment's
exp may round differently by one ulp):
  size = clamp(Particle::size / |pos - eye|, 1, 2047); clip = VP . (pos, 1) (VP given)
  a point whose vertex lies outside the clip volume vanishes
  window = ((ndc.xy + 1) / 2) * (W, H), depth = (ndc.z + 1) / 2
  pixels with centres in [x - s/2, x + s/2) x [y - s/2, y + s/2)
  offset = ((px + .5 - x) / s, -(py + .5 - y) / s); discard if |offset| > 0.5
  colour = particle colour * exp(-|offset|^2 * 3); nearest depth wins, then the lower index
"""
from __future__ import annotations

import numpy as np

F = np.float32
CLEAR = np.array([0.15, 0.15, 0.18, 1.0], dtype=F)


def _u8(c):
    return np.floor(np.clip(c, F(0), F(1)) * F(255) + F(0.5)).astype(np.uint8)


def render(particles: np.ndarray, vp: np.ndarray, eye, width: int, height: int) -> np.ndarray:
    """vp: float32 4x4 (m[row, col]); returns uint8 [height, width, 4], row 0 at the top."""
    pos = particles["position"].astype(F)
    eye = np.asarray(eye, dtype=F)
    dx, dy, dz = pos[:, 0] - eye[0], pos[:, 1] - eye[1], pos[:, 2] - eye[2]
    dist = np.sqrt(dx * dx + dy * dy + dz * dz)
    size = np.clip(particles["size"].astype(F) / dist, F(1), F(2047))
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    c = [vp[k, 0] * x + vp[k, 1] * y + vp[k, 2] * z + vp[k, 3] for k in range(4)]
    w = c[3]
    inside = (w > 0) & (np.abs(c[0]) <= w) & (np.abs(c[1]) <= w) & (np.abs(c[2]) <= w)
    with np.errstate(divide="ignore", invalid="ignore"):
        xw = (c[0] / w + F(1)) * F(0.5) * F(width)
        yw = (c[1] / w + F(1)) * F(0.5) * F(height)
        zw = (c[2] / w + F(1)) * F(0.5)
    colour = particles["color"].astype(F)
    depth = np.full((height, width), np.inf, dtype=np.float64)
    winner = np.full((height, width), -1, dtype=np.int64)
    order = np.lexsort((np.arange(len(pos)), zw))
    for i in order:
        if not inside[i] or not zw[i] < 1:
            continue
        s = size[i]
        x0 = max(0, int(np.ceil(xw[i] - F(0.5) * s - F(0.5))))
        x1 = min(width - 1, int(np.ceil(xw[i] + F(0.5) * s - F(0.5))) - 1)
        y0 = max(0, int(np.ceil(yw[i] - F(0.5) * s - F(0.5))))
        y1 = min(height - 1, int(np.ceil(yw[i] + F(0.5) * s - F(0.5))) - 1)
        if x0 > x1 or y0 > y1:
            continue
        px = np.arange(x0, x1 + 1, dtype=np.int64)[None, :]
        py = np.arange(y0, y1 + 1, dtype=np.int64)[:, None]
        ox = ((px.astype(F) + F(0.5)) - xw[i]) / s
        oy = -((py.astype(F) + F(0.5)) - yw[i]) / s
        d = np.sqrt(ox * ox + oy * oy)
        hit = d <= F(0.5)
        sub = winner[y0:y1 + 1, x0:x1 + 1]
        free = hit & (sub < 0)  # sorted by (depth, index): the first to reach a pixel wins
        sub[free] = i
        depth[y0:y1 + 1, x0:x1 + 1][free] = zw[i]
    img = np.empty((height, width, 4), dtype=np.uint8)
    img[:] = _u8(CLEAR)
    ys, xs = np.nonzero(winner >= 0)
    i = winner[ys, xs]
    ox = ((xs.astype(F) + F(0.5)) - xw[i]) / size[i]
    oy = -((ys.astype(F) + F(0.5)) - yw[i]) / size[i]
    d = np.sqrt(ox * ox + oy * oy)
    a = np.exp(-d * d * F(3))
    img[ys, xs] = _u8(colour[i] * a[:, None])
    return img[::-1].copy()  # window row 0 is the bottom
