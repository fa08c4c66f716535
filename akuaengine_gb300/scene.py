"""Initial particle sets in the reference's 108-byte Particle layout.

``reference_dam_break`` rebuilds the scene of AkuaEngine's Application::prepareDamBreak
(src/Application/Application.cpp:14-15, 162-192): a 30x30x30 lattice at spacing 0.05 in
[2, 3.5] x [1, 2.5] x [2, 3.5], mass 1, blue, size 50, inside the box [1.5, 4.5] x [0, 4] x [1.5, 4.5].

``dam_break`` builds the seeded synthetic workloads the benchmarks run (lattice blocks at spacing
0.5h with uniform jitter of +-0.01h); there is no public dataset for this path.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from ._abi import PARTICLE_DTYPE

F32 = np.float32


@dataclass
class Scene:
    particles: np.ndarray            # PARTICLE_DTYPE records
    box_min: tuple
    box_max: tuple
    dt: float
    name: str
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.particles.shape[0])


def lattice_block(counts, spacing, origin, jitter=0.0, seed=0, mass=1.0,
                  color=(0.0, 0.0, 1.0, 1.0), size=50.0) -> np.ndarray:
    """counts = (nx, ny, nz) particles per axis, x-major order as the reference's loops
    (Application.cpp:174-190); position = origin + index * spacing in float32, plus
    uniform(-jitter, +jitter) per axis when jitter > 0."""
    nx, ny, nz = (int(c) for c in counts)
    sp = F32(spacing)
    ix, iy, iz = np.meshgrid(np.arange(nx, dtype=np.int64), np.arange(ny, dtype=np.int64),
                             np.arange(nz, dtype=np.int64), indexing="ij")
    pos = np.empty((nx * ny * nz, 3), dtype=F32)
    for a, idx in enumerate((ix, iy, iz)):
        pos[:, a] = F32(origin[a]) + idx.reshape(-1).astype(F32) * sp
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        pos = (pos + rng.uniform(-jitter, jitter, size=pos.shape).astype(F32)).astype(F32)
    p = np.zeros(pos.shape[0], dtype=PARTICLE_DTYPE)
    p["position"] = pos
    p["mass"] = F32(mass)
    p["color"] = np.asarray(color, dtype=F32)
    p["size"] = F32(size)
    return p


def reference_dam_break() -> Scene:
    """Application.cpp:162-192 with the reference's dt of 0.016 (Application.h:32)."""
    spacing = F32(0.05)
    lo = np.array([2.0, 1.0, 2.0], dtype=F32)
    hi = np.array([3.5, 2.5, 3.5], dtype=F32)
    counts = [int(F32(hi[a] - lo[a]) / spacing) for a in range(3)]
    p = lattice_block(counts, spacing, lo)
    return Scene(p, (1.5, 0.0, 1.5), (4.5, 4.0, 4.5), 0.016, "reference_dam_break",
                 {"counts": counts})


def dam_break(block=(30, 30, 30), box_widths=(4.0, 4.0, 4.0), h=0.1, seed=0, dt=0.0083,
              jitter_frac=0.01) -> Scene:
    """A lattice block at spacing 0.5h, jitter +-jitter_frac*h, in the lower corner of a box whose
    extents are `box_widths` times the block's x width; the block starts one spacing from the
    walls so no particle starts inside the 0.025 clamp band."""
    spacing = F32(0.5 * h)
    width = float(block[0]) * float(spacing)
    box_min = (0.0, 0.0, 0.0)
    box_max = tuple(float(F32(w * width)) for w in box_widths)
    origin = (float(spacing),) * 3
    p = lattice_block(block, spacing, origin, jitter=float(F32(jitter_frac * h)), seed=seed)
    return Scene(p, box_min, box_max, dt, "dam_break_%dx%dx%d" % tuple(block),
                 {"block": tuple(block), "box_widths": tuple(box_widths), "seed": seed})


def double_dam_break(block=(200, 100, 200), box_widths=(6.0, 2.0, 2.0), h=0.1, seed=0,
                     dt=0.0083, jitter_frac=0.01) -> Scene:
    """Two lattice blocks at opposite corners of the box (low x/low z and high x/high z), box
    extents in units of the block's x width; they meet in the middle of the box."""
    spacing = F32(0.5 * h)
    width = float(block[0]) * float(spacing)
    box_max = tuple(float(F32(w * width)) for w in box_widths)
    o1 = (float(spacing), float(spacing), float(spacing))
    o2 = (box_max[0] - float(spacing) * block[0], float(spacing), box_max[2] - float(spacing) * block[2])
    jit = float(F32(jitter_frac * h))
    a = lattice_block(block, spacing, o1, jitter=jit, seed=seed)
    b = lattice_block(block, spacing, o2, jitter=jit, seed=seed + 1)
    return Scene(np.concatenate([a, b]), (0.0, 0.0, 0.0), box_max, dt,
                 "double_dam_break_2x%dx%dx%d" % tuple(block),
                 {"block": tuple(block), "box_widths": tuple(box_widths), "seed": seed})


@dataclass
class SceneBatch:
    """Independent scenes stepped by one batch solver: records of scene k at
    [first[k], first[k] + n_k) of `particles`."""
    particles: np.ndarray
    scenes: list            # per scene: dict(numParticles, gravity, box_min, box_max, seed, block)
    dt: float
    name: str

    @property
    def n(self) -> int:
        return int(self.particles.shape[0])

    @property
    def first(self) -> list:
        out, f = [], 0
        for d in self.scenes:
            out.append(f)
            f += d["numParticles"]
        return out

    def scene(self, k: int) -> Scene:
        """Scene k alone (its own records, box and gravity in `meta`)."""
        d, f = self.scenes[k], self.first[k]
        return Scene(self.particles[f:f + d["numParticles"]].copy(), d["box_min"], d["box_max"],
                     self.dt, "%s[%d]" % (self.name, k), {"gravity": d["gravity"]})


def batched_dam_breaks(count=256, n_min=2000, n_max=64000, h=0.1, seed=0, dt=0.0083,
                       jitter_frac=0.01) -> SceneBatch:
    """`count` independent dam breaks: particle counts log-uniform in [n_min, n_max], block
    aspect ratios uniform in [0.5, 2] per axis, gravity magnitude uniform in [5, 15] (along -y),
    box extents 2-4x the block's per axis, lattice spacing 0.5h with jitter +-jitter_frac*h, one
    seed per scene."""
    rng = np.random.default_rng(seed)
    spacing = F32(0.5 * h)
    parts, scenes = [], []
    for k in range(count):
        target = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        aspect = rng.uniform(0.5, 2.0, 3)
        c = (target / float(np.prod(aspect))) ** (1.0 / 3.0)
        block = [max(2, int(round(a * c))) for a in aspect]
        g = float(rng.uniform(5.0, 15.0))
        factor = rng.uniform(2.0, 4.0, 3)
        box_max = tuple(float(F32((b + 2) * float(spacing) * f)) for b, f in zip(block, factor))
        origin = (float(spacing),) * 3
        sseed = int(rng.integers(0, 2 ** 31))
        p = lattice_block(block, spacing, origin, jitter=float(F32(jitter_frac * h)), seed=sseed)
        parts.append(p)
        scenes.append({"numParticles": int(p.shape[0]), "gravity": (0.0, -g, 0.0),
                       "box_min": (0.0, 0.0, 0.0), "box_max": box_max, "seed": sseed,
                       "block": tuple(block)})
    return SceneBatch(np.concatenate(parts), scenes, dt, "batched_%d" % count)


# Workloads of the benchmark configurations (sizes and parameters; seeded synthetic data).
def workload(name: str, seed: int = 0) -> Scene:
    if name == "dam_break_27k":
        return dam_break((30, 30, 30), (4.0, 4.0, 4.0), seed=seed)
    if name == "dam_break_100k":
        return dam_break((50, 40, 50), (3.0, 1.5, 1.5), seed=seed)
    if name == "dam_break_1m":
        return dam_break((100, 100, 100), (3.0, 1.5, 1.5), seed=seed)
    if name == "double_dam_break_8m":
        return double_dam_break((200, 100, 200), (6.0, 2.0, 2.0), seed=seed)
    raise KeyError(name)


def benchmark_params(strong_pressure: bool = False):
    """Solver parameters of the benchmark workloads: the reference dam-break scene's values
    (PBFConfig.h:10-28), including its artificial pressure k=1e-4, n=4, delta_q=0.03.

    `strong_pressure` selects k=0.1, n=4, delta_q=0.2h instead.  With the reference's rest density
    7600 and unit masses that term is ~100x the constraint's own lambda and the block disintegrates
    within a few steps, so it is used by the tests as a sparse-neighbourhood case, not as the
    benchmark workload."""
    from .solver import LambdaCorrParams, PBFConfig
    cfg = PBFConfig()
    if strong_pressure:
        corr = LambdaCorrParams(k=0.1, n=4.0, delta_q=0.2 * cfg.smoothRadius)
    else:
        corr = LambdaCorrParams()
    return cfg, corr
