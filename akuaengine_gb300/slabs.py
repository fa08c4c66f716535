"""Slab decomposition of one scene over several ranks (GPUs), with a wide halo.

The scene's x range is cut into `world` slabs; rank r owns the particles whose position lies in
slab r.  A step of the reference algorithm reaches, from a particle, every particle within its
dependency radius: the neighbour lists (radius h around the predicted positions), each Jacobi
iteration (density and lambda of the neighbours, then their positions: 2h), vorticity,
confinement and XSPH (h each).  With K iterations that is (2K + 3) h, plus the distance a particle
can travel in the prediction.  Each rank therefore steps its own particles together with every
other particle within that halo of its slab, in the global record order, and keeps only its own
results: the neighbour lists, sums and corrections of its own particles see exactly the particles
the single-domain step sees, so they come out identical, and one exchange per step replaces the
K + 2 halo exchanges a thin halo needs (the ghosts are recomputed instead of communicated).

The record order matters for exactness: the step sorts stably by (hash, previous order), so each
rank steps its records in their global order, and the owned results of all ranks are put back in
global order by their (hash, previous global rank) keys (the previous rank travels through the
step in colour[3], `tag`).  The local step must use the whole scene's hash table size
(maxNeighbours * N), so hashes and bucket collisions are those of the single-domain step.

The local step is any callable that steps an array of records in place (the GPU solver on a box
with one GPU per rank; the host restatement in the tests).  Every rank gets the whole scene's
records at the start of a step and the owned results are gathered after it.  Two forms: numpy
record arrays (`decomposed_step`) and device-resident torch tensors of the attached-buffer layout
(`decomposed_step_device`, selection and reassembly on the GPU, exchange through
`all_gather_records`, which uses torch.distributed: NCCL for CUDA tensors).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Slabs:
    world: int
    x_min: float
    x_max: float
    halo: float

    def cuts(self) -> np.ndarray:
        return np.linspace(self.x_min, self.x_max, self.world + 1)

    def owner(self, x: np.ndarray) -> np.ndarray:
        """Rank owning each x (clamped to the end slabs)."""
        width = (self.x_max - self.x_min) / self.world
        r = np.floor((np.asarray(x, dtype=np.float64) - self.x_min) / width).astype(np.int64)
        return np.clip(r, 0, self.world - 1)

    def local_mask(self, x: np.ndarray, rank: int) -> np.ndarray:
        """Particles rank `rank` steps: its own plus those within the halo of its slab."""
        c = self.cuts()
        lo = -np.inf if rank == 0 else c[rank] - self.halo
        hi = np.inf if rank == self.world - 1 else c[rank + 1] + self.halo
        x = np.asarray(x, dtype=np.float64)
        return (x >= lo) & (x < hi)


def halo_width(h: float, iterations: int, max_speed: float, dt: float, gravity: float,
               margin: float = 0.0) -> float:
    """(2K + 3) h plus the largest prediction displacement |v| dt + |g| dt^2."""
    return (2 * iterations + 3) * h + max_speed * dt + abs(gravity) * dt * dt + margin


def make_slabs(records: np.ndarray, world: int, cfg, dt: float, margin: float = 0.0) -> Slabs:
    x = records["position"][:, 0].astype(np.float64)
    v = np.linalg.norm(records["velocity"].astype(np.float64), axis=1)
    g = float(np.linalg.norm(np.asarray(cfg.gravity, dtype=np.float64)))
    halo = halo_width(cfg.smoothRadius, cfg.solverIterations, float(v.max(initial=0.0)), dt, g,
                      margin)
    return Slabs(world, float(x.min()), float(np.nextafter(x.max(), np.inf)), halo)


def step_slab(records: np.ndarray, slabs: Slabs, rank: int, local_step,
              tag_field: str = "color") -> np.ndarray:
    """One decomposed step on rank `rank` over `records` tagged by `tag`: steps the owned and
    halo records (global order kept) with `local_step(records) -> None`, which reorders them,
    and returns the owned ones after the step (found again through their tags)."""
    x = records["position"][:, 0]
    own = slabs.owner(x) == rank
    idx = np.nonzero(slabs.local_mask(x, rank) | own)[0]  # global order preserved
    local = records[idx].copy()
    local_step(local)
    return local[own[local[tag_field][:, 3].astype(np.int64)]]


def global_records(parts, n: int, tag_field: str = "color") -> np.ndarray:
    """Reassembles the owned records of all ranks in global hash order: sorted by (hash, previous
    global rank), with the previous rank carried in colour[3] by the caller (see `tag`)."""
    allrec = np.concatenate(parts)
    assert allrec.shape[0] == n, "every particle must have exactly one owner"
    prev = allrec[tag_field][:, 3].astype(np.int64)
    order = np.lexsort((prev, allrec["hash"]))
    return allrec[order]


def tag(records: np.ndarray, tag_field: str = "color") -> np.ndarray:
    """Writes each record's index (its global rank) into colour[3], exactly representable for
    fewer than 2^24 particles; the step carries colour through unchanged."""
    r = records.copy()
    if r.shape[0] >= (1 << 24):
        raise ValueError("too many particles to tag in a float32")
    r[tag_field][:, 3] = np.arange(r.shape[0], dtype=np.float32)
    return r


def decomposed_step(records: np.ndarray, world: int, cfg, dt: float, local_step,
                    exchange=None, rank: int | None = None, margin: float = 0.0) -> np.ndarray:
    """A full decomposed step.  Without `exchange` all ranks run here in turn (one process);
    with it (a callable that all-gathers a list of numpy arrays across ranks, e.g. over
    torch.distributed), this process runs rank `rank` and the owned records are exchanged.
    Returns the records of the whole scene after the step in global hash order (colour
    untouched)."""
    tagged = tag(records)
    slabs = make_slabs(tagged, world, cfg, dt, margin)
    ranks = range(world) if exchange is None else [rank]
    mine = []
    for r in ranks:
        mine.append(step_slab(tagged, slabs, r, local_step))
    if exchange is not None:
        mine = exchange(mine[0])
    out = global_records(mine, records.shape[0])
    out["color"][:, 3] = records["color"][:, 3][out["color"][:, 3].astype(np.int64)]
    return out


# ------------------------------------------------------------------------------ device-resident
# The same decomposition on records that stay on the GPU: a torch uint8 tensor of N x 108-byte
# records (the attached-buffer layout).  Selection, tagging and reassembly are torch operations on
# the device; the local step is any callable stepping a record tensor in place (the CUDA solver).
REC_BYTES = 108
REC_WORDS = REC_BYTES // 4
_W_X, _W_V, _W_HASH, _W_TAG = 0, 3, 21, 25  # word offsets: position.x, velocity, hash, colour[3]


def _rows(buf):
    n = buf.numel() // REC_BYTES
    return buf.view(n, REC_BYTES), n


def decomposed_step_device(records, world: int, cfg, dt: float, local_step, exchange=None,
                           rank: int | None = None, margin: float = 0.0):
    """One decomposed step of device-resident records (`records`: contiguous torch uint8 tensor of
    N x 108 bytes on a GPU).  Without `exchange` every rank's slab is stepped here in turn; with it
    (a callable taking this rank's owned records and returning every rank's, e.g.
    `all_gather_records`), this process steps rank `rank` only.  Returns a new tensor with the whole
    scene's records in global hash order, equal to the single-domain step's."""
    import torch

    rows, n = _rows(records)
    if n >= (1 << 24):
        raise ValueError("too many particles to tag in a float32")
    tagged = rows.clone()
    tw = tagged.view(torch.float32)                       # [N, 27]
    tw[:, _W_TAG] = torch.arange(n, device=records.device, dtype=torch.float32)
    x = tw[:, _W_X].double()
    x_min = x.min()
    x_max = torch.nextafter(x.max(), torch.tensor(float("inf"), dtype=torch.float64,
                                                  device=records.device))
    v_max = float(tw[:, _W_V:_W_V + 3].double().norm(dim=1).max())
    g = float(np.linalg.norm(np.asarray(cfg.gravity, dtype=np.float64)))
    halo = halo_width(cfg.smoothRadius, cfg.solverIterations, v_max, dt, g, margin)
    width = (x_max - x_min) / world
    owner = torch.clamp(torch.floor((x - x_min) / width).long(), 0, world - 1)
    ranks = range(world) if exchange is None else [rank]
    mine = []
    for r in ranks:
        lo = -float("inf") if r == 0 else float(x_min + r * width) - halo
        hi = float("inf") if r == world - 1 else float(x_min + (r + 1) * width) + halo
        idx = torch.nonzero(((x >= lo) & (x < hi)) | (owner == r)).squeeze(1)  # global order kept
        local = tagged[idx].contiguous()
        local_step(local.view(-1))
        tags = local.view(torch.float32)[:, _W_TAG].long()
        mine.append(local[owner[tags] == r])
    if exchange is not None:
        mine = exchange(mine[0])
    allrec = torch.cat(mine)
    if allrec.shape[0] != n:
        raise RuntimeError("every particle must have exactly one owner")
    hashes = allrec.view(torch.int32)[:, _W_HASH].long() & 0xFFFFFFFF
    prev = allrec.view(torch.float32)[:, _W_TAG].long()
    out = allrec[torch.argsort(hashes * n + prev)]       # (hash, previous global rank): unique
    ow = out.view(torch.float32)
    ow[:, _W_TAG] = rows.view(torch.float32)[ow[:, _W_TAG].long(), _W_TAG]
    return out.view(-1)


def all_gather_records(mine, group=None):
    """Every rank's owned records (torch uint8 [k, 108], k differing between ranks) through
    torch.distributed.all_gather (NCCL for CUDA tensors, gloo for CPU ones): sizes first, then
    contributions padded to the largest."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    size = torch.tensor([mine.shape[0]], device=mine.device, dtype=torch.int64)
    sizes = [torch.zeros_like(size) for _ in range(world)]
    dist.all_gather(sizes, size, group=group)
    sizes = [int(s.item()) for s in sizes]
    padded = torch.zeros((max(sizes), REC_BYTES), dtype=torch.uint8, device=mine.device)
    padded[:mine.shape[0]] = mine
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    return [p[:k] for p, k in zip(parts, sizes)]
