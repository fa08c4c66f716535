"""Slab decomposition of one scene over several ranks (GPUs) with a halo exchange between
neighbouring slabs only.

The box's x range is cut into `world` fixed slabs; rank r owns the particles whose position lies in
slab r and holds, besides them, every particle within `halo` of its slab (its held region).  A step
of the reference algorithm reaches, from a particle, every particle within its dependency radius:
the neighbour lists (h around the predicted positions), each Jacobi iteration (density and lambda
of the neighbours, then their positions: 2h), vorticity, confinement and XSPH (h each), so
(2K + 3) h with K iterations, plus the distance a particle travels in the prediction.  Each rank
steps all its held particles and trusts the results of the particles it owned at the start of the
step (their whole dependency ball was held, with exact states); the ghosts' results are discarded.
After the step each rank sends each neighbour the trusted records that fall in the neighbour's held
region — the only communication, O(halo) per step — and keeps those in its own.  A particle that
crossed a cut is owned by the neighbour from the next step on, which already holds it.

Exactness needs more than the right particles: the step sorts stably by (cell hash, previous
order), so the neighbour lists — and every sum over them — depend on the global order of
particles that share a hash.  No rank knows the global order, but it only matters among particles
a walk can see together (same hash, cells at most two apart) and, one step later, among their
successors.  Each rank therefore orders its held records by (hash, w, particle id), where w is a
record's position, in the step's output order, among the records with the same hash whose cells
are linked to its own by a chain of cells at most `LINK_CELLS` apart (a cluster: normally the
particles of one cell; a few cells where the hash collides nearby).  The cluster of a trusted
particle lies inside the region its rank stepped exactly, so every rank that holds the particle
computes the same w, and within a cluster w follows the global order.  Particles with one hash in
different clusters are far apart, and no walk sees two of them together.  (The argument needs each
pair of particles that share a hash in consecutive steps while moving between clusters to stay
within the link distance; a particle pair in hash-colliding cells 3-4 cells apart on two
consecutive steps would break it: a chance of order 1e-7 per step for a million particles.)

Records carry their particle id as the bit pattern of colour[3] (uint32), which the step copies
unchanged; the caller's colour[3] values are kept aside and restored.  The local step must use the
whole scene's hash-table size (maxNeighbours * N) so hashes and collisions match the single-domain
step.

Two forms with one algorithm: numpy record arrays with any local step (`SlabRank`, the host
restatement in the CPU tests) and device-resident torch tensors of the attached-buffer layout
(`SlabRankDevice`, the CUDA solver on one GPU per rank), exchanging through `neighbour_exchange`
(torch.distributed point-to-point: NCCL for CUDA tensors, gloo for CPU ones) or, with every rank in
one process, `step_all`.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

LINK_CELLS = 4  # cells with one hash at most this far apart (Chebyshev) share a cluster


@dataclass(frozen=True)
class SlabPlan:
    world: int
    x_min: float
    x_max: float
    halo: float
    cell: float

    def cuts(self) -> np.ndarray:
        return np.linspace(self.x_min, self.x_max, self.world + 1)

    @property
    def width(self) -> float:
        return (self.x_max - self.x_min) / self.world

    def owner(self, x) -> np.ndarray:
        """Rank owning each x (positions outside the box belong to the end slabs)."""
        r = np.floor((np.asarray(x, dtype=np.float64) - self.x_min) / self.width).astype(np.int64)
        return np.clip(r, 0, self.world - 1)

    def held_range(self, rank: int) -> tuple[float, float]:
        """[lo, hi) of x that rank `rank` holds: its slab and `halo` either side."""
        c = self.cuts()
        lo = -np.inf if rank == 0 else c[rank] - self.halo
        hi = np.inf if rank == self.world - 1 else c[rank + 1] + self.halo
        return float(lo), float(hi)

    def held(self, x, rank: int) -> np.ndarray:
        lo, hi = self.held_range(rank)
        x = np.asarray(x, dtype=np.float64)
        return (x >= lo) & (x < hi)


def dependency_radius(h: float, iterations: int, travel: float) -> float:
    """How far one step reaches: (2K + 3) h plus a particle's travel in the prediction."""
    return (2 * iterations + 3) * h + travel


def plan_slabs(box_min, box_max, world: int, cfg, dt: float, max_speed: float,
               margin: float = 0.0) -> SlabPlan:
    """Slabs of the box along x.  The halo covers the dependency radius, the clusters of the
    trusted particles (LINK_CELLS + 1 cells) and two travels (the clusters are formed at the new
    positions).  `max_speed` bounds |v| over the run (a bound for all steps: the slabs are fixed)."""
    g = float(np.linalg.norm(np.asarray(cfg.gravity, dtype=np.float64)))
    travel = max_speed * dt + g * dt * dt
    cell = float(cfg.spatialHashCellSize)
    halo = (dependency_radius(cfg.smoothRadius, cfg.solverIterations, travel)
            + (LINK_CELLS + 1) * cell + 2 * travel + margin)
    plan = SlabPlan(world, float(box_min[0]), float(box_max[0]), halo, cell)
    if world > 1 and plan.width <= halo + travel:
        raise ValueError("slabs of width %.3g are too thin for a halo of %.3g: use fewer ranks"
                         % (plan.width, halo))
    return plan


# ------------------------------------------------------------------------------ order keys
def cluster_positions(hashes: np.ndarray, cells: np.ndarray) -> np.ndarray:
    """w of every record of a hash-sorted sequence: its position among the earlier records with
    the same hash whose cells are linked to its own (chains of cells at most LINK_CELLS apart).
    `cells`: int64 [n, 3] (any position of the step gives cells within a cell or two of the
    hashed one; the link distance absorbs that).  A run of one hash whose cells span at most
    LINK_CELLS per axis is one cluster (the usual case: one cell); only runs spread further — cells
    far apart that collide in the table — are split."""
    n = hashes.shape[0]
    w = np.zeros(n, dtype=np.uint32)
    if n == 0:
        return w
    h = hashes.astype(np.int64)
    start = np.flatnonzero(np.r_[True, h[1:] != h[:-1]])
    end = np.r_[start[1:], n]
    span = (np.maximum.reduceat(cells, start, axis=0)
            - np.minimum.reduceat(cells, start, axis=0)).max(axis=1)
    run_of = np.repeat(np.arange(start.size), end - start)
    w[:] = np.arange(n) - start[run_of]
    for k in np.flatnonzero(span > LINK_CELLS):
        a, b = start[k], end[k]
        w[a:b] = _cluster_positions_slow(cells[a:b])
    return w


def _cluster_positions_slow(cells: np.ndarray) -> np.ndarray:
    """One hash's records (in order) spanning several cells: link cells within LINK_CELLS,
    number each record within its linked cluster."""
    uniq, inv = np.unique(cells, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    parent = list(range(len(uniq)))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for a in range(len(uniq)):
        for b in range(a + 1, len(uniq)):
            if np.abs(uniq[a] - uniq[b]).max() <= LINK_CELLS:
                parent[find(a)] = find(b)
    root = np.array([find(c) for c in inv])
    w = np.zeros(len(cells), dtype=np.uint32)
    seen: dict[int, int] = {}
    for i, r in enumerate(root):
        w[i] = seen.get(r, 0)
        seen[r] = w[i] + 1
    return w


def order_key(hashes: np.ndarray, w: np.ndarray, gid: np.ndarray) -> np.ndarray:
    """Indices sorting records by (hash, w, particle id)."""
    return np.lexsort((gid.astype(np.int64), w.astype(np.int64), hashes.astype(np.int64)))


def cell_of(pos: np.ndarray, cell: float) -> np.ndarray:
    """Walk cell of each position, as the step computes it (floor(x / cell) in float32)."""
    return np.floor(pos.astype(np.float32) / np.float32(cell)).astype(np.int64)


# ------------------------------------------------------------------------------ host records
def gid_of(rec: np.ndarray) -> np.ndarray:
    return rec["color"][:, 3].view(np.uint32)


def set_gid(rec: np.ndarray, gid: np.ndarray) -> None:
    rec["color"][:, 3] = np.asarray(gid, dtype=np.uint32).view(np.float32)


def realign(values, gid_before, gid_after):
    """`values` aligned with records of ids `gid_before`, reordered to ids `gid_after` (the same
    set, permuted by a step)."""
    order = np.argsort(gid_before, kind="stable")
    return values[order[np.searchsorted(gid_before[order], gid_after)]]


class SlabRank:
    """Rank `rank`'s part of a decomposed scene over numpy records.

    `records`: the whole scene's initial records (global order) — each rank takes the records of
    its held region from them.  `local_step(rec)` steps a record array in place (hash-sorted on
    return) with the whole scene's table size.  A step is `advance` (step locally; returns
    {neighbour: (records, w, alpha)} to send) then `absorb` (the parts received); `step` does both
    through an exchange callable, `step_all` for every rank in one process."""

    def __init__(self, records: np.ndarray, plan: SlabPlan, rank: int):
        self.plan, self.rank, self.n_global = plan, rank, records.shape[0]
        x = records["position"][:, 0]
        sel = np.flatnonzero(plan.held(x, rank))           # global order kept
        self.rec = records[sel].copy()
        self.alpha = records["color"][sel, 3].copy()        # the caller's colour[3], per record
        set_gid(self.rec, sel.astype(np.uint32))
        self.sent_records = 0                               # exchange volume, for the tests
        self._kept = None

    def owned_mask(self) -> np.ndarray:
        return self.plan.owner(self.rec["position"][:, 0]) == self.rank

    def advance(self, local_step) -> dict:
        """Steps the held records and returns what to send: {neighbour: (records, w, alpha)}."""
        gid_before = gid_of(self.rec).copy()
        trusted_gid = gid_before[self.owned_mask()]
        local_step(self.rec)
        rec = self.rec
        gid = gid_of(rec)
        alpha = realign(self.alpha, gid_before, gid)
        w = cluster_positions(rec["hash"], cell_of(rec["position"], self.plan.cell))
        trusted = np.isin(gid, trusted_gid)
        x = rec["position"][:, 0]
        sends = {}
        for nb in (self.rank - 1, self.rank + 1):
            if 0 <= nb < self.plan.world:
                m = trusted & self.plan.held(x, nb)
                sends[nb] = (rec[m].copy(), w[m].copy(), alpha[m].copy())
                self.sent_records += int(m.sum())
        keep = trusted & self.plan.held(x, self.rank)
        self._kept = (rec[keep].copy(), w[keep].copy(), alpha[keep].copy())
        return sends

    def absorb(self, received) -> None:
        """Merges the kept trusted records with the neighbours' and orders them for the next
        step by (hash, w, particle id)."""
        parts = [self._kept] + list(received)
        new = np.concatenate([p[0] for p in parts])
        nw = np.concatenate([p[1] for p in parts])
        na = np.concatenate([p[2] for p in parts])
        order = order_key(new["hash"], nw, gid_of(new))
        self.rec, self.alpha = new[order], na[order]
        self._kept = None

    def step(self, local_step, exchange) -> None:
        """One step: `exchange(sends) -> received` (e.g. `neighbour_exchange`)."""
        self.absorb(exchange(self.advance(local_step)))

    def owned_records(self):
        """(owned records with the caller's colour[3] restored, their particle ids)."""
        m = self.owned_mask()
        out = self.rec[m].copy()
        gid = gid_of(out).copy()
        out["color"][:, 3] = self.alpha[m]
        return out, gid


def step_all(ranks, local_step) -> None:
    """One step of every rank of a decomposition held in this process (the exchange is a direct
    hand-over of each rank's sends to its neighbours)."""
    inbox = {r.rank: [] for r in ranks}
    for r in ranks:
        for dst, payload in r.advance(local_step).items():
            inbox[dst].append(payload)
    for r in ranks:
        r.absorb(inbox[r.rank])


def gather_by_gid(ranks_or_parts, n: int):
    """The owned records of all ranks, indexed by particle id (test and debugging aid: this is
    O(N) and not part of a step).  Accepts SlabRank objects or (records, gid) pairs."""
    parts = [r.owned_records() if hasattr(r, "owned_records") else r for r in ranks_or_parts]
    rec = np.concatenate([p[0] for p in parts])
    gid = np.concatenate([p[1] for p in parts]).astype(np.int64)
    if rec.shape[0] != n or np.unique(gid).size != n:
        raise RuntimeError("every particle must have exactly one owner")
    out = np.empty_like(rec)
    out[gid] = rec
    return out


def neighbour_exchange(sends, rank: int, world: int, group=None):
    """Point-to-point exchange of numpy (records, w, alpha) with the neighbouring ranks over
    torch.distributed (gloo): counts first, then the bytes.  Returns the received parts."""
    import torch
    import torch.distributed as dist

    from ._abi import PARTICLE_DTYPE

    recs = []
    nbs = [nb for nb in (rank - 1, rank + 1) if 0 <= nb < world]
    counts_out = {nb: torch.tensor([sends[nb][0].shape[0]], dtype=torch.int64) for nb in nbs}
    counts_in = {nb: torch.zeros(1, dtype=torch.int64) for nb in nbs}
    reqs = []
    for nb in nbs:
        reqs.append(dist.isend(counts_out[nb], nb, group=group))
        reqs.append(dist.irecv(counts_in[nb], nb, group=group))
    for q in reqs:
        q.wait()
    reqs, bufs = [], {}
    for nb in nbs:
        rec, w, alpha = sends[nb]
        payload = np.concatenate([rec.view(np.uint8).reshape(-1),
                                  w.astype(np.uint32).view(np.uint8),
                                  alpha.astype(np.float32).view(np.uint8)])
        reqs.append(dist.isend(torch.from_numpy(payload.copy()), nb, group=group))
        k = int(counts_in[nb].item())
        bufs[nb] = (k, torch.empty(k * (PARTICLE_DTYPE.itemsize + 8), dtype=torch.uint8))
        reqs.append(dist.irecv(bufs[nb][1], nb, group=group))
    for q in reqs:
        q.wait()
    for nb in nbs:
        k, buf = bufs[nb]
        b = buf.numpy()
        nb_rec = k * PARTICLE_DTYPE.itemsize
        rec = b[:nb_rec].view(PARTICLE_DTYPE).copy()
        w = b[nb_rec:nb_rec + 4 * k].view(np.uint32).copy()
        alpha = b[nb_rec + 4 * k:].view(np.float32).copy()
        recs.append((rec, w, alpha))
    return recs


# ------------------------------------------------------------------------------ device-resident
# The same decomposition over records that stay on a GPU: torch uint8 tensors of k x 108-byte
# records (the attached-buffer layout).  Every operation is a torch operation on the held records
# of this rank (O(held), never the whole scene); the local step is any callable stepping a record
# tensor in place (the CUDA solver).
REC_BYTES = 108
_W_X, _W_HASH, _W_TAG = 0, 21, 25  # word offsets: position.x, hash, colour[3]


def _words(rec):
    import torch

    return rec.view(torch.float32), rec.view(torch.int32)


def cluster_positions_device(hashes, cells):
    """cluster_positions on device tensors (hashes int64 [n], cells int64 [n, 3]); the rare runs
    spread over far-apart cells are finished on the host."""
    import torch

    n = hashes.numel()
    dev = hashes.device
    if n == 0:
        return torch.zeros(0, dtype=torch.int64, device=dev)
    new_run = torch.ones(n, dtype=torch.bool, device=dev)
    new_run[1:] = hashes[1:] != hashes[:-1]
    run_id = torch.cumsum(new_run.to(torch.int64), 0) - 1
    start = torch.nonzero(new_run).squeeze(1)
    w = torch.arange(n, device=dev) - start[run_id]
    runs = start.numel()
    idx = run_id.unsqueeze(1).expand(-1, 3)
    big = torch.iinfo(torch.int64).max
    mx = torch.full((runs, 3), -big, dtype=torch.int64, device=dev).scatter_reduce(
        0, idx, cells, "amax")
    mn = torch.full((runs, 3), big, dtype=torch.int64, device=dev).scatter_reduce(
        0, idx, cells, "amin")
    bad = torch.nonzero((mx - mn).amax(dim=1) > LINK_CELLS).squeeze(1).tolist()
    if bad:
        end = torch.cat([start[1:], torch.tensor([n], device=dev)])
        for k in bad:
            a, b = int(start[k]), int(end[k])
            w[a:b] = torch.from_numpy(
                _cluster_positions_slow(cells[a:b].cpu().numpy()).astype(np.int64)).to(dev)
    return w


def _realign_device(values, gid_before, gid_after):
    import torch

    order = torch.argsort(gid_before, stable=True)
    return values[order[torch.searchsorted(gid_before[order], gid_after)]]


class SlabRankDevice:
    """SlabRank over device-resident record tensors (uint8 [k, 108]); `local_step(buf)` steps the
    flat uint8 tensor `buf` in place (e.g. PBFSolver.step on an attached device buffer with the
    whole scene's table size)."""

    def __init__(self, records, plan: SlabPlan, rank: int):
        import torch

        rows = records.view(-1, REC_BYTES)
        f, _ = _words(rows)
        self.plan, self.rank, self.n_global = plan, rank, rows.shape[0]
        sel = torch.nonzero(self._held(f[:, _W_X], rank)).squeeze(1)  # global order kept
        self.rec = rows[sel].contiguous()
        self.alpha = f[sel, _W_TAG].clone()
        _words(self.rec)[1][:, _W_TAG] = sel.to(torch.int32)
        self.sent_records = 0
        self._kept = None

    def _held(self, x, rank):
        lo, hi = self.plan.held_range(rank)
        xd = x.double()
        return (xd >= lo) & (xd < hi)

    def _owner(self, x):
        import torch

        r = torch.floor((x.double() - self.plan.x_min) / self.plan.width).to(torch.int64)
        return torch.clamp(r, 0, self.plan.world - 1)

    def gid(self, rec=None):
        import torch

        rec = self.rec if rec is None else rec
        return _words(rec)[1][:, _W_TAG].to(torch.int64) & 0xFFFFFFFF

    def owned_mask(self):
        return self._owner(_words(self.rec)[0][:, _W_X]) == self.rank

    def advance(self, local_step) -> dict:
        import torch

        gid_before = self.gid()
        trusted_gid = gid_before[self.owned_mask()]
        local_step(self.rec.view(-1))
        rec = self.rec
        f, iw = _words(rec)
        gid = self.gid()
        alpha = _realign_device(self.alpha, gid_before, gid)
        hashes = iw[:, _W_HASH].to(torch.int64) & 0xFFFFFFFF
        cells = torch.floor(f[:, 0:3] / torch.tensor(self.plan.cell, dtype=torch.float32,
                                                     device=rec.device)).to(torch.int64)
        w = cluster_positions_device(hashes, cells)
        trusted = torch.isin(gid, trusted_gid)
        x = f[:, _W_X]
        sends = {}
        for nb in (self.rank - 1, self.rank + 1):
            if 0 <= nb < self.plan.world:
                m = trusted & self._held(x, nb)
                sends[nb] = (rec[m].contiguous(), w[m].to(torch.int32), alpha[m].contiguous())
                self.sent_records += int(m.sum())
        keep = trusted & self._held(x, self.rank)
        self._kept = (rec[keep].contiguous(), w[keep].to(torch.int32), alpha[keep].contiguous())
        return sends

    def absorb(self, received) -> None:
        import torch

        parts = [self._kept] + list(received)
        new = torch.cat([p[0] for p in parts])
        nw = torch.cat([p[1] for p in parts]).to(torch.int64)
        na = torch.cat([p[2] for p in parts])
        gid = self.gid(new)
        hashes = _words(new)[1][:, _W_HASH].to(torch.int64) & 0xFFFFFFFF
        # (hash, w, particle id): stable sorts from the last key to the first
        o1 = torch.argsort(gid, stable=True)
        o2 = torch.argsort(((hashes << 31) | nw)[o1], stable=True)
        order = o1[o2]
        self.rec, self.alpha = new[order].contiguous(), na[order].contiguous()
        self._kept = None

    def step(self, local_step, exchange) -> None:
        self.absorb(exchange(self.advance(local_step)))

    def owned_records(self):
        """(owned records [k, 108] with the caller's colour[3] restored, their particle ids)."""
        m = self.owned_mask()
        out = self.rec[m].clone()
        _words(out)[0][:, _W_TAG] = self.alpha[m]
        return out, self.gid()[m]


def gather_by_gid_device(ranks, n: int):
    """All ranks' owned device records indexed by particle id (O(N): tests and debugging)."""
    import torch

    parts = [r.owned_records() for r in ranks]
    rec = torch.cat([p[0] for p in parts])
    gid = torch.cat([p[1] for p in parts])
    if rec.shape[0] != n or torch.unique(gid).numel() != n:
        raise RuntimeError("every particle must have exactly one owner")
    out = torch.empty_like(rec)
    out[gid] = rec
    return out


def neighbour_exchange_device(sends, rank: int, world: int, group=None):
    """Point-to-point exchange of (records, w, alpha) tensors with the neighbouring ranks over
    torch.distributed: NCCL for CUDA tensors, gloo for CPU ones.  Counts first, then one byte
    payload per neighbour.  Returns the received parts."""
    import torch
    import torch.distributed as dist

    nbs = [nb for nb in (rank - 1, rank + 1) if 0 <= nb < world]
    dev = next(iter(sends.values()))[0].device if sends else torch.device("cpu")
    c_out = {nb: torch.tensor([sends[nb][0].shape[0]], dtype=torch.int64, device=dev) for nb in nbs}
    c_in = {nb: torch.zeros(1, dtype=torch.int64, device=dev) for nb in nbs}
    reqs = []
    for nb in nbs:
        reqs += [dist.isend(c_out[nb], nb, group=group), dist.irecv(c_in[nb], nb, group=group)]
    for q in reqs:
        q.wait()
    reqs, bufs = [], {}
    for nb in nbs:
        rec, w, alpha = sends[nb]
        payload = torch.cat([rec.reshape(-1), w.contiguous().view(torch.uint8),
                             alpha.contiguous().view(torch.uint8)])
        reqs.append(dist.isend(payload, nb, group=group))
        k = int(c_in[nb].item())
        bufs[nb] = (k, torch.empty(k * (REC_BYTES + 8), dtype=torch.uint8, device=dev))
        reqs.append(dist.irecv(bufs[nb][1], nb, group=group))
    for q in reqs:
        q.wait()
    out = []
    for nb in nbs:
        k, b = bufs[nb]
        rec = b[:k * REC_BYTES].view(k, REC_BYTES)
        w = b[k * REC_BYTES:k * (REC_BYTES + 4)].view(torch.int32)
        alpha = b[k * (REC_BYTES + 4):].view(torch.float32)
        out.append((rec, w, alpha))
    return out
