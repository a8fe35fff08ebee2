"""Domain-decomposed flock over the ranks of a process group: the
counterpart of BoidSimulationMultiNode (src/boid_simulation_mpi.{h,cpp}).

The field is cut into px x py x pz blocks, one per rank
(src/boid_simulation_mpi.cpp:151-160).  A rank owns the boids whose
position lies in its block and also holds those within a margin of it
(margin = the largest sight distance, :162-185), so that every neighbour of
an owned boid is local.  One update of a rank:

1. its local boids (owned and margin), in ascending global id, go through
   the engine's update (`BoidSimulation.set_population` + `update`): the
   accumulation order of the reference is ascending id, so the owned boids'
   new states are bit-identical to those of one engine holding the whole
   flock;
2. it keeps the new states of the boids it owned;
3. one exchange (`all_to_all_single`, the counts first): every owned boid
   goes to each other rank whose block-plus-margin region now contains it,
   the owner of its new block among them, as the reference's border
   exchange does (:474-499, there over MPI point-to-point to <= 26
   neighbours); a rank keeps those of its own that are still in its region.

`gather` collects the owned boids of all ranks in id order
(MPI_Gather + sort, :555-586).  The reference's MPI engine also changes the
periodic wrap (x >= F and an FLT_EPSILON fix-up, :362-388); this one keeps
the single-engine arithmetic, so that its result equals one GPU's.

The exchange runs on torch.distributed (NCCL between GPUs, gloo on CPU);
the local update runs on the rank's GPU through the library's C ABI.  A
test may pass another engine with the same four methods.
"""
from __future__ import annotations

import numpy as np


def dims_create(size: int) -> tuple[int, int, int]:
    """A balanced px * py * pz == size (as MPI_Dims_create): the prime
    factors, largest first, each to the smallest dimension so far."""
    dims = [1, 1, 1]
    f, n, primes = 2, size, []
    while f * f <= n:
        while n % f == 0:
            primes.append(f)
            n //= f
        f += 1
    if n > 1:
        primes.append(n)
    for q in sorted(primes, reverse=True):
        i = min(range(3), key=lambda j: (dims[j], -j))
        dims[i] *= q
    return tuple(sorted(dims))


class Decomposition:
    """Blocks of a periodic cube of side `field` over a px x py x pz grid of
    ranks (rank = (ix * py + iy) * pz + iz) and the margin around them."""

    def __init__(self, field: float, topology: tuple[int, int, int], margin: float):
        self.F = float(field)
        self.dims = tuple(int(d) for d in topology)
        self.margin = float(margin)
        for d in self.dims:
            if d < 1:
                raise ValueError("topology dimensions must be positive")
            # a boid reaches only the blocks next to its own
            if d > 1 and self.F / d < 2.0 * self.margin:
                raise ValueError("blocks thinner than twice the margin (%g / %d < 2 x %g)" % (self.F, d, self.margin))

    @property
    def size(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    def rank_of(self, b: np.ndarray) -> np.ndarray:
        """Rank of block indices b (..., 3)."""
        return (b[..., 0] * self.dims[1] + b[..., 1]) * self.dims[2] + b[..., 2]

    def block_of_rank(self, rank: int) -> np.ndarray:
        px, py, pz = self.dims
        return np.array([rank // (py * pz), (rank // pz) % py, rank % pz])

    def blocks(self, pos: np.ndarray) -> np.ndarray:
        """Block index along each axis of positions (n, 3) in [0, F]."""
        d = np.asarray(self.dims)
        w = self.F / d
        return np.minimum((np.asarray(pos, np.float64) / w).astype(np.int64), d - 1).clip(0)

    def owners(self, pos: np.ndarray) -> np.ndarray:
        return self.rank_of(self.blocks(pos))

    # the 26 offsets from a block to its neighbours
    _OFF = np.array([[ox, oy, oz] for ox in (-1, 0, 1) for oy in (-1, 0, 1) for oz in (-1, 0, 1)
                     if (ox, oy, oz) != (0, 0, 0)])

    def destinations(self, pos: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """(boid index, rank) pairs: every rank whose block or margin holds
        the boid, its owner first, each pair once."""
        pos = np.asarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        d = np.asarray(self.dims)
        w = self.F / d
        b = self.blocks(pos)
        owner = self.rank_of(b)
        # only boids within the margin of a face between two blocks reach
        # another block: the others go to their owner alone
        lo = b * w
        near_lo = ((pos - lo) < self.margin) & (d > 1)         # also in the margin of block b - 1
        near_hi = ((lo + w - pos) <= self.margin) & (d > 1)    # ... of block b + 1
        edge = np.nonzero(np.any(near_lo | near_hi, axis=1))[0]
        ei, er = [], []
        for off in self._OFF:
            if np.any((off != 0) & (d == 1)):
                continue
            m = np.ones(edge.size, bool)
            for a in range(3):
                if off[a] < 0:
                    m &= near_lo[edge, a]
                elif off[a] > 0:
                    m &= near_hi[edge, a]
            sel = edge[m]
            if sel.size:
                ei.append(sel)
                er.append(self.rank_of((b[sel] + off) % d))
        if ei:
            # a blocks-of-two axis reaches the same neighbour both ways: each pair once
            key = np.unique(np.concatenate(ei).astype(np.int64) * self.size + np.concatenate(er))
            ei, er = key // self.size, key % self.size
        else:
            ei, er = np.zeros(0, np.int64), np.zeros(0, np.int64)
        return np.concatenate([np.arange(n, dtype=np.int64), ei]), np.concatenate([owner.astype(np.int64), er])


class HaloFlock:
    """One rank's part of a domain-decomposed flock.

    engine: an object with set_population(pos, vel), update(1), state() and
    forces() (a `BoidSimulation` set up for the whole flock's N, made by
    default on the rank's GPU); group: a torch.distributed process group
    (None: one rank, no exchange)."""

    def __init__(self, n, field, sep, ali, coh, vmax, vmin, engine=None, group=None, topology=None,
                 device=None, record_forces=False):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.multi = group is not None
        self.rank = dist.get_rank(group) if self.multi else 0
        self.size = dist.get_world_size(group) if self.multi else 1
        topology = tuple(topology) if topology else dims_create(self.size)
        if topology[0] * topology[1] * topology[2] != self.size:
            raise ValueError("topology %r does not hold %d ranks" % (topology, self.size))
        self.N, self.F = int(n), float(field)
        radius = max(sep[0], ali[0], coh[0])
        # the margin keeps every boid within the largest radius of an owned
        # boid; the slack covers the rounding of the block bounds
        self.dec = Decomposition(field, topology, radius * (1.0 + 1e-3) + self.F * 1e-6)
        self.block = self.dec.block_of_rank(self.rank)
        if engine is None:
            from . import BoidSimulation
            engine = BoidSimulation("grid", device=0 if device is None else device, record_forces=record_forces)
            engine.setup(n, field, *sep, *ali, *coh, vmax, vmin)
        self.engine = engine
        self.ids = np.zeros(0, np.int64)
        self.pos = np.zeros((0, 3), np.float32)
        self.vel = np.zeros((0, 3), np.float32)
        self.force = None
        self.steps_done = 0

    def init(self, kind: str = "random_uniform", seed: int = 12345):
        """BoidSimulation::init of the whole flock on every rank (the same
        seeded draw everywhere, in place of the reference's MPI_Bcast,
        src/boid_simulation_mpi.cpp:186-199), then this rank's part."""
        self.engine.initialization_type = kind
        self.engine.rand_seed = seed
        self.engine.init()
        p, v = self.engine.state()
        self.set_global_state(p, v)

    # ---- the rank's local set
    def _owned(self) -> np.ndarray:
        return self.dec.owners(self.pos) == self.rank

    def set_global_state(self, pos, vel):
        """Take this rank's block and margin from a whole-flock state in id
        order (every rank holds the same state: no collective)."""
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        vel = np.asarray(vel, np.float32).reshape(-1, 3)
        if pos.shape[0] != self.N or vel.shape != pos.shape:
            raise ValueError("expected %d boids" % self.N)
        i, r = self.dec.destinations(pos)
        mine = np.unique(i[r == self.rank])
        self.ids, self.pos, self.vel = mine, pos[mine].copy(), vel[mine].copy()
        self.force = None

    # ---- one update of every rank
    def _exchange(self, send_idx: list, payload: np.ndarray) -> np.ndarray:
        """Rows payload[send_idx[r]] to rank r; the rows received, rank order."""
        import torch
        dist = self.dist
        dev = torch.device("cuda", torch.cuda.current_device()) \
            if dist.get_backend(self.group) == "nccl" else torch.device("cpu")
        counts = torch.tensor([len(s) for s in send_idx], dtype=torch.int64, device=dev)
        rcounts = torch.empty_like(counts)
        dist.all_to_all_single(rcounts, counts, group=self.group)
        width = payload.shape[1]
        out_rows = np.concatenate([payload[s] for s in send_idx]) if len(payload) else payload[:0]
        send = torch.from_numpy(np.ascontiguousarray(out_rows).reshape(-1)).to(dev)
        rc = rcounts.cpu().tolist()
        recv = torch.empty(sum(rc) * width, dtype=send.dtype, device=dev)
        dist.all_to_all_single(recv, send, output_split_sizes=[c * width for c in rc],
                               input_split_sizes=[len(s) * width for s in send_idx], group=self.group)
        return recv.cpu().numpy().reshape(-1, width)

    def update(self, steps: int = 1):
        for _ in range(int(steps)):
            self._update_once()

    def _update_once(self):
        own = self._owned()
        # 1. the local boids' update, ascending global id (self.ids is sorted)
        self.engine.set_population(self.pos, self.vel)
        self.engine.update(1)
        p, v = self.engine.state()
        f = self.engine.forces() if getattr(self.engine, "record_forces", False) else None
        ids, p, v = self.ids[own], p[own], v[own]
        self.force = (ids, f[own]) if f is not None else None
        # 2-3. the exchange: each owned boid to every rank whose region holds it
        bi, br = self.dec.destinations(p)
        keep = np.unique(bi[br == self.rank])
        if self.multi and self.size > 1:
            rows = np.concatenate([ids.astype(np.int64).view(np.float32).reshape(-1, 2), p, v], 1) \
                if len(ids) else np.zeros((0, 8), np.float32)
            send = [bi[br == r] if r != self.rank else np.zeros(0, np.int64) for r in range(self.size)]
            got = self._exchange(send, rows)
            rid = np.ascontiguousarray(got[:, :2]).view(np.int64).reshape(-1)
            ids = np.concatenate([ids[keep], rid])
            p = np.concatenate([p[keep], got[:, 2:5]])
            v = np.concatenate([v[keep], got[:, 5:8]])
        else:
            ids, p, v = ids[keep], p[keep], v[keep]
        order = np.argsort(ids, kind="stable")
        ids, p, v = ids[order], p[order], v[order]
        if ids.size > 1 and np.any(ids[1:] == ids[:-1]):
            raise RuntimeError("a boid arrived twice")
        self.ids, self.pos, self.vel = ids, np.ascontiguousarray(p), np.ascontiguousarray(v)
        self.steps_done += 1

    # ---- the whole flock
    def owned_state(self):
        """(ids, pos, vel) of the boids this rank owns."""
        own = self._owned()
        return self.ids[own], self.pos[own], self.vel[own]

    def _gather_rows(self, ids: np.ndarray, vals: np.ndarray) -> np.ndarray:
        """Rows vals (one per id, float32) of every rank's ids, in id order
        over the whole flock, on every rank (all_gather, padded to the
        largest count)."""
        vals = np.asarray(vals, np.float32).reshape(len(ids), -1)
        width = 2 + vals.shape[1]
        rows = np.concatenate([ids.astype(np.int64).view(np.float32).reshape(-1, 2), vals], 1) \
            if len(ids) else np.zeros((0, width), np.float32)
        if self.multi and self.size > 1:
            import torch
            dist = self.dist
            dev = torch.device("cuda", torch.cuda.current_device()) \
                if dist.get_backend(self.group) == "nccl" else torch.device("cpu")
            cnt = torch.tensor([len(ids)], dtype=torch.int64, device=dev)
            cnts = [torch.empty_like(cnt) for _ in range(self.size)]
            dist.all_gather(cnts, cnt, group=self.group)
            cmax = int(max(int(c.item()) for c in cnts))
            buf = torch.zeros(cmax * width, dtype=torch.float32, device=dev)
            buf[:rows.size] = torch.from_numpy(np.ascontiguousarray(rows).reshape(-1)).to(dev)
            outs = [torch.empty_like(buf) for _ in range(self.size)]
            dist.all_gather(outs, buf, group=self.group)
            rows = np.concatenate([o.cpu().numpy().reshape(-1, width)[:int(c.item())] for o, c in zip(outs, cnts)])
        gid = np.ascontiguousarray(rows[:, :2]).view(np.int64).reshape(-1)
        if gid.size != self.N or np.any(np.sort(gid) != np.arange(self.N)):
            raise RuntimeError("the ranks do not own every boid exactly once")
        return rows[np.argsort(gid), 2:].copy()

    def gather(self):
        """The whole flock in id order, (pos, vel) of shape (N, 3), on every
        rank (the reference's gather_data: MPI_Gather and a sort by id,
        src/boid_simulation_mpi.cpp:555-586)."""
        ids, p, v = self.owned_state()
        r = self._gather_rows(ids, np.concatenate([p, v], 1))
        return r[:, 0:3], r[:, 3:6]

    def gather_forces(self):
        """get_force of the last update for every boid, (N, 9) in id order
        (cohesion, separation, alignment xyz), on every rank; needs an
        engine that records forces."""
        if self.force is None:
            raise RuntimeError("no forces: no update yet, or an engine without force recording")
        ids, f = self.force
        return self._gather_rows(ids, f)
