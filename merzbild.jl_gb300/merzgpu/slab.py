"""Slab decomposition of a 1-D grid: one process per GPU, each owning a
contiguous range of cells (a slab), and the particle exchange after
convection.

The reference runs a chunked multithreaded simulation: the cells are split
into contiguous chunks (ChunkSplitters' `chunks(1:nx; n=n_chunks)`, equal
sizes with the remainder on the first chunks;
simulations/1D/couette_multithreaded.jl:14-37), each chunk with its own
ParticleVector and ParticleIndexerArray, and after convection
exchange_particles! / sort_particles_after_exchange! (parallel.jl:281-532)
move every particle that left a chunk into the chunk that now holds its cell.

Here a rank's Domain holds its slab's cells, keyed on their global cell ids
(Domain.set_cell_rng), and convects on the global grid and walls.  A particle
moves less than a slab's length in a step (|v| dt is a fraction of a cell in
the reference's set-ups), so it can only enter a neighbouring slab: the
exchange is neighbour to neighbour, a count and then the particles' 7-double
records (w, vx, vy, vz, x, y, z), staged through host memory and sent with
torch.distributed point-to-point calls.  There is no collective on the data
path.  The arrivals from the left go before the rank's own particles and
those from the right after them, which, with the stable sort by cell, gives
every cell the particle order of a single domain over the whole grid: a
sharded equal-weight run equals the single-domain run bit for bit.
"""
from __future__ import annotations

import numpy as np

RECORD = 7  # doubles per exchanged particle: w, vx, vy, vz, x, y, z


def slab_bounds(n_cells: int, n_slabs: int, i: int) -> tuple[int, int]:
    """(first global cell, number of cells) of slab i (0-based) of n_slabs:
    equal sizes, the first n_cells % n_slabs slabs one cell larger."""
    if not (0 <= i < n_slabs) or n_slabs > n_cells:
        raise ValueError("slab_bounds: need 0 <= i < n_slabs <= n_cells")
    base, extra = divmod(n_cells, n_slabs)
    c0 = i * base + min(i, extra)
    return c0, base + (1 if i < extra else 0)


def neighbour_exchange(to_left: np.ndarray, to_right: np.ndarray, rank: int, world_size: int, group=None):
    """Send to_left to rank - 1 and to_right to rank + 1, receive what they
    send back; returns (from the left, from the right), (n, 7) float64 each.

    Counts go first (one int64 each way), then the records; both directions
    are posted at once (isend / irecv), so no pair of ranks waits on the
    other.  The end slabs have no neighbour outside: a particle staged that
    way is an error (it left through a wall that did not reflect it)."""
    import torch
    import torch.distributed as dist

    to_left = np.ascontiguousarray(to_left, np.float64).reshape(-1, RECORD)
    to_right = np.ascontiguousarray(to_right, np.float64).reshape(-1, RECORD)
    left = rank - 1 if rank > 0 else None
    right = rank + 1 if rank < world_size - 1 else None
    if left is None and to_left.shape[0]:
        raise RuntimeError(f"slab exchange: {to_left.shape[0]} particles left the first slab through its left end")
    if right is None and to_right.shape[0]:
        raise RuntimeError(f"slab exchange: {to_right.shape[0]} particles left the last slab through its right end")
    peers = [(p, buf) for p, buf in ((left, to_left), (right, to_right)) if p is not None]
    n_out = {p: torch.tensor([buf.shape[0]], dtype=torch.int64) for p, buf in peers}
    n_in = {p: torch.zeros(1, dtype=torch.int64) for p, _ in peers}
    reqs = []
    for p, _ in peers:
        reqs.append(dist.isend(n_out[p], p, group=group, tag=1))
        reqs.append(dist.irecv(n_in[p], p, group=group, tag=1))
    for r in reqs:
        r.wait()
    data_in = {p: torch.empty((int(n_in[p].item()), RECORD), dtype=torch.float64) for p, _ in peers}
    reqs = []
    for p, buf in peers:
        if buf.shape[0]:
            reqs.append(dist.isend(torch.from_numpy(buf), p, group=group, tag=2))
        if data_in[p].shape[0]:
            reqs.append(dist.irecv(data_in[p], p, group=group, tag=2))
    for r in reqs:
        r.wait()
    empty = np.empty((0, RECORD))
    from_left = data_in[left].numpy() if left is not None else empty
    from_right = data_in[right].numpy() if right is not None else empty
    return from_left, from_right


class Slab:
    """One rank's slab: `engine` holds the cells [c0, c0 + n) of the global
    grid `grid` (a Domain, or any object with the Domain's slab_extract /
    slab_fetch / slab_insert methods), and exchange() moves the particles
    that left it to the neighbouring ranks and takes theirs in.

    Call order per step (the reference's chunked loop):
    collisions -> convection on the global grid and walls (without computing
    cells) -> exchange() -> props.  A Domain engine gets its cells' streams
    keyed on the global cell ids here."""

    def __init__(self, engine, grid, c0: int, rank: int, world_size: int, group=None, n_species: int = 1):
        self.engine = engine
        self.grid = grid
        self.c0 = int(c0)
        self.rank = int(rank)
        self.world_size = int(world_size)
        self.group = group
        self.n_species = int(n_species)
        n = getattr(engine, "n_cells")
        if self.c0 < 0 or self.c0 + n > grid.n_cells:
            raise ValueError("Slab: the slab lies outside the global grid")
        if hasattr(engine, "set_cell_rng"):
            engine.set_cell_rng(rids=self.c0 + np.arange(n, dtype=np.uint32))

    def exchange(self, species=None):
        """Exchange the particles of one species (default: every species);
        returns the number sent per species as (to the left, to the right)."""
        out = []
        for s in range(self.n_species) if species is None else [species]:
            nl, nr = self.engine.slab_extract(s, self.grid, self.c0)
            to_left, to_right = self.engine.slab_fetch(s)
            from_left, from_right = neighbour_exchange(to_left, to_right, self.rank, self.world_size, self.group)
            self.engine.slab_insert(s, self.grid, self.c0, from_left, from_right)
            out.append((nl, nr))
        return out


def exchange_local(slabs, species: int = 0):
    """The same exchange between slabs held by one process (consecutive in
    `slabs`, e.g. several slabs on one GPU): every slab's leaving particles
    are staged first, then every slab takes its neighbours'."""
    staged = []
    for sl in slabs:
        sl.engine.slab_extract(species, sl.grid, sl.c0)
        staged.append(sl.engine.slab_fetch(species))
    empty = np.empty((0, RECORD))
    for i, sl in enumerate(slabs):
        if i == 0 and staged[0][0].shape[0]:
            raise RuntimeError("slab exchange: particles left the first slab through its left end")
        if i == len(slabs) - 1 and staged[i][1].shape[0]:
            raise RuntimeError("slab exchange: particles left the last slab through its right end")
        from_left = staged[i - 1][1] if i > 0 else empty
        from_right = staged[i + 1][0] if i + 1 < len(slabs) else empty
        sl.engine.slab_insert(species, sl.grid, sl.c0, from_left, from_right)
