"""Slab decomposition of a 1-D grid on the CPU (merzgpu/slab.py): gloo ranks,
each holding one slab of a Couette grid in an oracle state keyed on its global
cells, run the reference's per-step loop (ntc_equal_weight!, convection on the
global grid and walls) with the slab exchange over torch.distributed between
neighbours; the slabs' particles together equal a single-domain oracle run bit
for bit.  The reference moves particles between the cell chunks of one grid
with exchange_particles! / sort_particles_after_exchange! (parallel.jl:281-532);
the chunks follow ChunkSplitters' batch split
(simulations/1D/couette_multithreaded.jl:31)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NX, PPC, L, NDENS, T0, V_WALL, STEPS, SEED = 48, 40, 5e-4, 1e23, 273.0, 500.0, 12, 77


def _paths():
    for p in (ROOT, os.path.join(ROOT, "merzbild.jl_gb300"), os.path.join(ROOT, "oracle"),
              os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _setup():
    """Initial particles (cell order, stable), the configuration and the
    single-domain oracle."""
    import merzgpu as mz
    import oracle

    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    grid = mz.Grid1DUniform(L, NX)
    Fnum = grid.dx * NDENS / PPC
    walls = mz.MaxwellWalls1D(sp, T0, T0, -V_WALL, V_WALL, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T0)
    rng = np.random.default_rng(SEED)
    n = PPC * NX
    cell = np.sort(rng.integers(0, NX, size=n))
    x = np.column_stack([(cell + rng.uniform(0.02, 0.98, size=n)) * grid.dx, rng.random(n), rng.random(n)])
    v = rng.normal(0.0, np.sqrt(mz.K_B * T0 / mz.AR_MASS), size=(n, 3))
    rows = np.column_stack([np.full(n, Fnum), v, x])
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T0, T0, Fnum)
    return oracle, grid, walls, dt, rows, cell, smax


def _oracle(oracle, n_cells, rows, cells0, smax):
    import merzgpu as mz

    o = oracle.Oracle(n_cells, 1, [mz.AR_MASS])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    o.set_particles_simple(0, cells0 + 1, rows)
    o.cf_set_smax(0, 0, smax)
    return o


class OracleSlabEngine:
    """The slab calls of a Domain restated on an oracle state: particles in
    logical order split by global cell (x * inv_dx, the device's mapping),
    arrivals placed [from the left | own | from the right], then grouped by
    cell stably."""

    def __init__(self, o, n_cells):
        self.o = o
        self.n_cells = n_cells
        self.pending = None

    def slab_extract(self, s, grid, c0):
        rows, _ = self.o.logical(s)
        g = np.clip(np.floor(rows[:, 4] * grid.inv_dx).astype(np.int64), 0, grid.n_cells - 1)
        left, right = g < c0, g >= c0 + self.n_cells
        own = ~(left | right)
        self.pending = (rows[left], rows[own], rows[right])
        return int(left.sum()), int(right.sum())

    def slab_fetch(self, s):
        return self.pending[0], self.pending[2]

    def slab_insert(self, s, grid, c0, from_left, from_right):
        rows = np.concatenate([np.asarray(from_left).reshape(-1, 7), self.pending[1],
                               np.asarray(from_right).reshape(-1, 7)])
        g = np.clip(np.floor(rows[:, 4] * grid.inv_dx).astype(np.int64), 0, grid.n_cells - 1)
        assert np.all((g >= c0) & (g < c0 + self.n_cells)), "an arrival beyond the neighbouring slab"
        self.o.set_particles_simple(s, g - c0 + 1, rows)
        self.pending = None


def _rank_main(rank, world, port, out):
    _paths()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    from merzgpu.slab import Slab, slab_bounds

    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle, grid, walls, dt, rows, cell, smax = _setup()
    c0, n = slab_bounds(NX, world, rank)
    mine = (cell >= c0) & (cell < c0 + n)
    o = _oracle(oracle, n, rows[mine], cell[mine] - c0, smax)
    o.set_cell_offset(c0)
    slab = Slab(OracleSlabEngine(o, n), grid, c0, rank, world)
    sent = np.zeros(2, np.int64)
    for step in range(1, STEPS + 1):
        o.ntc_cells(0, 0, dt, grid.V[:n], SEED, step, equal_weight=True)
        o.convect(0, L, NX, walls.as_flat_array(), dt, SEED, step)
        (nl, nr), = slab.exchange()
        sent += (nl, nr)
    rows_out, cells_out = o.logical(0)
    out.put((rank, rows_out, cells_out - 1 + c0, sent))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_slab_exchange_over_gloo_equals_the_single_domain_run(world):
    torch = pytest.importorskip("torch")
    _paths()
    import oracle

    oracle.build()
    _, grid, walls, dt, rows, cell, smax = _setup()
    ref = _oracle(oracle, NX, rows, cell, smax)
    for step in range(1, STEPS + 1):
        ref.ntc_cells(0, 0, dt, grid.V, SEED, step, equal_weight=True)
        ref.convect(0, L, NX, walls.as_flat_array(), dt, SEED, step)
        ref.sort(0, L=L, nx=NX)
    ref_rows, ref_cells = ref.logical(0)

    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in range(world)), key=lambda t: t[0])
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    rows_all = np.concatenate([r[1] for r in res])
    cells_all = np.concatenate([r[2] for r in res])
    sent = sum(r[3] for r in res)
    # particles crossed the slab boundaries in both directions
    assert sent[0] > 0 and sent[1] > 0
    assert np.array_equal(cells_all, ref_cells - 1)
    assert np.array_equal(rows_all, ref_rows)


def test_slab_bounds_follow_the_batch_split():
    _paths()
    from merzgpu.slab import slab_bounds

    assert [slab_bounds(10, 3, i) for i in range(3)] == [(0, 4), (4, 3), (7, 3)]
    assert [slab_bounds(50_000, 8, i)[1] for i in range(8)] == [6250] * 8
    with pytest.raises(ValueError):
        slab_bounds(2, 3, 0)
