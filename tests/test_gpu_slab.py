"""The slab exchange on the device (mz_slab_extract / mz_slab_fetch /
mz_slab_insert through merzgpu.slab): a Couette grid split into slabs, each
in its own Domain keyed on its global cells, stepped with ntc_equal_weight!
and convection on the global grid and walls, the slabs exchanging their
leaving particles after every convection, equals one Domain over the whole
grid bit for bit, and that Domain's cells equal the oracle's.  The slabs run
in one process on one GPU (merzgpu.slab.exchange_local); the exchange between
processes is the same calls with torch.distributed point-to-point transfers
in between (tests/test_slab_gloo.py).  Reference: exchange_particles! /
sort_particles_after_exchange!, parallel.jl:281-532."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import device_logical, oracle_state, species
from merzgpu.slab import Slab, exchange_local, slab_bounds

pytestmark = pytest.mark.gpu

NX, PPC, L, NDENS, T0, V_WALL, SEED = 96, 60, 5e-4, 1e23, 273.0, 500.0, 21


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _config():
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    grid = mz.Grid1DUniform(L, NX)
    Fnum = grid.dx * NDENS / PPC
    walls = mz.MaxwellWalls1D(sp, T0, T0, -V_WALL, V_WALL, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T0)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T0, T0, Fnum)
    rng = np.random.default_rng(SEED)
    n = PPC * NX
    cell = np.sort(rng.integers(0, NX, size=n)).astype(np.int32)
    x = np.column_stack([(cell + rng.uniform(0.02, 0.98, size=n)) * grid.dx, rng.random(n), rng.random(n)])
    v = rng.normal(0.0, np.sqrt(mz.K_B * T0 / mz.AR_MASS), size=(n, 3))
    w = np.full(n, Fnum)
    return sp, inter, grid, walls, dt, smax, (w, v, x, cell)


def _domain(ctx, sp, inter, n_cells, arrays, smax, grid):
    dom = mz.Domain(ctx, n_cells, sp, 4 * len(arrays[0]) + 1024, interactions=inter, seed=SEED)
    dom.upload(0, *arrays)
    dom.set_cell_volumes(np.full(n_cells, grid.dx))
    dom.set_sigma_g_w_max(0, 0, smax)
    return dom


@pytest.mark.parametrize("n_slabs", [2, 3])
def test_slabs_on_one_gpu_equal_the_single_domain(ctx, orc, n_slabs):
    sp, inter, grid, walls, dt, smax, (w, v, x, cell) = _config()
    steps = 10
    single = _domain(ctx, sp, inter, NX, (w, v, x, cell), smax, grid)
    for step in range(1, steps + 1):
        single.ntc(0, 0, dt, step, equal_weight=True)
        single.convect(0, grid, walls, dt, step)
        single.sort(0, grid)
    ref_rows, ref_cells = device_logical(single, 0)
    single.close()

    slabs = []
    for i in range(n_slabs):
        c0, n = slab_bounds(NX, n_slabs, i)
        m = (cell >= c0) & (cell < c0 + n)
        dom = _domain(ctx, sp, inter, n, (w[m], v[m], x[m], cell[m] - c0), smax, grid)
        slabs.append(Slab(dom, grid, c0, i, n_slabs))
    moved = 0
    for step in range(1, steps + 1):
        for sl in slabs:
            sl.engine.ntc(0, 0, dt, step, equal_weight=True)
            sl.engine.convect(0, grid, walls, dt, step)
        exchange_local(slabs)
        moved += sum(sum(sl.engine._slab_pending) for sl in slabs)
    rows, cells = [], []
    for sl in slabs:
        r, c = device_logical(sl.engine, 0)
        rows.append(r)
        cells.append(c + sl.c0)
        assert sl.engine.check_pia_is_correct(0) == (True, 0)
        sl.engine.close()
    assert moved > 0
    assert np.array_equal(np.concatenate(cells), ref_cells)
    assert np.array_equal(np.concatenate(rows), ref_rows)

    # the single domain follows the oracle's loop (cells exact)
    o = oracle_state(orc, NX, sp, mz.VHS, [(w, v, x, cell)])
    o.cf_set_smax(0, 0, smax)
    for step in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, grid.V, SEED, step, equal_weight=True)
        o.convect(0, L, NX, walls.as_flat_array(), dt, SEED, step)
        o.sort(0, L=L, nx=NX)
    _, oc = o.logical(0)
    assert np.array_equal(oc - 1, ref_cells)


def test_slab_arguments_are_checked(ctx):
    sp, inter, grid, walls, dt, smax, (w, v, x, cell) = _config()
    m = cell < 10
    dom = _domain(ctx, sp, inter, 10, (w[m], v[m], x[m], cell[m]), smax, grid)
    with pytest.raises(mz.MerzError):
        dom.slab_extract(0, grid, NX - 5)  # the slab would end beyond the grid
    with pytest.raises(mz.MerzError):
        dom._ck(mz.lib().mz_slab_fetch(dom.h, 0, None, None))  # no extraction pending
    # nothing left the slab: empty exchange, same particles
    before = device_logical(dom, 0)
    assert dom.slab_extract(0, grid, 0) == (0, 0)
    dom.slab_fetch(0)
    dom.slab_insert(0, grid, 0, np.empty((0, 7)), np.empty((0, 7)))
    after = device_logical(dom, 0)
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    dom.close()
