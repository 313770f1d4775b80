"""The variable-weight Couette loop (test/test_1D_couette_varweight.jl:60-90):
every step ntc! with weight splitting, octree N:2 merging of the cells above a
threshold, convection and sorting.  On the device against the oracle's loop
on the same streams, and per-cell conservation of mass, momentum and energy
through the splitting collisions and the merging."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import assert_close_rows, device_logical, interactions, oracle_logical, oracle_state, species

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _varweight_state(nx, ppc, seed, span=2.0):
    """Couette gas at 273 K, n = 1e23, weights log-uniform over `span` decades
    around Fnum, positions uniform in each cell."""
    sp = species(["Ar"])
    inter = interactions(sp)
    L, ndens, T = 5e-4, 1e23, 273.0
    grid = mz.Grid1DUniform(L, nx)
    Fnum = grid.dx * ndens / ppc
    rng = np.random.default_rng(seed)
    n = nx * ppc
    cell = np.repeat(np.arange(nx, dtype=np.int32), ppc)
    x = rng.random((n, 3))
    x[:, 0] = (cell + rng.uniform(0.01, 0.99, n)) * grid.dx
    v = rng.normal(0.0, np.sqrt(mz.K_B * T / sp[0].mass), (n, 3))
    w = Fnum * 10.0 ** (span * (rng.random(n) - 0.5))
    w *= n * Fnum / w.sum()  # the same total number of physical particles
    walls = mz.MaxwellWalls1D(sp, T, T, -500.0, 500.0, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, ndens, T)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T, T, Fnum)
    return sp, inter, grid, walls, dt, smax, (w, v, x, cell)


def test_varweight_couette_loop_vs_oracle(ctx, orc):
    nx, ppc, steps, threshold, target, seed = 16, 150, 4, 160, 80, 91
    sp, inter, grid, walls, dt, smax, arrays = _varweight_state(nx, ppc, seed)
    cap = 8 * nx * ppc
    o = oracle_state(orc, nx, sp, mz.VHS, [arrays], capacity=cap)
    o.cf_set_smax(0, 0, smax)
    dom = mz.Domain(ctx, nx, sp, cap, interactions=inter, seed=seed)
    dom.upload(0, *arrays)
    dom.set_cell_volumes(grid.V)
    dom.set_sigma_g_w_max(0, 0, smax)
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    oc = orc.Octree(orc.SPLIT_MID, mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit, 6000, 10)
    merged_total = 0
    for step in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, grid.V, seed, step, equal_weight=False)
        ind, _, _ = o.pia_get()
        expect = 0
        for c in range(nx):
            if ind[0, c, 0] > threshold:
                o.merge_octree(oc, 0, c + 1, target, L=grid.L, nx=nx, seed=seed, step=step)
                expect += 1
        o.squash(0)
        o.convect(0, grid.L, nx, walls.as_flat_array(), dt, seed, step)
        o.sort(0, L=grid.L, nx=nx)

        dom.ntc(0, 0, dt, step, equal_weight=False)
        merged = dom.merge_octree(0, octree, target, threshold=threshold, grid=grid, step=step)
        assert merged == expect, step
        merged_total += merged
        dom.convect(0, grid, walls, dt, step)
        dom.sort(0, grid)

        smax_o, cnt = o.cf_get(0, 0)
        cf = dom.collision_factors(0, 0)
        assert np.array_equal(cf["n_coll"], cnt[:, 2]) and np.array_equal(cf["n_coll_performed"], cnt[:, 3]), step
        orows, oc_cells = oracle_logical(o, 0)
        drows, dc_cells = device_logical(dom, 0)
        assert np.array_equal(oc_cells, dc_cells), step
        assert_close_rows(orows, drows, 1e-11, f"particles after step {step}")
    assert merged_total >= nx  # cells were merged


def _cell_moments(rows, cells, nx):
    w = rows[:, 0]
    v = rows[:, 1:4]
    m = np.zeros((nx, 5))
    for k, q in enumerate((w, w * v[:, 0], w * v[:, 1], w * v[:, 2], w * (v ** 2).sum(axis=1))):
        m[:, k] = np.bincount(cells, weights=q, minlength=nx)
    return m


def test_splitting_and_merging_conserve_per_cell(ctx):
    """Mass, momentum and energy of every cell before and after ntc! with
    splitting followed by merging, to FP64 round-off (relative to each cell's
    magnitudes)."""
    nx, ppc, threshold, target, seed = 64, 400, 450, 120, 5
    sp, inter, grid, walls, dt, smax, arrays = _varweight_state(nx, ppc, seed)
    dom = mz.Domain(ctx, nx, sp, 8 * nx * ppc, interactions=inter, seed=seed)
    dom.upload(0, *arrays)
    dom.set_cell_volumes(grid.V)
    dom.set_sigma_g_w_max(0, 0, smax)
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    merged = 0
    for step in range(1, 6):
        before = _cell_moments(*device_logical(dom, 0), nx)
        dom.ntc(0, 0, 3 * dt, step, equal_weight=False)
        merged += dom.merge_octree(0, octree, target, threshold=threshold, grid=grid, step=step)
        after = _cell_moments(*device_logical(dom, 0), nx)
        scale = np.abs(before).max(axis=0)
        scale[1:4] = np.abs(before[:, 1:4]).max()
        assert np.all(np.abs(after - before) <= 1e-13 * scale), step
        dom.convect(0, grid, walls, dt, step)
        dom.sort(0, grid)
    assert merged > 0 and dom.counters()["splits"] > 0
