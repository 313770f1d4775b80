"""Edge cases of the fused step: a domain without particles, ragged occupancy
(empty cells, cells of one and of two particles beside full ones) through
the 1-D step in every launch form against the oracle's loop of the
reference's time step, the batched 0-D step with empty and one-particle
instances, and the variable-weight step on ragged cells against the
standalone calls.  Cells below two particles draw no candidates
(compute_n_coll_single_species, collision_ntc.jl:173-181); empty cells give
zero properties."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import assert_close_rows, device_logical, interactions, oracle_logical, oracle_state, species

pytestmark = pytest.mark.gpu

L, NDENS, T0 = 5e-4, 1e23, 273.0


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _plan_1d(grid, walls, dt, launches=0, graph=True, props=True, avg_start=0, n_avg=1):
    p = mz._lib.StepPlan()
    p.dims, p.collide, p.equal_weight, p.props = 1, 1, 1, 1 if props else 0
    p.avg_start, p.n_avg, p.dt, p.dw_tol, p.step0 = avg_start, n_avg, dt, 1e-16, 0
    p.use_graph, p.launches = 1 if graph else 0, launches
    p.grid, p.walls = grid.c_struct(), walls.c_struct()
    return p


def _ragged(rng, nx, grid, Fnum):
    """Counts per cell: every fourth cell empty, some cells of one and of two
    particles, the others full; particles inside their cells."""
    counts = rng.integers(150, 300, nx)
    counts[::4] = 0
    counts[1::7] = 1
    counts[2::9] = 2
    cell = np.repeat(np.arange(nx, dtype=np.int32), counts)
    n = cell.size
    x = np.column_stack([(cell + rng.uniform(0.02, 0.98, n)) * grid.dx, rng.random(n), rng.random(n)])
    v = rng.normal(0.0, np.sqrt(mz.K_B * T0 / mz.AR_MASS), (n, 3))
    return counts, (np.full(n, Fnum), v, x, cell)


def _oracle_loop(orc, o, grid, walls, dt, seed, steps):
    for t in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, grid.V, seed, t, equal_weight=True)
        o.convect(0, grid.L, grid.n_cells, walls.as_flat_array(), dt, seed, t)
        o.sort(0, L=grid.L, nx=grid.n_cells)


@pytest.mark.parametrize("launches,graph", [(1, True), (2, True), (3, True), (2, False)])
def test_domain_without_particles_steps_cleanly(ctx, launches, graph):
    sp = species(["Ar"])
    inter = interactions(sp)
    nx = 64
    grid = mz.Grid1DUniform(L, nx)
    walls = mz.MaxwellWalls1D(sp, T0, T0, -500.0, 500.0, 1.0, 1.0)
    dom = mz.Domain(ctx, nx, sp, 1000, interactions=inter, seed=3)
    dom.set_cell_volumes(grid.V)
    dom.set_sigma_g_w_max(0, 0, 1e-10)
    inst, avg = mz.PhysProps(dom), mz.PhysProps(dom)
    dom.step(_plan_1d(grid, walls, 1e-9, launches, graph, avg_start=1, n_avg=3), 4, inst, avg)
    r, a = inst.fetch(), avg.fetch()
    for k in ("np", "n", "T"):
        assert not np.any(r[k]) and not np.any(a[k]), k
    assert dom.info(0)["n_total"] == 0
    assert dom.counters()["candidates"] == 0
    dom.close()


@pytest.mark.parametrize("launches", [1, 2, 3])
def test_ragged_cells_through_the_1d_step_match_the_oracle(ctx, orc, launches):
    sp = species(["Ar"])
    inter = interactions(sp)
    nx, steps, seed = 72, 5, 13
    grid = mz.Grid1DUniform(L, nx)
    Fnum = grid.dx * NDENS / 200
    walls = mz.MaxwellWalls1D(sp, T0, T0, -500.0, 500.0, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T0)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T0, T0, Fnum)
    rng = np.random.default_rng(seed)
    counts, arrays = _ragged(rng, nx, grid, Fnum)
    dom = mz.Domain(ctx, nx, sp, 3 * arrays[0].size, interactions=inter, seed=seed)
    dom.upload(0, *arrays)
    dom.set_cell_volumes(grid.V)
    dom.set_sigma_g_w_max(0, 0, smax)
    o = oracle_state(orc, nx, sp, mz.VHS, [arrays], capacity=3 * arrays[0].size)
    o.cf_set_smax(0, 0, smax)
    inst = mz.PhysProps(dom)
    dom.step(_plan_1d(grid, walls, dt, launches), steps, inst)
    _oracle_loop(orc, o, grid, walls, dt, seed, steps)
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-11, "particles")
    ref = o.compute_props(mode=2)
    r = inst.fetch()
    assert np.array_equal(r["np"][:, 0], ref["np"][0])
    assert_close_rows(r["T"][:, 0:1], ref["T"][0].reshape(-1, 1), 1e-11, "T")
    cf = dom.collision_factors(0, 0)
    _, cnt = o.cf_get(0, 0)
    assert np.array_equal(cf["n_coll"], cnt[:, 2]) and np.array_equal(cf["n_coll_performed"], cnt[:, 3])
    dom.close()


@pytest.mark.parametrize("big_cell", [0, -1])
def test_batched_0d_with_empty_and_single_particle_instances(ctx, orc, big_cell):
    sp = species(["Ar"])
    inter = interactions(sp)
    counts = np.array([0, 1, 2, 3, 0, 500, 1, 2500, 0, 40])
    n_cells, steps, dt, Fnum, T = len(counts), 5, 0.05, 1e13, 500.0
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T, T, Fnum)
    dom = mz.Domain(ctx, n_cells, sp, int(counts.sum()) + 64, interactions=inter, seed=52)
    dom.sample_cells(0, counts, T, Fnum, step=0)
    dom.set_sigma_g_w_max(0, 0, smax)
    o = orc.Oracle(n_cells, 1, [sp[0].mass])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    o.pv_create(0, int(counts.sum()) + 64)
    for c in range(n_cells):
        o.sample_equal_weight(0, c + 1, int(counts[c]), T, Fnum, seed=52, step=0)
    o.cf_set_smax(0, 0, smax)
    plan = mz._lib.StepPlan()
    plan.dims, plan.collide, plan.equal_weight, plan.props, plan.dt = 0, 1, 1, 1, dt
    plan.use_graph, plan.big_cell = 1, big_cell
    inst = mz.PhysProps(dom)
    dom.step(plan, steps, inst)
    for t in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, None, 52, t, equal_weight=True)
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-11, "particles")
    r = inst.fetch()
    ref = o.compute_props(mode=0)
    assert np.array_equal(r["np"][:, 0], counts)
    empty = counts == 0
    assert not np.any(r["n"][empty, 0]) and not np.any(r["T"][empty, 0])
    assert_close_rows(r["T"][~empty, 0:1], ref["T"][0][~empty].reshape(-1, 1), 1e-11, "T")
    dom.close()


def test_varweight_step_on_ragged_cells_equals_the_standalone_calls(ctx):
    sp = species(["Ar"])
    inter = interactions(sp)
    nx, steps, seed = 48, 4, 29
    grid = mz.Grid1DUniform(L, nx)
    Fnum = grid.dx * NDENS / 200
    walls = mz.MaxwellWalls1D(sp, T0, T0, -500.0, 500.0, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T0)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T0, T0, Fnum)
    rng = np.random.default_rng(seed)
    counts, (w, v, x, cell) = _ragged(rng, nx, grid, Fnum)
    w = Fnum * 10.0 ** (rng.random(w.size) - 0.5)
    octree = mz.OctreeN2Merge(max_Nbins=4096)
    threshold, target = 260, 80
    runs = []
    for fused in (True, False):
        dom = mz.Domain(ctx, nx, sp, 20 * w.size, interactions=inter, seed=seed)
        dom.upload(0, w, v, x, cell)
        dom.set_cell_volumes(grid.V)
        dom.set_sigma_g_w_max(0, 0, smax)
        if fused:
            p = _plan_1d(grid, walls, dt, graph=True)
            p.equal_weight = 0
            p.merge_threshold, p.merge_target, p.octree = threshold, target, octree.params
            dom.step(p, steps, mz.PhysProps(dom))
        else:
            for t in range(1, steps + 1):
                dom.ntc(0, 0, dt, t, equal_weight=False)
                dom.merge_octree(0, octree, target, threshold=threshold, grid=grid, step=t)
                dom.convect(0, grid, walls, dt, t)
                dom.sort(0, grid)
        runs.append((device_logical(dom, 0), dom.counters()))
        dom.close()
    (a, ca), na = runs[0]
    (b, cb), nb = runs[1]
    assert na["splits"] > 0 and na["merges"] > 0
    assert np.array_equal(ca, cb) and np.array_equal(a, b)
