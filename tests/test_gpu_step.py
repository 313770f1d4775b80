"""The fused, graph-replayed step (mz_step) against the oracle running the
reference's time loops step by step."""
import ctypes as C

import numpy as np
import pytest

import merzgpu as mz
from helpers import assert_close_rows, device_logical, interactions, oracle_logical, species

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def couette_plan(grid, walls, dt, step0=0, avg_start=0, n_avg=1, graph=True, props=True):
    plan = mz._lib.StepPlan()
    plan.dims = 1
    plan.collide = 1
    plan.equal_weight = 1
    plan.props = 1 if props else 0
    plan.avg_start = avg_start
    plan.n_avg = n_avg
    plan.dt = dt
    plan.dw_tol = 1e-16
    plan.step0 = step0
    plan.use_graph = 1 if graph else 0
    plan.grid = grid.c_struct()
    plan.walls = walls.c_struct()
    return plan


def couette_setup(ctx, orc, nx=80, ppc=120, seed=17):
    sp = species(["Ar"])
    inter = interactions(sp)
    L, ndens, T = 5e-4, 1e23, 273.0
    grid = mz.Grid1DUniform(L, nx)
    Fnum = grid.dx * ndens / ppc
    walls = mz.MaxwellWalls1D(sp, T, T, -500.0, 500.0, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, ndens, T)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T, T, Fnum)
    o = orc.Oracle(nx, 1, [sp[0].mass])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    o.pv_create(0, 2 * ppc * nx)
    o.sample_grid_ndens(0, L, nx, ndens, T, Fnum, seed=seed, step=0)
    o.cf_set_smax(0, 0, smax)
    dom = mz.Domain(ctx, nx, sp, 2 * ppc * nx, interactions=inter, seed=seed)
    dom.set_cell_volumes(grid.V)
    dom.sample_grid_ndens(0, grid, ndens, T, Fnum, step=0)
    dom.set_sigma_g_w_max(0, 0, smax)
    return sp, grid, walls, dt, o, dom, seed


def oracle_couette(orc, o, grid, walls, dt, seed, steps, avg_start):
    avg = np.zeros((6, grid.n_cells))
    n_avg = steps - avg_start + 1
    for t in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, grid.V, seed, t, equal_weight=True)
        o.convect(0, grid.L, grid.n_cells, walls.as_flat_array(), dt, seed, t)
        o.sort(0, L=grid.L, nx=grid.n_cells)
        if t >= avg_start:
            r = o.compute_props(mode=2)
            inst = np.vstack([r["np"][0], r["n"][0], r["v"][0].T, r["T"][0]])
            for k in range(6):
                a = np.ascontiguousarray(avg[k])
                b = np.ascontiguousarray(inst[k])
                orc.lib().orc_avg_props(grid.n_cells, a.ctypes.data_as(C.POINTER(C.c_double)),
                                        b.ctypes.data_as(C.POINTER(C.c_double)), float(n_avg))
                avg[k] = a
    return avg


@pytest.mark.parametrize("graph,steps", [(True, 6), (False, 3), (True, 1), (True, 2)])
def test_fused_couette_matches_reference_loop(ctx, orc, graph, steps):
    sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc)
    avg_start = max(1, steps - 2)
    ref_avg = oracle_couette(orc, o, grid, walls, dt, seed, steps, avg_start)
    inst = mz.PhysProps(dom)
    avg = mz.PhysProps(dom)
    dom.step(couette_plan(grid, walls, dt, avg_start=avg_start, n_avg=steps - avg_start + 1, graph=graph), steps,
             inst, avg)
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-11, "particles after fused steps")
    r = inst.fetch()
    ref = o.compute_props(mode=2)
    assert np.array_equal(r["np"][:, 0], ref["np"][0])
    assert_close_rows(r["T"][:, 0:1], ref["T"][0].reshape(-1, 1), 1e-11, "T")
    a = avg.fetch()
    assert_close_rows(a["T"][:, 0:1], ref_avg[5].reshape(-1, 1), 1e-11, "averaged T")
    assert_close_rows(a["v"][:, :, 0].T, ref_avg[2:5].T, 1e-11, "averaged v")
    assert_close_rows(a["np"][:, 0:1], ref_avg[0].reshape(-1, 1), 1e-14, "averaged np")
    cf = dom.collision_factors(0, 0)
    smax, cnt = o.cf_get(0, 0)
    assert np.array_equal(cf["n_coll_performed"], cnt[:, 3])
    # the device counters add up the per-cell collisions of every step
    assert dom.counters()["accepted"] >= int(cf["n_coll_performed"].sum()) > 0


def test_fused_0d_two_species_matches_reference_loop(ctx, orc):
    """README.md:91-106 / test_2species.jl:52-66: ntc! for (Ar,Ar), (He,Ar),
    (He,He) then compute_props! every step, on 8 independent 0-D cells."""
    sp = species(["Ar", "He"])
    inter = interactions(sp)
    n_cells, steps = 8, 5
    rng = np.random.default_rng(5)
    counts = [rng.integers(50, 400, n_cells), rng.integers(200, 900, n_cells)]
    Fnum = 5e12
    o = orc.Oracle(n_cells, 2, [s.mass for s in sp])
    t = mz.VHS
    o.load_interactions([[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]],
                        [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]], 273.0)
    dom = mz.Domain(ctx, n_cells, sp, 8000, interactions=inter, seed=8)
    for s, T0 in enumerate((3000.0, 360.0)):
        o.pv_create(s, 8000)
        for c in range(n_cells):
            o.sample_equal_weight(s, c + 1, int(counts[s][c]), T0, Fnum, seed=8, step=0)
        dom.sample_cells(s, counts[s], T0, Fnum, step=0)
    o.estimate_sigma_g_w_max([3000.0, 360.0], Fnum)
    for s1 in range(2):
        for s2 in range(2):
            smax, _ = o.cf_get(s1, s2)
            dom.set_sigma_g_w_max(s1, s2, smax)
    dt = 2.5e-3
    for tt in range(1, steps + 1):
        for s2 in range(2):
            for s1 in range(s2, 2):
                o.ntc_cells(s1, s2, dt, None, 8, tt, equal_weight=False)
    plan = mz._lib.StepPlan()
    plan.dims = 0
    plan.collide = 1
    plan.equal_weight = 1
    plan.props = 1
    plan.dt = dt
    plan.use_graph = 1
    inst = mz.PhysProps(dom)
    dom.step(plan, steps, inst)
    for s in range(2):
        orows, oc = oracle_logical(o, s)
        drows, dc = device_logical(dom, s)
        assert np.array_equal(oc, dc)
        assert_close_rows(orows, drows, 1e-11, f"species {s}")
    r = inst.fetch()
    ref = o.compute_props(mode=0)
    assert_close_rows(r["T"].T.reshape(-1, 1), ref["T"].reshape(-1, 1), 1e-11, "T")
    for s1, s2 in [(0, 0), (1, 0), (1, 1)]:
        cf = dom.collision_factors(s1, s2)
        _, cnt = o.cf_get(s1, s2)
        assert np.array_equal(cf["n_coll_performed"], cnt[:, 3])


def test_fused_equals_standalone_ops_bitwise(ctx, orc):
    """The fused kernel and the standalone kernels run the same per-cell
    routines: identical particle state after the same steps."""
    sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc, nx=50, ppc=100, seed=23)
    _, _, _, _, o2, dom2, _ = couette_setup(ctx, orc, nx=50, ppc=100, seed=23)
    steps = 4
    dom.step(couette_plan(grid, walls, dt, props=False), steps)
    for t in range(1, steps + 1):
        dom2.ntc(0, 0, dt, t, equal_weight=True)
        dom2.convect(0, grid, walls, dt, t)
        dom2.sort(0, grid)
    a, ca = device_logical(dom, 0)
    b, cb = device_logical(dom2, 0)
    assert np.array_equal(ca, cb)
    assert np.array_equal(a, b)


def test_fused_0d_block_per_cell_equals_warp_groups_and_oracle(ctx, orc):
    """Large 0-D cells collide one block per cell (ntc_cell_block) and small
    ones in 8-lane groups; the mapping changes no result: block-per-cell for
    cells of >= 2,048 particles, >= 64 particles, and never give identical
    states, equal to the oracle's ntc_equal_weight! loop."""
    sp = species(["Ar"])
    inter = interactions(sp)
    counts = np.array([100, 800, 2500, 5000, 3000, 50, 2048, 2047, 7000, 300])
    n_cells, steps, dt, Fnum, T0 = len(counts), 6, 0.05, 1e13, 300.0
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T0, T0, Fnum)
    states = []
    for big in (0, 64, -1):
        dom = mz.Domain(ctx, n_cells, sp, int(counts.sum()) + 64, interactions=inter, seed=41)
        dom.sample_cells(0, counts, T0, Fnum, step=0)
        dom.set_sigma_g_w_max(0, 0, smax)
        plan = mz._lib.StepPlan()
        plan.dims, plan.collide, plan.equal_weight, plan.props, plan.dt = 0, 1, 1, 1, dt
        plan.use_graph, plan.big_cell = 1, big
        inst = mz.PhysProps(dom)
        dom.step(plan, steps, inst)
        cnt = dom.counters()
        states.append((device_logical(dom, 0), inst.fetch(), cnt))
        dom.close()
    (a, ca), pa, na = states[0]
    assert na["accepted"] > 1000
    for (b, cb), pb, nb in states[1:]:
        assert np.array_equal(ca, cb) and np.array_equal(a, b)
        assert na["accepted"] == nb["accepted"]
        # the block-per-cell props sum in another order: equal to round-off
        assert np.array_equal(pa["np"], pb["np"])
        assert np.allclose(pa["T"], pb["T"], rtol=1e-13, atol=0) and np.allclose(pa["n"], pb["n"], rtol=1e-14)
    o = orc.Oracle(n_cells, 1, [sp[0].mass])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    o.pv_create(0, int(counts.sum()) + 64)
    for c in range(n_cells):
        o.sample_equal_weight(0, c + 1, int(counts[c]), T0, Fnum, seed=41, step=0)
    o.cf_set_smax(0, 0, smax)
    for tt in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, None, 41, tt, equal_weight=True, nthreads=8)
    orows, oc = oracle_logical(o, 0)
    assert np.array_equal(oc, ca)
    assert_close_rows(orows, a, 1e-11, "0-D cells after 6 steps")


def test_autotuned_mapping_changes_no_result(ctx, orc):
    """mz_step_autotune runs real steps under every mapping; the state after
    tuning plus further steps equals the same number of steps run with the
    default mapping, bit for bit (0-D and 1-D)."""
    sp = species(["Ar"])
    inter = interactions(sp)
    counts = np.array([60, 900, 2600, 40, 5000, 1200, 300, 8200])
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 300.0, 300.0, 1e13)
    runs = []
    for tune in (True, False):
        dom = mz.Domain(ctx, len(counts), sp, int(counts.sum()) + 64, interactions=inter, seed=77)
        dom.sample_cells(0, counts, 300.0, 1e13, step=0)
        dom.set_sigma_g_w_max(0, 0, smax)
        plan = mz._lib.StepPlan()
        plan.dims, plan.collide, plan.equal_weight, plan.props, plan.dt, plan.use_graph = 0, 1, 1, 1, 0.05, 1
        done = 0
        if tune:
            lanes, big = dom.autotune(plan, trial_steps=1)
            assert lanes in (8, 16, 32) and big in (512, 2048, 8192, -1)
            done = 24
        plan.step0 = done
        dom.step(plan, 27 - done)
        runs.append(device_logical(dom, 0))
        dom.close()
    assert np.array_equal(runs[0][1], runs[1][1]) and np.array_equal(runs[0][0], runs[1][0])

    states = []
    for tune in (True, False):
        _, grid, walls, dt, _, dom, _ = couette_setup(ctx, orc, nx=40, ppc=100, seed=9)
        plan = couette_plan(grid, walls, dt, props=False)
        done = 0
        if tune:
            dom.autotune(plan, trial_steps=1)
            done = 18
        dom.step(couette_plan(grid, walls, dt, step0=done, props=False), 22 - done)
        states.append(device_logical(dom, 0))
        dom.close()
    assert np.array_equal(states[0][1], states[1][1]) and np.array_equal(states[0][0], states[1][0])


def test_two_launch_step_equals_fused(ctx, orc):
    """The 1-D step as one fused launch, as two (sort + gather + props, then
    NTC + convection in place) and as one launch with gathering and physics
    warps side by side gives the same particles and the same averaged and
    instantaneous properties, and all equal the oracle loop's averages."""
    results = []
    for launches in (1, 2, 3):
        sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc, nx=60, ppc=100, seed=23)
        inst, avg = mz.PhysProps(dom), mz.PhysProps(dom)
        plan = couette_plan(grid, walls, dt, avg_start=3, n_avg=5)
        plan.launches = launches
        dom.step(plan, 7, inst, avg)
        results.append((device_logical(dom, 0), inst.fetch(), avg.fetch()))
        if launches == 2:
            ref_avg = oracle_couette(orc, o, grid, walls, dt, seed, 7, 3)
        dom.close()
    (r1, i1, a1) = results[0]
    for r2, i2, a2 in results[1:]:
        assert np.array_equal(r1[1], r2[1]) and np.array_equal(r1[0], r2[0])
        for k in ("np", "n", "v", "T"):
            assert np.array_equal(i1[k], i2[k]) and np.array_equal(a1[k], a2[k]), k
    assert_close_rows(a2["T"][:, 0:1], ref_avg[5].reshape(-1, 1), 1e-11, "averaged T, two launches")


def test_launch_forms_with_cells_above_1024_particles(ctx, orc):
    """Cells of ~1,500 particles take the gathers' sorts for large segments
    (in place in global memory in these kernels): the three launch forms give
    the same particles and properties, equal to the oracle loop's."""
    results = []
    for launches in (1, 2, 3):
        sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc, nx=10, ppc=1500, seed=31)
        n_before = device_logical(dom, 0)[1]
        assert np.bincount(n_before, minlength=10).min() > 1024
        inst, avg = mz.PhysProps(dom), mz.PhysProps(dom)
        plan = couette_plan(grid, walls, dt, avg_start=2, n_avg=3)
        plan.launches = launches
        dom.step(plan, 4, inst, avg)
        results.append((device_logical(dom, 0), inst.fetch(), avg.fetch()))
        if launches == 1:
            ref_avg = oracle_couette(orc, o, grid, walls, dt, seed, 4, 2)
        dom.close()
    (r1, i1, a1) = results[0]
    for r2, i2, a2 in results[1:]:
        assert np.array_equal(r1[1], r2[1]) and np.array_equal(r1[0], r2[0])
        for k in ("np", "n", "v", "T"):
            assert np.array_equal(i1[k], i2[k]) and np.array_equal(a1[k], a2[k]), k
    assert_close_rows(a1["T"][:, 0:1], ref_avg[5].reshape(-1, 1), 1e-11, "averaged T")


def test_two_species_couette_step_matches_reference_loop(ctx, orc):
    """An Ar + He mixture between the Couette walls: the fused and the
    two-launch 1-D step give the same particles, and both follow the
    reference loop (ntc_equal_weight! for (Ar,Ar), (He,Ar), (He,He), then
    convection and sorting of both species) run by the oracle on the same
    streams."""
    sp = species(["Ar", "He"])
    inter = interactions(sp)
    nx, L, T, seed, steps = 30, 5e-4, 273.0, 61, 4
    grid = mz.Grid1DUniform(L, nx)
    walls = mz.MaxwellWalls1D(sp, T, T, -500.0, 500.0, 1.0, 1.0)
    ndens = (6e22, 4e22)
    Fnum = [grid.dx * n / 60 for n in ndens]
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, 1e23, T)
    t = mz.VHS
    o = orc.Oracle(nx, 2, [s.mass for s in sp])
    o.load_interactions([[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]],
                        [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]], 273.0)
    smax = {}
    for s in range(2):
        o.pv_create(s, 4 * 60 * nx)
        o.sample_grid_ndens(s, L, nx, ndens[s], T, Fnum[s], seed=seed, step=0)
    for s1 in range(2):
        for s2 in range(2):
            smax[s1, s2] = mz.estimate_sigma_g_w_max(inter[s1][s2], sp[s1], sp[s2], T, T, max(Fnum[s1], Fnum[s2]))
            o.cf_set_smax(s1, s2, smax[s1, s2])
    for step in range(1, steps + 1):
        for s2 in range(2):
            for s1 in range(s2, 2):
                o.ntc_cells(s1, s2, dt, grid.V, seed, step, equal_weight=True)
        for s in range(2):
            o.convect(s, L, nx, walls.as_flat_array(), dt, seed, step)
            o.sort(s, L=L, nx=nx)
    states = []
    for launches in (1, 2, 3):
        dom = mz.Domain(ctx, nx, sp, 4 * 60 * nx, interactions=inter, seed=seed)
        dom.set_cell_volumes(grid.V)
        for s in range(2):
            dom.sample_grid_ndens(s, grid, ndens[s], T, Fnum[s], step=0)
        for (s1, s2), v in smax.items():
            dom.set_sigma_g_w_max(s1, s2, v)
        plan = couette_plan(grid, walls, dt, props=False)
        plan.launches = launches
        dom.step(plan, steps)
        states.append([device_logical(dom, s) for s in range(2)])
        dom.close()
    for s in range(2):
        (r1, c1) = states[0][s]
        for other in states[1:]:
            (r2, c2) = other[s]
            assert np.array_equal(c1, c2) and np.array_equal(r1, r2), f"species {s}: the launch forms differ"
        orows, oc = oracle_logical(o, s)
        assert np.array_equal(oc, c1), f"species {s}: cells"
        assert_close_rows(orows, r1, 1e-11, f"species {s} after {steps} steps")


def test_async_snapshots_equal_fetched_properties(ctx, orc):
    """mz_props_snapshot: each step's read-back, taken without stopping the
    device (two slots, each read two steps later), equals the properties a
    synchronous fetch returns after the same step of an identical run."""
    runs = []
    for use_snapshot in (True, False):
        sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc, nx=50, ppc=80, seed=29)
        inst = mz.PhysProps(dom)
        m = grid.n_cells
        snaps = [mz.PinnedArray(ctx, 6 * m), mz.PinnedArray(ctx, 6 * m)]
        got = []
        for k in range(5):
            dom.step(couette_plan(grid, walls, dt, step0=k), 1, inst)
            if use_snapshot:
                if k >= 2:
                    inst.snapshot_wait(k % 2)
                    got.append(inst.unpack(snaps[k % 2].array.copy()))
                inst.snapshot(k % 2, snaps[k % 2])
            else:
                got.append(inst.fetch())
        if use_snapshot:
            for k in (3, 4):
                inst.snapshot_wait(k % 2)
                got.append(inst.unpack(snaps[k % 2].array.copy()))
        runs.append(got)
        for a in snaps:
            a.close()
        dom.close()
    assert len(runs[0]) == len(runs[1]) == 5
    for a, b in zip(*runs):
        for key in ("np", "n", "v", "T"):
            assert np.array_equal(a[key], b[key]), key
