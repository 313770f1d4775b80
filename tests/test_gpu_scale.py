"""Parity at the sizes the benchmark runs: the device against the oracle on
the same initial state (the device's sampled particles are handed to the
oracle bit for bit), at 50,000 cells x 400 particles (the scaled Couette
configuration of simulations/1D/couette_benchmarking.jl), at 65,536 batched
0-D cells, and on grids of several scan tiles where particles move hundreds
of cells per step (the windowed histograms' and the scatter's fallback paths,
and a wall-hit queue too small for the step's hitters).

Integer outcomes (cells, indexers, candidate and collision counts) must be
equal; particle state and cell properties within 1e-11 of each quantity's
scale (FMA contraction and CUDA's pow/log against glibc's differ by an ulp)."""
import os

import numpy as np
import pytest

import merzgpu as mz
from helpers import assert_close_rows, device_logical, oracle_logical, species

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))
L_COUETTE, NDENS, T_WALL, V_WALL = 5e-4, 1e23, 273.0, 500.0


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _oracle_from_device(orc, dom, sp):
    """An oracle holding the device's particles in the device's logical order."""
    o = orc.Oracle(dom.n_cells, len(sp), [s.mass for s in sp])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    for s in range(len(sp)):
        w, v, x, cell = dom.download(s)
        o.set_particles_simple(s, cell.astype(np.int64) + 1, np.column_stack([w, v, x]))
        o.pv_resize(s, int(dom.info(s)["capacity"]))
    return o


def _plan(grid, walls, dt, launches, steps, hitq=0):
    p = mz._lib.StepPlan()
    p.dims, p.collide, p.equal_weight, p.props = 1, 1, 1, 1
    p.avg_start, p.n_avg = 2, steps - 1
    p.dt, p.dw_tol, p.step0, p.use_graph = dt, 1e-16, 0, 1
    p.launches, p.hit_queue_capacity = launches, hitq
    p.grid, p.walls = grid.c_struct(), walls.c_struct()
    return p


def _oracle_loop(o, grid, walls, dt, seed, steps, avg_start):
    """The reference loop (ntc_equal_weight! -> convect_particles! ->
    sort_particles! -> compute_props_sorted! -> avg_props!) on the oracle."""
    nx = grid.n_cells
    n_avg = steps - avg_start + 1
    avg = {k: np.zeros(sh) for k, sh in (("np", nx), ("n", nx), ("v", (nx, 3)), ("T", nx))}
    last = None
    for t in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, grid.V, seed, t, equal_weight=True, nthreads=THREADS)
        o.convect(0, grid.L, nx, walls.as_flat_array(), dt, seed, t, nthreads=THREADS)
        o.sort(0, L=grid.L, nx=nx)
        last = o.compute_props(mode=2, nthreads=THREADS)
        if t >= avg_start:
            # avg_props! (physical_props.jl:281-299): avg + inst * (1 / n_avg)
            inv = 1.0 / n_avg
            for k in ("np", "n", "v", "T"):
                avg[k] += last[k][0] * inv
    return last, avg


def _compare_couette(o, dom, inst, avg, last, ref_avg, what):
    smax_o, cnt = o.cf_get(0, 0)
    cf = dom.collision_factors(0, 0)
    assert np.array_equal(cf["n_coll"], cnt[:, 2]), f"{what}: n_coll"
    assert np.array_equal(cf["n_coll_performed"], cnt[:, 3]), f"{what}: n_coll_performed"
    assert np.allclose(cf["sigma_g_w_max"], smax_o, rtol=1e-12, atol=0), f"{what}: (sigma g w)_max"
    oind, ont, _ = o.pia_get()
    dind, dnt = dom.indexer(0)
    assert dnt == ont[0], f"{what}: n_total"
    assert np.array_equal(dind[:, 3], oind[0, :, 3]), f"{what}: n_group1 per cell"
    nz = dind[:, 3] > 0
    assert np.array_equal(dind[nz, 1] + 1, oind[0, nz, 1]), f"{what}: start1 per cell"
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc), f"{what}: cells"
    assert_close_rows(orows, drows, 1e-11, f"{what}: particles")
    r = inst.fetch()
    assert np.array_equal(r["np"][:, 0], last["np"][0]), f"{what}: np"
    assert_close_rows(r["T"][:, 0:1], last["T"][0].reshape(-1, 1), 1e-11, f"{what}: T")
    assert_close_rows(r["v"][:, :, 0].T, last["v"][0], 1e-11, f"{what}: v")
    a = avg.fetch()
    assert_close_rows(a["np"][:, 0:1], ref_avg["np"].reshape(-1, 1), 1e-13, f"{what}: averaged np")
    assert_close_rows(a["n"][:, 0:1], ref_avg["n"].reshape(-1, 1), 1e-11, f"{what}: averaged n")
    assert_close_rows(a["T"][:, 0:1], ref_avg["T"].reshape(-1, 1), 1e-11, f"{what}: averaged T")
    assert_close_rows(a["v"][:, :, 0].T, ref_avg["v"], 1e-11, f"{what}: averaged v")


def _couette_device(ctx, nx, ppc, seed, dt=None, cap_factor=1.1):
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    grid = mz.Grid1DUniform(L_COUETTE, nx)
    Fnum = grid.dx * NDENS / ppc
    walls = mz.MaxwellWalls1D(sp, T_WALL, T_WALL, -V_WALL, V_WALL, 1.0, 1.0)
    if dt is None:
        dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T_WALL)
    dom = mz.Domain(ctx, nx, sp, int(nx * ppc * cap_factor) + 1024, interactions=inter, seed=seed)
    dom.set_cell_volumes(grid.V)
    dom.sample_grid_ndens(0, grid, NDENS, T_WALL, Fnum, step=0)
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T_WALL, T_WALL, Fnum))
    return sp, grid, walls, dt, dom


def _oracle_couette(orc, dom, sp):
    """The oracle of a Couette domain: the device's particles and (sigma g w)_max."""
    o = _oracle_from_device(orc, dom, sp)
    o.cf_set_smax(0, 0, dom.collision_factors(0, 0)["sigma_g_w_max"])
    return o


@pytest.fixture(scope="module")
def bench_reference(ctx, orc):
    """The oracle's reference loop on the benchmark's own workload: 50,000
    cells x 400 particles (2e7 Ar), n = 1e23, diffuse walls at 273 K and
    -/+500 m/s, dt = 0.2 / nu, 4 steps, averages over steps 2-4."""
    nx, ppc, seed, steps = 50_000, 400, 1234, 4
    sp, grid, walls, dt, dom = _couette_device(ctx, nx, ppc, seed)
    o = _oracle_couette(orc, dom, sp)
    init = dom.download(0)
    dom.close()
    last, ref_avg = _oracle_loop(o, grid, walls, dt, seed, steps, 2)
    return dict(nx=nx, ppc=ppc, seed=seed, steps=steps, sp=sp, grid=grid, walls=walls, dt=dt, o=o, init=init,
                last=last, avg=ref_avg)


@pytest.mark.parametrize("launches", [2, 1, 3])
def test_bench_couette_steps_match_oracle(ctx, bench_reference, launches):
    """mz_step on the benchmark workload (the graph-replayed step, fused or
    two launches per step) equals the reference loop: 50,000 cells exceed
    one scan tile (2,048 cells) 25 times over, and particles move ~280 cells
    per step, so the windowed histograms' fallbacks run too."""
    R = bench_reference
    sp = R["sp"]
    dom = mz.Domain(ctx, R["nx"], sp, int(R["nx"] * R["ppc"] * 1.1) + 1024,
                    interactions=mz.interactions_from_vhs(sp, mz.VHS), seed=R["seed"])
    dom.set_cell_volumes(R["grid"].V)
    dom.upload(0, *R["init"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    Fnum = R["grid"].dx * NDENS / R["ppc"]
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T_WALL, T_WALL, Fnum))
    inst, avg = mz.PhysProps(dom), mz.PhysProps(dom)
    dom.step(_plan(R["grid"], R["walls"], R["dt"], launches, R["steps"]), R["steps"], inst, avg)
    assert dom.counters()["wall_hits"] > 0
    _compare_couette(R["o"], dom, inst, avg, R["last"], R["avg"], f"50,000 cells, {launches} launch(es)")
    dom.close()


@pytest.mark.parametrize("launches,hitq", [(1, 0), (2, 0), (3, 0), (1, 64), (2, 64), (3, 64)])
def test_far_movers_on_a_multi_tile_grid_match_oracle(ctx, orc, launches, hitq):
    """7,000 cells (four scan tiles) and dt = 2e-7 s: particles move ~670
    cells per step (a standard deviation), so many destinations fall outside
    the step kernel's 1,536-cell histogram window and the scatter's
    2,048-cell window and take the direct-count paths; with a 64-entry
    wall-hit queue most hitters are reflected inside the step kernel."""
    nx, ppc, seed, steps = 7000, 24, 77, 4
    sp, grid, walls, dt, dom = _couette_device(ctx, nx, ppc, seed, dt=2e-7, cap_factor=1.5)
    o = _oracle_couette(orc, dom, sp)
    last, ref_avg = _oracle_loop(o, grid, walls, dt, seed, steps, 2)
    inst, avg = mz.PhysProps(dom), mz.PhysProps(dom)
    dom.step(_plan(grid, walls, dt, launches, steps, hitq=hitq), steps, inst, avg)
    assert dom.counters()["wall_hits"] > 4 * 64
    _compare_couette(o, dom, inst, avg, last, ref_avg, f"far movers, {launches} launch(es), queue {hitq}")
    dom.close()


@pytest.mark.parametrize("n_cells,n,seed", [(7000, 300_000, 4), (20_000, 1_000_000, 5)])
def test_sort_over_several_scan_tiles_bit_exact(ctx, orc, n_cells, n, seed):
    """sort_particles! (grid_sorting.jl:58-113) with 4 and 10 scan tiles: of
    particles moved anywhere in the domain (the permutation, the indexers and
    the particles in order are equal), and of the state a splitting ntc!
    leaves (group-2 particles, dead reserved slots)."""
    rng = np.random.default_rng(seed)
    L = 5e-4
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    cell = np.sort(rng.integers(0, n_cells, n)).astype(np.int32)
    x = rng.random((n, 3))
    x[:, 0] = (cell + rng.uniform(0.05, 0.95, n)) * (L / n_cells)
    v = rng.normal(0.0, 300.0, (n, 3))
    w = 1e12 * 10.0 ** (rng.random(n) - 0.5)
    dom = mz.Domain(ctx, n_cells, sp, 2 * n, interactions=inter, seed=seed)
    dom.upload(0, w, v, x, cell)
    o = _oracle_from_device(orc, dom, sp)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 300.0, 300.0, 1e12)
    dom.set_sigma_g_w_max(0, 0, smax)
    o.cf_set_smax(0, 0, smax)
    # a splitting ntc! appends group-2 particles (V = 1 per cell, so a long
    # dt gives a few collisions per cell); then every particle moves
    o.ntc_cells(0, 0, 20.0, None, seed, 1, equal_weight=False, nthreads=THREADS)
    dom.ntc(0, 0, 20.0, 1, equal_weight=False)
    assert dom.counters()["splits"] > 1000
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    xs = drows[:, 4].copy()
    xn = rng.random(xs.size) * L * 0.999999 + L * 5e-7
    # new positions through a fresh upload on both sides, in the current order
    dom2 = mz.Domain(ctx, n_cells, sp, 2 * n, interactions=inter, seed=seed)
    rows = drows.copy()
    rows[:, 4] = xn
    rows[:, 5] = np.arange(rows.shape[0])  # y carries an id tag
    dom2.upload(0, rows[:, 0], rows[:, 1:4], rows[:, 4:7], dc.astype(np.int32))
    o2 = _oracle_from_device(orc, dom2, sp)
    o2.sort(0, L=L, nx=n_cells)
    perm = dom2.sort(0, mz.Grid1DUniform(L, n_cells), return_index=True)
    orows, ocell = oracle_logical(o2, 0)
    drows2, dcell = device_logical(dom2, 0)
    assert np.array_equal(orows, drows2) and np.array_equal(ocell, dcell)
    assert np.array_equal(perm, o2.pv_get(0)["index"][: rows.shape[0]] - 1)
    oind, _, _ = o2.pia_get()
    dind, nt = dom2.indexer(0)
    assert nt == rows.shape[0]
    assert np.array_equal(dind[:, 3], oind[0, :, 3]) and np.array_equal(dind[:, 0], oind[0, :, 0])
    # the split state itself sorted on the grid (split particles share their
    # parent's position, so every particle stays in its cell): group 1 of
    # every cell, then group 2 in cell order, dead reserved slots skipped
    o.sort(0, L=L, nx=n_cells)
    dom.sort(0, mz.Grid1DUniform(L, n_cells))
    orows, ocell = oracle_logical(o, 0)
    drows, dcell = device_logical(dom, 0)
    assert np.array_equal(ocell, dcell)
    # positions are copied exactly (collisions change velocities and splits
    # weights, equal to round-off): equal positions mean the same order
    assert np.array_equal(orows[:, 4:7], drows[:, 4:7])
    assert_close_rows(orows, drows, 1e-12, "split state sorted")
    oind, _, _ = o.pia_get()
    dind, _ = dom.indexer(0)
    assert np.array_equal(dind[:, 3], oind[0, :, 3]) and np.all(dind[:, 6] == 0)
    dom.close()
    dom2.close()


def test_batched_0d_full_size_matches_oracle(ctx, orc):
    """The batched 0-D workload itself: 65,536 independent Ar cells with
    seeded log-uniform counts in [50, 4000] (5.9e7 particles), bi-Maxwellian
    2000 / 300 / 300 K, Fnum 1e13, V 1; two graph steps at dt = 1e-6 s, then
    two at dt = 1e-4 s (more collisions), cells of 2,048 particles and more
    colliding one block per cell.  Collision counts per cell equal, particles
    and compute_props! within 1e-11."""
    n_cells, seed = 65536, 1234
    rng = np.random.default_rng(seed)
    counts = np.floor(np.exp(rng.uniform(np.log(50), np.log(4000), n_cells))).astype(np.int64)
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    dom = mz.Domain(ctx, n_cells, sp, int(counts.sum()) + 1024, interactions=inter, seed=seed)
    dom.sample_cells(0, counts, [2000.0, 300.0, 300.0], 1e13, step=0)
    Tm = (2000.0 + 300.0 + 300.0) / 3
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], Tm, Tm, 1e13)
    dom.set_sigma_g_w_max(0, 0, smax)
    o = _oracle_from_device(orc, dom, sp)
    o.cf_set_smax(0, 0, smax)
    inst = mz.PhysProps(dom)
    done = 0
    for dt, k in ((1e-6, 2), (1e-4, 2)):
        p = mz._lib.StepPlan()
        p.dims, p.collide, p.equal_weight, p.props, p.dt, p.step0, p.use_graph = 0, 1, 1, 1, dt, done, 1
        p.big_cell = 2048
        dom.step(p, k, inst)
        for t in range(done + 1, done + k + 1):
            o.ntc_cells(0, 0, dt, None, seed, t, equal_weight=True, nthreads=THREADS)
        done += k
        smax_o, cnt = o.cf_get(0, 0)
        cf = dom.collision_factors(0, 0)
        assert np.array_equal(cf["n_coll"], cnt[:, 2]), dt
        assert np.array_equal(cf["n_coll_performed"], cnt[:, 3]), dt
        assert np.allclose(cf["sigma_g_w_max"], smax_o, rtol=1e-12, atol=0)
    assert dom.counters()["accepted"] > 10_000
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-11, "65,536 0-D cells after 4 steps")
    r = inst.fetch()
    ref = o.compute_props(mode=0, nthreads=THREADS)
    assert np.array_equal(r["np"][:, 0], ref["np"][0])
    assert_close_rows(r["T"][:, 0:1], ref["T"][0].reshape(-1, 1), 1e-11, "T")
    assert_close_rows(r["n"][:, 0:1], ref["n"][0].reshape(-1, 1), 1e-13, "n")
    dom.close()
