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


def _vw_plan(grid, walls, dt, octree, threshold, target, dims=1, step0=0, graph=True, avg_start=0, n_avg=1,
             split_lanes=0):
    """mz_step with equal_weight = 0: ntc! with splitting, merging of the cells
    above `threshold` down to `target`, (1-D) convection, sort, props."""
    p = mz._lib.StepPlan()
    p.dims, p.collide, p.equal_weight, p.props = dims, 1, 0, 1
    p.avg_start, p.n_avg, p.dt, p.dw_tol, p.step0 = avg_start, n_avg, dt, 1e-16, step0
    p.use_graph = 1 if graph else 0
    if grid is not None:
        p.grid = grid.c_struct()
    if walls is not None:
        p.walls = walls.c_struct()
    p.merge_threshold, p.merge_target, p.octree = threshold, target, octree.params
    p.split_lanes = split_lanes
    return p


def _oracle_varweight_loop(o, oc, grid, walls, dt, seed, steps, threshold, target, step0=0, threads=8):
    """The reference loop of couette_varweight_octree.jl:85-135 on the oracle:
    ntc! per cell, merge of the cells above the threshold, squash_pia!,
    convect, sort."""
    nx = o.n_cells
    merged = 0
    for step in range(step0 + 1, step0 + steps + 1):
        o.ntc_cells(0, 0, dt, None if grid is None else grid.V, seed, step, equal_weight=False, nthreads=threads)
        ind, _, _ = o.pia_get()
        for c in np.nonzero(ind[0, :, 0] > threshold)[0]:
            if grid is None:
                o.merge_octree(oc, 0, int(c) + 1, target, seed=seed, step=step)
            else:
                o.merge_octree(oc, 0, int(c) + 1, target, L=grid.L, nx=nx, seed=seed, step=step)
            merged += 1
        o.squash(0)
        if grid is not None:
            o.convect(0, grid.L, nx, walls.as_flat_array(), dt, seed, step, nthreads=threads)
            o.sort(0, L=grid.L, nx=nx)
    return merged


@pytest.mark.parametrize("graph", [True, False])
def test_fused_varweight_step_equals_standalone_loop(ctx, orc, graph):
    """mz_step with splitting and merging (one graph-replayed step, no host
    synchronisation inside) gives the particles of the standalone calls
    ntc! -> merge -> convect -> sort bit for bit, and both follow the oracle."""
    nx, ppc, steps, threshold, target, seed = 24, 150, 5, 160, 80, 93
    sp, inter, grid, walls, dt, smax, arrays = _varweight_state(nx, ppc, seed)
    cap = 8 * nx * ppc
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    doms = []
    for fused in (True, False):
        dom = mz.Domain(ctx, nx, sp, cap, interactions=inter, seed=seed)
        dom.upload(0, *arrays)
        dom.set_cell_volumes(grid.V)
        dom.set_sigma_g_w_max(0, 0, smax)
        if fused:
            inst = mz.PhysProps(dom)
            dom.step(_vw_plan(grid, walls, dt, octree, threshold, target, graph=graph), steps, inst)
        else:
            for step in range(1, steps + 1):
                dom.ntc(0, 0, dt, step, equal_weight=False)
                dom.merge_octree(0, octree, target, threshold=threshold, grid=grid, step=step)
                dom.convect(0, grid, walls, dt, step)
                dom.sort(0, grid)
        doms.append(dom)
    a, ca = device_logical(doms[0], 0)
    b, cb = device_logical(doms[1], 0)
    assert np.array_equal(ca, cb) and np.array_equal(a, b)
    cnt = doms[0].counters()
    assert cnt["merges"] >= nx and cnt["splits"] > 0
    assert doms[0].info(0)["n_total"] == a.shape[0]
    o = oracle_state(orc, nx, sp, mz.VHS, [arrays], capacity=cap)
    o.cf_set_smax(0, 0, smax)
    oc = orc.Octree(orc.SPLIT_MID, mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit, 6000, 10)
    _oracle_varweight_loop(o, oc, grid, walls, dt, seed, steps, threshold, target)
    orows, oc_cells = oracle_logical(o, 0)
    assert np.array_equal(oc_cells, ca)
    assert_close_rows(orows, a, 1e-11, "fused variable-weight step")
    r = inst.fetch()
    ref = o.compute_props(mode=2)
    assert np.array_equal(r["np"][:, 0], ref["np"][0])
    assert_close_rows(r["T"][:, 0:1], ref["T"][0].reshape(-1, 1), 1e-11, "T after the fused steps")
    for dom in doms:
        dom.close()


def test_varweight_lanes_per_cell_change_no_result(ctx):
    """8, 16 or 32 lanes per cell in the splitting NTC, set by the plan or
    chosen by mz_step_autotune on real steps: the same particles after the
    same steps."""
    nx, ppc, steps, threshold, target, seed = 40, 150, 14, 170, 90, 55
    sp, inter, grid, walls, dt, smax, arrays = _varweight_state(nx, ppc, seed)
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    runs = []
    for lanes in ("tune", 8, 16, 32):
        dom = mz.Domain(ctx, nx, sp, 8 * nx * ppc, interactions=inter, seed=seed)
        dom.upload(0, *arrays)
        dom.set_cell_volumes(grid.V)
        dom.set_sigma_g_w_max(0, 0, smax)
        done = 0
        if lanes == "tune":
            chosen, big = dom.autotune(_vw_plan(grid, walls, dt, octree, threshold, target), trial_steps=1)
            assert chosen in (8, 16, 32) and big == 0
            done = 6
        dom.step(_vw_plan(grid, walls, dt, octree, threshold, target, step0=done,
                          split_lanes=0 if lanes == "tune" else lanes), steps - done)
        runs.append(device_logical(dom, 0))
        assert dom.counters()["splits"] > 0
        dom.close()
    for r in runs[1:]:
        assert np.array_equal(runs[0][1], r[1]) and np.array_equal(runs[0][0], r[0])


@pytest.mark.parametrize("split_lanes", [32, 8])
def test_fused_varweight_couette_at_the_benchmark_size_matches_oracle(ctx, orc, split_lanes):
    """The variable-weight Couette configuration: 1,000 cells, 1,000 initial
    particles per cell with weights log-uniform over two decades, merging of
    cells above 1,200 particles down to 300; four fused steps against the
    oracle's reference loop: candidate and collision counts per cell, cells
    and indexers equal, particles within 1e-11."""
    nx, ppc, steps, threshold, target, seed = 1000, 1000, 4, 1200, 300, 1234
    sp, inter, grid, walls, dt, smax, arrays = _varweight_state(nx, ppc, seed)
    cap = 5_000_000
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    dom = mz.Domain(ctx, nx, sp, cap, interactions=inter, seed=seed)
    dom.upload(0, *arrays)
    dom.set_cell_volumes(grid.V)
    dom.set_sigma_g_w_max(0, 0, smax)
    inst = mz.PhysProps(dom)
    dom.step(_vw_plan(grid, walls, dt, octree, threshold, target, split_lanes=split_lanes), steps, inst)
    o = oracle_state(orc, nx, sp, mz.VHS, [arrays], capacity=cap)
    o.cf_set_smax(0, 0, smax)
    oc = orc.Octree(orc.SPLIT_MID, mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit, 6000, 10)
    merged = _oracle_varweight_loop(o, oc, grid, walls, dt, seed, steps, threshold, target, threads=16)
    cnt = dom.counters()
    assert cnt["merges"] == merged and merged > 100
    smax_o, ccnt = o.cf_get(0, 0)
    cf = dom.collision_factors(0, 0)
    assert np.array_equal(cf["n_coll"], ccnt[:, 2]) and np.array_equal(cf["n_coll_performed"], ccnt[:, 3])
    orows, oc_cells = oracle_logical(o, 0)
    drows, dc_cells = device_logical(dom, 0)
    assert np.array_equal(oc_cells, dc_cells)
    assert_close_rows(orows, drows, 1e-11, "variable-weight Couette, 1,000 cells")
    oind, _, _ = o.pia_get()
    dind, _ = dom.indexer(0)
    assert np.array_equal(dind[:, 3], oind[0, :, 3])
    r = inst.fetch()
    ref = o.compute_props(mode=2)
    assert np.array_equal(r["np"][:, 0], ref["np"][0])
    assert_close_rows(r["T"][:, 0:1], ref["T"][0].reshape(-1, 1), 1e-11, "T")
    dom.close()


def test_fused_varweight_step_grows_storage_and_resumes(ctx):
    """Storage too small for a step's split reservations, and a 0-D cell larger
    than the merge scratch: the step is abandoned before it changes a
    particle, the host grows the storage (MZ_E_CAPACITY's remedy,
    collision_ntc.jl:241-243 resizes the ParticleVector) or the scratch and
    resumes; the result equals a run that never ran short."""
    sp = species(["Ar"])
    inter = interactions(sp)
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    # 1-D: capacity just above the initial particles
    nx, ppc, threshold, target, seed = 16, 150, 160, 80, 71
    _, _, grid, walls, dt, smax, arrays = _varweight_state(nx, ppc, seed)
    runs = []
    for cap in (nx * ppc + 10, 8 * nx * ppc):
        dom = mz.Domain(ctx, nx, sp, cap, interactions=inter, seed=seed)
        dom.upload(0, *arrays)
        dom.set_cell_volumes(grid.V)
        dom.set_sigma_g_w_max(0, 0, smax)
        dom.step(_vw_plan(grid, walls, 3 * dt, octree, threshold, target), 6)
        runs.append((device_logical(dom, 0), dom.info(0)["capacity"]))
        dom.close()
    (a, ca), cap_small = runs[0]
    (b, cb), _ = runs[1]
    assert cap_small > nx * ppc + 10  # the storage grew
    assert np.array_equal(ca, cb) and np.array_equal(a, b)
    # 0-D: a cell of 5,000 particles is beyond the default merge scratch
    # (2 x threshold or threshold + 2,048)
    counts = np.array([300, 5000, 800, 120])
    states = []
    for mode in ("graph", "direct", "standalone"):
        dom = mz.Domain(ctx, len(counts), sp, 4 * int(counts.sum()), interactions=inter, seed=seed)
        dom.sample_cells(0, counts, 300.0, 1e12, step=0, log10_weight_span=2.0)
        dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 300.0, 300.0, 1e12))
        if mode == "standalone":
            for step in range(1, 4):
                dom.ntc(0, 0, 1e-3, step, equal_weight=False)
                dom.merge_octree(0, octree, 100, threshold=200, step=step)
                dom.squash(0)
        else:
            dom.step(_vw_plan(None, None, 1e-3, octree, 200, 100, dims=0, graph=mode == "graph"), 3)
        states.append(device_logical(dom, 0))
        # three cells above the threshold, merged to a target below it
        assert dom.counters()["merges"] >= 3
        dom.close()
    for a, ca in states[1:]:
        assert np.array_equal(states[0][1], ca) and np.array_equal(states[0][0], a)


def _one_cell_oracle(orc, sp, rows_by_species, smax, capacity):
    """A one-cell oracle (the reference's 0-D variable-weight tests simulate
    one cell: with several cells and no sort between steps, a cell's next
    split would extend its group 2 over the next cell's, particles.jl:311-315)."""
    t = mz.VHS
    o = orc.Oracle(1, len(sp), [s.mass for s in sp])
    if len(sp) == 1:
        o.load_interactions(*t["Ar,Ar"])
    else:
        o.load_interactions([[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]],
                            [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]], 273.0)
    for s, rows in enumerate(rows_by_species):
        o.set_particles_simple(s, np.ones(rows.shape[0], np.int64), rows)
        o.pv_resize(s, capacity)
    for (s1, s2), v in smax.items():
        o.cf_set_smax(s1, s2, v)
    return o


def test_fused_varweight_0d_and_mixture_match_oracle(ctx, orc):
    """0-D variable-weight steps (test_bkw_varweight_octree.jl's loop: ntc!,
    merge, compute_props!) on the device-resident path, and a two-species
    mixture with unequal weights (test_2species_varweight_octree.jl), which
    mz_step runs with the standalone kernels step by step.  Every device cell
    draws the streams of cell 0 (mz_set_cell_rng), so each equals a one-cell
    oracle run of the reference loop on that cell's particles."""
    sp = species(["Ar"])
    inter = interactions(sp)
    counts = np.array([300, 1800, 800, 120, 2600, 40])
    n_cells = len(counts)
    seed, steps, threshold, target, dt, Fnum = 19, 4, 1000, 400, 0.2, 1e12
    dom = mz.Domain(ctx, n_cells, sp, 6 * int(counts.sum()), interactions=inter, seed=seed)
    dom.set_cell_rng(rids=np.zeros(n_cells, np.uint32))
    dom.sample_cells(0, counts, 500.0, Fnum, step=0, log10_weight_span=2.0)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 500.0, 500.0, Fnum)
    dom.set_sigma_g_w_max(0, 0, smax)
    w, v, x, cell = dom.download(0)
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    inst = mz.PhysProps(dom)
    dom.step(_vw_plan(None, None, dt, octree, threshold, target, dims=0), steps, inst)
    assert dom.counters()["splits"] > 100
    drows, dc_cells = device_logical(dom, 0)
    r = inst.fetch()
    oc = orc.Octree(orc.SPLIT_MID, mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit, 6000, 10)
    merged = 0
    for c in range(n_cells):
        rows = np.column_stack([w, v, x])[cell == c]
        o = _one_cell_oracle(orc, sp, [rows], {(0, 0): smax}, 6 * int(counts.sum()))
        merged += _oracle_varweight_loop(o, oc, None, None, dt, seed, steps, threshold, target)
        orows, _ = oracle_logical(o, 0)
        assert_close_rows(orows, drows[dc_cells == c], 1e-11, f"0-D variable-weight cell {c}")
        ref = o.compute_props(mode=0)
        assert abs(r["T"][c, 0] - ref["T"][0][0]) <= 1e-11 * ref["T"][0][0], c
    assert dom.counters()["merges"] == merged and merged >= 2
    dom.close()

    # two species, unequal weights: ntc! for (Ar,Ar), (He,Ar), (He,He), then
    # merging of each species (test_2species_varweight_octree.jl:57-80)
    sp2 = species(["Ar", "He"])
    inter2 = interactions(sp2)
    n_cells, seed, steps = 4, 23, 3
    cnt2 = [np.array([400, 900, 150, 600]), np.array([1200, 300, 800, 500])]
    Fn = (2e12, 5e11)
    dom = mz.Domain(ctx, n_cells, sp2, 20000, interactions=inter2, seed=seed)
    dom.set_cell_rng(rids=np.zeros(n_cells, np.uint32))
    for s, T0 in enumerate((3000.0, 360.0)):
        dom.sample_cells(s, cnt2[s], T0, Fn[s], step=0, log10_weight_span=1.0)
    arrays = [dom.download(s) for s in range(2)]
    smax2 = {}
    for s1 in range(2):
        for s2 in range(2):
            T1, T2 = (3000.0, 360.0)[s1], (3000.0, 360.0)[s2]
            smax2[s1, s2] = mz.estimate_sigma_g_w_max(inter2[s1][s2], sp2[s1], sp2[s2], T1, T2, max(Fn))
            dom.set_sigma_g_w_max(s1, s2, smax2[s1, s2])
    dom.step(_vw_plan(None, None, 0.2, octree, 1000, 500, dims=0), steps)
    assert dom.counters()["splits"] > 100
    dev = [device_logical(dom, s) for s in range(2)]
    for c in range(n_cells):
        rows = [np.column_stack(a[:3])[a[3] == c] for a in arrays]
        o = _one_cell_oracle(orc, sp2, rows, smax2, 20000)
        for step in range(1, steps + 1):
            for s2 in range(2):
                for s1 in range(s2, 2):
                    o.ntc(s1, s2, 1, 0.2, 1.0, seed, step, equal_weight=False)
            ind, _, _ = o.pia_get()
            for s in range(2):
                if ind[s, 0, 0] > 1000:
                    o.merge_octree(oc, s, 1, 500, seed=seed, step=step)
        for s in range(2):
            orows, _ = oracle_logical(o, s)
            drows, dcells = dev[s]
            assert_close_rows(orows, drows[dcells == c], 1e-11, f"mixture cell {c} species {s}")
    dom.close()
