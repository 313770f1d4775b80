"""Parity of the CUDA path (through the C ABI) with the oracle on the same
seeded inputs, plus the reference's known-answer vectors run on the device.

Tolerances: integer / index / permutation results are compared bit-exactly;
floating-point particle state and moments within 1e-12 relative to the
magnitude of the quantity (the replay tolerance of the collision routine)."""
import numpy as np
import pytest

import merzgpu as mz
from conftest import scenario
from helpers import (EPS, assert_close_rows, device_logical, device_state, interactions, oracle_logical, oracle_state,
                     random_particles, species)

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


# ---------------------------------------------------------------- sorting
def test_sort_golden_on_device(ctx, golden):
    """test/test_grid_sorting.jl:8-235 on the device; y carries particle ids."""
    sc = scenario(golden, "grid_sorting_coarse_fine_uneven")
    sp = species(["Ar"])
    parts = np.array(sc["particles"])
    st = sc["steps"]
    # coarse: sampled 4 per cell (cells [1-4], [5-8]) then positions overwritten
    dom = mz.Domain(ctx, 2, sp, 16)
    dom.upload(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7], np.array([0] * 4 + [1] * 4, np.int32))
    perm = dom.sort(0, mz.Grid1DUniform(8.0, 2), return_index=True)
    ids = dom.download(0)[2][:, 1]
    assert ids.tolist() == st[0]["expect_index"]
    assert perm.tolist() == [i - 1 for i in st[0]["expect_index"]]
    ind, nt = dom.indexer(0)
    exp = np.array(st[0]["expect_indexer"])
    exp[:, 1:3] -= 1  # 0-based slots
    assert ind.tolist() == exp.tolist()
    # fine grid continuing from the sorted state, all 8 in cell 0 group 1
    w, v, x, _ = dom.download(0)
    dom4 = mz.Domain(ctx, 4, sp, 16)
    dom4.upload(0, w, v, x, np.zeros(8, np.int32))
    dom4.sort(0, mz.Grid1DUniform(8.0, 4))
    assert dom4.download(0)[2][:, 1].tolist() == st[1]["expect_index"]
    ind, _ = dom4.indexer(0)
    assert ind[:, 3].tolist() == [2, 2, 2, 2] and ind[:, 1].tolist() == [0, 2, 4, 6]
    # uneven split after resetting the order to particle ids 1..8
    x2 = parts[:, 4:7].copy()
    x2[:, 0] = st[2]["x"]
    dom4.upload(0, parts[:, 0], parts[:, 1:4], x2, np.zeros(8, np.int32))
    dom4.sort(0, mz.Grid1DUniform(8.0, 4))
    assert dom4.download(0)[2][:, 1].tolist() == st[2]["expect_index"]
    ind, _ = dom4.indexer(0)
    assert ind[:, 3].tolist() == st[2]["expect_counts"]
    assert ind[:, 1].tolist() == [s - 1 if s > 0 else 0 for s in st[2]["expect_starts"]]
    assert ind[:, 2].tolist() == [e - 1 if e > 0 else -1 for e in st[2]["expect_ends"]]
    p = mz.PhysProps(dom4)
    mz.compute_props(dom4, p)
    r = p.fetch()
    assert np.all(np.abs(r["n"][:, 0] - np.array(st[2]["expect_n"])) < 2 * EPS)
    assert r["np"][:, 0].tolist() == st[2]["expect_counts"]
    # stored-cell variant (cells given at upload == sort_particles! without grid)
    dom4.upload(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7], np.array(st[3]["cell"], np.int32) - 1)
    assert dom4.download(0)[2][:, 1].tolist() == st[3]["expect_index"]


@pytest.mark.parametrize("n_cells,n,seed", [(7, 300, 1), (100, 20000, 2), (2000, 40000, 3)])
def test_sort_random_bit_exact(ctx, orc, n_cells, n, seed):
    rng = np.random.default_rng(seed)
    L = 5e-4
    sp = species(["Ar"])
    w, v, x, cell = random_particles(rng, n, n_cells, L=L)
    # move every particle somewhere else in the domain; y carries an id tag
    x[:, 0] = rng.random(n) * L * 0.999999 + L * 5e-7
    x[:, 1] = np.arange(n)
    o = oracle_state(orc, n_cells, sp, mz.VHS, [(w, v, x, cell)])
    dom = device_state(ctx, n_cells, sp, interactions(sp), [(w, v, x, cell)])
    o.sort(0, L=L, nx=n_cells)
    perm = dom.sort(0, mz.Grid1DUniform(L, n_cells), return_index=True)
    orows, ocell = oracle_logical(o, 0)
    drows, dcell = device_logical(dom, 0)
    assert np.array_equal(orows, drows)  # bit-exact: same particles in the same order
    assert np.array_equal(ocell, dcell)
    opv = o.pv_get(0)
    assert np.array_equal(perm, opv["index"][:n] - 1)
    oind, _, _ = o.pia_get()
    dind, nt = dom.indexer(0)
    assert nt == n
    assert np.array_equal(dind[:, 3], oind[0, :, 3])
    assert np.array_equal(dind[:, 0], oind[0, :, 0])


def test_sort_large_segments_bit_exact(ctx, orc):
    """Destination segments of up to 1,024 particles (register sort), of
    1,025-2,048 (sorted in a shared-memory buffer) and above 2,048 (sorted in
    place in global memory) end bit for bit like the oracle's sort."""
    rng = np.random.default_rng(9)
    L = 5e-4
    counts = np.array([5, 1024, 1025, 1500, 2048, 2049, 3000])
    n_cells, n = len(counts), int(counts.sum())
    sp = species(["Ar"])
    w, v, x, cell = random_particles(rng, n, n_cells, L=L)
    dest = rng.permutation(np.repeat(np.arange(n_cells), counts))
    x[:, 0] = (dest + rng.uniform(0.01, 0.99, n)) * (L / n_cells)
    x[:, 1] = np.arange(n)
    o = oracle_state(orc, n_cells, sp, mz.VHS, [(w, v, x, cell)])
    dom = device_state(ctx, n_cells, sp, interactions(sp), [(w, v, x, cell)])
    o.sort(0, L=L, nx=n_cells)
    perm = dom.sort(0, mz.Grid1DUniform(L, n_cells), return_index=True)
    orows, ocell = oracle_logical(o, 0)
    drows, dcell = device_logical(dom, 0)
    assert np.array_equal(np.bincount(dcell, minlength=n_cells), counts)
    assert np.array_equal(orows, drows) and np.array_equal(ocell, dcell)
    assert np.array_equal(perm, o.pv_get(0)["index"][:n] - 1)
    dom.close()


# ---------------------------------------------------------------- convection
def test_convection_golden_on_device(ctx, golden):
    sc = scenario(golden, "convection_specular_4particles")
    sp = species(["Ar"])
    parts = np.array(sc["particles"])
    grid = mz.Grid1DUniform(sc["L"], sc["nx"])
    walls = mz.MaxwellWalls1D(sp, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0)
    for compute_cell in (False, True):
        dom = mz.Domain(ctx, sc["nx"], sp, 16)
        dom.upload(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7], np.zeros(4, np.int32))
        dom.convect(0, grid, walls, sc["dt"], step=0, compute_cell=compute_cell)
        perm = dom.sort(0, None if compute_cell else grid, return_index=True)
        assert (perm + 1).tolist() == sc["expect_index_after_sort"]
        rows, cells = device_logical(dom, 0)
        for k, e in enumerate(sc["expect_sorted"]):
            tol = 2 * EPS if e["x_tol"] == "2eps" else e["x_tol"]
            assert np.max(np.abs(rows[k, 4:7] - np.array(e["x"]))) < tol
            assert rows[k, 1:4].tolist() == e["v"] and rows[k, 0] == e["w"]
        assert (cells + 1).tolist() == sorted(sc["expect_cells_after_convect"])


def test_convection_noncontiguous_on_device(ctx, golden):
    sc = scenario(golden, "convection_noncontiguous")
    sp = species(["Ar"])
    parts = np.array(sc["particles"])
    nx = sc["nx"]
    ind = np.zeros((nx, 7), np.int64)
    ind[:, 2] = -1
    ind[:, 5] = -1
    r = sc["indexer_cell2"]
    ind[1] = [r[0], r[1] - 1, r[2] - 1, r[3], r[4] - 1, r[5] - 1, r[6]]
    dom = mz.Domain(ctx, nx, sp, 64)
    dom.upload_indexed(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7], ind)
    p = mz.PhysProps(dom)
    mz.compute_props(dom, p)
    f = p.fetch()
    assert abs(f["n"][1, 0] - 15.0) < EPS and abs(f["v"][0, 1, 0] - 1.0) < EPS
    dom.convect(0, mz.Grid1DUniform(sc["L"], nx), mz.MaxwellWalls1D(sp, 1.0, 1.0, 0, 0, 0, 0), sc["dt"], step=0)
    dom.sort(0, mz.Grid1DUniform(sc["L"], nx))
    mz.compute_props(dom, p)
    f = p.fetch()
    assert abs(f["n"][3, 0] - 15.0) < EPS
    assert np.all(np.abs(np.delete(f["n"][:, 0], 3)) <= EPS)
    assert abs(f["v"][0, 3, 0] - 1.0) < EPS


@pytest.mark.parametrize("acc", [(1.0, 1.0), (0.2, 1.0), (0.0, 0.0)])
def test_convect_diffuse_vs_oracle(ctx, orc, acc):
    rng = np.random.default_rng(7)
    n_cells, n, L = 50, 20000, 5e-4
    sp = species(["Ar"])
    w, v, x, cell = random_particles(rng, n, n_cells, T=300.0, L=L)
    v *= 20.0  # many wall hits
    walls = mz.MaxwellWalls1D(sp, 273.0, 300.0, -500.0, 500.0, acc[0], acc[1])
    grid = mz.Grid1DUniform(L, n_cells)
    dt = 2e-9
    o = oracle_state(orc, n_cells, sp, mz.VHS, [(w, v, x, cell)])
    dom = device_state(ctx, n_cells, sp, interactions(sp), [(w, v, x, cell)], seed=99)
    o.convect(0, L, n_cells, walls.as_flat_array(), dt, seed=99, step=5, compute_cell=True)
    dom.convect(0, grid, walls, dt, step=5, compute_cell=True)
    ocells = o.pv_get(0)["cell"]
    o.sort(0)
    dom.sort(0)
    orows, ocell = oracle_logical(o, 0)
    drows, dcell = device_logical(dom, 0)
    assert np.array_equal(ocell, dcell)
    assert_close_rows(orows, drows, RTOL, "convected particles")
    assert dom.counters()["wall_hits"] > 0 if acc != (0.0, 0.0) else True


# ---------------------------------------------------------------- props
@pytest.mark.parametrize("mode", ["all", "sorted", "moments", "ndens"])
def test_props_vs_oracle(ctx, orc, mode):
    rng = np.random.default_rng(11)
    n_cells = 300
    sp = species(["Ar", "He"])
    arrays = [random_particles(rng, 30000, n_cells, T=500.0, mass=sp[0].mass, wspan=1.0, drift=(100, -50, 10)),
              random_particles(rng, 9000, n_cells, T=800.0, mass=sp[1].mass, w=3e11)]
    arrays[1][3][:] = np.minimum(arrays[1][3], n_cells - 5)  # a few empty cells for species 2
    o = oracle_state(orc, n_cells, sp, mz.VHS, arrays)
    dom = device_state(ctx, n_cells, sp, interactions(sp), arrays)
    powers = [4, 6, 8, 10] if mode == "moments" else []
    V = np.linspace(1.0, 2.0, n_cells)
    p = mz.PhysProps(dom, powers, ndens_not_Np=(mode == "ndens"), Tref=273.0)
    if mode == "ndens":
        dom.set_cell_volumes(V)
    {"all": mz.compute_props, "sorted": mz.compute_props_sorted, "moments": mz.compute_props_with_total_moments,
     "ndens": mz.compute_props_sorted}[mode](dom, p)
    r = p.fetch()
    omode = {"all": 0, "sorted": 2, "moments": 1, "ndens": 3}[mode]
    ref = o.compute_props(mode=omode, powers=powers, Tref=273.0, inv_V=(1.0 / V if mode == "ndens" else None))
    assert np.array_equal(r["np"].T, ref["np"])
    assert_close_rows(r["n"].T.reshape(-1, 1), ref["n"].reshape(-1, 1), RTOL, "n")
    assert_close_rows(r["v"].transpose(2, 1, 0).reshape(-1, 3), ref["v"].reshape(-1, 3), RTOL, "v")
    assert_close_rows(r["T"].T.reshape(-1, 1), ref["T"].reshape(-1, 1), RTOL, "T")
    if powers:
        a = r["moments"].transpose(2, 1, 0).reshape(-1, len(powers))
        b = ref["moments"].reshape(-1, len(powers))
        ok = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), ok)
        assert_close_rows(a[ok.all(1)], b[ok.all(1)], 1e-11, "moments")


# ---------------------------------------------------------------- NTC
def _ntc_case(ctx, orc, names, n_per, n_cells, equal_weight, wspan, seed, steps=1, cand_per_cell=60.0):
    """Matched oracle/device NTC runs.  dt is chosen so the first pair sees
    about cand_per_cell candidates per cell per step."""
    rng = np.random.default_rng(seed)
    sp = species(names)
    table = mz.VHS
    inter = interactions(sp, table)
    arrays = [random_particles(rng, n_per[s], n_cells, T=[2000.0, 600.0][s], mass=sp[s].mass, w=1e12 * (s + 1),
                               wspan=wspan) for s in range(len(sp))]
    o = oracle_state(orc, n_cells, sp, table, arrays, capacity=sum(n_per) * 4)
    dom = device_state(ctx, n_cells, sp, inter, arrays, capacity=sum(n_per) * 4, seed=seed)
    V = np.full(n_cells, 1.0)
    smax0 = None
    for s1 in range(len(sp)):
        for s2 in range(len(sp)):
            smax = mz.estimate_sigma_g_w_max(inter[s1][s2], sp[s1], sp[s2], 1000.0, 1000.0, 1e12 * (max(s1, s2) + 1))
            smax0 = smax if smax0 is None else smax0
            o.cf_set_smax(s1, s2, smax)
            dom.set_sigma_g_w_max(s1, s2, smax)
    npc = n_per[0] / n_cells
    dt = cand_per_cell / (0.5 * npc * npc * smax0)
    pairs = [(s1, s2) for s2 in range(len(sp)) for s1 in range(s2, len(sp))]
    for step in range(1, steps + 1):
        for s1, s2 in pairs:
            o.ntc_cells(s1, s2, dt, V, seed, step, equal_weight=equal_weight)
            dom.ntc(s1, s2, dt, step, equal_weight=equal_weight)
    return o, dom, sp, pairs


@pytest.mark.parametrize("equal_weight", [True, False])
def test_ntc_single_species_vs_oracle(ctx, orc, equal_weight):
    o, dom, sp, pairs = _ntc_case(ctx, orc, ["Ar"], [40000], 100, equal_weight, 0.0, seed=21, steps=3)
    cf = dom.collision_factors(0, 0)
    smax, cnt = o.cf_get(0, 0)
    assert np.array_equal(cf["n_coll"], cnt[:, 2]) and np.array_equal(cf["n_coll_performed"], cnt[:, 3])
    assert np.array_equal(cf["n_eq_w_coll_performed"], cnt[:, 4])
    assert cnt[:, 3].sum() > 1000
    assert_close_rows(cf["sigma_g_w_max"].reshape(-1, 1), smax.reshape(-1, 1), RTOL, "smax")
    orows, _ = oracle_logical(o, 0)
    drows, _ = device_logical(dom, 0)
    assert_close_rows(orows, drows, RTOL, "particles after ntc")


@pytest.mark.parametrize("n_cells,steps", [(20, 1), (1, 4)])
def test_ntc_variable_weight_splits_vs_oracle(ctx, orc, n_cells, steps):
    """Splitting (collision_ntc.jl:235-267).  The reference appends split
    particles at position n_total, so repeated calls stay consistent only on a
    single cell (0-D) or with a sort in between -- the two usages tested."""
    o, dom, sp, pairs = _ntc_case(ctx, orc, ["Ar"], [300 * n_cells], n_cells, False, 1.0, seed=33, steps=steps,
                                  cand_per_cell=40.0)
    smax, cnt = o.cf_get(0, 0)
    cf = dom.collision_factors(0, 0)
    assert np.array_equal(cf["n_coll"], cnt[:, 2])
    assert np.array_equal(cf["n_coll_performed"], cnt[:, 3])
    assert np.array_equal(cf["n_eq_w_coll_performed"], cnt[:, 4])
    ind, nt = dom.indexer(0)
    oind, ont, _ = o.pia_get()
    assert nt == ont[0] and nt > 300 * n_cells  # splits happened
    assert np.array_equal(ind[:, 0], oind[0, :, 0])
    orows, _ = oracle_logical(o, 0)
    drows, _ = device_logical(dom, 0)
    assert_close_rows(orows, drows, RTOL, "particles after split ntc")
    assert np.isclose(orows[:, 0].sum(), drows[:, 0].sum(), rtol=1e-14)


@pytest.mark.parametrize("equal_weight,n_cells,steps", [(True, 16, 2), (False, 1, 3)])
def test_ntc_two_species_vs_oracle(ctx, orc, equal_weight, n_cells, steps):
    o, dom, sp, pairs = _ntc_case(ctx, orc, ["Ar", "He"], [250 * n_cells, 750 * n_cells], n_cells, equal_weight,
                                  0.0 if equal_weight else 0.5, seed=44, steps=steps, cand_per_cell=30.0)
    for s1, s2 in pairs:
        smax, cnt = o.cf_get(s1, s2)
        cf = dom.collision_factors(s1, s2)
        assert np.array_equal(cf["n_coll"], cnt[:, 2]), (s1, s2)
        assert np.array_equal(cf["n_coll_performed"], cnt[:, 3]), (s1, s2)
    for s in range(2):
        orows, _ = oracle_logical(o, s)
        drows, _ = device_logical(dom, s)
        assert_close_rows(orows, drows, RTOL, f"species {s}")


# ---------------------------------------------------------------- sampling
@pytest.mark.parametrize("dist", [0, 1])
def test_sampler_vs_oracle(ctx, orc, dist):
    sp = species(["Ar"])
    n_cells = 5
    o = orc.Oracle(n_cells, 1, [sp[0].mass])
    o.pv_create(0, 5000)
    dom = mz.Domain(ctx, n_cells, sp, 5000, seed=77)
    counts = [1000, 0, 700, 50, 3]
    T = 500.0
    for c, n in enumerate(counts):
        if n:
            o.sample_equal_weight(0, c + 1, n, T, 1e13, box=(c * 1.0, c + 1.0, 0, 1, 0, 1), seed=77, step=3,
                                  distribution=dist)
    box = np.array([[c, c + 1.0, 0, 1, 0, 1] for c in range(n_cells)])
    dom.sample_cells(0, counts, T, 1e13, step=3, box=box, distribution=dist)
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-13, "sampled")


def test_grid_ndens_sampler_vs_oracle(ctx, orc):
    sp = species(["Ar"])
    nx, L, ndens, T = 40, 5e-4, 1e23, 273.0
    grid = mz.Grid1DUniform(L, nx)
    Fnum = grid.dx * ndens / 97.3
    o = orc.Oracle(nx, 1, [sp[0].mass])
    o.pv_create(0, 5000)
    o.sample_grid_ndens(0, L, nx, ndens, T, Fnum, seed=5, step=0)
    dom = mz.Domain(ctx, nx, sp, 5000, seed=5)
    dom.sample_grid_ndens(0, grid, ndens, T, Fnum, step=0)
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-13, "grid sampled")


# ---------------------------------------------------------------- a 1D step sequence
def test_couette_steps_vs_oracle(ctx, orc):
    """ntc_equal_weight! -> convect -> sort -> compute_props_sorted!, 5 steps,
    the loop of simulations/1D/couette_benchmarking.jl:58-85."""
    sp = species(["Ar"])
    inter = interactions(sp)
    nx, L, ndens, T = 60, 5e-4, 1e23, 273.0
    grid = mz.Grid1DUniform(L, nx)
    ppc = 150
    Fnum = grid.dx * ndens / ppc
    walls = mz.MaxwellWalls1D(sp, T, T, -500.0, 500.0, 1.0, 1.0)
    nu = mz.mean_collision_frequency(inter, sp, 0, ndens, T)
    dt = 0.2 / nu
    o = orc.Oracle(nx, 1, [sp[0].mass])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    o.pv_create(0, ppc * nx * 2)
    o.sample_grid_ndens(0, L, nx, ndens, T, Fnum, seed=3, step=0)
    dom = mz.Domain(ctx, nx, sp, ppc * nx * 2, interactions=inter, seed=3)
    dom.sample_grid_ndens(0, grid, ndens, T, Fnum, step=0)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T, T, Fnum)
    o.cf_set_smax(0, 0, smax)
    dom.set_sigma_g_w_max(0, 0, smax)
    dom.set_cell_volumes(grid.V)
    p = mz.PhysProps(dom)
    for step in range(1, 6):
        o.ntc_cells(0, 0, dt, grid.V, 3, step, equal_weight=True)
        dom.ntc(0, 0, dt, step, equal_weight=True)
        o.convect(0, L, nx, walls.as_flat_array(), dt, 3, step)
        dom.convect(0, grid, walls, dt, step)
        o.sort(0, L=L, nx=nx)
        dom.sort(0, grid)
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, 1e-11, "state after 5 Couette steps")
    mz.compute_props_sorted(dom, p)
    r = p.fetch()
    ref = o.compute_props(mode=2)
    assert np.array_equal(r["np"].T, ref["np"])
    assert_close_rows(r["T"].T.reshape(-1, 1), ref["T"].reshape(-1, 1), 1e-11, "T")


def test_close_order_is_safe(ctx):
    """Closing a context closes its domains and their property sets first;
    later finalizers are no-ops (no use after free)."""
    c2 = mz.Context(0)
    sp = species(["Ar"])
    dom = mz.Domain(c2, 4, sp, 16)
    p = mz.PhysProps(dom)
    q = mz.PhysProps(dom)
    q.close()
    c2.close()
    assert not dom.h and not p.h
    del p, dom


# ---------------------------------------------------------------- squash_pia!
SQUASH_CASES = [
    # (cell positions, 1-based indexer rows, deletions (cell, group or 0 for delete_particle_end!))
    # test/test_pia_contiguous.jl:1-320
    ([10.0] * 10, [[10, 1, 10, 10, -1, -1, 0]], [(1, 1)]),
    ([10.0] * 10, [[10, 1, 5, 5, 6, 10, 5]], [(1, 1), (1, 2)]),
    ([1.0, 1.0, 1.0, 2.0, 2.0, 3.0, 3.0, 1.0, 3.0, 3.0],
     [[4, 1, 3, 3, 8, 8, 1], [2, 4, 5, 2, -1, -1, 0], [4, 6, 7, 2, 9, 10, 2]], [(1, 0), (1, 0), (1, 0), (3, 1)]),
    ([1.0, 1.0, 1.0, 2.0, 3.0, 3.0, 3.0, 2.0, 2.0, 2.0],
     [[3, 1, 3, 3, -1, -1, 0], [4, 4, 4, 1, 8, 10, 3], [3, 5, 7, 3, -1, -1, 0]], [(1, 0), (3, 0), (3, 0), (2, 1)]),
    # test/test_pia_contiguous.jl:440-615: cells deleted to empty
    ([1.0, 1.0, 1.0, 2.0, 3.0, 3.0, 3.0, 2.0, 2.0, 2.0],
     [[3, 1, 3, 3, -1, -1, 0], [4, 4, 4, 1, 8, 10, 3], [3, 5, 7, 3, -1, -1, 0]], [(1, 0), (1, 0), (1, 0)]),
    ([1.0, 1.0, 1.0, 2.0, 3.0, 3.0, 3.0, 2.0, 2.0, 2.0],
     [[3, 1, 3, 3, -1, -1, 0], [4, 4, 4, 1, 8, 10, 3], [3, 5, 7, 3, -1, -1, 0]], [(1, 0), (3, 0), (3, 0), (3, 0)]),
]


@pytest.mark.parametrize("case", range(len(SQUASH_CASES)))
def test_squash_known_answers_vs_oracle(ctx, orc, case):
    """The reference's hand-built states after deletions, squashed on the
    device (every cell into one contiguous list, logical order kept) and by
    the oracle's squash_pia!: the same particles in the same cell order."""
    x, rows, dels = SQUASH_CASES[case]
    n, nc = len(x), len(rows)
    parts = np.array([[float(i + 1), 0.0, 0.0, 0.0, x[i], 0.0, 1.0] for i in range(n)])
    o = orc.Oracle(nc, 1, [mz.AR_MASS])
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = o.pia_get()
    for c, r in enumerate(rows):
        ind[0, c] = r
    nt[0] = n
    o.pia_set(ind, nt, cg)
    for cell, group in dels:
        if group:
            o.delete_particle_end_group(0, cell, group)
        else:
            o.delete_particle_end(0, cell)
    # the device gets the post-deletion state: logical position p holds
    # particle index[p]; positions no indexer entry covers (the deleted ones,
    # which may lie below the last position in use) are dead slots
    pv = o.pv_get(0)
    ind, nt, cg = o.pia_get()
    slots = parts[pv["index"] - 1]
    dev_rows = [[r[0], r[1] - 1, r[2] - 1, r[3], (r[4] - 1) if r[6] else 0, (r[5] - 1) if r[6] else -1, r[6]]
                for r in ind[0]]
    dom = mz.Domain(ctx, nc, species(["Ar"]), n + 16)
    dom.upload_indexed(0, slots[:, 0], slots[:, 1:4], slots[:, 4:7], dev_rows)
    cg[0] = 0
    o.pia_set(ind, nt, cg)
    o.squash(0)
    dom.squash(0)
    orows, ocells = oracle_logical(o, 0)
    drows, dcells = device_logical(dom, 0)
    assert np.array_equal(ocells, dcells)
    assert np.array_equal(orows, drows)
    dind, dnt = dom.indexer(0)
    oind, ont, _ = o.pia_get()
    assert dnt == ont[0] and dind[:, 0].tolist() == oind[0, :, 0].tolist()
    dom.close()
