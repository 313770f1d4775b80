"""N:2 octree merging on the device (mz_merge_octree_n2) against the oracle's
restatement of merge_octree_N2_based! and against the reference's
known-answer vectors (test/test_octree_merging.jl).

Particle counts, indexer groups and the bin structure are compared exactly;
the merged particles' weights, velocities and positions within 1e-12 of the
column scale (the moments are FMA-contracted sums on both sides)."""
import numpy as np
import pytest

import merzgpu as mz
from conftest import scenario
from helpers import EPS, assert_close_rows, device_logical, oracle_logical, oracle_state, species

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _golden_device(ctx, parts, indexer=None, seed=1234):
    parts = np.asarray(parts, float)
    n = parts.shape[0]
    dom = mz.Domain(ctx, 1, species(["Ar"]), n + 64, seed=seed)
    if indexer is None:
        dom.upload(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7], np.zeros(n, np.int32))
    else:
        n_local, s1, e1, n1, s2, e2, n2 = indexer
        dom.upload_indexed(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7],
                           [[n_local, s1 - 1, e1 - 1, n1, s2 - 1, e2 - 1, n2]])
    return dom


def _golden_oracle(orc, parts, indexer=None):
    parts = np.asarray(parts, float)
    n = parts.shape[0]
    o = orc.Oracle(1, 1, [mz.AR_MASS])
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = o.pia_get()
    ind[0, 0] = indexer if indexer is not None else [n, 1, n, n, 0, -1, 0]
    nt[0] = n
    o.pia_set(ind, nt, cg)
    return o


def _props(dom):
    p = mz.PhysProps(dom)
    mz.compute_props(dom, p)
    return p.fetch()


def test_merge_known_answers_on_device(ctx, orc, golden):
    """test/test_octree_merging.jl:129-290: merge 24 -> 16 -> 2, zero weights,
    two groups, a two-particle cell; conserved n, v, T."""
    sc = scenario(golden, "octree_merge_24")
    octc = mz.OctreeN2Merge(init_bin_bounds=mz.OctreeInitBinC)
    dom = _golden_device(ctx, sc["particles24"])
    r0 = _props(dom)
    assert r0["n"][0, 0] == 108.0
    assert dom.merge_octree(0, octc, 16, step=0) == 1
    _, nt = dom.indexer(0)
    assert nt == 16 and dom.info(0)["n_total"] == 16
    r = _props(dom)
    assert r["np"][0, 0] == 16
    assert abs(r["n"][0, 0] - r0["n"][0, 0]) < EPS
    assert abs(r["T"][0, 0] - r0["T"][0, 0]) < 1e-14
    assert np.max(np.abs(r["v"][:, 0, 0] - r0["v"][:, 0, 0])) < 1e-14
    # the same merge in the oracle, same stream
    o = _golden_oracle(orc, sc["particles24"])
    oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
    o.merge_octree(oc, 0, 1, 16, seed=1234, step=0)
    assert oc.summary()["Nbins"] == 8
    assert_close_rows(oracle_logical(o, 0)[0], device_logical(dom, 0)[0], RTOL, "merge 24 -> 16")

    dom.merge_octree(0, octc, 2, step=1)
    rows, _ = device_logical(dom, 0)
    assert rows.shape[0] == 2 and rows[0, 0] == 54.0 and rows[1, 0] == 54.0
    r = _props(dom)
    assert abs(r["n"][0, 0] - r0["n"][0, 0]) < EPS
    assert abs(r["T"][0, 0] - r0["T"][0, 0]) < 1e-14
    assert np.max(np.abs(r["v"][:, 0, 0] - r0["v"][:, 0, 0])) < 1e-14
    o.merge_octree(oc, 0, 1, 2, seed=1234, step=1)
    assert_close_rows(oracle_logical(o, 0)[0], rows, RTOL, "merge 16 -> 2")

    for key in ("zero_weight_last", "zero_weight_two_groups"):
        z = sc[key]
        dom = _golden_device(ctx, z["particles"], indexer=z.get("indexer"), seed=99)
        r0 = _props(dom)
        dom.merge_octree(0, octc, z["target"], step=0)
        ind, nt = dom.indexer(0)
        assert nt == z["expect_n_total"]
        r = _props(dom)
        assert r["np"][0, 0] == nt
        assert abs(r["n"][0, 0] - r0["n"][0, 0]) < EPS
        assert abs(r["T"][0, 0] - r0["T"][0, 0]) < 1e-14
        assert np.max(np.abs(r["v"][:, 0, 0] - r0["v"][:, 0, 0])) < 1e-14
        rows, _ = device_logical(dom, 0)
        assert np.all(rows[:, 0] > 0) and not np.any(np.isnan(rows[:, 4]))
        if key == "zero_weight_last":
            assert ind[0, 6] == 0 and ind[0, 3] == nt
        else:
            assert ind[0, 3] > 0 and ind[0, 6] > 0
        o = _golden_oracle(orc, z["particles"], z.get("indexer"))
        o.merge_octree(oc, 0, 1, z["target"], seed=99, step=0)
        assert_close_rows(oracle_logical(o, 0)[0], rows, RTOL, key)
        oind, _, _ = o.pia_get()
        assert [ind[0, 3], ind[0, 6]] == [oind[0, 0, 3], oind[0, 0, 6]]

    t = sc["two_particles"]
    dom = _golden_device(ctx, t["particles"])
    dom.merge_octree(0, octc, t["target"])
    rows, _ = device_logical(dom, 0)
    assert_close_rows(np.asarray(t["particles"], float), rows, 0.0, "two particles kept")


def _random_cells(rng, n_cells, nmax, wspan):
    counts = np.floor(np.exp(rng.uniform(np.log(1), np.log(nmax), n_cells))).astype(int)
    counts[rng.integers(0, n_cells, 2)] = 0
    cells = np.repeat(np.arange(n_cells), counts).astype(np.int32)
    n = cells.size
    w = 1e12 * 10.0 ** (wspan * (2 * rng.random(n) - 1))
    v = rng.normal(0.0, 300.0, (n, 3)) + rng.normal(0.0, 50.0, (n_cells, 3))[cells]
    L = 1e-3
    x = rng.random((n, 3))
    x[:, 0] = (cells + rng.uniform(0.0, 1.0, n)) * (L / n_cells)
    return (w, v, x, cells), L


CASES = [
    # init bounds, bound rule, max_Nbins, max_depth, target, threshold, grid
    (mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit, 4096, 10, 40, 60, False),
    (mz.OctreeInitBinMinMaxVelSym, mz.OctreeBinBoundsRecompute, 4096, 10, 100, -1, True),
    (mz.OctreeInitBinC, mz.OctreeBinBoundsInherit, 24, 10, 300, 20, True),
    (mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsRecompute, 4096, 2, 300, 16, False),
]



@pytest.mark.parametrize("weights", ["beyond_fp32", "equal"])
def test_merge_bin_choice_on_exact_weights_vs_oracle(ctx, orc, weights):
    """Bins chosen on exact weights: weights beyond the FP32 range (each
    split sums its octants exactly at once) and equal weights (octants of
    equal counts tie, so the contenders' exact sums decide), in cells of up
    to 1,500 particles whose first splits run on every warp of the block."""
    rng = np.random.default_rng(7 if weights == "equal" else 8)
    n_cells = 24
    (w, v, x, cells), L = _random_cells(rng, n_cells, 1500, 1.0)
    if weights == "equal":
        w = np.full(w.size, 1e12)
    else:
        w = 10.0 ** (35.0 + 10.0 * rng.random(w.size))
    arrays = (w, v, x, cells)
    init, bounds, max_bins, max_depth, target, threshold = (mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit,
                                                            4096, 10, 60, 100)
    sp = species(["Ar"])
    o = oracle_state(orc, n_cells, sp, mz.VHS, [arrays])
    dom = mz.Domain(ctx, n_cells, sp, w.size + 64, seed=77)
    dom.upload(0, *arrays)
    octree = mz.OctreeN2Merge(init_bin_bounds=init, bin_bounds_compute=bounds, max_Nbins=max_bins,
                              max_depth=max_depth)
    merged = dom.merge_octree(0, octree, target, threshold=threshold, step=5)
    oc = orc.Octree(orc.SPLIT_MID, init, bounds, max_bins, max_depth)
    counts = np.bincount(cells, minlength=n_cells)
    expect = 0
    for c in range(n_cells):
        if counts[c] <= threshold:
            continue
        o.merge_octree(oc, 0, c + 1, target, seed=77, step=5)
        expect += 1
    assert merged == expect and expect > 5 and counts.max() > 1000
    orows, ocells = oracle_logical(o, 0)
    drows, dcells = device_logical(dom, 0)
    assert np.array_equal(ocells, dcells)
    assert_close_rows(orows, drows, RTOL, "merged cells")
    oind, ont, _ = o.pia_get()
    ind, nt = dom.indexer(0)
    assert nt == ont[0] == dom.info(0)["n_total"]
    assert np.array_equal(ind[:, 3], oind[0, :, 3]) and np.array_equal(ind[:, 6], oind[0, :, 6])


@pytest.mark.parametrize("init,bounds,max_bins,max_depth,target,threshold,grid", CASES)
def test_merge_cells_vs_oracle(ctx, orc, init, bounds, max_bins, max_depth, target, threshold, grid):
    """Cells of 0..1500 variable-weight particles merged in one launch against
    the oracle merging the same cells one by one with the same streams."""
    rng = np.random.default_rng(1000 + max_bins + target)
    n_cells = 48
    arrays, L = _random_cells(rng, n_cells, 1500, 1.0)
    sp = species(["Ar"])
    o = oracle_state(orc, n_cells, sp, mz.VHS, [arrays])
    dom = mz.Domain(ctx, n_cells, sp, arrays[0].size + 64, seed=77)
    dom.upload(0, *arrays)
    octree = mz.OctreeN2Merge(init_bin_bounds=init, bin_bounds_compute=bounds, max_Nbins=max_bins,
                              max_depth=max_depth)
    g = mz.Grid1DUniform(L, n_cells) if grid else None
    merged = dom.merge_octree(0, octree, target, threshold=threshold, grid=g, step=5)
    oc = orc.Octree(orc.SPLIT_MID, init, bounds, max_bins, max_depth)
    counts = np.bincount(arrays[3], minlength=n_cells)
    expect = 0
    for c in range(n_cells):
        if counts[c] == 0 or (threshold >= 0 and counts[c] <= threshold):
            continue
        o.merge_octree(oc, 0, c + 1, target, L=L if grid else None, nx=n_cells, seed=77, step=5)
        expect += 1
    assert merged == expect
    orows, ocells = oracle_logical(o, 0)
    drows, dcells = device_logical(dom, 0)
    assert np.array_equal(ocells, dcells)
    assert_close_rows(orows, drows, RTOL, "merged cells")
    oind, ont, _ = o.pia_get()
    ind, nt = dom.indexer(0)
    assert nt == ont[0] == dom.info(0)["n_total"]
    assert np.array_equal(ind[:, 3], oind[0, :, 3]) and np.array_equal(ind[:, 6], oind[0, :, 6])
    if grid:
        # clamped positions stay on the grid: the merged state (with dead
        # slots) sorts like any other
        dom.sort(0, g)
        assert dom.info(0)["n_total"] == nt
        assert dom.info(0)["high_water"] == nt


def test_merge_1d_keeps_particles_in_the_grid(ctx, orc):
    """test/test_octree_merging_1D.jl: 4 particles in each of 2 unit-grid cells
    placed so that mean(x) -/+ std(x) leaves the domain; merged to 2 per cell
    without the grid some land outside, with the grid none does, and the
    device matches the oracle's merge with the same streams."""
    x1, x2 = [0.05, 0.05, 0.05, 0.45], [0.55, 0.95, 0.85, 0.99]
    parts = np.array([[2.0, 0.5, -3.0, 4.0, x, 0.0, 0.0] for x in x1] +
                     [[3.0, 0.5, -3.0, 4.0, x, 0.0, 0.0] for x in x2])
    cells = np.array([0, 0, 0, 0, 1, 1, 1, 1], np.int32)
    g = mz.Grid1DUniform(1.0, 2)
    for with_grid in (False, True):
        dom = mz.Domain(ctx, 2, species(["Ar"]), 64, seed=1234)
        dom.upload(0, parts[:, 0], parts[:, 1:4], parts[:, 4:7], cells)
        octree = mz.OctreeN2Merge(init_bin_bounds=mz.OctreeInitBinC)
        merged = dom.merge_octree(0, octree, 2, threshold=-1, grid=g if with_grid else None, step=0)
        assert merged == 2
        ind, nt = dom.indexer(0)
        assert nt == 4 and ind[:, 3].tolist() == [2, 2]
        drows, dcells = device_logical(dom, 0)
        for c in (0, 1):
            x = drows[dcells == c, 4]
            assert bool(np.any((x < 0.0) | (x > 1.0))) == (not with_grid), (with_grid, c, x)
        o = orc.Oracle(2, 1, [mz.AR_MASS])
        o.set_particles_simple(0, cells + 1, parts)
        oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
        for c in (1, 2):
            o.merge_octree(oc, 0, c, 2, L=1.0 if with_grid else None, nx=2, seed=1234, step=0)
        orows, ocells = oracle_logical(o, 0)
        assert np.array_equal(ocells, dcells)
        assert_close_rows(orows, drows, RTOL, "1-D merge")
        if with_grid:
            dom.sort(0, g)
            p = _props(dom)
            assert p["np"][:, 0].tolist() == [2, 2]
            assert p["n"][:, 0].tolist() == [8.0, 12.0]
        dom.close()
