"""SWPM collisions (swpm!, collision_swpm.jl:170-288) on the device against the
oracle's restatement on the same draws, and the reference's statistical test
test/test_bkw_varweight_octree_swpm.jl (BKW moments against the analytic
solution, conservation of number density and temperature through SWPM and
octree merging)."""
import math

import numpy as np
import pytest

import merzgpu as mz
from helpers import (assert_close_rows, device_logical, device_state, interactions, oracle_logical, oracle_state,
                     random_particles, species)

pytestmark = pytest.mark.gpu
RTOL = 1e-12
L_GRID = 1e-3


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _ragged(rng, n_cells, npc, wspan):
    """Variable-weight particles; with 4 cells or more, cell 0 is empty, cell 1
    holds one particle and cell 2 two."""
    w, v, x, cell = random_particles(rng, n_cells * npc, n_cells, T=800.0, wspan=wspan, drift=(50.0, 0.0, -20.0),
                                     L=L_GRID)
    keep = np.ones(len(w), bool)
    for c, n in ((0, 0), (1, 1), (2, 2)):
        if n_cells >= 4:
            idx = np.flatnonzero(cell == c)
            keep[idx[n:]] = False
    return w[keep], v[keep], x[keep], cell[keep]


@pytest.mark.parametrize("n_cells,steps,G", [(24, 1, 1.0), (1, 5, 1.5), (16, 3, 0.0)])
def test_swpm_vs_oracle(ctx, orc, n_cells, steps, G):
    """Counts of candidates and accepted collisions exact, indexers exact,
    particles within 1e-12 of each quantity's scale.  Repeated calls on many
    cells sort by position in between, as the reference's 1-D SWPM loop does
    (test/test_1D_couette_varweight_swpm.jl:76-93): swpm! appends at n_total,
    so its group 2 stays contiguous only within one call or on a single cell,
    and new particles take their parent's position but no stored cell."""
    rng = np.random.default_rng(int(G * 10) + n_cells)
    sp = species(["Ar"])
    inter = interactions(sp)
    arrays = _ragged(rng, n_cells, 300, 1.0)
    cap = len(arrays[0]) * 6 + 1024
    o = oracle_state(orc, n_cells, sp, mz.VHS, [arrays], capacity=cap)
    dom = device_state(ctx, n_cells, sp, inter, [arrays], capacity=cap, seed=77)
    sgm = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 800.0, 800.0, 1.0)
    o.cf_set_smax(0, 0, sgm)
    dom.set_sigma_g_w_max(0, 0, sgm)
    wmax = arrays[0].max()
    dt = 50.0 / (0.5 * 300 * 300 * sgm * wmax * (G + 1))  # about 50 candidates per full cell
    accepted = 0
    for step in range(1, steps + 1):
        if step > 1 and n_cells > 1:
            o.sort(0, L=L_GRID, nx=n_cells)
            dom.sort(0, mz.Grid1DUniform(L_GRID, n_cells))
        o.swpm_cells(0, G, dt, None, 77, step)
        dom.swpm(0, G, dt, step)
        accepted += int(o.cf_get(0, 0)[1][:, 3].sum())
    smax, cnt = o.cf_get(0, 0)
    cf = dom.collision_factors(0, 0)
    assert np.array_equal(cf["n_coll"], cnt[:, 2])
    assert np.array_equal(cf["n_coll_performed"], cnt[:, 3])
    assert cnt[:, 3].sum() > 20
    assert_close_rows(cf["sigma_g_w_max"].reshape(-1, 1), smax.reshape(-1, 1), RTOL, "(sigma g)_max")
    ind, nt = dom.indexer(0)
    oind, ont, _ = o.pia_get()
    assert nt == ont[0] == len(arrays[0]) + 2 * accepted
    assert np.array_equal(ind[:, 0], oind[0, :, 0])
    orows, oc = oracle_logical(o, 0)
    drows, dc = device_logical(dom, 0)
    assert np.array_equal(oc, dc)
    assert_close_rows(orows, drows, RTOL, "particles after swpm")
    # weight, momentum and energy are conserved by every collision
    w0 = arrays[0]
    assert np.isclose(drows[:, 0].sum(), w0.sum(), rtol=1e-13)
    p0 = (w0[:, None] * arrays[1]).sum(axis=0)
    p1 = (drows[:, :1] * drows[:, 1:4]).sum(axis=0)
    assert np.allclose(p1, p0, rtol=0, atol=1e-12 * np.abs(w0[:, None] * arrays[1]).sum())
    e0 = (w0 * (arrays[1] ** 2).sum(axis=1)).sum()
    e1 = (drows[:, 0] * (drows[:, 1:4] ** 2).sum(axis=1)).sum()
    assert abs(e1 - e0) <= 1e-12 * e0


def test_collision_factors_swpm_estimate(ctx):
    """test/test_collision_utils_swpm.jl: the SWPM (sigma g)_max estimate is the
    NTC estimate with Fnum = 1."""
    sp = species(["Ar", "He"])
    inter = interactions(sp)
    dom = mz.Domain(ctx, 40, sp, 64, interactions=inter)
    mz.create_collision_factors_swpm_array(dom, inter, sp, [300.0, 600.0], mult_factor=2.0)
    for s1 in range(2):
        for s2 in range(2):
            ref = mz.estimate_sigma_g_w_max(inter[s1][s2], sp[s1], sp[s2], [300.0, 600.0][s1], [300.0, 600.0][s2],
                                            1.0, 2.0)
            got = dom.collision_factors(s1, s2)["sigma_g_w_max"]
            assert np.all(np.abs(got - ref) <= 2 * np.finfo(float).eps * ref)
    dom.close()


def _bkw_analytic(t, magic, N):
    # test/test_bkw_varweight_octree_swpm.jl:26-30
    C = 1.0 - 0.4 * np.exp(-t * magic / 6.0)
    kk = N / 2
    return C ** (kk - 1) * (kk - (kk - 1) * C)


def test_bkw_swpm_octree_moments_and_conservation(ctx):
    """test/test_bkw_varweight_octree_swpm.jl:32-140 on the device: pseudo-
    Maxwell Ar, G = 1, swpm! every step, octree N:2 merging of cells above
    10,000 particles down to 8,000, total moments every step for 500 steps of
    0.025 t_ref.  The reference samples one cell on a velocity grid; here 32
    independent cells of 10,000 BKW-sampled particles each, averaged.  Bounds:
    M4, M6, M8 within 2 %, 7 %, 15 % of the analytic solution; T within 5e-4 K
    and the number density within 1e-11 of their initial values; the particle
    count stays below the threshold."""
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.PSEUDO_MAXWELL)
    n_cells, n0, n_t, G = 32, 10000, 500, 1.0
    threshold, target = 10000, 8000
    T0, n_dens = 273.0, 1e23
    sigma_ref = math.pi * mz.PSEUDO_MAXWELL["Ar,Ar"][0] ** 2
    vref = math.sqrt(2 * mz.K_B * T0 / sp[0].mass)
    tref = 1.0 / (n_dens * sigma_ref) / vref
    kappa_mult = sigma_ref * (inter[0][0].m_r / (2 * mz.K_B * T0)) ** (-0.5) / math.gamma(1.5)
    magic = tref / (1.0 / (4 * math.pi * n_dens * kappa_mult)) / (4 * math.pi)
    Fnum = n_dens / n0
    dom = mz.Domain(ctx, n_cells, sp, n_cells * 4 * n0, interactions=inter, seed=1234)
    dom.sample_cells(0, [n0] * n_cells, T0, Fnum, step=0, distribution=1)
    mz.create_collision_factors_swpm_array(dom, inter, sp, T0)
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    props = mz.PhysProps(dom, moments_list=[4, 6, 8, 10], Tref=T0)
    dt = 0.025 * tref
    rng = mz.PhiloxRNG(1234)
    mz.compute_props_with_total_moments(dom, props)
    r = props.fetch()
    moms = [r["moments"][:, :, 0].mean(axis=1)]
    T_first, n_first = r["T"][:, 0].copy(), r["n"][:, 0].copy()
    for ts in range(1, n_t + 1):
        rng.next_step()
        mz.swpm(rng, dom, (0, n_cells), 0, G, dt)
        dom.merge_octree(0, octree, target, threshold=threshold, step=rng.step)
        mz.compute_props_with_total_moments(dom, props)
        r = props.fetch()
        moms.append(r["moments"][:, :, 0].mean(axis=1))
    moms = np.array(moms)
    assert dom.counters()["accepted"] > n_cells * n_t * 50
    assert np.all(np.abs(r["T"][:, 0] - T_first) < 5e-4)
    assert np.all(np.abs(r["n"][:, 0] / n_first - 1.0) < 1e-11)
    assert np.all(r["np"][:, 0] <= threshold)
    t = np.arange(n_t + 1) * 0.025
    for k, (N, tol) in enumerate(((4, 0.02), (6, 0.07), (8, 0.15))):
        a = _bkw_analytic(t, magic, N)
        rel = np.abs(a - moms[:, k]) / a
        assert np.max(rel) < tol, f"M{N}: worst relative deviation {np.max(rel):.4f}"
