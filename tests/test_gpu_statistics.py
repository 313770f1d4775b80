"""Statistical checks of the device path against analytic solutions and
against ensembles of the oracle (the reference's own statistical tests,
test/test_bkw.jl and test/test_2species.jl, plus an ensemble comparison).

The device and the oracle draw from independent streams here (different
seeds), so these are comparisons of distributions, not replays."""
import math

import numpy as np
import pytest

import merzgpu as mz
from helpers import species

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _bkw_analytic(t, magic, N):
    # test/test_bkw.jl:22-26
    C = 1.0 - 0.4 * np.exp(-t * magic / 6.0)
    kk = N / 2
    return C ** (kk - 1) * (kk - (kk - 1) * C)


def test_bkw_moments_follow_the_analytic_solution(ctx):
    """test/test_bkw.jl:31-128 on the device: pseudo-Maxwell Ar, 20,000
    particles sampled from the BKW distribution, ntc! + total moments every
    step for 500 steps of 0.025 t_ref; M4, M6, M8 within 5 %, 5.5 %, 15 % of the
    analytic BKW solution.  Eight independent cells, averaged."""
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.PSEUDO_MAXWELL)
    n_cells, n_particles, n_t = 8, 20000, 500
    T0, n_dens = 273.0, 1e23
    d_ref = mz.PSEUDO_MAXWELL["Ar,Ar"][0]
    sigma_ref = math.pi * d_ref ** 2
    vref = math.sqrt(2 * mz.K_B * T0 / sp[0].mass)
    tref = 1.0 / (n_dens * sigma_ref) / vref
    kappa_mult = sigma_ref * (inter[0][0].m_r / (2 * mz.K_B * T0)) ** (-0.5) / math.gamma(1.5)
    magic = tref / (1.0 / (4 * math.pi * n_dens * kappa_mult)) / (4 * math.pi)
    Fnum = n_dens / n_particles
    dom = mz.Domain(ctx, n_cells, sp, n_cells * n_particles + 64, interactions=inter, seed=4321)
    dom.sample_cells(0, [n_particles] * n_cells, T0, Fnum, step=0, distribution=1)
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T0, T0, Fnum))
    props = mz.PhysProps(dom, moments_list=[4, 6, 8, 10], Tref=T0)
    dt = 0.025 * tref
    mz.compute_props_with_total_moments(dom, props)
    moms = [props.fetch()["moments"][:, :, 0].mean(axis=1)]
    for ts in range(1, n_t + 1):
        dom.ntc(0, 0, dt, ts)
        mz.compute_props_with_total_moments(dom, props)
        r = props.fetch()
        assert np.all(r["np"][:, 0] == n_particles)
        moms.append(r["moments"][:, :, 0].mean(axis=1))
    moms = np.array(moms)
    t = np.arange(n_t + 1) * 0.025
    for k, (N, tol) in enumerate(((4, 0.05), (6, 0.055), (8, 0.15))):
        a = _bkw_analytic(t, magic, N)
        rel = np.abs(a - moms[:, k]) / a
        assert np.max(rel) < tol, f"M{N}: worst relative deviation {np.max(rel):.4f}"


def _relax_plan(dt, step0):
    plan = mz._lib.StepPlan()
    plan.dims = 0
    plan.collide = 1
    plan.equal_weight = 1
    plan.props = 1
    plan.dt = dt
    plan.step0 = step0
    plan.use_graph = 1
    return plan


CHECK = (25, 50, 100, 200, 400, 800)


def _oracle_relaxation(orc, n_cells, seed, dt):
    """The README two-species case (README.md:91-106) in the oracle: ntc! for
    (Ar,Ar), (He,Ar), (He,He), props at the check steps."""
    t = mz.VHS
    o = orc.Oracle(n_cells, 2, [mz.AR_MASS, mz.HE_MASS])
    o.load_interactions([[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]],
                        [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]], 273.0)
    for s, (n, T0) in enumerate(((400, 3000.0), (4000, 360.0))):
        o.pv_create(s, n * n_cells + 64)
        for c in range(n_cells):
            o.sample_equal_weight(s, c + 1, n, T0, 5e12, seed=seed, step=0)
    o.estimate_sigma_g_w_max([3000.0, 360.0], 5e12)
    out = {}
    for tt in range(1, CHECK[-1] + 1):
        for s2 in range(2):
            for s1 in range(s2, 2):
                o.ntc_cells(s1, s2, dt, None, seed, tt, equal_weight=True, nthreads=8)
        if tt in CHECK:
            out[tt] = o.compute_props(mode=0)["T"].copy()  # (species, cells)
    return out


def test_two_species_relaxation_ensemble_matches_the_oracle(ctx, orc):
    """test/test_2species.jl: Ar 400 at 3000 K + He 4000 at 360 K relax to
    600 K.  64 device instances (one fused graph step per time step) against 48
    oracle instances with other seeds: mean T of each species at every check
    step within 3 combined standard errors, and both within 12 % of 600 K at
    step 800."""
    sp = species(["Ar", "He"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    n_dev, dt = 64, 2.5e-3
    dom = mz.Domain(ctx, n_dev, sp, 4000 * n_dev + 64, interactions=inter, seed=2024)
    dom.sample_cells(0, [400] * n_dev, 3000.0, 5e12, step=0)
    dom.sample_cells(1, [4000] * n_dev, 360.0, 5e12, step=0)
    for s1 in range(2):
        for s2 in range(2):
            T1, T2 = (3000.0, 360.0)[s1], (3000.0, 360.0)[s2]
            dom.set_sigma_g_w_max(s1, s2, mz.estimate_sigma_g_w_max(inter[s1][s2], sp[s1], sp[s2], T1, T2, 5e12))
    inst = mz.PhysProps(dom)
    dev = {}
    done = 0
    for tt in CHECK:
        dom.step(_relax_plan(dt, done), tt - done, inst)
        done = tt
        dev[tt] = inst.fetch()["T"].T.copy()  # (species, cells)
    ora = _oracle_relaxation(orc, 48, 99, dt)
    for tt in CHECK:
        for s in range(2):
            a, b = dev[tt][s], ora[tt][s]
            se = math.sqrt(a.var(ddof=1) / a.size + b.var(ddof=1) / b.size)
            assert abs(a.mean() - b.mean()) <= 3 * se, (tt, s, a.mean(), b.mean(), se)
    for s in range(2):
        assert abs(dev[800][s].mean() - 600.0) / 600.0 < 0.12


def test_couette_profiles_ensemble_matches_the_oracle(ctx, orc):
    """Couette flow (simulations/1D/couette_benchmarking.jl:58-85 at a small
    size): time-averaged velocity and temperature profiles of 16 device runs
    (the fused graph step with avg_props!) against 16 oracle runs of the
    reference loop, other seeds; per cell and quantity z = difference of the
    ensemble means over its standard error, sum of z^2 below the chi-square
    99.9 % quantile."""
    scipy_stats = pytest.importorskip("scipy.stats")
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    nx, ppc, L, ndens, T = 20, 200, 5e-4, 1e23, 273.0
    n_steps, avg_from, runs = 400, 201, 16
    grid = mz.Grid1DUniform(L, nx)
    Fnum = grid.dx * ndens / ppc
    walls = mz.MaxwellWalls1D(sp, T, T, -500.0, 500.0, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, ndens, T)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T, T, Fnum)
    n_avg = n_steps - avg_from + 1

    dev_v, dev_T = [], []
    for r in range(runs):
        dom = mz.Domain(ctx, nx, sp, 3 * ppc * nx, interactions=inter, seed=500 + r)
        dom.set_cell_volumes(grid.V)
        dom.sample_grid_ndens(0, grid, ndens, T, Fnum, step=0)
        dom.set_sigma_g_w_max(0, 0, smax)
        plan = mz._lib.StepPlan()
        plan.dims, plan.collide, plan.equal_weight, plan.props = 1, 1, 1, 1
        plan.avg_start, plan.n_avg, plan.dt, plan.dw_tol = avg_from, n_avg, dt, 1e-16
        plan.step0, plan.use_graph = 0, 1
        plan.grid, plan.walls = grid.c_struct(), walls.c_struct()
        avg = mz.PhysProps(dom)
        dom.step(plan, n_steps, None, avg)
        a = avg.fetch()
        dev_v.append(a["v"][1, :, 0].copy())
        dev_T.append(a["T"][:, 0].copy())
        dom.close()

    ora_v, ora_T = [], []
    for r in range(runs):
        seed = 900 + r
        o = orc.Oracle(nx, 1, [sp[0].mass])
        o.load_interactions(*mz.VHS["Ar,Ar"])
        o.pv_create(0, 3 * ppc * nx)
        o.sample_grid_ndens(0, L, nx, ndens, T, Fnum, seed=seed, step=0)
        o.cf_set_smax(0, 0, smax)
        sv, sT = np.zeros(nx), np.zeros(nx)
        for step in range(1, n_steps + 1):
            o.ntc_cells(0, 0, dt, grid.V, seed, step, equal_weight=True)
            o.convect(0, L, nx, walls.as_flat_array(), dt, seed, step)
            o.sort(0, L=L, nx=nx)
            if step >= avg_from:
                pr = o.compute_props(mode=2)
                sv += pr["v"][0, :, 1] / n_avg
                sT += pr["T"][0] / n_avg
        ora_v.append(sv)
        ora_T.append(sT)

    chi2 = 0.0
    for dev, ora in ((np.array(dev_v), np.array(ora_v)), (np.array(dev_T), np.array(ora_T))):
        se = np.sqrt(dev.var(axis=0, ddof=1) / runs + ora.var(axis=0, ddof=1) / runs)
        chi2 += float(np.sum(((dev.mean(axis=0) - ora.mean(axis=0)) / se) ** 2))
    limit = scipy_stats.chi2.ppf(0.999, 2 * nx)
    assert chi2 < limit, f"chi2 {chi2:.1f} over {2 * nx} cells x quantities, limit {limit:.1f}"
    # the profiles are Couette profiles: the averaged velocity runs from the
    # left wall's -500 m/s towards the right wall's +500 m/s
    vmean = np.array(dev_v).mean(axis=0)
    assert vmean[0] < -100.0 and vmean[-1] > 100.0 and np.all(np.diff(vmean) > -30.0)
