"""test/test_grid_1D_uniform.jl on the device: a 4 m grid of 8 cells filled
with 1,000 particles per cell (Fnum = 1e10 / 1000) and by number density
(1e23 m^-3, Fnum 1e20: 500 per cell), then compute_props! and the
number-density form of compute_props_sorted!.  Counts, number densities and
the agreement of the two props forms are exact as in the reference; the
sampled temperature and mean velocity are checked to 4.5 standard errors of
a Maxwellian sample of that size (the reference's fixed bounds, 7.5 % and
24 m/s, are about 3 and 2.4 standard errors, met by its own random stream)."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import species

pytestmark = pytest.mark.gpu

EPS = np.finfo(float).eps


def bounds(T, mass, n):
    """4.5 standard errors of the sample temperature (relative) and of a mean
    velocity component, for n Maxwellian particles at T."""
    return 4.5 * np.sqrt(2.0 / (3.0 * n)), 4.5 * np.sqrt(mz.K_B * T / mass / n)


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def test_grid_sampling_and_props(ctx):
    grid = mz.Grid1DUniform(4.0, 8)
    assert grid.L == 4.0 and grid.n_cells == 8 and grid.dx == 0.5
    assert np.all(grid.V == 0.5)
    # get_cell (0-based here): test_grid_1D_uniform.jl:97-100
    assert [grid.get_cell(x) for x in (0.001, 0.4, 0.501, 3.999)] == [0, 0, 1, 7]

    sp = species(["Ar"])
    ppc, n_per_cell, T = 1000, 1e10, 500.0
    dom = mz.Domain(ctx, grid.n_cells, sp, 2 * ppc * grid.n_cells, seed=1234)
    dom.set_cell_volumes(grid.V)
    box = [[c * grid.dx, (c + 1) * grid.dx, 0.0, 1.0, 0.0, 1.0] for c in range(grid.n_cells)]
    dom.sample_cells(0, ppc, T, n_per_cell / ppc, step=0, box=box)
    ind, nt = dom.indexer(0)
    assert nt == ppc * grid.n_cells
    assert ind[:, 0].tolist() == [ppc] * 8 and ind[:, 3].tolist() == [ppc] * 8
    p = mz.PhysProps(dom, Tref=1.0)
    mz.compute_props(dom, p)
    r = p.fetch()
    assert r["np"][:, 0].tolist() == [ppc] * 8
    assert np.all(np.abs(r["n"][:, 0] - n_per_cell) < 2 * EPS)
    tb, vb = bounds(T, sp[0].mass, ppc)
    assert np.all(np.abs(r["T"][:, 0] - T) / T < tb)
    assert np.all(np.abs(r["v"][:, :, 0]) < vb)
    pn = mz.PhysProps(dom, Tref=1.0, ndens_not_Np=True)
    mz.compute_props_sorted(dom, pn)
    rn = pn.fetch()
    assert np.all(np.abs(rn["n"][:, 0] - n_per_cell / 0.5) < 2 * EPS)
    assert rn["np"][:, 0].tolist() == [ppc] * 8
    assert np.all(np.abs(rn["T"][:, 0] - r["T"][:, 0]) / r["T"][:, 0] < 2.5 * EPS)
    assert np.all(np.abs(rn["v"] - r["v"]) < 2 * EPS)
    dom.close()

    # filling by number density: 0.5 m^3 cells hold 500 particles each
    dom = mz.Domain(ctx, grid.n_cells, sp, 2 * ppc * grid.n_cells, seed=1234)
    dom.sample_grid_ndens(0, grid, 1e23, T, 1e20, step=0)
    p = mz.PhysProps(dom, Tref=1.0)
    mz.compute_props(dom, p)
    r = p.fetch()
    assert r["np"].sum() == 0.5 * round(1e23 / 1e20) * grid.n_cells
    tb, vb = bounds(T, sp[0].mass, 500)
    assert np.all(np.abs(r["T"][:, 0] - T) / T < tb)
    assert np.all(np.abs(r["v"][:, :, 0]) < vb)
    dom.close()


def test_sampling_with_drift_matches_the_oracle(ctx, orc):
    """The keywords vx0, vy0, vz0 of sample_particles_equal_weight!
    (distributions_and_sampling.jl:477-509, grid_uniform1D.jl:198-219): a
    different offset per cell, one offset for every cell, and the
    number-density form, against the oracle on the same streams (the
    oracle's restatement of the drift is pinned statistically by
    tests/test_oracle_statistics.py)."""
    sp = species(["Ar"])
    n_cells, ppc, T, Fn, seed = 6, 700, 400.0, 1e12, 29
    v0 = np.array([[100.0 * c, -50.0 * c, 3.0 * c] for c in range(n_cells)])
    for per_cell in (True, False):
        dom = mz.Domain(ctx, n_cells, sp, 2 * ppc * n_cells, seed=seed)
        if per_cell:
            dom.sample_cells(0, ppc, T, Fn, step=0, v0=v0)
        else:
            dom.sample_cells(0, ppc, T, Fn, step=0, v0=v0[2])
        o = orc.Oracle(n_cells, 1, [sp[0].mass])
        o.pv_create(0, 2 * ppc * n_cells)
        for c in range(n_cells):
            o.sample_equal_weight(0, c + 1, ppc, T, Fn, seed=seed, step=0, v0=v0[c] if per_cell else v0[2])
        rows, cells = o.logical(0)
        w, v, x, cell = dom.download(0)
        assert np.array_equal(cells - 1, cell)
        drows = np.column_stack([w, v, x])
        scale = np.maximum(np.abs(rows).max(axis=0), np.abs(drows).max(axis=0))
        assert np.all(np.abs(rows - drows) <= 1e-13 * scale), per_cell
        # the offsets are there: mean velocity per cell near v0
        for c in range(n_cells):
            vc = v[cell == c].mean(axis=0)
            assert np.all(np.abs(vc - (v0[c] if per_cell else v0[2])) < 5 * np.sqrt(mz.K_B * T / sp[0].mass / ppc))
        dom.close()
    grid = mz.Grid1DUniform(5e-4, n_cells)
    drift = np.array([250.0, -120.0, 40.0])
    dom = mz.Domain(ctx, n_cells, sp, 4000 * n_cells, seed=seed)
    dom.sample_grid_ndens(0, grid, 1e23, T, grid.dx * 1e23 / 800.5, step=0, v0=drift)
    o = orc.Oracle(n_cells, 1, [sp[0].mass])
    o.pv_create(0, 4000 * n_cells)
    o.sample_grid_ndens(0, grid.L, n_cells, 1e23, T, grid.dx * 1e23 / 800.5, seed=seed, step=0, v0=drift)
    rows, cells = o.logical(0)
    w, v, x, cell = dom.download(0)
    assert np.array_equal(cells - 1, cell)
    drows = np.column_stack([w, v, x])
    scale = np.maximum(np.abs(rows).max(axis=0), np.abs(drows).max(axis=0))
    assert np.all(np.abs(rows - drows) <= 1e-13 * scale)
    dom.close()
