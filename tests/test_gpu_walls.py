"""Wall reflection on the device after test/test_convection_1D.jl:75-212:
10,000 particles driven into a diffuse wall (left at 2000 K moving at 1100
m/s, right at 500 K moving at -820 m/s), into a cold wall with accommodation
0.2 (80 % specular), and variable-weight particles into specular walls.

Exact as in the reference: every reflected velocity points away from the
wall, the cell weights, and the specular cases.  The mean tangential
velocities are checked to 4.5 standard errors of the wall's Maxwellian
(sqrt(kT/m) / sqrt(N)) and the specular count to 4.5 binomial standard
errors; the reference's fixed bounds (2.25e-3 relative, 3 m/s, 100
particles) sit at 0.4 to 2.5 standard errors and are met by its own random
stream."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import species

pytestmark = pytest.mark.gpu

N = 10_000


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _run(ctx, w, v, x, walls, dt, step):
    sp = species(["Ar"])
    grid = mz.Grid1DUniform(50.0, 100)
    dom = mz.Domain(ctx, grid.n_cells, sp, 2 * N, seed=1234)
    cells = np.array([grid.get_cell(xx) for xx in x[:, 0]], np.int32)
    dom.upload(0, w, v, x, cells)
    dom.convect(0, grid, mz.MaxwellWalls1D(sp, *walls), dt, step)
    dom.sort(0, grid)
    wd, vd, xd, cd = dom.download(0)
    p = mz.PhysProps(dom, Tref=1.0)
    mz.compute_props(dom, p)
    r = p.fetch()
    dom.close()
    return vd, r, sp[0].mass


def _sigma_mean(T, mass):
    return np.sqrt(mz.K_B * T / mass / N)


def test_diffuse_walls(ctx):
    n = 1e10
    w = np.full(N, n / N)
    # left wall: 2000 K, moving at 1100 m/s
    v = np.tile([-1000.0, 0.0, 0.0], (N, 1))
    x = np.tile([0.999e-4, 0.0, 0.0], (N, 1))
    vd, r, m = _run(ctx, w, v, x, (2000.0, 500.0, 1100.0, -820.0, 1.0, 1.0), 1e-7, 1)
    assert np.all(vd[:, 0] >= 0.0)
    assert abs(r["n"][0, 0] - n) < np.finfo(float).eps
    s = _sigma_mean(2000.0, m)
    assert abs(r["v"][1, 0, 0] - 1100.0) < 4.5 * s, (r["v"][:, 0, 0], s)
    assert abs(r["v"][2, 0, 0]) < 4.5 * s
    # right wall: 500 K, moving at -820 m/s
    v = np.tile([1000.0, 0.0, 0.0], (N, 1))
    x = np.tile([50.0 - 0.999e-4, 0.0, 0.0], (N, 1))
    vd, r, m = _run(ctx, w, v, x, (2000.0, 500.0, 1100.0, -820.0, 1.0, 1.0), 1e-7, 2)
    assert np.all(vd[:, 0] <= 0.0)
    assert abs(r["n"][99, 0] - n) < np.finfo(float).eps
    s = _sigma_mean(500.0, m)
    assert abs(r["v"][1, 99, 0] + 820.0) < 4.5 * s, (r["v"][:, 99, 0], s)
    assert abs(r["v"][2, 99, 0]) < 4.5 * s


def test_partially_accommodating_cold_wall(ctx):
    w = np.full(N, 1e6)
    v = np.tile([-1000.0, 0.0, 0.0], (N, 1))
    x = np.tile([0.999e-4, 0.0, 0.0], (N, 1))
    vd, r, m = _run(ctx, w, v, x, (10.0, 10.0, 1100.0, -820.0, 0.2, 1.0), 1e-7, 3)
    assert np.all(vd[:, 0] >= 0.0)
    nspecular = int(np.sum(np.abs(vd[:, 0] - 1000.0) < 2 * np.finfo(float).eps))
    assert abs(nspecular - 0.8 * N) < 4.5 * np.sqrt(N * 0.8 * 0.2), nspecular


def test_variable_weight_specular_walls(ctx):
    i = np.arange(1, N + 1)
    even = i % 2 == 0
    w = np.where(even, 2.0, 1.0)
    v = np.zeros((N, 3))
    v[:, 0] = np.where(even, 2.0, -1.0)
    x = np.tile([1e-4, 0.0, 0.0], (N, 1))
    vd, r, m = _run(ctx, w, v, x, (1.0, 1.0, 0.0, 0.0, 0.0, 0.0), 0.5, 4)
    assert np.all(vd[:, 0] >= 0.0)
    assert abs(r["n"][0, 0] - N / 2) < np.finfo(float).eps
    assert abs(r["n"][2, 0] - 2 * N / 2) < np.finfo(float).eps
