"""Surface sampling of the 1-D walls (SurfProps, convect_particles! with
surf_props) on the device against the oracle's restatement, which is pinned
to test/test_surface_props_1D_uniform.jl.  Counts exact; the other sums
within 1e-12 of the largest magnitude of each quantity (the device adds the
wall hits in a varying order)."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import device_logical, interactions, oracle_logical, oracle_state, random_particles, species

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def as_q(r, s=0):
    """device SurfProps arrays -> (2 elements, 11) in the oracle's order"""
    q = np.zeros((2, 11))
    for e in range(2):
        q[e] = [r["np"][e, s], r["flux_incident"][e, s], r["flux_reflected"][e, s], *r["force"][:, e, s],
                r["normal_pressure"][e, s], *r["shear_pressure"][:, e, s], r["kinetic_energy_flux"][e, s]]
    return q


def assert_surf_close(dev, ref, what):
    assert np.array_equal(dev[:, 0], ref[:, 0]), f"{what}: wall hit counts"
    scale = np.maximum(np.abs(dev).max(axis=0), np.abs(ref).max(axis=0))
    err = np.abs(dev - ref)
    assert np.all(err <= 1e-12 * scale + 1e-300), f"{what}: worst {np.max(err / np.maximum(scale, 1e-300)):.2e}"


@pytest.mark.parametrize("acc", [1.0, 0.0, 0.6])
def test_convect_surface_sums_vs_oracle(ctx, orc, acc):
    sp = species(["Ar"])
    inter = interactions(sp)
    rng = np.random.default_rng(int(acc * 10) + 3)
    nx, L = 20, 5e-4
    arrays = random_particles(rng, 6000, nx, T=600.0, L=L, wspan=1.0, drift=(0.0, 150.0, 0.0))
    o = oracle_state(orc, nx, sp, mz.VHS, [arrays])
    dom = mz.Domain(ctx, nx, sp, 2 * 6000, interactions=inter, seed=21)
    dom.upload(0, *arrays)
    grid = mz.Grid1DUniform(L, nx)
    walls = mz.MaxwellWalls1D(sp, 273.0, 400.0, -300.0, 250.0, acc, acc)
    surf = mz.SurfProps(dom)
    dt = 4e-7  # many particles reach a wall, some twice
    for step in (1, 2, 3):
        mz.convect_particles(mz.PhiloxRNG(21, step), grid, walls, dom, 0, dt, surf_props=surf)
        ref = o.convect_surf(0, L, nx, walls.as_flat_array(), dt, 21, step)
        dev = as_q(surf.fetch())
        assert dev[:, 0].sum() > 100
        assert_surf_close(dev, ref, f"step {step}")
        drows, dc = device_logical(dom, 0)
        orows, oc = oracle_logical(o, 0)
        assert np.allclose(drows, orows, rtol=0, atol=1e-11 * np.abs(orows).max())


def test_fused_step_surface_average_vs_oracle(ctx, orc):
    """Couette steps with surface sampling attached to the fused step: the
    averaged wall sums (avg_props! from step 2 on) equal the oracle loop's."""
    from test_gpu_step import couette_plan, couette_setup

    sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc, nx=40, ppc=100, seed=31)
    inst, avg = mz.SurfProps(dom), mz.SurfProps(dom)
    dom.set_step_surface(inst, avg)
    steps, avg_start = 5, 2
    n_avg = steps - avg_start + 1
    dom.step(couette_plan(grid, walls, dt, avg_start=avg_start, n_avg=n_avg, props=False), steps)
    ref_avg = np.zeros((2, 11))
    ref_last = None
    for t in range(1, steps + 1):
        o.ntc_cells(0, 0, dt, grid.V, seed, t, equal_weight=True)
        ref_last = o.convect_surf(0, grid.L, grid.n_cells, walls.as_flat_array(), dt, seed, t)
        o.sort(0, L=grid.L, nx=grid.n_cells)
        if t >= avg_start:
            ref_avg += ref_last / n_avg
    assert_surf_close(as_q(inst.fetch()), ref_last, "last step")
    da = as_q(avg.fetch())
    assert np.allclose(da[:, 0], ref_avg[:, 0], rtol=1e-14, atol=0)
    assert_surf_close(np.column_stack([ref_avg[:, :1], da[:, 1:]]), ref_avg, "average")
    # the shear on the moving walls pulls along their velocity: -y on the left wall, +y on the right
    assert da[0, 8] * da[1, 8] < 0
