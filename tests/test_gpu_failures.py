"""Failure detection without a GPU fault: the device status word, bad
arguments and storage that runs short.  Every kernel clamps what it cannot
use and raises a status bit; the host turns the bit into MZ_E_STATE at the
entry point's synchronisation, clears it, and the context stays usable.
Storage that a splitting ntc! or the fused variable-weight step outgrows is
grown on the host (the reference's resize!, collision_ntc.jl:241-243) and the
result equals a run that never ran short."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import device_logical, interactions, random_particles, species

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def test_particle_outside_the_grid_is_reported_and_the_context_survives(ctx):
    sp = species(["Ar"])
    rng = np.random.default_rng(1)
    n_cells, L = 10, 1.0
    w, v, x, cell = random_particles(rng, 200, n_cells, L=L)
    x[7, 0] = 1.5 * L  # beyond the last cell
    dom = mz.Domain(ctx, n_cells, sp, 400, interactions=interactions(sp))
    dom.upload(0, w, v, x, cell)
    with pytest.raises(mz.MerzError) as e:
        dom.sort(0, mz.Grid1DUniform(L, n_cells))
    assert e.value.code == mz._lib.MZ_E_STATE and "outside the grid" in str(e.value)
    # clamped into the last cell, nothing lost; the status was cleared, so a
    # call that does not map positions again (a sort by the stored cells) is clean
    _, c2 = device_logical(dom, 0)
    assert c2.size == 200 and c2.max() == n_cells - 1
    dom.sort(0)
    _, c3 = device_logical(dom, 0)
    assert np.array_equal(np.sort(c2), c3)
    dom.close()


def test_sampling_into_an_occupied_cell_is_reported(ctx):
    sp = species(["Ar"])
    dom = mz.Domain(ctx, 3, sp, 1000, interactions=interactions(sp))
    dom.sample_cells(0, [10, 0, 0], 300.0, 1e10)
    with pytest.raises(mz.MerzError) as e:
        dom.sample_cells(0, [5, 0, 0], 300.0, 1e10)
    assert e.value.code == mz._lib.MZ_E_STATE
    dom.sample_cells(0, [0, 4, 0], 300.0, 1e10)  # an empty cell still works
    assert dom.indexer(0)[0][1, 3] == 4
    dom.close()


def test_bad_arguments_are_refused_before_any_launch(ctx):
    sp = species(["Ar"])
    dom = mz.Domain(ctx, 4, sp, 100, interactions=interactions(sp))
    with pytest.raises(mz.MerzError) as e:
        dom.sort(0, mz.Grid1DUniform(1.0, 5))  # grid of another size
    assert e.value.code == mz._lib.MZ_E_ARG
    with pytest.raises(mz.MerzError) as e:
        dom.ntc(3, 0, 1e-3, 1)  # no such species
    assert e.value.code == mz._lib.MZ_E_ARG
    plan = mz._lib.StepPlan()
    plan.dims, plan.collide, plan.equal_weight, plan.props, plan.dt = 7, 1, 1, 1, 1e-3
    with pytest.raises(mz.MerzError):
        dom.step(plan, 1)
    dom.close()


def test_splitting_ntc_outgrowing_its_storage_equals_an_ample_run(ctx):
    """ntc! with splitting in a domain whose storage holds only the initial
    particles: the reservation outgrows it, the host grows the storage and
    the collisions run as in a domain that was large enough."""
    sp = species(["Ar"])
    inter = interactions(sp)
    rng = np.random.default_rng(4)
    n_cells, n = 30, 3000
    arrays = random_particles(rng, n, n_cells, wspan=1.0)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 300.0, 300.0, 1e12)
    runs = []
    for cap in (n, 10 * n):
        dom = mz.Domain(ctx, n_cells, sp, cap, interactions=inter, seed=4)
        dom.upload(0, *arrays)
        dom.set_sigma_g_w_max(0, 0, smax)
        for step in range(1, 4):
            dom.ntc(0, 0, 50.0, step, equal_weight=False)
        runs.append((device_logical(dom, 0), dom.info(0)["capacity"], dom.counters()["splits"]))
        dom.close()
    (a, ca), cap_small, splits = runs[0]
    (b, cb), _, _ = runs[1]
    assert splits > 100 and cap_small > n
    assert np.array_equal(ca, cb) and np.array_equal(a, b)
