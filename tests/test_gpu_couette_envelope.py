"""The 1-D Couette configuration at its base size against an ensemble of
oracle runs (the reference envelope, tests/golden/couette_c3_envelope.json,
made by tests/golden/make_couette_envelope.py): 2,000 cells x 200 Ar
particles, n = 1e23 m^-3, diffuse walls at 273 K and -/+500 m/s, dt = 0.2 /
nu, 20,000 steps of the fused graph-replayed step, time averages over the last
10,000 (simulations/1D/couette_benchmarking.jl:58-85).

16 device runs with seeds other than the oracle's.  Per block of 50 cells and
quantity (y velocity, temperature), the difference of the two ensemble means
over its standard error follows Student's t with Welch's degrees of freedom;
mapped to a standard normal, the sum of squares over the 80 blocks x
quantities must stay below its chi-square 99.9 % quantile, and no block may
lie more than 4.5 standard errors out (3-sigma agreement of every block holds
with probability ~0.7 for 80 blocks; 4.5 keeps the false-alarm rate near
1e-3).  The profiles are Couette profiles: y velocity from about -V_wall
towards +V_wall, heated in the middle."""
import json
import os

import numpy as np
import pytest

import merzgpu as mz
from helpers import species

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "couette_c3_envelope.json")


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _device_run(ctx, cfg, seed):
    sp = species(["Ar"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    nx, ppc = cfg["cells"], cfg["ppc"]
    grid = mz.Grid1DUniform(cfg["L"], nx)
    Fnum = grid.dx * cfg["ndens"] / ppc
    walls = mz.MaxwellWalls1D(sp, cfg["T_wall"], cfg["T_wall"], -cfg["v_wall"], cfg["v_wall"], 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, cfg["ndens"], cfg["T_wall"])
    dom = mz.Domain(ctx, nx, sp, 3 * ppc * nx, interactions=inter, seed=seed)
    dom.set_cell_volumes(grid.V)
    dom.sample_grid_ndens(0, grid, cfg["ndens"], cfg["T_wall"], Fnum, step=0)
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], cfg["T_wall"],
                                                          cfg["T_wall"], Fnum))
    plan = mz._lib.StepPlan()
    plan.dims, plan.collide, plan.equal_weight, plan.props = 1, 1, 1, 1
    plan.avg_start, plan.n_avg = cfg["avg_from"], cfg["steps"] - cfg["avg_from"] + 1
    plan.dt, plan.dw_tol, plan.step0, plan.use_graph = dt, 1e-16, 0, 1
    plan.grid, plan.walls = grid.c_struct(), walls.c_struct()
    avg = mz.PhysProps(dom)
    dom.step(plan, cfg["steps"], None, avg)
    a = avg.fetch()
    dom.close()
    return a["v"][1, :, 0].copy(), a["T"][:, 0].copy()


def test_couette_profiles_lie_in_the_oracle_envelope(ctx):
    stats = pytest.importorskip("scipy.stats")
    with open(FIXTURE) as f:
        env = json.load(f)
    cfg = env["config"]
    runs, block = 16, cfg["block"]
    nb = cfg["cells"] // block
    dev_vy, dev_T = [], []
    for r in range(runs):
        vy, T = _device_run(ctx, cfg, 31_000 + r)
        dev_vy.append(vy.reshape(nb, block).mean(axis=1))
        dev_T.append(T.reshape(nb, block).mean(axis=1))
    u_sq, worst = 0.0, 0.0
    for dev, ora in ((np.array(dev_vy), np.array(env["block_vy"])), (np.array(dev_T), np.array(env["block_T"]))):
        n1, n2 = dev.shape[0], ora.shape[0]
        v1, v2 = dev.var(axis=0, ddof=1) / n1, ora.var(axis=0, ddof=1) / n2
        se = np.sqrt(v1 + v2)
        t = (dev.mean(axis=0) - ora.mean(axis=0)) / se
        dof = (v1 + v2) ** 2 / (v1 ** 2 / (n1 - 1) + v2 ** 2 / (n2 - 1))
        z = stats.norm.ppf(stats.t.cdf(t, dof))
        u_sq += float(np.sum(z ** 2))
        worst = max(worst, float(np.max(np.abs(t))))
    limit = stats.chi2.ppf(0.999, 2 * nb)
    assert u_sq < limit, f"sum of squared block deviations {u_sq:.1f} over {2 * nb}, limit {limit:.1f}"
    assert worst < 4.5, f"a block lies {worst:.2f} standard errors from the oracle ensemble"
    vmean = np.array(dev_vy).mean(axis=0)
    Tmean = np.array(dev_T).mean(axis=0)
    assert vmean[0] < -200.0 and vmean[-1] > 200.0 and np.all(np.diff(vmean) > 0)
    assert Tmean[nb // 2] > Tmean[0] and Tmean[nb // 2] > Tmean[-1]
