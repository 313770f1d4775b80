"""The Couette case of test/test_1D_couette.jl (50 cells over 5e-4 m, Ar at
5e22 m^-3, diffuse walls at 300 K moving at -/+500 m/s, 1,000 particles per
cell, dt 2.59e-9 s, 50,000 steps) run through the fused device step with
averaging from step 14,001 and wall sampling, against the SPARTA solution of
the same case that ships with the reference's tests
(tests/golden/sparta_couette.json, made by tests/golden/make_sparta_couette.py).
Both are single stochastic runs; the bounds are a few times the statistical
scatter of the time averages."""
import json
import os

import numpy as np
import pytest

import merzgpu as mz
from helpers import interactions, species

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sparta_couette.json")


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def couette(ctx):
    ref = json.load(open(GOLDEN))
    st = ref["setup"]
    sp = species(["Ar"])
    inter = interactions(sp)
    nx, ppc, n, T, vw, dt = st["n_cells"], st["ppc"], st["nrho"], st["T_wall"], st["v_wall"], st["dt"]
    grid = mz.Grid1DUniform(st["L"], nx)
    Fnum = grid.dx * n / ppc
    walls = mz.MaxwellWalls1D(sp, T, T, -vw, vw, 1.0, 1.0)
    dom = mz.Domain(ctx, nx, sp, 3 * ppc * nx, interactions=inter, seed=2024)
    dom.set_cell_volumes(grid.V)
    dom.sample_grid_ndens(0, grid, n, T, Fnum, step=0)
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T, T, Fnum))
    avg = mz.PhysProps(dom)
    s_inst, s_avg = mz.SurfProps(dom), mz.SurfProps(dom)
    dom.set_step_surface(s_inst, s_avg)
    n_steps, avg_from = st["n_steps"], st["avg_from"]
    plan = mz._lib.StepPlan()
    plan.dims, plan.collide, plan.equal_weight, plan.props = 1, 1, 1, 1
    plan.avg_start, plan.n_avg, plan.dt, plan.dw_tol = avg_from, n_steps - avg_from + 1, dt, 1e-16
    plan.step0, plan.use_graph = 0, 1
    plan.grid, plan.walls = grid.c_struct(), walls.c_struct()
    dom.step(plan, n_steps, None, avg)
    # the gas shear stress P_xy = sum m w (vx - ux)(vy - uy) / V of the final
    # state, averaged over the cells
    w, v, x, cell = dom.download(0)
    pxy = []
    for c in range(nx):
        sel = cell == c
        ww, vv = w[sel], v[sel]
        u = (ww[:, None] * vv).sum(axis=0) / ww.sum()
        pxy.append(sp[0].mass * (ww * (vv[:, 0] - u[0]) * (vv[:, 1] - u[1])).sum() / grid.dx)
    out = {"props": avg.fetch(), "surf": s_avg.fetch(), "V": grid.dx, "ref": ref, "pxy": float(np.mean(pxy))}
    dom.close()
    return out


def test_cell_profiles_match_sparta(couette):
    ref = np.array(couette["ref"]["cells"])  # temp, press, n, nrho, u, v
    p = couette["props"]
    T = p["T"][:, 0]
    nrho = p["n"][:, 0] / couette["V"]
    vy = p["v"][1, :, 0]
    vx = p["v"][0, :, 0]
    dT = np.abs(T / ref[:, 0] - 1.0)
    dn = np.abs(nrho / ref[:, 3] - 1.0)
    dv = np.abs(vy - ref[:, 5])
    assert dT.max() < 0.015, f"temperature: worst relative difference {dT.max():.4f} (mean {dT.mean():.4f})"
    assert dn.max() < 0.015, f"number density: worst relative difference {dn.max():.4f} (mean {dn.mean():.4f})"
    assert dv.max() < 8.0, f"y velocity: worst difference {dv.max():.2f} m/s (mean {dv.mean():.2f})"
    assert np.abs(vx).max() < 5.0
    # the profiles' shapes: hottest in the middle, densest at the walls, v_y antisymmetric
    assert T.argmax() in range(20, 30) and nrho.argmin() in range(20, 30)
    assert abs(vy[0] + vy[-1]) < 8.0 and vy[0] < -400.0


def test_wall_quantities(couette):
    """Normal pressure against SPARTA's; the wall shear equal on both walls and
    equal to the gas shear stress P_xy (steady-state momentum balance; SPARTA's
    boundary shear output is 20 % above both while the velocity profiles agree
    within 1 m/s, so it is not compared); the net kinetic energy flux into each
    wall (heat in minus the wall's work, a small residual of two large terms in
    steady state) below 1 % of the work, like SPARTA's (63 W/m^2 of 33 kW/m^2)."""
    ref = np.array(couette["ref"]["walls"])  # nflux, mflux, press, shx, shy, shz, ke
    s = couette["surf"]
    pn = np.abs(s["normal_pressure"][:, 0])
    shy = s["shear_pressure"][1, :, 0]
    ke = s["kinetic_energy_flux"][:, 0]
    msg = f"pn {pn}, shear_y {shy}, ke {ke}, gas P_xy {couette['pxy']:.2f}, SPARTA {ref[:, [2, 4, 6]].tolist()}"
    assert np.all(np.abs(pn / ref[:, 2] - 1.0) < 0.02), msg
    assert abs(abs(shy[0]) / abs(shy[1]) - 1.0) < 0.02, msg
    assert abs(abs(shy[0]) / abs(couette["pxy"]) - 1.0) < 0.1, msg
    work = np.abs(shy) * couette["ref"]["setup"]["v_wall"]
    assert np.all(np.abs(ke) < 0.01 * work), msg
    assert np.all(np.abs(ref[:, 6]) < 0.01 * np.abs(ref[:, 4]) * couette["ref"]["setup"]["v_wall"])
    # incident and reflected mass fluxes balance at steady state
    fi, fr = s["flux_incident"][:, 0], s["flux_reflected"][:, 0]
    assert np.all(np.abs(fi / np.abs(fr) - 1.0) < 0.01), (fi, fr)
