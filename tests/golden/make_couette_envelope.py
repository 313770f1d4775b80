"""Ensemble of oracle runs of the 1-D Couette configuration at its base size,
the reference envelope that tests/test_gpu_couette_envelope.py holds the
device's runs against.

Configuration (simulations/1D/couette_benchmarking.jl:58-85 with the sizes of
the benchmark's Couette case): argon, L = 5e-4 m, 2,000 uniform cells, 200
particles per cell sampled at n = 1e23 m^-3 and 273 K, diffuse walls at 273 K
moving at -500 / +500 m/s, dt = 0.2 / nu (nu the mean collision frequency,
collisional_props.jl:42-47), 20,000 steps of ntc_equal_weight! ->
convect_particles! -> sort_particles! -> compute_props_sorted!, time averages
(avg_props!) over the last 10,000 steps.

Each run has its own seed (RUN_SEED0 + r).  The fixture keeps, per run, the
time-averaged y velocity and temperature averaged over blocks of BLOCK
consecutive cells, and the ensemble mean of both per cell.

Usage: python tests/golden/make_couette_envelope.py [runs] [workers]
(about 20 minutes per run on one core)."""
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "merzbild.jl_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

NX, PPC, L, NDENS, T_WALL, V_WALL = 2000, 200, 5e-4, 1e23, 273.0, 500.0
N_STEPS, AVG_FROM = 20_000, 10_001
BLOCK = 50
RUN_SEED0 = 9000
OUT = os.path.join(HERE, "couette_c3_envelope.json")


def config():
    import merzgpu as mz

    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    grid = mz.Grid1DUniform(L, NX)
    Fnum = grid.dx * NDENS / PPC
    walls = mz.MaxwellWalls1D(sp, T_WALL, T_WALL, -V_WALL, V_WALL, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T_WALL)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T_WALL, T_WALL, Fnum)
    return sp, grid, Fnum, walls, dt, smax


def one_run(r):
    import merzgpu as mz
    import oracle

    sp, grid, Fnum, walls, dt, smax = config()
    seed = RUN_SEED0 + r
    o = oracle.Oracle(NX, 1, [sp[0].mass])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    o.pv_create(0, 3 * PPC * NX)
    o.sample_grid_ndens(0, L, NX, NDENS, T_WALL, Fnum, seed=seed, step=0)
    o.cf_set_smax(0, 0, smax)
    n_avg = N_STEPS - AVG_FROM + 1
    inv = 1.0 / n_avg
    vy, T = np.zeros(NX), np.zeros(NX)
    t0 = time.time()
    for step in range(1, N_STEPS + 1):
        o.ntc_cells(0, 0, dt, grid.V, seed, step, equal_weight=True)
        o.convect(0, L, NX, walls.as_flat_array(), dt, seed, step)
        o.sort(0, L=L, nx=NX)
        if step >= AVG_FROM:
            pr = o.compute_props(mode=2)
            vy += pr["v"][0, :, 1] * inv
            T += pr["T"][0] * inv
    print(f"run {r} (seed {seed}) done in {time.time() - t0:.0f} s", flush=True)
    return vy, T


def main():
    import oracle

    runs = int(sys.argv[1]) if len(sys.argv) > 1 else 16
    workers = int(sys.argv[2]) if len(sys.argv) > 2 else min(runs, os.cpu_count() or 1)
    oracle.build()
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(one_run, range(runs))
    vy = np.array([a for a, _ in res])
    T = np.array([b for _, b in res])
    nb = NX // BLOCK
    out = {
        "config": {"cells": NX, "ppc": PPC, "L": L, "ndens": NDENS, "T_wall": T_WALL, "v_wall": V_WALL,
                   "steps": N_STEPS, "avg_from": AVG_FROM, "block": BLOCK, "run_seed0": RUN_SEED0,
                   "runs": runs},
        "block_vy": [[float("%.10g" % x) for x in row] for row in vy.reshape(runs, nb, BLOCK).mean(axis=2)],
        "block_T": [[float("%.10g" % x) for x in row] for row in T.reshape(runs, nb, BLOCK).mean(axis=2)],
        "cell_mean_vy": [float("%.8g" % x) for x in vy.mean(axis=0)],
        "cell_mean_T": [float("%.8g" % x) for x in T.mean(axis=0)],
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
