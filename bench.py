#!/usr/bin/env python
"""Benchmark: 1-D Couette flow in argon, the batched (fused, graph-replayed)
DSMC step on one GB300.

Workload (the scaled Couette configuration): 50,000 uniform cells over
L = 5e-4 m, 400 particles per cell (2e7 Ar particles), n = 1e23 m^-3,
T0 = T_wall = 273 K, diffuse walls moving at -/+500 m/s, dt = 0.2 / nu
(mean_collision_frequency), VHS Ar.  One step = ntc_equal_weight! ->
convect + wall reflection -> counting sort -> compute_props_sorted! ->
avg_props! (the averaging phase of simulations/1D/couette_benchmarking.jl).
Synthetic, seeded initial state sampled on the device.  The particle state
(2.9 GB) is larger than L2, so no flush is needed between steps.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl merzgpu|reference]
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "merzbild.jl_gb300"))

L_DOMAIN, NDENS, T_WALL, V_WALL = 5e-4, 1e23, 273.0, 500.0
ALG_BYTES = 112  # per particle-step: every particle read once and written once (7 FP64)
# ncu figures of the Couette step's particle kernels at 10,000 cells x 400
# particles (the capture-size rule keeps full-size launches out of ncu):
# DRAM bytes moved per particle by the two-launch step (gather + props, then
# NTC + convection) and by the one-launch step, and the FP64 warp
# instructions per particle of a whole step
DRAM_BYTES_PER_PARTICLE_TWO_LAUNCH = 276.5
DRAM_BYTES_PER_PARTICLE_FUSED = 386.6
FORMS = ("one fused launch", "two launches", "gathering and physics warps side by side")
FP64_WARP_INST_PER_PARTICLE = 0.814


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="merzgpu", choices=["merzgpu", "reference"])
    p.add_argument("--cells", type=int, default=50000)
    p.add_argument("--ppc", type=int, default=400)
    p.add_argument("--plain-steps", type=int, default=5)
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the batched 0-D, variable-weight Couette, serving and largest-request measurements")
    p.add_argument("--only-extra", default=None,
                   choices=["batched_0d", "varweight", "serving", "largest_request", "readme_0d"],
                   help="run one of the extra measurements alone and print its result")
    p.add_argument("--seed", type=int, default=1234)
    p.add_argument("--launches", type=int, default=0, choices=[0, 1, 2, 3],
                   help="1 or 2 kernel launches per step instead of the autotuner's choice (no autotuning; for "
                        "profiling runs)")
    return p.parse_args()


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Barrier:
    """Host barrier across ranks (gloo); a no-op for one process."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def __call__(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload(args):
    return {"workload": "1D Couette, Ar, diffuse walls 273 K at -/+500 m/s, n=1e23 m^-3, dt=0.2/nu, "
                        f"{args.cells} cells x {args.ppc} ppc",
            "cells": args.cells, "ppc": args.ppc, "particles": args.cells * args.ppc,
            "step": "ntc_equal_weight -> convect -> sort -> compute_props_sorted -> avg_props",
            "l2": "inputs larger than L2 (particle state %.1f GB)" % (args.cells * args.ppc * 144 / 1e9)}


def setup_device(mz, ctx, args, seed):
    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    grid = mz.Grid1DUniform(L_DOMAIN, args.cells)
    Fnum = grid.dx * NDENS / args.ppc
    walls = mz.MaxwellWalls1D(sp, T_WALL, T_WALL, -V_WALL, V_WALL, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T_WALL)
    cap = int(args.cells * args.ppc * 1.05) + 1024
    dom = mz.Domain(ctx, args.cells, sp, cap, interactions=inter, seed=seed)
    dom.set_cell_volumes(grid.V)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T_WALL, T_WALL, Fnum)
    dom.set_sigma_g_w_max(0, 0, smax)
    return sp, inter, grid, Fnum, walls, dt, dom, smax


def make_plan(mz, grid, walls, dt, step0, n_avg, graph=True, launches=0):
    plan = mz._lib.StepPlan()
    plan.dims = 1
    plan.collide = 1
    plan.equal_weight = 1
    plan.props = 1
    plan.avg_start = 1
    plan.n_avg = n_avg
    plan.dt = dt
    plan.dw_tol = 1e-16
    plan.step0 = step0
    plan.use_graph = 1 if graph else 0
    plan.launches = launches
    plan.grid = grid.c_struct()
    plan.walls = walls.c_struct()
    return plan


AR_MASS = 66.3e-27                 # data/particles.toml
AR_VHS = (4.11e-10, 0.81, 273.0)   # data/vhs.toml: vhs_d, vhs_o, vhs_Tref


def batched_0d(mz, ctx, seed, steps=20, warmup=2):
    """Batched 0-D relaxation: 65,536 independent Ar cells with seeded
    log-uniform particle counts in [50, 4000], bi-Maxwellian velocities (Tx =
    2000 K, Ty = Tz = 300 K), Fnum = 1e13, V = 1, dt = 1e-6 s; one fused step =
    ntc_equal_weight! + compute_props! for every cell, graph-replayed.  The
    plain form launches ntc! cell by cell, then props, for one step."""
    import numpy as np

    n_cells = 65536
    rng = np.random.default_rng(seed)
    counts = np.floor(np.exp(rng.uniform(np.log(50), np.log(4000), n_cells))).astype(np.int64)
    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    dom = mz.Domain(ctx, n_cells, sp, int(counts.sum()) + 1024, interactions=inter, seed=seed)
    dom.sample_cells(0, counts, [2000.0, 300.0, 300.0], 1e13, step=0)
    Tm = (2000.0 + 300.0 + 300.0) / 3
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], Tm, Tm, 1e13))
    n = int(counts.sum())
    dt = 1e-6
    inst = mz.PhysProps(dom)

    def plan(step0):
        p = mz._lib.StepPlan()
        p.dims, p.collide, p.equal_weight, p.props, p.dt, p.step0, p.use_graph = 0, 1, 1, 1, dt, step0, 1
        return p

    lanes, big = dom.autotune(plan(0), trial_steps=1)
    dom.step(plan(24), warmup, inst)
    warmup += 24
    dom.counters(reset=True)
    ctx.synchronize()
    ctx.timer_start()
    dom.step(plan(warmup), steps, inst)
    ms = ctx.timer_stop()
    cnt = dom.counters(reset=True)
    # plain: whole-domain standalone calls per step (ntc_equal_weight! over
    # every cell, then compute_props!), no graph, no fusion
    plain_steps = 3
    ctx.synchronize()
    t0 = time.perf_counter()
    for k in range(plain_steps):
        dom.ntc(0, 0, dt, warmup + steps + 1 + k, equal_weight=True)
        mz.compute_props(dom, inst)
    ctx.synchronize()
    plain_s = (time.perf_counter() - t0) / plain_steps
    # secondary: one ntc! launch per cell (the reference's call granularity)
    ctx.synchronize()
    t0 = time.perf_counter()
    for c in range(n_cells):
        dom.ntc(0, 0, dt, warmup + steps + plain_steps + 1, cells=(c, c + 1), equal_weight=True)
    mz.compute_props(dom, inst)
    ctx.synchronize()
    per_cell_s = time.perf_counter() - t0
    value = n * steps / (ms / 1e3)
    out = {"workload": "0-D Ar relaxation, 65,536 cells, N log-uniform [50, 4000], bi-Maxwellian 2000/300/300 K",
           "particles": n, "steps": steps, "mapping": {"lanes_per_cell": lanes, "block_per_cell_from": big},
           "value": value, "unit": "particle-steps/s", "ms_per_step": ms / steps,
           "collisions_per_s": cnt["accepted"] / (ms / 1e3),
           "plain_value": n / plain_s, "plain_ms_per_step": 1e3 * plain_s,
           "plain_form": "whole-domain standalone calls per step (ntc over every cell, compute_props), no graph",
           "batched_over_plain": value / (n / plain_s),
           "per_cell_value": n / per_cell_s, "batched_over_per_cell": value / (n / per_cell_s),
           # 0-D step: v and w read (32 B) and v written (24 B) per particle-step
           "hbm_frac_algorithmic": 56.0 * value / (measured_peaks()[0] * 1e9)}
    dom.close()
    return out


def readme_0d(mz, ctx, seed, batch=4096, n_steps=800):
    """The README's 0-D case (README.md:91-106, test_2species.jl): 400 Ar at
    3000 K and 4000 He at 360 K in one cell, Fnum 5e12, V 1, dt 2.5e-3 s, 800
    steps of ntc! for (Ar,Ar), (He,Ar), (He,He) and compute_props!.  Plain:
    one instance, mz_step over its 800 steps (graph-replayed).  Batched:
    `batch` instances with their own random streams as the cells of one
    domain, the same 800 steps.  The oracle runs one instance on one host
    core."""
    import numpy as np

    sp = [mz.Species("Ar", mz.AR_MASS), mz.Species("He", mz.HE_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    T0, N0, Fnum, dt = (3000.0, 360.0), (400, 4000), 5e12, 2.5e-3

    def run(cells):
        dom = mz.Domain(ctx, cells, sp, [N0[0] * cells + 64, N0[1] * cells + 64], interactions=inter, seed=seed)
        for s in range(2):
            dom.sample_cells(s, [N0[s]] * cells, T0[s], Fnum, step=0)
        for s1 in range(2):
            for s2 in range(2):
                dom.set_sigma_g_w_max(s1, s2, mz.estimate_sigma_g_w_max(inter[s1][s2], sp[s1], sp[s2], T0[s1],
                                                                        T0[s2], Fnum))
        inst = mz.PhysProps(dom)
        p = mz._lib.StepPlan()
        p.dims, p.collide, p.equal_weight, p.props, p.dt, p.step0, p.use_graph = 0, 1, 1, 1, dt, 0, 1
        ctx.synchronize()
        dom.counters(reset=True)
        ctx.timer_start()
        dom.step(p, n_steps, inst)
        ms = ctx.timer_stop()
        cnt = dom.counters(reset=True)
        T = inst.fetch()["T"].mean(axis=0)
        dom.close()
        ps = cells * sum(N0) * n_steps
        return {"instances": cells, "value": ps / (ms / 1e3), "unit": "particle-steps/s", "ms_total": ms,
                "ms_per_step": ms / n_steps, "collisions_per_s": cnt["accepted"] / (ms / 1e3),
                "T_final_mean": [float(T[0]), float(T[1])]}

    plain = run(1)
    batched = run(batch)
    # the oracle: one instance on one host core
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    o = oracle.Oracle(1, 2, [s.mass for s in sp])
    t = mz.VHS
    o.load_interactions([[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]],
                        [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]], 273.0)
    for s in range(2):
        o.pv_create(s, N0[s] + 64)
        o.sample_equal_weight(s, 1, N0[s], T0[s], Fnum, seed=seed, step=0)
    o.estimate_sigma_g_w_max(list(T0), Fnum)
    t0 = time.perf_counter()
    for tt in range(1, n_steps + 1):
        for s2 in range(2):
            for s1 in range(s2, 2):
                o.ntc_cells(s1, s2, dt, None, seed, tt, equal_weight=True)
        o.compute_props(mode=0)
    cpu_s = time.perf_counter() - t0
    cpu = {"value": sum(N0) * n_steps / cpu_s, "unit": "particle-steps/s", "cores": 1, "kind": "port",
           "sample": f"one instance, {n_steps} steps"}
    return {"workload": "README 0-D Ar/He relaxation: 400 Ar at 3000 K + 4000 He at 360 K, Fnum 5e12, V 1, "
                        "dt 2.5e-3, 800 steps, ntc! for every pair + compute_props! per step",
            "plain": plain, "batched": batched, "batched_over_plain": batched["value"] / plain["value"],
            "cpu_oracle": cpu}


def varweight_couette(mz, ctx, seed, steps=40, warmup=5):
    """Variable-weight Couette (couette_varweight_octree.jl's loop at the
    configuration's size): 1,000 cells over L = 5e-4 m, Ar at n = 1e23 and
    273 K, 1,000 particles per cell with seeded log-uniform weights over two
    decades, diffuse walls at -/+500 m/s, dt = 0.2 / nu.  One step = ntc! with
    splitting for every cell, octree N:2 merging of the cells above 1,200
    particles down to 300, convection, sort, compute_props_sorted!.  Batched:
    mz_step (device-resident, graph-replayed).  Plain: the same step as
    whole-domain standalone calls; secondary: ntc! and the merge cell by cell
    (the reference's loop)."""
    import numpy as np

    nx, ppc, threshold, target = 1000, 1000, 1200, 300
    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    grid = mz.Grid1DUniform(L_DOMAIN, nx)
    Fnum = grid.dx * NDENS / ppc
    walls = mz.MaxwellWalls1D(sp, T_WALL, T_WALL, -V_WALL, V_WALL, 1.0, 1.0)
    dt = 0.2 / mz.mean_collision_frequency(inter, sp, 0, NDENS, T_WALL)
    rng = np.random.default_rng(seed)
    n0 = nx * ppc
    cell = np.repeat(np.arange(nx, dtype=np.int32), ppc)
    x = rng.random((n0, 3))
    x[:, 0] = (cell + rng.uniform(0.01, 0.99, n0)) * grid.dx
    v = rng.normal(0.0, (mz.K_B * T_WALL / mz.AR_MASS) ** 0.5, (n0, 3))
    w = Fnum * 10.0 ** (2.0 * (rng.random(n0) - 0.5))
    w *= n0 * Fnum / w.sum()
    dom = mz.Domain(ctx, nx, sp, 5_000_000, interactions=inter, seed=seed)
    dom.upload(0, w, v, x, cell)
    dom.set_cell_volumes(grid.V)
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], T_WALL, T_WALL, Fnum))
    octree = mz.OctreeN2Merge(max_Nbins=6000)
    props = mz.PhysProps(dom)

    def plan(step0, k, graph=True):
        p = mz._lib.StepPlan()
        p.dims, p.collide, p.equal_weight, p.props = 1, 1, 0, 1
        p.dt, p.dw_tol, p.step0, p.use_graph = dt, 1e-16, step0, 1 if graph else 0
        p.grid, p.walls = grid.c_struct(), walls.c_struct()
        p.merge_threshold, p.merge_target, p.octree = threshold, target, octree.params
        return p

    def standalone_step(step, per_cell=False):
        if per_cell:
            for c in range(nx):
                dom.ntc(0, 0, dt, step, cells=(c, c + 1), equal_weight=False)
                dom.merge_octree(0, octree, target, threshold=threshold, cells=(c, c + 1), grid=grid, step=step)
        else:
            dom.ntc(0, 0, dt, step, equal_weight=False)
            dom.merge_octree(0, octree, target, threshold=threshold, grid=grid, step=step)
        dom.convect(0, grid, walls, dt, step)
        dom.sort(0, grid)
        mz.compute_props_sorted(dom, props)

    # the mapping (lanes per cell of the splitting NTC) from timed trial steps
    lanes, _ = dom.autotune(plan(0, 1), trial_steps=2)
    tuned = 3 * 2 * 2  # three mappings, two rounds, two steps each
    dom.step(plan(tuned, warmup), warmup, props)
    warmup += tuned
    # per-kernel shares: the same steps with every launch bracketed by events
    # (no graph: a graph's launches are not timed one by one)
    ctx.set_kernel_timing(True)
    dom.step(plan(warmup, steps, graph=False), steps, props)
    ctx.synchronize()
    timings = ctx.kernel_timings()
    ctx.set_kernel_timing(False)
    ctx.synchronize()
    n_start = dom.info(0)["n_total"]
    dom.counters(reset=True)
    ctx.timer_start()
    dom.step(plan(warmup + steps, steps), steps, props)
    ms = ctx.timer_stop()
    cnt = dom.counters(reset=True)
    n_end = dom.info(0)["n_total"]
    live = 0.5 * (n_start + n_end)
    # plain: whole-domain standalone calls, then the per-cell form
    t_plain = warmup + 2 * steps + 1
    ctx.synchronize()
    n_plain = dom.info(0)["n_total"]
    t0 = time.perf_counter()
    for k in range(3):
        standalone_step(t_plain + k)
    ctx.synchronize()
    plain_s = (time.perf_counter() - t0) / 3
    n_pc = dom.info(0)["n_total"]
    t0 = time.perf_counter()
    standalone_step(t_plain + 3, per_cell=True)
    ctx.synchronize()
    per_cell_s = time.perf_counter() - t0
    value = live * steps / (ms / 1e3)
    tot = sum(v[0] for v in timings.values()) or 1.0
    out = {"workload": "1-D Couette, variable weight (2 decades), 1,000 cells x 1,000 initial particles, "
                       "ntc! with splitting + octree merge 1,200 -> 300 + convect + sort + props",
           "mean_live_particles": live, "steps": steps, "value": value, "unit": "particle-steps/s",
           "ms_per_step": ms / steps, "collisions_per_s": cnt["accepted"] / (ms / 1e3),
           "splits_per_step": cnt["splits"] / steps, "merged_cells_per_step": cnt["merges"] / steps,
           "form": "mz_step, device-resident and graph-replayed", "lanes_per_cell": lanes,
           "plain_value": n_plain / plain_s, "plain_ms_per_step": 1e3 * plain_s,
           "plain_form": "whole-domain standalone calls per step (ntc, merge, convect, sort, props)",
           "batched_over_plain": value / (n_plain / plain_s),
           "per_cell_value": n_pc / per_cell_s, "batched_over_per_cell": value / (n_pc / per_cell_s),
           "kernel_share": {k: round(v[0] / tot, 4) for k, v in sorted(timings.items(), key=lambda kv: -kv[1][0])},
           # 1-D step: every live particle read and written once (56 B each way)
           "hbm_frac_algorithmic": 112.0 * value / (measured_peaks()[0] * 1e9)}
    dom.close()
    return out


def serving(mz, ctx, seed, window_s=3.0, rate=200.0, plain_sample=50):
    """Serving loop: seeded Poisson arrivals (mean `rate` per s over `window_s`)
    of 0-D relaxation requests, 70 % Ar and 30 % Ar + He, particles
    log-uniform in [200, 200,000] per species, temperatures uniform in [300,
    5000] K, steps uniform in [50, 2000]; a common number density (Fnum = n V /
    N), dt = 2.5e-3 s.  Requests are admitted by free slots and free device
    memory (the server's storage grows into free HBM, 2 GiB kept free), and
    co-batched per step; p50 / p99 latency from arrival to result.  The plain
    form runs the first `plain_sample` requests one at a time on the same
    GPU."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sp = [mz.Species("Ar", mz.AR_MASS), mz.Species("He", mz.HE_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, int(rate * window_s * 1.5)))
    arrivals = arrivals[arrivals < window_s]
    reqs = []
    for k, t in enumerate(arrivals):
        two = rng.random() < 0.3
        c = [int(np.exp(rng.uniform(np.log(200), np.log(200_000)))),
             int(np.exp(rng.uniform(np.log(200), np.log(200_000)))) if two else 0]
        T = [rng.uniform(300.0, 5000.0), rng.uniform(300.0, 5000.0) if two else 0.0]
        reqs.append((float(t), dict(counts=c, T=T, Fnum=2.2e16 / sum(c), n_steps=int(rng.integers(50, 2001)),
                                    seed=int(seed) * 100_000 + k)))
    srv = mz.Server(ctx, sp, inter, 2.5e-3, 1024, 0)
    lat, ids, elapsed = srv.serve(reqs)
    info = srv.info()
    srv.close()
    lat = np.array(lat)
    # plain: the first requests one at a time (arrival at 0, no overlap)
    one = mz.Server(ctx, sp, inter, 2.5e-3, 1, 0)
    ps = 0
    t0 = time.perf_counter()
    for _, kw in reqs[:plain_sample]:
        one.serve([(0.0, kw)])
        ps += sum(kw["counts"]) * kw["n_steps"]
    plain_s = time.perf_counter() - t0
    one.close()
    return {"workload": f"Poisson {rate:g}/s over {window_s:g} s, {len(reqs)} requests, 70 % Ar / 30 % Ar+He, "
                        "N log-uniform [200, 2e5] per species, T [300, 5000] K, steps [50, 2000]",
            "requests": len(reqs), "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "value": info["particle_steps"] / elapsed,
            "unit": "particle-steps/s", "elapsed_s": elapsed, "server_steps": info["steps"],
            "admission": "free slots and free device memory (cudaMemGetInfo less 2 GiB)",
            "plain_value": ps / plain_s, "plain_sample": f"first {plain_sample} requests one at a time",
            "batched_over_plain": (info["particle_steps"] / elapsed) / (ps / plain_s)}


def largest_request(mz, ctx, seed, steps=20, warmup=3):
    """The step of the serving mix's largest request alone: one 0-D Ar cell of
    200,000 particles at 3000 K (Fnum = 2.2e16 / N, V = 1, dt = 2.5e-3),
    collided block-per-cell (k_ntc_big) without per-step props, as the server
    runs it.  Its candidate loop is sequential in batches, so this step time
    is the floor of a serving step while the request runs."""
    import numpy as np

    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    n = 200_000
    Fnum = 2.2e16 / n
    dom = mz.Domain(ctx, 1, sp, n + 1024, interactions=inter, seed=seed)
    dom.sample_cells(0, np.array([n], dtype=np.int64), [3000.0, 3000.0, 3000.0], Fnum, step=0)
    dom.set_sigma_g_w_max(0, 0, mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 3000.0, 3000.0, Fnum))
    p = mz._lib.StepPlan()
    p.dims, p.collide, p.equal_weight, p.props, p.dt, p.step0, p.use_graph = 0, 1, 1, 0, 2.5e-3, 0, 0
    p.big_cell = 2048
    dom.step(p, warmup)
    dom.counters(reset=True)
    ctx.synchronize()
    ctx.timer_start()
    p.step0 = warmup
    dom.step(p, steps)
    ms = ctx.timer_stop()
    cnt = dom.counters(reset=True)
    dom.close()
    return {"workload": "one 0-D Ar cell, 200,000 particles, 3000 K, dt 2.5e-3, block-per-cell NTC, no per-step props",
            "steps": steps, "ms_per_step": ms / steps, "value": n * steps / (ms / 1e3), "unit": "particle-steps/s",
            "candidates_per_step": cnt["candidates"] / steps, "accepted_per_step": cnt["accepted"] / steps}


def cpu_oracle_run(args, steps, time_budget=None, nthreads=None, warmup=0):
    """The oracle (C++ restatement of the reference path) on the host cores:
    the same workload, `warmup` untimed steps, then `steps` timed steps (or
    until time_budget seconds).  Uses nothing from the GPU package."""
    import math

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    nthreads = nthreads or os.cpu_count() or 1
    g = oracle.grid(L_DOMAIN, args.cells)
    Fnum = g["dx"] * NDENS / args.ppc
    d, om, tr = AR_VHS
    # mean_collision_frequency (collisional_props.jl:42-47)
    nu = 4.0 * d * d * NDENS * math.sqrt(math.pi * 1.380649e-23 * tr / AR_MASS) * (T_WALL / tr) ** (1.0 - om)
    dt = 0.2 / nu
    walls = [T_WALL, T_WALL, 0.0, -V_WALL, 0.0, 0.0, V_WALL, 0.0, 1.0, 1.0]
    V = [g["dx"]] * args.cells
    o = oracle.Oracle(args.cells, 1, [AR_MASS])
    o.load_interactions(d, om, tr)
    o.pv_create(0, int(args.cells * args.ppc * 1.05) + 1024)
    o.sample_grid_ndens(0, L_DOMAIN, args.cells, NDENS, T_WALL, Fnum, seed=args.seed, step=0)
    o.cf_set_smax(0, 0, o.estimate_single(0, 0, T_WALL, T_WALL, Fnum))
    _, nt, _ = o.pia_get()
    n = int(nt[0])
    for t in range(1, warmup + 1):
        o.ntc_cells(0, 0, dt, V, args.seed, t, equal_weight=True, nthreads=nthreads)
        o.convect(0, L_DOMAIN, args.cells, walls, dt, args.seed, t, nthreads=nthreads)
        o.sort(0, L=L_DOMAIN, nx=args.cells)
        o.compute_props(mode=2, nthreads=nthreads)
    done = 0
    t0 = time.perf_counter()
    for t in range(warmup + 1, warmup + steps + 1):
        o.ntc_cells(0, 0, dt, V, args.seed, t, equal_weight=True, nthreads=nthreads)
        o.convect(0, L_DOMAIN, args.cells, walls, dt, args.seed, t, nthreads=nthreads)
        o.sort(0, L=L_DOMAIN, nx=args.cells)
        o.compute_props(mode=2, nthreads=nthreads)
        done += 1
        if time_budget and time.perf_counter() - t0 > time_budget:
            break
    el = time.perf_counter() - t0
    return {"value": done * n / el, "unit": "particle-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{done} full steps of the same workload ({args.cells} cells, {n} particles), "
                      "C++ oracle restating the reference path, OpenMP over cells",
            "seconds": el, "steps": done}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # a bounded sample: at most the first W steps as warm-up and the timed
    # steps until 60 s have passed, so the run ends within a few minutes
    steps = max(1, args.steps)
    r = cpu_oracle_run(args, steps, time_budget=60.0, warmup=min(args.warmup, 3))
    out = {"impl": "reference", "metric": "particle-steps/s", "value": r["value"], "unit": "particle-steps/s",
           "n_gpus": args.gpus, "device": "host cores (no GPU used)", "steps": r["steps"], "warmup": args.warmup,
           "ms_per_step": 1e3 * r["seconds"] / r["steps"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload(args),
           "cpu_baseline": {"value": r["value"], "unit": r["unit"], "cores": r["cores"], "kind": r["kind"],
                            "sample": r["sample"]},
           "e2e": {"value": r["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "note": "reference Julia path unavailable here (no Julia toolchain); timed: the oracle's C++ "
                   "restatement of the reference algorithm on the host cores"}
    print(json.dumps(out), flush=True)


def run_gpu(args):
    rank, world, local = dist_env()
    import numpy as np

    import merzgpu as mz
    from merzgpu import build as b

    b.build()
    log("library ready")
    barrier = Barrier(world)
    ctx = mz.Context(local)
    seed = args.seed + 7919 * rank  # independent replicas
    if args.only_extra:
        fn = {"batched_0d": batched_0d, "varweight": varweight_couette, "serving": serving,
              "largest_request": largest_request, "readme_0d": readme_0d}[args.only_extra]
        print(json.dumps({args.only_extra: fn(mz, ctx, seed)}), flush=True)
        ctx.close()
        return
    sp, inter, grid, Fnum, walls, dt, dom, smax = setup_device(mz, ctx, args, seed)
    log("domain created")
    dom.sample_grid_ndens(0, grid, NDENS, T_WALL, Fnum, step=0)
    n = dom.info(0)["n_total"]
    log(f"sampled {n} particles")
    inst = mz.PhysProps(dom)
    avg = mz.PhysProps(dom)
    K, W = args.steps, args.warmup
    # the autotuner times each mapping (lanes per cell x the three launch
    # forms: one fused launch, two launches, gathering and physics warps side
    # by side) on real steps, two rounds of 8 steps each before the warm-up,
    # then W untimed warm-up steps
    if args.launches:
        # a fixed mapping: the default lanes per cell and the launches asked for
        tune_steps = 0
        mapping = (8 if args.cells >= 4096 else (16 if args.cells >= 1024 else 32), args.launches - 1)
    else:
        tune_steps = 18 * 8
        mapping = dom.autotune(make_plan(mz, grid, walls, dt, 0, K), trial_steps=8)
    dom.step(make_plan(mz, grid, walls, dt, tune_steps, K, launches=args.launches), W, inst, avg)
    ctx.synchronize()
    log(f"warm-up done (mapping: {mapping[0]} lanes per cell, launch form {FORMS[mapping[1]]})")
    mz.clear_props(avg)
    dom.counters(reset=True)
    step0 = tune_steps + W
    plan = make_plan(mz, grid, walls, dt, step0, K, launches=args.launches)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launch_count()
    barrier()
    ctx.synchronize()
    ctx.timer_start()
    dom.step(plan, K, inst, avg)
    ms = ctx.timer_stop()
    ctx.synchronize()
    barrier()
    launches = ctx.launch_count() - launches0
    log(f"timed {K} steps: {ms:.3f} ms")
    clk = clocks.stop()
    cnt = dom.counters(reset=True)
    t_max = barrier.max(ms / 1e3)
    total_ps = barrier.sum(float(n) * K)
    value = total_ps / t_max
    coll = barrier.sum(float(cnt["accepted"])) / t_max
    cand = barrier.sum(float(cnt["candidates"])) / t_max

    # per-kernel CUDA-event timing (direct launches, same stream) for the roofline
    log("kernel timing pass")
    ctx.set_kernel_timing(True)
    kt_steps = max(3, min(K, 6))
    dom.step(make_plan(mz, grid, walls, dt, step0 + K, kt_steps, graph=False, launches=args.launches), kt_steps,
             inst, avg)
    timings = ctx.kernel_timings()
    ctx.set_kernel_timing(False)
    tot = sum(v[0] for v in timings.values())
    # the step's particle kernel: one fused launch, or (when the autotuner
    # chose two launches per step) the gather + props launch and the NTC +
    # convection launch together, each launched once per step
    two = "step_cell" not in timings and "step_cell_final" in timings and "step_cell_inplace" in timings
    if two:
        kname = "step_cell_final+step_cell_inplace"
        avg_launch_s = sum(timings[k][0] / timings[k][1] for k in ("step_cell_final", "step_cell_inplace")) / 1e3
    else:
        kname = "step_cell" if "step_cell" in timings else max(timings.items(), key=lambda kv: kv[1][0])[0]
        kms, klaunch = timings[kname]
        avg_launch_s = kms / klaunch / 1e3
    peak, peak_kind = measured_peaks()
    achieved = ALG_BYTES * n / avg_launch_s / 1e9
    # DRAM bytes per particle of the step's particle kernel(s), measured with
    # ncu (dram__bytes_read.sum + dram__bytes_write.sum) on the same step at
    # 10,000 cells x 400 particles; traffic scales with the particles a launch
    # moves, so it is scaled to this launch's particle count
    traffic = None
    if two:
        traffic = DRAM_BYTES_PER_PARTICLE_TWO_LAUNCH * n
    elif mapping[1] == 0:
        traffic = DRAM_BYTES_PER_PARTICLE_FUSED * n
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": ALG_BYTES * n,
                "kernel_share": {k: v[0] / tot for k, v in sorted(timings.items(), key=lambda kv: -kv[1][0])}}
    # secondary bound: the FP64 pipe.  GB300 spends 16 SM cycles on every FP64
    # warp instruction (2 DFMA per SM per clock); the step's FP64 warp
    # instructions per particle (collisions, convection, both props passes)
    # were counted with ncu on the full-step kernel, so their pipe time at the
    # clock seen during the timed region is a floor
    ck = clk if isinstance(clk, dict) else {}
    sm_hz = 1e6 * (ck.get("sm_mhz") or ck.get("sm_max_mhz") or 2070.0)
    import torch

    n_sms = torch.cuda.get_device_properties(local).multi_processor_count
    floor_s = FP64_WARP_INST_PER_PARTICLE * n * 16.0 / (n_sms * sm_hz)
    roofline["secondary"] = {
        "bound": "fp64", "fp64_warp_inst_per_particle": FP64_WARP_INST_PER_PARTICLE,
        "pipe_cycles_per_warp_inst": 16, "sm_mhz": sm_hz / 1e6, "floor_ms_per_step": floor_s * 1e3,
        "frac": floor_s / (ms / K / 1e3),
        "source": "ncu instruction counts of the full-step kernel at 10,000 cells x 400 particles"}

    # plain form: the same step as whole-domain standalone entry points, one
    # call each per step with no graph and no fusion (ntc_equal_weight! over
    # every cell, convect_particles!, sort_particles!, compute_props_sorted!);
    # secondary: the reference's call granularity, one ntc! call per cell
    plain = None
    log("roofline: " + json.dumps({k: (v if not isinstance(v, dict) else None) for k, v in roofline.items()}))
    if not args.no_plain and rank == 0:
        rng = mz.PhiloxRNG(seed, step0 + K + kt_steps)
        pp = mz.PhysProps(dom)
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.plain_steps):
            rng.next_step()
            dom.ntc(0, 0, dt, rng.step, equal_weight=True)
            mz.convect_particles(rng, grid, walls, dom, 0, dt)
            mz.sort_particles(dom, 0, grid)
            mz.compute_props_sorted(dom, pp)
        ctx.synchronize()
        el = time.perf_counter() - t0
        pv = n * args.plain_steps / el
        rng.next_step()
        ctx.synchronize()
        t0 = time.perf_counter()
        for c in range(args.cells):
            mz.ntc_equal_weight(rng, dom, c, 0, dt)
        mz.convect_particles(rng, grid, walls, dom, 0, dt)
        mz.sort_particles(dom, 0, grid)
        mz.compute_props_sorted(dom, pp)
        ctx.synchronize()
        el1 = time.perf_counter() - t0
        plain = {"value": pv, "unit": "particle-steps/s", "steps": args.plain_steps,
                 "ms_per_step": 1e3 * el / args.plain_steps, "launches_per_step": 7,
                 "form": "whole-domain standalone entry points per step (ntc, convect, sort, props), no graph",
                 "batched_over_plain": value / world / pv,
                 "per_cell": {"value": n / el1, "ms_per_step": 1e3 * el1, "launches_per_step": args.cells + 6,
                              "form": "one ntc! call per cell (the reference's call granularity), then "
                                      "convect, sort, props",
                              "batched_over_per_cell": value / world / (n / el1)}}

    # end to end through the C ABI with host buffers: upload the initial state,
    # K steps, read the cell properties back every step
    e2e = None
    log(f"plain: {plain}")
    if not args.no_e2e:
        # the initial state in page-locked host memory (prepared outside the
        # timed region), uploaded inside it; every step's cell properties
        # come back to the host through double-buffered asynchronous
        # snapshots, each read on the host two steps later
        w, v, x, cell = dom.download(0)
        hw, hv = mz.PinnedArray(ctx, w.shape), mz.PinnedArray(ctx, v.shape)
        hx, hc = mz.PinnedArray(ctx, x.shape), mz.PinnedArray(ctx, cell.shape, np.int32)
        hw.array[:], hv.array[:], hx.array[:], hc.array[:] = w, v, x, cell
        m = grid.n_cells * len(sp)
        snaps = [mz.PinnedArray(ctx, 6 * m), mz.PinnedArray(ctx, 6 * m)]
        ctx.synchronize()
        barrier()
        t0 = time.perf_counter()
        dom.upload(0, hw.array, hv.array, hx.array, hc.array)
        d2h, seen = 0, 0.0
        for k in range(K):
            dom.step(make_plan(mz, grid, walls, dt, 1000 + k, 1, launches=args.launches), 1, inst, None)
            slot = k % 2
            if k >= 2:
                inst.snapshot_wait(slot)
                seen += float(snaps[slot].array[:m].sum())  # particles counted by the step k - 2
            inst.snapshot(slot, snaps[slot])
            d2h += snaps[slot].array.nbytes
        for k in range(max(0, K - 2), K):
            inst.snapshot_wait(k % 2)
            seen += float(snaps[k % 2].array[:m].sum())
        ctx.synchronize()
        el = barrier.max(time.perf_counter() - t0)
        h2d = w.nbytes + v.nbytes + x.nbytes + cell.nbytes
        assert abs(seen - float(n) * K) < 0.5, (seen, n * K)  # every step's read-back holds all particles
        e2e = {"value": barrier.sum(float(n) * K) / el, "unit": "particle-steps/s",
               "h2d_bytes_per_step": int(h2d / K), "d2h_bytes_per_step": int(d2h / K),
               "note": f"initial state uploaded once from page-locked memory ({h2d} B) inside the timed region, "
                       f"amortised over {K} steps; every step's cell properties (np, n, v, T) read back to the "
                       "host through asynchronous double-buffered snapshots that overlap the next step"}
        for a in (hw, hv, hx, hc, *snaps):
            a.close()

    extra_0d = extra_srv = extra_vw = extra_big = extra_readme = None
    log(f"e2e: {e2e}")
    if not args.no_extra and rank == 0:
        extra_0d = batched_0d(mz, ctx, seed)
        log(f"batched 0-D: {extra_0d}")
        extra_vw = varweight_couette(mz, ctx, seed)
        log(f"variable-weight Couette: {extra_vw}")
        extra_srv = serving(mz, ctx, seed)
        log(f"serving: {extra_srv}")
        extra_big = largest_request(mz, ctx, seed)
        log(f"largest request: {extra_big}")
        extra_readme = readme_0d(mz, ctx, seed)
        log(f"README 0-D: {extra_readme}")

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        r = cpu_oracle_run(args, 20, time_budget=15.0)
        cpu = {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        out = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
               "steps": K, "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, sampled on the device)",
               "config": workload(args),
               "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
               "mapping": {"lanes_per_cell": mapping[0], "launch_form": FORMS[mapping[1]],
                           "autotune_steps": tune_steps},
               "collisions_per_s": coll, "candidates_per_s": cand,
               "hbm_frac_algorithmic": ALG_BYTES * value / world / (peak * 1e9),
               "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
               "plain": plain, "batched_0d": extra_0d, "varweight_couette": extra_vw, "serving": extra_srv,
               "largest_request": extra_big, "readme_0d": extra_readme}
        print(json.dumps(out), flush=True)
    ctx.close()


def main():
    import faulthandler

    faulthandler.enable()
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
