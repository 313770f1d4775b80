"""The continuous-batching server (mz_server_*): a request's result is the same
alone and in a mix of requests of other sizes arriving at other times, and it
equals the oracle running the same problem (the README relaxation loop) with
the same streams."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import species

pytestmark = pytest.mark.gpu

DT = 2.5e-3


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def _server(ctx, max_requests=16, capacity=200_000):
    sp = species(["Ar", "He"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    return mz.Server(ctx, sp, inter, DT, max_requests, capacity)


REQUESTS = [
    # counts (Ar, He), temperatures, steps, seed
    ((400, 4000), (3000.0, 360.0), 40, 11),
    ((1500, 0), (800.0, 0.0), 25, 12),
    ((250, 600), (5000.0, 300.0), 60, 13),
    ((6000, 0), (300.0, 0.0), 10, 14),
    ((90, 3000), (1200.0, 2500.0), 33, 15),
    ((3000, 3000), (450.0, 4400.0), 20, 16),
]


def _fnum(counts):
    # a common number density across requests: Fnum = n V / N
    return 2.2e16 / max(1, sum(counts))


def _run(server, reqs, stagger=False, max_steps=1):
    """Submit (all at once, or one every few calls) and step until done."""
    ids = {}
    pending = list(reqs)
    k = 0
    while pending or any(server.result(i)["state"] != mz._lib.MZ_REQ_DONE for i in ids.values()):
        if pending and (not stagger or k % 3 == 0):
            c, T, n, seed = pending.pop(0)
            ids[seed] = server.submit(c, T, _fnum(c), n, seed)
        server.step(max_steps)
        k += 1
        assert k < 10_000
    return {seed: server.result(i) for seed, i in ids.items()}


def test_results_alone_equal_results_in_the_mix(ctx):
    alone = {}
    for r in REQUESTS:
        sv = _server(ctx)
        alone.update(_run(sv, [r]))
        sv.close()
    sv = _server(ctx, max_requests=4, capacity=16_000)  # queueing and storage reuse
    mixed = _run(sv, REQUESTS, stagger=True)
    for seed, a in alone.items():
        m = mixed[seed]
        assert a["state"] == m["state"] == mz._lib.MZ_REQ_DONE
        assert a["steps_done"] == m["steps_done"]
        for key in ("np", "n", "T"):
            assert a[key] == m[key], (seed, key)
        assert a["v"] == m["v"], seed
    sv.close()


def test_multi_step_calls_give_the_same_results(ctx):
    """mz_server_step_many: up to 7 steps per call (never past a running
    request's end; admissions between calls) gives every request the results
    of single steps."""
    sv = _server(ctx, max_requests=4, capacity=16_000)
    single = _run(sv, REQUESTS, stagger=True)
    sv.close()
    sv = _server(ctx, max_requests=4, capacity=16_000)
    many = _run(sv, REQUESTS, stagger=True, max_steps=7)
    sv.close()
    for seed, a in single.items():
        m = many[seed]
        assert m["state"] == mz._lib.MZ_REQ_DONE and a["steps_done"] == m["steps_done"]
        for key in ("np", "n", "T", "v"):
            assert a[key] == m[key], (seed, key)


def test_served_request_matches_the_oracle(ctx, orc):
    """Request seed s occupies a cell with stream keys (s, stream id 0, its own
    step count): the oracle's one-cell run with seed s replays it."""
    counts, T, n_steps, seed = REQUESTS[0]
    sv = _server(ctx)
    res = _run(sv, REQUESTS[:3], stagger=True)[seed]
    sv.close()
    t = mz.VHS
    o = orc.Oracle(1, 2, [mz.AR_MASS, mz.HE_MASS])
    o.load_interactions([[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]],
                        [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]], 273.0)
    F = _fnum(counts)
    for s in range(2):
        o.pv_create(s, counts[s] + 64)
        o.sample_equal_weight(s, 1, counts[s], T[s], F, seed=seed, step=0)
    o.estimate_sigma_g_w_max(list(T), F)
    for tt in range(1, n_steps + 1):
        for s2 in range(2):
            for s1 in range(s2, 2):
                o.ntc_cells(s1, s2, DT, None, seed, tt, equal_weight=True)
    ref = o.compute_props(mode=0)
    for s in range(2):
        assert res["np"][s] == ref["np"][s, 0]
        assert abs(res["n"][s] - ref["n"][s, 0]) <= 1e-12 * ref["n"][s, 0]
        assert abs(res["T"][s] - ref["T"][s, 0]) <= 1e-11 * ref["T"][s, 0]
        # mean velocities lie near zero: absolute bound, far below the
        # thermal speed (hundreds of m/s); the He list spans two props chunks
        for a in range(3):
            assert abs(res["v"][s][a] - ref["v"][s, 0, a]) <= 1e-8, (s, a, res["v"][s][a], ref["v"][s, 0, a])


def test_poisson_request_loop_completes_every_request(ctx):
    rng = np.random.default_rng(3)
    sv = _server(ctx, max_requests=8, capacity=30_000)
    arrivals = np.cumsum(rng.exponential(1 / 200.0, 24))
    reqs = []
    for k, t in enumerate(arrivals):
        two = rng.random() < 0.3
        c = (int(np.exp(rng.uniform(np.log(200), np.log(8000)))),
             int(np.exp(rng.uniform(np.log(200), np.log(8000)))) if two else 0)
        T = (rng.uniform(300, 5000), rng.uniform(300, 5000) if two else 0.0)
        reqs.append((float(t), dict(counts=c, T=T, Fnum=_fnum(c), n_steps=int(rng.integers(5, 60)), seed=100 + k)))
    lat, ids, elapsed = sv.serve(reqs)
    assert len(lat) == len(reqs) and all(x > 0 for x in lat)
    for rid, (_, kw) in zip(ids, reqs):
        r = sv.result(rid)
        assert r["state"] == mz._lib.MZ_REQ_DONE and r["steps_done"] == kw["n_steps"]
        assert r["np"][0] == kw["counts"][0]
    info = sv.info()
    assert info["particle_steps"] == sum(sum(kw["counts"]) * kw["n_steps"] for _, kw in reqs)
    sv.close()


def test_two_lanes_give_the_results_of_one(ctx):
    """Requests of at least 3,000 particles in the lane of large requests (its
    own domain and stream, stepping while the small lane takes batches of
    steps) against all requests in one lane: identical results."""
    out = []
    for split in (0, 3000):
        sv = _server(ctx, max_requests=4, capacity=16_000)
        sv.set_lane_split(split)
        out.append(_run(sv, REQUESTS, stagger=True, max_steps=5))
        sv.close()
    one, two = out
    for seed, a in one.items():
        m = two[seed]
        assert m["state"] == mz._lib.MZ_REQ_DONE and a["steps_done"] == m["steps_done"]
        for key in ("np", "n", "T", "v"):
            assert a[key] == m[key], (seed, key)


def test_admission_by_free_device_memory_queues_what_does_not_fit(ctx):
    """A server created with capacity 0 admits by free device memory: with the
    headroom set just below the free memory, a request of 1.5 M particles
    (216 MB of particle storage) waits in its queue while a small request
    runs and finishes; once the headroom is lowered it is admitted, and its
    result equals the same request served alone."""
    torch = pytest.importorskip("torch")
    big = ((1_500_000, 0), (2000.0, 0.0), 3, 41)
    small = ((500, 700), (900.0, 400.0), 12, 42)
    sp = species(["Ar", "He"])
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    srv = mz.Server(ctx, sp, inter, DT, 8, 0)
    srv.set_lane_split(4096)
    free, _ = torch.cuda.mem_get_info(0)
    srv.set_hbm_headroom(free - (64 << 20))
    ids = {}
    for c, T, n, seed in (big, small):
        ids[seed] = srv.submit(c, T, _fnum(c), n, seed)
    for _ in range(40):
        srv.step(1)
        if srv.result(ids[42])["state"] == mz._lib.MZ_REQ_DONE:
            break
    assert srv.result(ids[42])["state"] == mz._lib.MZ_REQ_DONE
    assert srv.result(ids[41])["state"] == mz._lib.MZ_REQ_QUEUED
    srv.set_hbm_headroom(1 << 30)
    for _ in range(40):
        srv.step(1)
        if srv.result(ids[41])["state"] == mz._lib.MZ_REQ_DONE:
            break
    mixed = srv.result(ids[41])
    assert mixed["state"] == mz._lib.MZ_REQ_DONE
    srv.close()
    alone = _run(_server(ctx, capacity=2_000_000), [big])[41]
    for k in ("np", "n", "v", "T"):
        assert np.array_equal(np.asarray(mixed[k]), np.asarray(alone[k])), k
    # a request larger than the whole device memory less the headroom is refused
    srv = mz.Server(ctx, sp, inter, DT, 4, 0)
    _, total = torch.cuda.mem_get_info(0)
    with pytest.raises(Exception):
        srv.submit((total // 100, 0), (300.0, 0.0), 1e10, 1, 7)
    srv.close()
