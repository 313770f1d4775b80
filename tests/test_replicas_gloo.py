"""The N > 1 path of bench.py on the CPU: replicas joined by a gloo process
group (barrier, max over ranks, sum over ranks), and the reference arm under
torch.distributed.run, where rank 0 alone runs and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    b = bench.Barrier(world)
    b()
    # per-rank time and work: the job's time is the slowest rank's, its work the sum
    t = b.max(0.5 + rank)
    w = b.sum(1000.0 * (rank + 1))
    b()
    out.put((rank, t, w))


def test_replica_barrier_max_and_sum_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.SimpleQueue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert [r[1] for r in res] == [1.5, 1.5]
    assert [r[2] for r in res] == [3000.0, 3000.0]


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    import oracle

    oracle.build()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cells", "64", "--ppc", "20"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["value"] > 0 and out["cpu_baseline"]["kind"] == "port"
