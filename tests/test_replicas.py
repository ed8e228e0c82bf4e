"""The N-GPU path of bench.py on CPU: replicas over gloo (world size 2).

The step engine does not shard a network (every box has one GPU): N ranks run
N independent networks (weak scaling) and only the timing is combined, the
slowest rank's time and the sum of all ranks' events."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=2)
    sys.path.insert(0, ROOT)
    import bench
    t, e = bench.reduce_ranks(dist, 1.0 + rank, 10 * (rank + 1))
    bench.sync_all(dist)
    q.put((rank, t, e))
    dist.destroy_process_group()


def test_reduce_ranks_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun_two_ranks():
    """`bench.py --impl reference` launched as the multi-GPU run is: rank 0
    alone times the reference's CPU path and prints one JSON line, the other
    rank exits 0 without work."""
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
                        os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--reference-sample", "subnetwork"],
                       capture_output=True, text=True, cwd=ROOT, timeout=280)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] in ("reference", "port")
