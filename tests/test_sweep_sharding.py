"""A batched sweep split over ranks (host logic, CPU): the split covers every
instance once and balances the neurons; with world_size 2 over gloo each rank
builds and runs only its own instances (here on the oracle, standing in for
the GPU) and the gathered rasters equal those of one process running all."""
import os
import socket
import subprocess
import sys

import numpy as np

from brian2_gb300 import batched

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_covers_every_instance_and_balances():
    sizes = [int(x) for x in np.random.default_rng(3).integers(500, 8001, size=256)]
    for world in (1, 2, 4, 8):
        parts = batched.shard(sizes, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[k] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)


WORKER = r"""
import os, sys, json
ROOT = sys.argv[1]
sys.path.insert(0, ROOT); sys.path.insert(0, os.path.join(ROOT, "oracle"))
import numpy as np
import torch.distributed as dist
from brian2_gb300 import batched, workloads as W
from oracle import oracle_from_built
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
spec = W.load_spec("cuba_f32")
params = batched.sweep_parameters(n=6, seed=5, n_lo=200, n_hi=600)

def oracle_runner(spec, builts, steps, threads):
    out = []
    for b in builts:
        o = oracle_from_built(spec, b); o.run(steps)
        i, ts, _ = o.spikes(0); out.append((i, ts))
    return 0.0, out

built_here = []
orig = batched.build_sweep
def counting_build(spec, ps, workers=16):
    built_here.extend(p["seed"] for p in ps)
    return orig(spec, ps, workers)
batched.build_sweep = counting_build
ms, res = batched.run_sharded(spec, params, 200, rank, world, dist, runner=oracle_runner)
mine = batched.shard([p["N"] for p in params], world)[rank]
assert sorted(built_here) == sorted(params[k]["seed"] for k in mine), (built_here, mine)
if rank == 0:
    batched.build_sweep = orig
    _, ref = batched.run_sharded(spec, params, 200, 0, 1, None, runner=oracle_runner)
    assert sorted(res) == list(range(len(params)))
    for k in res:
        assert np.array_equal(res[k][0], ref[k][0]) and np.array_equal(res[k][1], ref[k][1]), k
    print("OK", {k: len(v[0]) for k, v in res.items()})
dist.barrier()
dist.destroy_process_group()
"""


def test_two_ranks_run_their_shares_and_gather(tmp_path):
    script = tmp_path / "worker.py"
    script.write_text(WORKER)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(script), ROOT],
                       capture_output=True, text=True, timeout=280, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "OK" in r.stdout
