"""Batched parameter sweeps: many independent networks in one persistent launch.

Each network of the sweep is one *instance* of the same compiled model with its
own size, its own namespace constants (here ``taum`` and the excitatory weight
``we``) and its own synapses.  All instances run in one launch of the step
kernel in queue mode: resident CTAs take instances from a work queue (largest
first, so the long ones start early), each instance on one CTA with its state
in shared memory, every launch replayed from a captured CUDA graph.  The plain
path for comparison runs the same networks one after another, twice: all at
one fixed launch shape (512 threads, one CTA), and each at the shape the
autotuner picks for its size class (the networks binned by size, one tuning
per bin).

Sweep of the benchmark (configuration "batched parameter sweep"): 256 CUBA
networks, N uniform in 500..8000 (80/20 E/I), taum uniform in 10..30 ms,
excitatory weight scale uniform in 0.5..2.0, Bernoulli p=0.02 from seed s+k,
float32, dt = 0.1 ms, 500 ms.
"""
from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import workloads as W


def sweep_parameters(n=256, seed=2024, n_lo=500, n_hi=8000):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(n_lo, n_hi + 1, size=n)
    taum = rng.uniform(0.010, 0.030, size=n)
    wscale = rng.uniform(0.5, 2.0, size=n)
    return [dict(N=int(sizes[k]), taum=float(taum[k]), wscale=float(wscale[k]), seed=int(seed) + k)
            for k in range(n)]


def build_sweep(spec, params, workers=16):
    """Constructs every instance (host construction releases the GIL, so a
    thread pool builds them in parallel)."""
    we0 = W.const(spec, "we")

    def one(p):
        return W.build_cuba(spec, N=p["N"], seed=p["seed"],
                            consts=dict(taum=p["taum"], we=we0 * p["wscale"]))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(one, params))


class Sweep:
    """All instances of a sweep on the device, in one network handle."""

    def __init__(self, spec, builts, threads=512, use_graph=True, chunk_steps=0):
        order = sorted(range(len(builts)), key=lambda k: -sum(builts[k].sizes))
        self.order = order                  # instance slot -> sweep index (largest first)
        self.builts = [builts[k] for k in order]
        self.net = W.instantiate(spec, self.builts, threads=threads, queue_mode=True, chunk_steps=chunk_steps)
        if use_graph:
            self.net.configure(threads=threads, ctas_per_inst=1, queue_mode=True, chunk_steps=chunk_steps,
                               use_graph=True)

    def run(self, steps):
        self.net.run(steps)
        return self.net.last_kernel_ms()

    def spikes(self, k):
        """Spike raster of sweep index k."""
        slot = self.order.index(k)
        return self.net.spikes(slot, 0)


def run_sequential(spec, builts, steps, shape=None, shapes=None):
    """The plain GPU path: every network alone, one after another (at `shape`,
    or at its own entry of `shapes`); returns the summed device time (ms) and
    the per-network spike counts."""
    total_ms = 0.0
    counts = []
    for k, b in enumerate(builts):
        s = (shapes[k] if shapes else shape) or dict(threads=512, ctas_per_inst=1)
        net = W.instantiate(spec, [b], threads=s["threads"], ctas_per_inst=s.get("ctas_per_inst", 1))
        net.run(steps)
        total_ms += net.last_kernel_ms()
        counts.append(len(net.spikes(0, 0)[0]))
        net.close()
    return total_ms, counts


def tuned_shapes(spec, builts, bins=8):
    """The autotuner's launch shape for every network: the networks are binned
    by size (equal counts per bin), the median network of each bin is tuned,
    and its shape serves the bin.  Returns (shape per network, tuned shapes)."""
    from . import autotune
    order = sorted(range(len(builts)), key=lambda k: sum(builts[k].sizes))
    groups = [order[i * len(order) // bins:(i + 1) * len(order) // bins] for i in range(bins)]
    shapes = [None] * len(builts)
    tuned = []
    for g in groups:
        if not g:
            continue
        rep_ = builts[g[len(g) // 2]]
        sh = autotune.tune(spec, [rep_])
        tuned.append(dict(neurons=int(sum(rep_.sizes)), threads=sh["threads"], ctas_per_inst=sh["ctas_per_inst"]))
        for k in g:
            shapes[k] = dict(threads=sh["threads"], ctas_per_inst=sh["ctas_per_inst"])
    return shapes, tuned


def compare(spec, builts, steps, threads=512, seq_shape=None, tuned=True):
    """Batched vs sequential: device ms of each and the speed-ups, against the
    sequential networks at one fixed shape and (tuned) each at its size
    class's tuned shape."""
    t0 = time.perf_counter()
    sw = Sweep(spec, builts, threads=threads)
    batched_ms = sw.run(steps)
    b_counts = [len(sw.spikes(k)[0]) for k in range(len(builts))]
    sw.net.close()
    seq_ms, s_counts = run_sequential(spec, builts, steps, seq_shape)
    out = dict(batched_ms=batched_ms, sequential_ms=seq_ms, speedup=seq_ms / batched_ms,
               sequential_shape=seq_shape or dict(threads=512, ctas_per_inst=1),
               same_spike_counts=b_counts == s_counts)
    if tuned:
        shapes, tuned_list = tuned_shapes(spec, builts)
        t_ms, t_counts = run_sequential(spec, builts, steps, shapes=shapes)
        out.update(sequential_tuned_ms=t_ms, speedup_vs_tuned=t_ms / batched_ms, tuned_shapes=tuned_list,
                   same_spike_counts_tuned=b_counts == t_counts)
    out["wall_s"] = time.perf_counter() - t0
    return out


# ---------------------------------------------------------------------------
# A sweep over several GPUs: the instances are independent, so they are split
# over the ranks (one process per GPU) with no exchange during the run; only
# the per-instance results are gathered at the end.
# ---------------------------------------------------------------------------
def shard(sizes, world):
    """Instance indices per rank: largest first, each to the rank with the
    fewest neurons so far (a greedy longest-processing-time split, so every
    rank's queue-mode launch has about the same work)."""
    load = [0] * world
    out = [[] for _ in range(world)]
    for k in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(world), key=lambda r: (load[r], r))
        out[r].append(k)
        load[r] += sizes[k]
    return [sorted(x) for x in out]


def _device_runner(spec, builts, steps, threads=512):
    """This rank's instances in one queue-mode launch on its GPU."""
    sw = Sweep(spec, builts, threads=threads)
    ms = sw.run(steps)
    res = [sw.spikes(k) for k in range(len(builts))]
    sw.net.close()
    return ms, [(np.asarray(i), np.asarray(t)) for i, t, _ in res]


def run_sharded(spec, params, steps, rank=0, world=1, dist=None, runner=None, threads=512):
    """Runs this rank's share of a sweep and gathers every instance's raster
    on every rank (torch.distributed object all-gather; none with one rank).
    Returns (device ms of this rank, {sweep index: (i, ts)})."""
    mine = shard([p["N"] for p in params], world)[rank]
    builts = build_sweep(spec, [params[k] for k in mine])
    ms, res = (runner or _device_runner)(spec, builts, steps, threads) if builts else (0.0, [])
    local = {k: r for k, r in zip(mine, res)}
    if dist is None or world == 1:
        return ms, local
    gathered = [None] * world
    dist.all_gather_object(gathered, local)
    allres = {}
    for part in gathered:
        allres.update(part)
    return ms, allres
