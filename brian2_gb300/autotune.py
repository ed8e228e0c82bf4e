"""Launch-shape autotuner for the step kernel.

The best shape depends on the network: small float64 networks are FP64-bound
per SM and want several SMs in one thread-block cluster; small float32
networks want one CTA with the state in shared memory; very large networks
want one CTA per SM.  The tuner times a short run of each candidate on a
throwaway copy of the network (same construction, so the real run's state is
not touched) and keeps the fastest.  Results are cached per (model, sizes).
"""
from __future__ import annotations

import json
import os

from . import native

_CACHE_FILE = os.path.join(native.BUILD, "autotune.json")


def _load_cache():
    try:
        with open(_CACHE_FILE) as f:
            return json.load(f)
    except Exception:
        return {}


def _save_cache(c):
    os.makedirs(os.path.dirname(_CACHE_FILE), exist_ok=True)
    tmp = _CACHE_FILE + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(c, f, indent=1, sort_keys=True)
    os.replace(tmp, _CACHE_FILE)


def candidates(total_neurons: int, n_inst: int):
    """Shapes worth trying: (threads, ctas_per_inst, queue_mode)."""
    if n_inst > 1:
        return [(t, 1, True) for t in (256, 512, 1024)]
    out = [(512, 1, False), (1024, 1, False)]
    for c in (2, 4, 8, 16):
        if total_neurons >= 128 * c:
            out.append((256, c, False))
    # one CTA per SM: FP64-bound or arithmetic-heavy models (e.g. Hodgkin-Huxley
    # in either precision) and large networks
    if total_neurons >= 2000:
        out.append((256, 152, False))
        out.append((1024, 152, False))
    if total_neurons >= 100_000:  # two CTAs per SM
        out.append((512, 304, False))
        out.append((256, 304, False))
    return out


def tune(spec, builts, steps=None, make_network=None, verbose=False):
    """Returns the fastest {threads, ctas_per_inst, queue_mode} for these
    instances; `make_network(threads, ctas, queue)` builds a fresh network."""
    from .codegen import spec_hash
    from .workloads import instantiate
    sizes = [list(b.sizes) for b in builts]
    key = f"{spec['name']}:{spec_hash(spec)}:{len(builts)}:{sum(sum(s) for s in sizes)}"
    cache = _load_cache()
    if key in cache:
        return cache[key]
    total = max(sum(s) for s in sizes)
    if steps is None:  # sweeps: long enough that the state load at launch start does not decide
        steps = 1000 if len(builts) > 1 else 300
    best = None
    for threads, ctas, queue in candidates(total, len(builts)):
        try:
            net = (make_network(threads, ctas, queue) if make_network else
                   instantiate(spec, builts, threads=threads, ctas_per_inst=ctas, queue_mode=queue))
            net.run(steps)
            ms = net.last_kernel_ms()
            net.close()
        except Exception as e:  # a shape that cannot launch (too many CTAs, smem) is skipped
            if verbose:
                print("autotune: skip", threads, ctas, queue, e)
            continue
        if verbose:
            print(f"autotune: threads={threads} ctas={ctas} queue={queue}: {ms / steps * 1e3:.2f} us/step")
        if best is None or ms < best[0]:
            best = (ms, dict(threads=threads, ctas_per_inst=ctas, queue_mode=queue, us_per_step=ms / steps * 1e3))
    if best is None:
        raise RuntimeError("no launch shape could run this network")
    cache[key] = best[1]
    _save_cache(cache)
    return best[1]
