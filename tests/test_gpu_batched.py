"""Batched sweeps and graph replay (GPU only)."""
import numpy as np
import pytest

from brian2_gb300 import batched, workloads as W
from oracle import oracle_from_built

pytestmark = pytest.mark.gpu


def test_graph_replay_equals_direct_launch():
    spec = W.load_spec("delays_f64")
    b = W.build_delays(spec, N=2000, K=100, seed=5)
    outs = []
    for graph in (False, True):
        net = W.instantiate(spec, [b], threads=256, ctas_per_inst=4, chunk_steps=250)
        net.configure(threads=256, ctas_per_inst=4, chunk_steps=250, use_graph=graph)
        net.run(1000)
        outs.append((net.spikes(0, 0)[0], net.download(0, "neurongroup", "v")))
        assert net.launches() == 4
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_float32_sweep_matches_oracle_instances():
    """Every instance of a float32 sweep against its own oracle run: identical
    rasters up to the first divergence, which must not come in the first 50 ms
    (the device keeps float32 constants, the reference float32 mode doubles)."""
    spec = W.load_spec("cuba_f32")
    params = batched.sweep_parameters(n=12, seed=7, n_lo=300, n_hi=2500)
    builts = batched.build_sweep(spec, params)
    sw = batched.Sweep(spec, builts, threads=256)
    sw.run(1000)
    for k, b in enumerate(builts):
        o = oracle_from_built(spec, b)
        o.run(1000)
        oi, ots, _ = o.spikes(0)
        i, ts, _ = sw.spikes(k)
        n = min(len(i), len(oi))
        bad = np.flatnonzero((i[:n] != oi[:n]) | (ts[:n] != ots[:n]))
        first = ts[bad[0]] if len(bad) else None
        assert first is None or first >= 500, (k, first)
        assert abs(len(i) - len(oi)) <= 0.05 * len(oi) + 10
