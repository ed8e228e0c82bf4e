"""Device-side construction (GPU only): bit-exact with its CPU restatement,
and the step loop on a device-built network equals the oracle on the same
synapse lists."""
import numpy as np
import pytest

import scale_ref
from brian2_gb300 import workloads as W
from brian2_gb300.scale import DeviceCSR, build_delays_scale

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_src,n_post,K", [(1600, 2000, 80), (400, 2000, 20), (50, 300, 50)])
def test_device_csr_equals_cpu_restatement(n_src, n_post, K):
    we, wi, dmin, dspan = W.delay_constants()
    d = DeviceCSR(99, 1, n_src, 7, n_post, K, dmin, dspan, W.DT)
    seg, post, pre = d.host_arrays()
    ref = scale_ref.fixed_indegree_csr(99, 1, n_src, 7, n_post, K, dmin, dspan, W.DT)
    d.free()
    np.testing.assert_array_equal(seg, ref["seg"])
    np.testing.assert_array_equal(post, ref["post"])
    np.testing.assert_array_equal(pre, ref["pre"])
    # fixed in-degree: every target has exactly K distinct sources
    assert np.all(np.bincount(post, minlength=n_post) == K)


def test_step_loop_on_device_built_network_matches_oracle():
    from oracle import OracleNet
    spec = W.load_spec("delays_f64")
    N, K = 3000, 200
    net, csrs = build_delays_scale(spec, N=N, K=K, seed=17, keep_csr=True)
    o = OracleNet(spec, [N], W.DT)
    o.upload("neurongroup", "v", net.download(0, "neurongroup", "v"))
    o.upload("neurongroup", "i", np.arange(N, dtype=np.int32))
    Ne = int(0.8 * N)
    for pw, d, (lo, hi) in zip(("synapses_pre", "synapses_1_pre"), csrs, ((0, Ne), (Ne, N))):
        seg, post, pre = d.host_arrays()
        slots = np.repeat(np.arange(len(seg) - 1) % d.W + d.slot_min, np.diff(seg)).astype(np.int32)
        o.set_synapses(pw, pre - lo, post, slots, 0, (lo, hi), (0, N))
        o.upload_synapse_var(pw, "w", net.download_synapse_var(0, pw, "w"))
        d.free()
    net.run(1500)
    o.run(1500)
    i, ts, _ = net.spikes(0, 0)
    oi, ots, _ = o.spikes(0)
    assert len(oi) > 100
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(ts, ots)
    np.testing.assert_array_equal(net.download(0, "neurongroup", "v"), o.download(0, "v"))
