"""Push-mode delivery against its oracle and the reference (GPU only).

In push mode each CTA delivers its own neurons' spikes one step ahead into
accumulators that the target's owner adds to its state after the next
barrier.  The one change to the reference's arithmetic is the order of the
additions into a target: a step's deliveries are summed first, then added.
The oracle restates exactly that with ``"push_order": true``
(oracle/oracle.py), so for models whose increments into a variable are equal
within a step (every model here) the device must reproduce it bit for bit,
whatever order its atomics take.  Against the reference's own runs: rasters
identical, float64 state within 1e-12 relative (observed: a few ulp).
Covered: the delay networks of the benchmark in several launch shapes
(including the headline's, in float32), delays up to 25 ms with runs split
across launches, the scenarios whose model allows push mode (one pathway
adding into a variable that the target's reset also writes: its deliveries
must reach it before the reset), and the refusal to switch delivery modes
while spikes are in flight."""
import json
import os

import numpy as np
import pytest

from brian2_gb300 import workloads as W
from brian2_gb300.job import load_job, run_job
from cases import CASES
from oracle import oracle_from_built, run_job_on_oracle
from test_gpu_parity import first_divergence

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
RTOL = 1e-12


def push_net(spec, built, threads, ctas):
    net = W.instantiate(spec, [built], threads=threads, ctas_per_inst=ctas)
    net.set_push(True)
    assert net.delivery_mode() == "push"
    return net


def assert_same_as_push_oracle(net, spec, built, steps):
    o = oracle_from_built(dict(spec, push_order=True), built)
    o.run(steps)
    i, ts, cnt = net.spikes(0, 0)
    oi, ots, ocnt = o.spikes(0)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(ts, ots)
    np.testing.assert_array_equal(cnt, ocnt)
    for var in ("v", "ge", "gi"):
        np.testing.assert_array_equal(net.download(0, "neurongroup", var), o.download(0, var), err_msg=var)
    return i, ts


@pytest.mark.parametrize("case", ["delays_small_f64", "delays_f64", "delays_1s_f64"])
@pytest.mark.parametrize("threads,ctas", [(256, 4), (128, 16), (256, 40), (512, 1)])
def test_push_float64(case, threads, ctas, golden):
    """Bit-exact with the push-order oracle; against the reference's run:
    identical raster and rate counts, state within 1e-12 relative."""
    spec_name, build, steps = CASES[case]
    spec = W.load_spec(spec_name)
    meta, z = golden(case)
    b = build(spec)
    net = push_net(spec, b, threads, ctas)
    net.run(steps)
    i, ts = assert_same_as_push_oracle(net, spec, b, steps)
    assert len(i) == meta["n_spikes"]
    np.testing.assert_array_equal(i, z["spk_i"])
    np.testing.assert_array_equal(ts, z["spk_ts"])
    np.testing.assert_array_equal(net.rate_counts(0, 0), np.bincount(z["spk_ts"], minlength=steps))
    for var in ("v", "ge", "gi"):
        np.testing.assert_allclose(net.download(0, "neurongroup", var), z[var], rtol=RTOL, atol=1e-300, err_msg=var)
    net.close()


@pytest.mark.parametrize("threads,ctas", [(256, 8), (128, 4), (256, 1)])
def test_push_long_delays_split_runs(threads, ctas):
    """Delays up to 25 ms (a spike history of 251 steps, more than shared
    memory holds of it), runs split across launches: the history, the slot
    counts and the deliveries due at the next step carry over."""
    spec = W.load_spec("delays_f64")
    b = W.build_delays(spec, N=2000, K=100, seed=9, dmin_ms=0.1, dmax_ms=25.0)
    net = push_net(spec, b, threads, ctas)
    for chunk in (1, 300, 1199):
        net.run(chunk)
    i, _ = assert_same_as_push_oracle(net, spec, b, 1500)
    assert len(i) > 100
    net.close()


def test_push_float32_headline_shape():
    """The float32 delay network of 10,000 neurons in the headline's launch
    shape (256 threads, two CTAs per SM): bit-exact with the float32
    push-order oracle's raster and state over 2000 steps."""
    spec = W.load_spec("delays_f32")
    b = W.build_delays(spec, N=10000, K=1000, seed=1234)
    net = push_net(spec, b, 256, 304)
    net.run(2000)
    i, _ = assert_same_as_push_oracle(net, spec, b, 2000)
    assert len(i) > 1000
    net.close()


def test_push_mode_switch_refused():
    """Spikes in flight are held in push mode's history and accumulators: a
    switch to another delivery mode before the next run is refused."""
    from brian2_gb300.runtime import B200Error
    spec_name, build, _ = CASES["delays_small_f64"]
    spec = W.load_spec(spec_name)
    net = push_net(spec, build(spec), 256, 4)
    net.run(100)
    net.set_push(False)
    with pytest.raises(B200Error):
        net.run(10)
    net.close()


SCENARIOS = sorted(d for d in os.listdir(os.path.join(HERE, "golden", "jobs"))
                   if os.path.exists(os.path.join(HERE, "golden", "scenarios", d + ".npz")))


@pytest.mark.parametrize("name", SCENARIOS)
@pytest.mark.parametrize("ctas", [4, 20])
def test_push_scenarios(name, ctas):
    """Each scenario whose model allows push mode: bit-exact with the
    push-order oracle (monitors, rate counts, state, state-monitor traces)
    and the same raster as the reference's run."""
    jobdir = os.path.join(HERE, "golden", "jobs", name)
    spec, init, job = load_job(jobdir)
    out = run_job(jobdir, threads=128, ctas_per_inst=ctas, write=False, push=True)
    if not int(out["push"]):
        pytest.skip("push mode does not apply to this model (spike generators, custom events, on_post, "
                    "summed or per-synapse code, delays of 0 steps or an on_pre that is not an addition)")
    orc = run_job_on_oracle(jobdir, push_order=True)
    for k, v in orc.items():
        if k in out and isinstance(v, np.ndarray) and v.dtype != object:
            np.testing.assert_array_equal(out[k], v, err_msg=k)
    with np.load(os.path.join(HERE, "golden", "scenarios", name + ".npz")) as zf:
        ref = {k: zf[k] for k in zf.files}
    with open(os.path.join(HERE, "golden", "scenarios", name + ".json")) as f:
        meta = json.load(f)
    mons = [m["name"] for m in spec["spike_monitors"]]
    sm = mons.index(meta.get("spike_monitor", mons[0]))
    i, ts = out[f"sm{sm}_i"], out[f"sm{sm}_ts"]
    d = first_divergence(i, ts, ref["spk_i"], ref["spk_ts"])
    print(f"push {name} ({ctas} CTAs): {len(i)} spikes, reference {len(ref['spk_i'])}; first step differing "
          f"from the reference: {d} of {meta.get('n_steps')}")
    assert d is None
