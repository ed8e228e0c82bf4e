"""The oracle against the reference's own outputs (fixtures made by running
Brian2 cpp_standalone, single thread, strict IEEE flags): spike rasters and
final states must be identical, bit for bit, in float64 and float32."""
import numpy as np
import pytest

from brian2_gb300 import workloads as W
from cases import CASES
from oracle import oracle_from_built


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_reproduces_reference(case, golden):
    spec_name, build, steps = CASES[case]
    spec = W.load_spec(spec_name)
    meta, z = golden(case)
    assert meta["n_steps"] == steps
    o = oracle_from_built(spec, build(spec))
    o.run(steps)
    i, ts, cnt = o.spikes(0)
    assert len(i) == meta["n_spikes"]
    np.testing.assert_array_equal(i, z["spk_i"])
    np.testing.assert_array_equal(ts, z["spk_ts"])
    for var in ("v", "ge", "gi", "m", "n", "h"):
        if var in z:
            np.testing.assert_array_equal(o.download(0, var), z[var], err_msg=var)
    # rate monitor: count per step equals the raster's histogram
    np.testing.assert_array_equal(o.rate_counts(0), np.bincount(z["spk_ts"], minlength=steps))


@pytest.mark.parametrize("case", ["delays_small_f64", "delays_f64"])
def test_push_order_oracle_close_to_reference(case, golden):
    """The oracle of push-mode delivery (each step's deliveries summed into an
    accumulator, then added to their targets) on the reference's delay
    networks: the same raster as the reference's run, the float64 state within
    1e-12 relative -- the push order changes only the rounding of the sums."""
    spec_name, build, steps = CASES[case]
    spec = dict(W.load_spec(spec_name), push_order=True)
    meta, z = golden(case)
    o = oracle_from_built(spec, build(spec))
    o.run(steps)
    i, ts, _ = o.spikes(0)
    np.testing.assert_array_equal(i, z["spk_i"])
    np.testing.assert_array_equal(ts, z["spk_ts"])
    for var in ("v", "ge", "gi"):
        np.testing.assert_allclose(o.download(0, var), z[var], rtol=1e-12, atol=1e-300, err_msg=var)


def test_push_order_oracle_explicit_methods_scenario():
    """A pathway adding into a variable that its target's reset also writes
    (the explicit-methods scenario): the push-order oracle keeps the
    reference's raster (deliveries reach the variable before the reset)."""
    import os
    from oracle import run_job_on_oracle
    here = os.path.dirname(os.path.abspath(__file__))
    out = run_job_on_oracle(os.path.join(here, "golden", "jobs", "explicit_methods"), push_order=True)
    with np.load(os.path.join(here, "golden", "scenarios", "explicit_methods.npz")) as z:
        np.testing.assert_array_equal(out["sm0_i"], z["spk_i"])
        np.testing.assert_array_equal(out["sm0_ts"], z["spk_ts"])
        np.testing.assert_allclose(out["g0_v"], z["v"], rtol=1e-12, atol=1e-300)
