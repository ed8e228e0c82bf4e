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
