"""The drop-in path end to end: a job that set_device('b200') wrote from the
reference's own script (tests/golden/jobs) runs on the GPU through
brian2_gb300.job and reproduces the reference's fixture of the same case."""
import os

import numpy as np
import pytest

from brian2_gb300.job import run_job

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("case,ctas", [("cuba_small_f64", 1), ("delays_small_f64", 1), ("cobahh_small_f64", 1),
                                       ("cuba_small_f64", 4), ("delays_small_f64", 4)])
def test_plugin_job_reproduces_reference(case, ctas, golden):
    meta, z = golden(case)
    out = run_job(os.path.join(HERE, "golden", "jobs", case), ctas_per_inst=ctas, write=False)
    np.testing.assert_array_equal(out["sm0_i"], z["spk_i"])
    np.testing.assert_array_equal(out["sm0_ts"], z["spk_ts"])
    assert int(out["ts_end"]) == meta["n_steps"]
    if case.startswith("cobahh"):   # device exp/expm1: last-ulp differences in the state
        np.testing.assert_allclose(out["g0_v"], z["v"], rtol=1e-9, atol=0)
    else:
        np.testing.assert_array_equal(out["g0_v"], z["v"])
        np.testing.assert_array_equal(out["g0_ge"], z["ge"])
    np.testing.assert_array_equal(out["rm0_counts"], np.bincount(z["spk_ts"], minlength=meta["n_steps"]))


@pytest.mark.parametrize("case", ["delays_small_f64", "cuba_small_f64"])
def test_profiled_job_reports_every_code_object(case, golden):
    """run(profile=True) through the plugin: the device profile has cycles in
    the slots of the group's update, threshold and reset, of every delivery
    pass's events and of the monitors; profiling does not change the results."""
    from brian2_gb300.codegen import delivery_passes
    from brian2_gb300.job import load_job
    meta, z = golden(case)
    out = run_job(os.path.join(HERE, "golden", "jobs", case), write=False, profile=True)
    np.testing.assert_array_equal(out["sm0_i"], z["spk_i"])
    prof = dict(zip((str(x) for x in out["prof_names"]), out["prof_cycles"]))
    spec, _, _ = load_job(os.path.join(HERE, "golden", "jobs", case))
    passes = [f"events:{spec['pathways'][pis[0]]['name']}" for _, pis, _ in delivery_passes(spec["pathways"])]
    for slot in ["update:neurongroup", "threshold:neurongroup", "reset:neurongroup", "ring:neurongroup",
                 "spikemon:spikemonitor", "ratemon:ratemonitor"] + passes:
        assert prof.get(slot, 0) > 0, (slot, prof)
    assert float(out["kernel_ms"]) > 0
