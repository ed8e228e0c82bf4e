"""Parity scenarios through the drop-in path (GPU only): for each script of
oracle/brian_configs.py:SCENARIOS, the job the set_device('b200') plugin
wrote runs on the GPU and is compared with the reference's own run of the
same script (tests/golden/make_scenarios.py).

Bit-exact where every per-target increment of a pathway is equal (timed
refractoriness, subgroup monitors and a state monitor, a separate input
group, a spike generator, Poisson inputs -- which add after every delivery of
the step, as in the reference); where increments differ (random weights, a
presynaptic factor, plastic weights) the order of the float64 sums into a
target differs from the reference's queue order, so the raster must match and
the state (and the plastic synapses' variables) agree to 1e-12 relative."""
import json
import os

import numpy as np
import pytest

from brian2_gb300.job import load_job, run_job

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
EXACT = {"lif_refractory": True, "hetero_delays": False, "subgroup_monitors": True, "input_group": True,
         "presynaptic_read": False, "spike_generator": True, "stdp": False,
         "gap_junctions": True, "explicit_methods": True, "poisson_input": False, "poisson_drive": True,
         "noise_inputs": False, "regular_ops": True,
         "end_monitor": True, "host_sets": True, "spike_vars": True,
         "custom_events": True, "synaptic_state": False}


@pytest.mark.parametrize("name", sorted(EXACT))
@pytest.mark.parametrize("ctas,owner", [(1, "auto"), (4, True), (4, False), (20, "auto")])
def test_scenario_matches_reference(name, ctas, owner):
    jobdir = os.path.join(HERE, "golden", "jobs", name)
    spec, init, job = load_job(jobdir)
    with np.load(os.path.join(HERE, "golden", "scenarios", name + ".npz")) as z:
        ref = {k: z[k] for k in z.files}
    with open(os.path.join(HERE, "golden", "scenarios", name + ".json")) as f:
        meta = json.load(f)
    out = run_job(jobdir, threads=128, ctas_per_inst=ctas, write=False, owner=owner)
    mons = [m["name"] for m in spec["spike_monitors"]]
    sm = mons.index(meta.get("spike_monitor", mons[0]))
    assert len(out[f"sm{sm}_i"]) == meta["n_spikes"]
    np.testing.assert_array_equal(out[f"sm{sm}_i"], ref["spk_i"])
    np.testing.assert_array_equal(out[f"sm{sm}_ts"], ref["spk_ts"])
    if "other_monitor" in meta:                   # a second monitored group
        om = mons.index(meta["other_monitor"])
        np.testing.assert_array_equal(out[f"sm{om}_i"], ref["other_i"])
        np.testing.assert_array_equal(out[f"sm{om}_ts"], ref["other_ts"])
    if "gen_monitor" in meta:                     # the spike generator's raster and final cursor
        gm = mons.index(meta["gen_monitor"])
        np.testing.assert_array_equal(out[f"sm{gm}_i"], ref["gen_i"])
        np.testing.assert_array_equal(out[f"sm{gm}_ts"], ref["gen_ts"])
        gg = [g["name"] for g in spec["groups"]].index(meta["gen_group"])
        assert int(out[f"g{gg}_gen_last"]) == meta["gen_lastindex"]
    for mname, names in meta.get("spike_var_monitors", {}).items():  # recorded variables at each spike
        mi = mons.index(mname)
        m = spec["spike_monitors"][mi]
        gvars = [v["name"] for v in spec["groups"][m["group"]]["vars"]]
        for col, k in enumerate(m["vars"]):
            np.testing.assert_array_equal(out[f"sm{mi}_vals"][:, col], ref[f"smv_{mname}_{gvars[k]}"],
                                          err_msg=f"{mname}.{gvars[k]}")
        assert sorted(gvars[k] for k in m["vars"]) == sorted(names)
    np.testing.assert_array_equal(out["rm0_counts"], ref["rate_counts"])
    gi = [g["name"] for g in spec["groups"]].index(meta["group"])
    for var in ("v", "ge", "gi", "a", "Igap", "u"):
        if var in ref:
            if EXACT[name]:
                np.testing.assert_array_equal(out[f"g{gi}_{var}"], ref[var], err_msg=var)
            else:
                np.testing.assert_allclose(out[f"g{gi}_{var}"], ref[var], rtol=1e-12, atol=1e-18, err_msg=var)
    if "state_v" in ref:
        tr = out["stm0_trace"][:, 0, :].T            # [n_rec, steps]
        np.testing.assert_array_equal(tr, ref["state_v"])
    if "state_Igap" in ref:                        # a second recorded variable (a summed one)
        np.testing.assert_array_equal(out["stm0_trace"][:, 1, :].T, ref["state_Igap"])
    for mname, names in meta.get("syn_state_monitors", {}).items():  # synaptic variables over time
        mi = [m["name"] for m in spec["state_monitors"]].index(mname)
        cols = [str(x) for x in init[f"stm{mi}_vars"]]
        for var in names:
            np.testing.assert_array_equal(out[f"stm{mi}_trace"][:, cols.index(var), :].T, ref[f"sst_{mname}_{var}"],
                                          err_msg=f"{mname}.{var}")
    for var in meta.get("syn_vars", []):           # plastic synapses (on_pre and on_post share them)
        pi = next(k for k, p in enumerate(spec["pathways"])
                  if p["name"].startswith(meta["synapses"] + "_") and p.get("alias", -1) < 0)
        np.testing.assert_allclose(out[f"p{pi}_{var}"], ref["syn_" + var], rtol=1e-12, atol=1e-15, err_msg=var)
