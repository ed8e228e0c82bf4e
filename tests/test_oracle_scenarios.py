"""The oracle pinned on the parity scenarios (no GPU): each job that the
set_device('b200') plugin wrote from a script of
oracle/brian_configs.py:SCENARIOS runs on the oracle and must reproduce the
reference's own run of the same script (tests/golden/make_scenarios.py) bit
for bit -- the oracle keeps the reference's queue order, so even the
scenarios with unequal increments sum in the same order."""
import json
import os

import numpy as np
import pytest

from oracle import run_job_on_oracle

HERE = os.path.dirname(os.path.abspath(__file__))
SCENARIOS = sorted(f[:-5] for f in os.listdir(os.path.join(HERE, "golden", "scenarios")) if f.endswith(".json"))


@pytest.mark.parametrize("name", SCENARIOS)
def test_oracle_reproduces_reference_scenario(name):
    jobdir = os.path.join(HERE, "golden", "jobs", name)
    with open(os.path.join(jobdir, "spec.json")) as f:
        spec = json.load(f)
    with np.load(os.path.join(HERE, "golden", "scenarios", name + ".npz")) as z:
        ref = {k: z[k] for k in z.files}
    with open(os.path.join(HERE, "golden", "scenarios", name + ".json")) as f:
        meta = json.load(f)
    out = run_job_on_oracle(jobdir)
    init = np.load(os.path.join(jobdir, "init.npz"))
    mons = [m["name"] for m in spec["spike_monitors"]]
    sm = mons.index(meta.get("spike_monitor", mons[0]))
    np.testing.assert_array_equal(out[f"sm{sm}_i"], ref["spk_i"])
    np.testing.assert_array_equal(out[f"sm{sm}_ts"], ref["spk_ts"])
    np.testing.assert_array_equal(out["rm0_counts"], ref["rate_counts"])
    if "other_monitor" in meta:                   # a second monitored group
        om = mons.index(meta["other_monitor"])
        np.testing.assert_array_equal(out[f"sm{om}_i"], ref["other_i"])
        np.testing.assert_array_equal(out[f"sm{om}_ts"], ref["other_ts"])
    if "gen_monitor" in meta:
        gm = mons.index(meta["gen_monitor"])
        np.testing.assert_array_equal(out[f"sm{gm}_i"], ref["gen_i"])
        np.testing.assert_array_equal(out[f"sm{gm}_ts"], ref["gen_ts"])
        gg = [g["name"] for g in spec["groups"]].index(meta["gen_group"])
        assert int(out[f"g{gg}_gen_last"]) == meta["gen_lastindex"]
    for mname, names in meta.get("spike_var_monitors", {}).items():  # recorded variables at each spike
        mi = mons.index(mname)
        m = spec["spike_monitors"][mi]
        gvars = [v["name"] for v in spec["groups"][m["group"]]["vars"]]
        assert sorted(gvars[k] for k in m["vars"]) == sorted(names)
        for col, k in enumerate(m["vars"]):
            np.testing.assert_array_equal(out[f"sm{mi}_vals"][:, col], ref[f"smv_{mname}_{gvars[k]}"],
                                          err_msg=f"{mname}.{gvars[k]}")
    gi = [g["name"] for g in spec["groups"]].index(meta["group"])
    for var in ("v", "ge", "gi", "a", "Igap", "u"):
        if var in ref:
            np.testing.assert_array_equal(out[f"g{gi}_{var}"], ref[var], err_msg=var)
    if "state_v" in ref:
        np.testing.assert_array_equal(out["stm0_trace"][:, 0, :].T, ref["state_v"])
    if "state_Igap" in ref:                      # a second recorded variable (a summed one)
        np.testing.assert_array_equal(out["stm0_trace"][:, 1, :].T, ref["state_Igap"])
    for mname, names in meta.get("syn_state_monitors", {}).items():  # synaptic variables over time
        mi = [m["name"] for m in spec["state_monitors"]].index(mname)
        cols = [str(x) for x in init[f"stm{mi}_vars"]]
        for var in names:
            np.testing.assert_array_equal(out[f"stm{mi}_trace"][:, cols.index(var), :].T, ref[f"sst_{mname}_{var}"],
                                          err_msg=f"{mname}.{var}")
    for var in meta.get("syn_vars", []):        # plastic synapses: final synaptic variables
        pi = next(k for k, p in enumerate(spec["pathways"])
                  if p["name"].startswith(meta["synapses"] + "_") and p.get("alias", -1) < 0)
        np.testing.assert_array_equal(out[f"p{pi}_{var}"], ref["syn_" + var], err_msg=var)
