"""The set_device('b200') plugin end to end without a GPU: a scenario script of
oracle/brian_configs.py runs under the plugin (the job is written, not run),
the job runs on the oracle in place of the device, and the plugin imports the
outputs into the standalone results files; Brian's own monitor objects must
then hold what the reference's run of the same script recorded
(tests/golden/scenarios), times included (a state monitor on a clock of 5
steps).  Needs the reference importable (oracle/make_ref_env.sh)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PYENV = os.path.join(ROOT, "oracle", "_ref", "pyenv")

SCRIPT = r"""
import os, sys, json
import numpy as np
ROOT, NAME, DIR, OUT = sys.argv[1:5]
sys.path.insert(0, ROOT); sys.path.insert(0, os.path.join(ROOT, "oracle"))
import brian2_gb300.brian_device  # noqa: F401  (registers the device)
from brian2 import set_device, prefs, defaultclock, device, ms
import brian_configs as bc
from oracle import run_job_on_oracle
multi = getattr(bc.SCENARIOS[NAME], "multiple_runs", False)
set_device("b200", directory=DIR, build_on_run=not multi, b200_defer=True)
prefs.devices.cpp_standalone.openmp_threads = 0
prefs.codegen.cpp.extra_compile_args_gcc = ['-w', '-O3', '-std=c++17', '-ffp-contract=off', '-fno-fast-math']
prefs.core.default_float_dtype = np.float64
defaultclock.dt = 0.1 * ms
r = bc.SCENARIOS[NAME]()
if multi:  # several run() calls: one explicit build
    device.build(directory=DIR, b200_defer=True)
jobdir = device.b200_job_dir
out = run_job_on_oracle(jobdir)
with open(os.path.join(jobdir, "job.json")) as f:
    job = json.load(f)
init = np.load(os.path.join(jobdir, "init.npz"))
out["ts0"] = np.int64(int(init["ts0"]))
out["ts_end"] = np.int64(int(init["ts0"]) + sum(int(n) for n in job["runs"]))
out["device_ms"] = np.float64(0.0)
np.savez(os.path.join(jobdir, "out.npz"), **out)
device.b200_import_results(jobdir)
spk = r["spikes"]
res = dict(spk_i=np.asarray(spk.i[:]), spk_t=np.asarray(spk.t_[:]), v=np.asarray(r["P"].v_[:]),
           count=np.asarray(spk.count[:]), rate=np.asarray(r["rate"].rate_[:]))
if "I" in r["P"].variables:
    res["I"] = np.asarray(r["P"].I_[:])
if "state" in r:
    res.update(state_t=np.asarray(r["state"].t_[:]), state_v=np.asarray(r["state"].v_[:]))
if "G" in r and hasattr(r["G"], "_lastindex"):   # a spike generator's cursor
    res["gen_last"] = np.asarray(r["G"]._lastindex[:])
for var in r.get("syn_vars", ()):               # plastic synapses
    res["syn_" + var] = np.asarray(getattr(r["S"], var + "_")[:])
np.savez(OUT, **res)
"""


@pytest.mark.skipif(not os.path.isdir(os.path.join(PYENV, "brian2")), reason="the reference is not importable here")
@pytest.mark.parametrize("name", ["regular_ops", "spike_generator", "stdp", "noise_inputs", "host_sets"])
def test_plugin_imports_results_into_brian_monitors(tmp_path, name):
    out = tmp_path / "got.npz"
    env = dict(os.environ, PYTHONPATH=PYENV, PYTHONHASHSEED="0")  # (the fixtures' hash seed: the order of noise terms)
    p = subprocess.run([sys.executable, "-c", SCRIPT, ROOT, name, str(tmp_path / "proj"), str(out)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert p.returncode == 0, p.stderr[-3000:]
    got = np.load(out)
    with np.load(os.path.join(HERE, "golden", "scenarios", name + ".npz")) as z:
        ref = {k: z[k] for k in z.files}
    with open(os.path.join(HERE, "golden", "scenarios", name + ".json")) as f:
        meta = json.load(f)
    np.testing.assert_array_equal(got["spk_i"], ref["spk_i"])
    np.testing.assert_array_equal(np.round(got["spk_t"] / 1e-4).astype(np.int32), ref["spk_ts"])
    np.testing.assert_array_equal(got["count"], np.bincount(ref["spk_i"], minlength=len(got["count"])))
    np.testing.assert_array_equal(got["v"], ref["v"])
    n = len(got["v"])  # the rate monitor's rates: counts / dt / N
    np.testing.assert_array_equal(np.round(got["rate"] * 1e-4 * n).astype(np.int32), ref["rate_counts"])
    if "state_v" in ref:
        np.testing.assert_array_equal(got["state_v"], ref["state_v"])
        every = 5 if name == "regular_ops" else 1  # (a monitor on a clock of 5 steps there)
        rows = meta["n_steps"] // every
        assert got["state_t"].shape == (rows,)
        np.testing.assert_array_equal(got["state_t"], np.arange(rows) * (every * 1e-4))
    if "gen_lastindex" in meta:
        assert int(got["gen_last"].reshape(-1)[0]) == meta["gen_lastindex"]
    for var in meta.get("syn_vars", []):
        np.testing.assert_array_equal(got["syn_" + var], ref["syn_" + var], err_msg=var)
    if name == "host_sets":  # the assignment after the last run reaches the results
        np.testing.assert_array_equal(got["I"], np.full(len(got["I"]), 0.003))
