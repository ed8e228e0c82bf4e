"""Reference fixtures and b200 jobs of the parity scenarios.

For each scenario of ``oracle/brian_configs.py:SCENARIOS`` this runs the same
Brian2 script twice, each in its own process (a standalone device builds once
per process):

* with the reference's ``cpp_standalone`` device (one thread, strict IEEE
  flags, float64) -> ``tests/golden/scenarios/<name>.npz``: the spike monitor's
  indices and time steps, the rate monitor's per-step counts, the state
  monitor's trace, the final state of the monitored group (and, for a spike
  generator, its raster and final cursor; for plastic synapses, their final
  synaptic variables);
* with the ``b200`` plugin in deferred mode -> ``tests/golden/jobs/<name>/``:
  the job the plugin writes from the script (spec, initial state, synapses).

Run where the reference is importable::

    bash oracle/make_ref_env.sh <reference checkout>
    PYTHONPATH=oracle/_ref/pyenv python tests/golden/make_scenarios.py [name ...]
"""
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(ROOT, "oracle", "_ref", "scenario_build")
STRICT = ['-w', '-O3', '-std=c++17', '-ffp-contract=off', '-fno-fast-math']


def setup(device_name, directory, build_on_run=True, **kw):
    import numpy as np
    from brian2 import set_device, prefs, defaultclock, ms
    set_device(device_name, directory=directory, build_on_run=build_on_run, **kw)
    prefs.devices.cpp_standalone.openmp_threads = 0
    prefs.codegen.cpp.extra_compile_args_gcc = STRICT
    prefs.core.default_float_dtype = np.float64
    defaultclock.dt = 0.1 * ms


def run_ref(name):
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import brian_configs as bc
    d = os.path.join(BUILD, name + "_ref")
    shutil.rmtree(d, ignore_errors=True)
    multi = getattr(bc.SCENARIOS[name], "multiple_runs", False)
    setup("cpp_standalone", d, build_on_run=not multi)
    r = bc.SCENARIOS[name]()
    if multi:  # several run() calls: one explicit build
        from brian2 import device
        device.build(directory=d)
    P, spk, rate = r["P"], r["spikes"], r["rate"]
    out = {}
    t = np.asarray(spk.t_[:])
    out["spk_i"] = np.asarray(spk.i[:], dtype=np.int32)
    out["spk_ts"] = np.round(t / 1e-4).astype(np.int32)
    n_rate = len(rate.source)
    out["rate_counts"] = np.round(np.asarray(rate.rate_[:]) * 1e-4 * n_rate).astype(np.int32)
    if "state" in r:
        out["state_v"] = np.asarray(r["state"].v_[:]).copy()        # [n_rec, steps]
        out["state_idx"] = np.asarray(r["state"].record, dtype=np.int32)
    for var in ("v", "ge", "gi", "a", "Igap", "u"):
        if var in P.variables:
            out[var] = np.asarray(getattr(P, var + "_")[:]).copy()
    for var in r.get("state_extra", ()):        # more recorded variables: [n_rec, steps]
        out["state_" + var] = np.asarray(getattr(r["state"], var + "_")[:]).copy()
    meta = dict(group=P.name, n_spikes=int(len(t)), n_steps=int(len(out["rate_counts"])), spike_monitor=spk.name)
    if "gen_spikes" in r:                       # a spike generator's own raster and cursor
        g = r["gen_spikes"]
        out["gen_i"] = np.asarray(g.i[:], dtype=np.int32)
        out["gen_ts"] = np.round(np.asarray(g.t_[:]) / 1e-4).astype(np.int32)
        meta["gen_monitor"] = g.name
        meta["gen_group"] = r["G"].name
        from brian2 import device             # the results file (get_value returns the cached initial 0)
        fn = os.path.join(device.results_dir, device.get_array_filename(r["G"].variables["_lastindex"]))
        meta["gen_lastindex"] = int(np.fromfile(fn, dtype=np.int32)[0])
    if "other_spikes" in r:                    # a second monitored group (its raster)
        o = r["other_spikes"]
        out["other_i"] = np.asarray(o.i[:], dtype=np.int32)
        out["other_ts"] = np.round(np.asarray(o.t_[:]) / 1e-4).astype(np.int32)
        meta["other_monitor"] = o.name
    if "spike_var_monitors" in r:              # spike monitors' recorded variables
        meta["spike_var_monitors"] = {}
        for mon in r["spike_var_monitors"]:
            names = [v for v in mon.record_variables if v not in ("i", "t")]
            for var in names:
                out[f"smv_{mon.name}_{var}"] = np.asarray(getattr(mon, var + "_")[:]).copy()
            meta["spike_var_monitors"][mon.name] = names
    if "syn_state" in r:                       # state monitors of synaptic variables: [n_rec, steps]
        meta["syn_state_monitors"] = {}
        for mon in r["syn_state"]:
            for var in mon.record_variables:
                out[f"sst_{mon.name}_{var}"] = np.asarray(getattr(mon, var + "_")[:]).copy()
            meta["syn_state_monitors"][mon.name] = list(mon.record_variables)
    if "syn_vars" in r:                        # synaptic variables (creation order)
        for var in r["syn_vars"]:
            out["syn_" + var] = np.asarray(getattr(r["S"], var + "_")[:]).copy()
        meta["synapses"] = r["S"].name
        meta["syn_vars"] = list(r["syn_vars"])
    np.savez_compressed(os.path.join(HERE, "scenarios", name + ".npz"), **out)
    with open(os.path.join(HERE, "scenarios", name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "reference:", len(t), "spikes")


def run_job(name):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import brian2_gb300.brian_device  # noqa: F401  (registers the device)
    from brian2 import device
    import brian_configs as bc
    d = os.path.join(BUILD, name + "_job")
    shutil.rmtree(d, ignore_errors=True)
    multi = getattr(bc.SCENARIOS[name], "multiple_runs", False)
    setup("b200", d, build_on_run=not multi, b200_defer=True)
    bc.SCENARIOS[name]()
    if multi:
        device.build(directory=d, b200_defer=True)
    out = os.path.join(HERE, "jobs", name)
    shutil.rmtree(out, ignore_errors=True)
    shutil.copytree(device.b200_job_dir, out)
    print(name, "job ->", out)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--ref"]:
        run_ref(sys.argv[2])
        sys.exit(0)
    if sys.argv[1:2] == ["--job"]:
        run_job(sys.argv[2])
        sys.exit(0)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import brian_configs as bc
    os.makedirs(os.path.join(HERE, "scenarios"), exist_ok=True)
    # Brian orders the noise terms of a stochastic equation by iterating a set of
    # names, so the order of randn() calls in its generated code follows Python's
    # string hashing: both runs of a script use the same hash seed
    env = dict(os.environ, PYTHONHASHSEED="0")
    for n in sys.argv[1:] or list(bc.SCENARIOS):
        for phase in ("--ref", "--job"):
            subprocess.run([sys.executable, os.path.abspath(__file__), phase, n], check=True, env=env)
