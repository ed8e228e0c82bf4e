"""Generates the reference's own ``cpp_standalone`` projects of the CPU baselines.

Test infrastructure only (the timed CPU baselines; never on the product path).
Each project is a benchmark network written as a Brian script
(``brian_configs.py``) and turned into C++ by the reference's code generator for
its OpenMP standalone path (``brian2/devices/cpp_standalone/device.py``,
``openmp_threads`` preference), so what runs on the host cores is the
reference's generated step loop unchanged.  Workloads:

* ``delays`` -- the 10,000-neuron subnetwork of the large delay network
  (in-degree 1000, delays uniform in 0.1-5 ms, ``brian_configs.cuba_delays``),
  float64, one run of 1 s;
* ``delays1e6`` -- the large delay network itself: 1,000,000 neurons, 1e9
  synapses, float32; a run of 50 ms lets the activity settle, then a run of
  100 ms (1000 clock steps) reports its progress through Brian's own progress
  report (``run(report=..., report_period=...)``: for the standalone device
  C++ code of the report function, ``device.py:1889-1907``, called from the
  step loop with the run's elapsed time and completed fraction about every
  0.5 s of wall time, ``templates/network.cpp:59-90``).  One execution thus
  gives many timed samples after a single construction;
* ``cuba`` -- CUBA, 4000 neurons, float64, 1 s (``brian_configs.cuba``);
* ``cobahh`` / ``cobahh32`` -- COBAHH, 4000 neurons, 1 s, float64 / float32
  (``brian_configs.cobahh``);
* ``sweep8`` -- 8 networks of the 256-network CUBA sweep (float32, 500 ms
  each), one per size stratum: the sweep's networks sorted by size, the middle
  one of each run of 32 (``brian_configs.cuba_sweep``, the sweep's own sizes,
  seeds and parameters), run one after another, each reporting its own run
  time;
* ``adjoint`` -- the forward pass of the gradient workload written as a Brian
  network (200 spike-generator inputs -> 1000 LIF -> 10 readout, 5000 steps,
  float32, ``brian_configs.adjoint_network``).

Generation needs the reference importable, so it runs here::

    bash oracle/make_ref_env.sh <reference checkout>
    PYTHONPATH=oracle/_ref/pyenv python oracle/make_ref_standalone.py [workload:threads ...]

Output (git-ignored, compiled where it runs by ``ref_standalone.build``): one
project per workload and OpenMP thread count (the count is fixed at generation,
``brian2/devices/cpp_standalone/codeobject.py:17-40``) in
``oracle/_ref/standalone_<workload>_t<threads>/``, each with the generated
sources and ``manifest.json``, which names the result files (spike monitor
indices and times, the synapses' presynaptic indices) that the timing reads
back.  The generated ``makefile`` is not used: its default flags include
``-march=native``.
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# the marker the report function prints at each call: elapsed seconds and completed fraction
RUN_MARK = "REF_RUN_TIME"
REPORT = ('std::cout.precision(12); std::cout << "' + RUN_MARK +
          ' " << elapsed << " " << completed << std::endl;')
# name: (float dtype, builder arguments)
WORKLOADS = {
    "delays": ("float64", dict(kind="delays", N=10_000, K=1000, warmup_ms=0.0, duration_ms=1000.0, period=None)),
    "delays1e6": ("float32", dict(kind="delays", N=1_000_000, K=1000, warmup_ms=50.0, duration_ms=100.0,
                                  period=0.5)),
    "cuba": ("float64", dict(kind="cuba", N=4000, duration_ms=1000.0, seed=1234)),
    "cobahh": ("float64", dict(kind="cobahh", N=4000, duration_ms=1000.0, seed=1234)),
    "cobahh32": ("float32", dict(kind="cobahh", N=4000, duration_ms=1000.0, seed=1234)),
    "sweep8": ("float32", dict(kind="sweep", networks=256, strata=8, duration_ms=500.0)),
    "adjoint": ("float32", dict(kind="adjoint", steps=5000)),
}
DEFAULT = ("delays:1", "delays:16", "delays1e6:16", "cuba:1", "cuba:16", "cobahh:1", "cobahh:16",
           "cobahh32:1", "cobahh32:16", "sweep8:1", "sweep8:16", "adjoint:1", "adjoint:16")


def sweep_sample(networks=256, strata=8):
    """Indices into the sweep's parameter list: sorted by size, the middle
    network of each of ``strata`` equal strata."""
    sys.path.insert(0, ROOT)
    from brian2_gb300.batched import sweep_parameters
    params = sweep_parameters(networks)
    order = sorted(range(networks), key=lambda k: (params[k]["N"], k))
    per = networks // strata
    return params, [order[j * per + per // 2] for j in range(strata)]


def generate(workload, threads, seed_value=1234):
    """One project (the standalone device builds once per process)."""
    fdt, a = WORKLOADS[workload]
    OUT = os.path.join(HERE, "_ref", f"standalone_{workload}_t{threads}")
    sys.path.insert(0, HERE)
    sys.path.insert(0, ROOT)
    import numpy as np
    from brian2 import set_device, device, prefs, defaultclock, ms
    import brian_configs as bc
    shutil.rmtree(OUT, ignore_errors=True)
    set_device("cpp_standalone", directory=OUT, build_on_run=False)
    prefs.devices.cpp_standalone.openmp_threads = int(threads)
    prefs.core.default_float_dtype = getattr(np, fdt)
    defaultclock.dt = 0.1 * ms
    fname = device.get_array_filename
    man = dict(workload=workload, kind=a["kind"], dt=1e-4, threads=int(threads), float_dtype=fdt)
    if a["kind"] == "delays":
        r = bc.cuba_delays(N=a["N"], K=a["K"], duration_ms=a["duration_ms"], seed_value=seed_value,
                           warmup_ms=a["warmup_ms"], report=REPORT if a["period"] else None,
                           report_period_s=a["period"] or 10.0)
        man.update(N=a["N"], K=a["K"], seed=seed_value, warmup_ms=a["warmup_ms"], duration_ms=a["duration_ms"],
                   report_period_s=a["period"], run_mark=RUN_MARK if a["period"] else None)
    elif a["kind"] in ("cuba", "cobahh"):
        r = getattr(bc, a["kind"])(N=a["N"], duration_ms=a["duration_ms"], seed_value=a["seed"])
        man.update(N=a["N"], seed=a["seed"], warmup_ms=0.0, duration_ms=a["duration_ms"])
    elif a["kind"] == "sweep":
        params, pick = sweep_sample(a["networks"], a["strata"])
        nets = bc.cuba_sweep([params[k] for k in pick], duration_ms=a["duration_ms"], report=REPORT)
        man.update(duration_ms=a["duration_ms"], run_mark=RUN_MARK, sweep_networks=a["networks"],
                   sweep_indices=pick, networks=[dict(
                       N=params[k]["N"], spike_i=fname(n["spikes"].variables["i"]),
                       pre={s: fname(n[s].variables["_synaptic_pre"]) for s in ("Ce", "Ci")})
                       for k, n in zip(pick, nets)])
    elif a["kind"] == "adjoint":
        r = bc.adjoint_network(steps=a["steps"])
        man.update(N=1000, warmup_ms=0.0, duration_ms=a["steps"] * 0.1,
                   # the hidden layer's spikes reach the 10 readout neurons; the
                   # input layer's events are not counted (forward time is the figure)
                   pre={"Sout": fname(r["Sout"].variables["_synaptic_pre"])})
    if a["kind"] != "sweep":
        man.update(spike_i=fname(r["spikes"].variables["i"]), spike_t=fname(r["spikes"].variables["t"]))
        if "pre" not in man:
            # presynaptic indices in the underlying group (not the source subgroup)
            man["pre"] = {k: fname(r[k].variables["_synaptic_pre"]) for k in ("Ce", "Ci")}
    device.build(directory=OUT, compile=False, run=False)
    man["sources"] = sorted(os.path.relpath(os.path.join(d, f), OUT)
                            for d, _, fs in os.walk(OUT) for f in fs
                            if f.endswith((".cpp", ".c")) and "results" not in d)
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump(man, f, indent=1)
    print("generated", OUT, len(man["sources"]), "sources")


if __name__ == "__main__":
    if sys.argv[1:2] == ["--one"]:
        generate(sys.argv[2], int(sys.argv[3]))
    else:
        import subprocess
        for item in sys.argv[1:] or DEFAULT:
            w, t = item.split(":")
            subprocess.run([sys.executable, os.path.abspath(__file__), "--one", w, t], check=True)
