"""Generates the reference's own ``cpp_standalone`` projects of the CPU baseline.

Test infrastructure only (the timed CPU baseline; never on the product path).
Each project is a network with delays (in-degree 1000, delays uniform in
0.1-5 ms, ``brian_configs.cuba_delays``) written by the reference's code
generator for its OpenMP standalone path
(``brian2/devices/cpp_standalone/device.py``, ``openmp_threads`` preference),
so what runs on the host cores is the reference's generated step loop
unchanged.  Two workloads:

* ``delays`` -- the 10,000-neuron subnetwork, float64, one run of 1 s;
* ``delays1e6`` -- the headline network itself: 1,000,000 neurons, 1e9
  synapses, float32; a run of 50 ms lets the activity settle, then a run of
  100 ms (1000 clock steps) reports its progress through Brian's own progress
  report (``run(report=..., report_period=...)``: for the standalone device
  C++ code of the report function, ``device.py:1889-1907``, called from the
  step loop with the run's elapsed time and completed fraction about every
  0.5 s of wall time, ``templates/network.cpp:59-90``).  One execution thus
  gives many timed samples after a single construction.

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
# the marker the report function prints at each call: elapsed seconds and completed fraction
RUN_MARK = "REF_RUN_TIME"
REPORT = ('std::cout.precision(12); std::cout << "' + RUN_MARK +
          ' " << elapsed << " " << completed << std::endl;')
WORKLOADS = {
    # name: (N, K, float dtype, warm-up run in ms, reported run in ms, report period in s or None)
    "delays": (10_000, 1000, "float64", 0.0, 1000.0, None),
    "delays1e6": (1_000_000, 1000, "float32", 50.0, 100.0, 0.5),
}
DEFAULT = ("delays:1", "delays:16", "delays1e6:16")


def generate(workload, threads, seed_value=1234):
    """One project (the standalone device builds once per process)."""
    N, K, fdt, warm_ms, duration_ms, period = WORKLOADS[workload]
    OUT = os.path.join(HERE, "_ref", f"standalone_{workload}_t{threads}")
    sys.path.insert(0, HERE)
    import numpy as np
    from brian2 import set_device, device, prefs, defaultclock, ms
    import brian_configs as bc
    shutil.rmtree(OUT, ignore_errors=True)
    set_device("cpp_standalone", directory=OUT, build_on_run=False)
    prefs.devices.cpp_standalone.openmp_threads = int(threads)
    prefs.core.default_float_dtype = getattr(np, fdt)
    defaultclock.dt = 0.1 * ms
    r = bc.cuba_delays(N=N, K=K, duration_ms=duration_ms, seed_value=seed_value, warmup_ms=warm_ms,
                       report=REPORT if period else None, report_period_s=period or 10.0)
    device.build(directory=OUT, compile=False, run=False)
    man = dict(
        workload=workload, N=N, K=K, seed=seed_value, warmup_ms=warm_ms, duration_ms=duration_ms,
        report_period_s=period, dt=1e-4, threads=int(threads), float_dtype=fdt,
        run_mark=RUN_MARK if period else None,
        spike_i=device.get_array_filename(r["spikes"].variables["i"]),
        spike_t=device.get_array_filename(r["spikes"].variables["t"]),
        # presynaptic indices in the underlying group (not the source subgroup)
        pre={k: device.get_array_filename(r[k].variables["_synaptic_pre"]) for k in ("Ce", "Ci")},
        sources=sorted(os.path.relpath(os.path.join(d, f), OUT)
                       for d, _, fs in os.walk(OUT) for f in fs
                       if f.endswith((".cpp", ".c")) and "results" not in d),
    )
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
