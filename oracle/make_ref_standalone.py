"""Generates the reference's own ``cpp_standalone`` project of the CPU baseline.

Test infrastructure only (the timed CPU baseline; never on the product path).
The project is the 10,000-neuron network with delays (in-degree 1000, delays
uniform in 0.1-5 ms, ``brian_configs.cuba_delays``) written by the reference's
code generator for its OpenMP standalone path
(``brian2/devices/cpp_standalone/device.py``, ``openmp_threads`` preference),
so what runs on the host cores is the reference's generated step loop
unchanged.  Generation needs the reference importable, so it runs here::

    bash oracle/make_ref_env.sh <reference checkout>
    PYTHONPATH=oracle/_ref/pyenv python oracle/make_ref_standalone.py [threads ...]

Output (git-ignored, compiled where it runs by ``ref_standalone.build``): one
project per OpenMP thread count (the count is fixed at generation,
``brian2/devices/cpp_standalone/codeobject.py:17-40``), default 1 and 16, in
``oracle/_ref/standalone_delays_t<threads>/``, each with the generated sources
and ``manifest.json``, which names the result files (spike monitor indices and
the synapses' presynaptic indices) that the timing reads back.  The generated
``makefile`` is not used: its default flags include ``-march=native``.
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
THREADS = (1, 16)


def generate(threads, duration_ms=1000.0, N=10000, K=1000, seed_value=1234):
    """One project (the standalone device builds once per process)."""
    OUT = os.path.join(HERE, "_ref", f"standalone_delays_t{threads}")
    sys.path.insert(0, HERE)
    import numpy as np
    from brian2 import set_device, device, prefs, defaultclock, ms
    import brian_configs as bc
    shutil.rmtree(OUT, ignore_errors=True)
    set_device("cpp_standalone", directory=OUT, build_on_run=False)
    prefs.devices.cpp_standalone.openmp_threads = int(threads)
    prefs.core.default_float_dtype = np.float64
    defaultclock.dt = 0.1 * ms
    r = bc.cuba_delays(N=N, K=K, duration_ms=duration_ms, seed_value=seed_value)
    device.build(directory=OUT, compile=False, run=False)
    man = dict(
        workload="cuba_delays", N=N, K=K, seed=seed_value, duration_ms=duration_ms, dt=1e-4,
        threads=int(threads), float_dtype="float64",
        spike_i=device.get_array_filename(r["spikes"].variables["i"]),
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
        generate(int(sys.argv[2]))
    else:
        import subprocess
        for t in [int(x) for x in sys.argv[1:]] or THREADS:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--one", str(t)], check=True)
