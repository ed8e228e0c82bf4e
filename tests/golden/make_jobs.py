"""Job directories written by ``set_device('b200')`` for the golden cases.

Each case runs a workload script of ``oracle/brian_configs.py`` with the
``b200`` device plugin in deferred mode (``build(..., b200_defer=True)``):
Brian2 generates and runs the standalone ``main`` (network construction,
initial values), the plugin records the step loop as a spec and writes the job
(``spec.json``, ``init.npz``, ``job.json``) instead of running it.  The jobs
are committed under ``tests/golden/jobs/<case>/`` so that the GPU tests run
exactly what the plugin produced from the reference's own script, and compare
the result with the reference's fixture of the same case.

Run where the reference is importable (single-threaded, strict flags, as the
golden fixtures)::

    bash oracle/make_ref_env.sh <reference checkout>
    PYTHONPATH=oracle/_ref/pyenv python tests/golden/make_jobs.py
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(ROOT, "oracle", "_ref", "job_build")
STRICT = ['-w', '-O3', '-std=c++17', '-ffp-contract=off', '-fno-fast-math']

# case: (builder, kwargs) -- the same constructions as the golden fixtures
CASES = {
    "cuba_small_f64": ("cuba", dict(N=500, duration_ms=500.0, seed_value=7)),
    "delays_small_f64": ("cuba_delays", dict(N=2000, K=100, duration_ms=300.0, seed_value=5)),
    "cobahh_small_f64": ("cobahh", dict(N=400, duration_ms=100.0, seed_value=3)),
}


def one(name):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    from brian2 import set_device, device, prefs, defaultclock, ms
    import brian2_gb300.brian_device  # noqa: F401  (registers the device)
    import brian_configs as bc
    builder, kw = CASES[name]
    d = os.path.join(BUILD, name)
    shutil.rmtree(d, ignore_errors=True)
    set_device("b200", directory=d, build_on_run=True, b200_defer=True)
    prefs.devices.cpp_standalone.openmp_threads = 0
    prefs.codegen.cpp.extra_compile_args_gcc = STRICT
    prefs.core.default_float_dtype = np.float64
    defaultclock.dt = 0.1 * ms
    getattr(bc, builder)(**kw)
    out = os.path.join(HERE, "jobs", name)
    shutil.rmtree(out, ignore_errors=True)
    shutil.copytree(device.b200_job_dir, out)
    print(name, "->", out)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--one"]:
        one(sys.argv[2])
        sys.exit(0)
    for n in sys.argv[1:] or list(CASES):
        subprocess.run([sys.executable, os.path.abspath(__file__), "--one", n], check=True)
