"""Generate the golden fixtures by running the reference Brian2 itself.

Each case builds a workload from ``oracle/brian_configs.py`` with Brian2's own
``cpp_standalone`` device, single-threaded (OpenMP changes the random stream,
``brian2/devices/cpp_standalone/codeobject.py:135-155``), with strict IEEE
compile flags so the results are the reference's exact arithmetic.  It stores:

* ``<case>.npz``: spike raster (neuron index, integer time step), initial and
  final state variables, and (small cases only) the synapse arrays;
* ``<case>.json``: sizes, counts and SHA-256 digests of the synapse arrays
  (pre, post, quantised delays) so the full construction is pinned even where
  the arrays themselves are too large to commit.

Run where the reference is importable (it is not needed afterwards)::

    bash oracle/make_ref_env.sh <reference checkout>
    PYTHONPATH=oracle/_ref/pyenv python tests/golden/make_golden.py [case ...]
"""
import hashlib
import json
import os
import shutil
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
BUILD = os.path.join(ROOT, "oracle", "_ref", "golden_build")

STRICT = ['-w', '-O3', '-std=c++17', '-ffp-contract=off', '-fno-fast-math']


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# name: (builder, kwargs, float dtype, store synapse arrays?)
CASES = {
    "cuba_f64": ("cuba", dict(N=4000, duration_ms=1000.0, seed_value=1234), "float64", False),
    "cuba_small_f64": ("cuba", dict(N=500, duration_ms=500.0, seed_value=7), "float64", True),
    "cobahh_f64": ("cobahh", dict(N=4000, duration_ms=100.0, seed_value=1234), "float64", False),
    "cobahh_f32": ("cobahh", dict(N=4000, duration_ms=100.0, seed_value=1234), "float32", False),
    "cobahh_small_f64": ("cobahh", dict(N=400, duration_ms=100.0, seed_value=3), "float64", True),
    "delays_f64": ("cuba_delays", dict(N=10000, K=1000, duration_ms=200.0, seed_value=1234), "float64", False),
    "delays_small_f64": ("cuba_delays", dict(N=2000, K=100, duration_ms=300.0, seed_value=5), "float64", True),
    # the full simulated second of the benchmark configurations
    "cobahh_1s_f64": ("cobahh", dict(N=4000, duration_ms=1000.0, seed_value=1234), "float64", False),
    "delays_1s_f64": ("cuba_delays", dict(N=10000, K=1000, duration_ms=1000.0, seed_value=1234), "float64", False),
}


def run_phase(name, phase):
    """One Brian2 build+run per process (the standalone device runs once)."""
    from brian2 import set_device, device, prefs, defaultclock, ms
    import brian_configs as bc
    builder, kw, fdt, store_syn = CASES[name]
    out = {}
    meta = {}
    dur = 0.0 if phase == "init" else kw["duration_ms"]
    if True:
        d = os.path.join(BUILD, f"{name}_{phase}")
        shutil.rmtree(d, ignore_errors=True)
        set_device('cpp_standalone', directory=d, build_on_run=True)
        prefs.devices.cpp_standalone.openmp_threads = 0
        prefs.codegen.cpp.extra_compile_args_gcc = STRICT
        prefs.core.default_float_dtype = getattr(np, fdt)
        defaultclock.dt = 0.1 * ms
        args = dict(kw); args["duration_ms"] = dur
        r = getattr(bc, builder)(**args)
        P = r["P"]
        paths = {k: v for k, v in r.items() if k in ("Ce", "Ci", "S")}
        if phase == "init":
            out["v0"] = np.asarray(P.v_[:]).copy()
            syn = {}
            for k, S in sorted(paths.items()):
                pre = np.asarray(S.i[:], dtype=np.int32)
                post = np.asarray(S.j[:], dtype=np.int32)
                e = dict(n=int(len(pre)), pre_sha=sha(pre), post_sha=sha(post))
                dl = np.asarray(S.delay_[:])
                if dl.size > 1:
                    slots = (dl / 1e-4 + 0.5).astype(np.int32)
                    e["delay_slot_sha"] = sha(slots)
                    e["delay_slot_minmax"] = [int(slots.min()), int(slots.max())]
                    if store_syn:
                        out[f"{k}_delay"] = dl.copy()
                if "w" in S.variables:
                    w = np.asarray(S.w_[:])
                    e["w_sha"] = sha(w)
                    if store_syn:
                        out[f"{k}_w"] = w.copy()
                if store_syn:
                    out[f"{k}_pre"] = pre
                    out[f"{k}_post"] = post
                syn[k] = e
            meta.update(case=name, builder=builder, kwargs=kw, float_dtype=fdt, dt=1e-4,
                        N=int(len(P)), synapses=syn)
        else:
            spk = r["spikes"]
            t = np.asarray(spk.t_[:])
            ts = np.round(t / 1e-4).astype(np.int32)
            assert np.array_equal(ts.astype(np.float64) * 1e-4, t), "t is not timestep*dt"
            out["spk_i"] = np.asarray(spk.i[:], dtype=np.int32)
            out["spk_ts"] = ts
            for var in ("v", "ge", "gi", "m", "n", "h"):
                if var in P.variables:
                    out[var] = np.asarray(getattr(P, var + "_")[:]).copy()
            rate = np.asarray(r["rate"].rate_[:])
            meta["rate_sha"] = sha(rate)
            meta["n_steps"] = int(len(rate))
            meta["n_spikes"] = int(len(ts))
            meta["run_time_s"] = float(device._last_run_time)
    np.savez(os.path.join(BUILD, f"{name}_{phase}.npz"), **out)
    with open(os.path.join(BUILD, f"{name}_{phase}.json"), "w") as f:
        json.dump(meta, f)


def run_case(name):
    import subprocess
    out, meta = {}, {}
    for phase in ("init", "run"):
        subprocess.run([sys.executable, os.path.abspath(__file__), "--phase", name, phase],
                       check=True)
        with np.load(os.path.join(BUILD, f"{name}_{phase}.npz")) as z:
            out.update({k: z[k] for k in z.files})
        with open(os.path.join(BUILD, f"{name}_{phase}.json")) as f:
            meta.update(json.load(f))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(name, meta["n_spikes"], "spikes", {k: v["n"] for k, v in meta["synapses"].items()},
          f"{meta['run_time_s']:.3f}s", flush=True)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--phase"]:
        run_phase(sys.argv[2], sys.argv[3])
        sys.exit(0)
    names = sys.argv[1:] or list(CASES)
    os.makedirs(BUILD, exist_ok=True)
    for n in names:
        t0 = time.time()
        run_case(n)
        print(f"  ({time.time() - t0:.1f}s wall)", flush=True)
