"""Reference fixture and plugin job of the adjoint benchmark's forward pass.

The network of the "adjoint gradients" configuration written as a Brian
script (``oracle/brian_configs.py:adjoint_network``: SpikeGeneratorGroup
inputs, exact-linear LIF hidden layer, readout by on_pre) is run by the
reference itself (``cpp_standalone``, one thread, strict IEEE flags), giving
``adjoint_forward_f64.npz`` (hidden spike raster, readout potentials after
every step); the same script under ``set_device('b200')`` in deferred mode
gives the job ``jobs/adjoint_forward``.  Run where the reference is
importable::

    bash oracle/make_ref_env.sh <reference checkout>
    PYTHONPATH=oracle/_ref/pyenv python tests/golden/make_adjoint_forward.py
"""
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(ROOT, "oracle", "_ref", "golden_build")
STRICT = ['-w', '-O3', '-std=c++17', '-ffp-contract=off', '-fno-fast-math']


def one(device_name):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    from brian2 import set_device, device, prefs, defaultclock, ms
    import brian_configs as bc
    d = os.path.join(BUILD, f"adjoint_forward_{device_name}")
    shutil.rmtree(d, ignore_errors=True)
    if device_name == "b200":
        import brian2_gb300.brian_device  # noqa: F401  (registers the device)
        set_device("b200", directory=d, build_on_run=True, b200_defer=True)
    else:
        set_device("cpp_standalone", directory=d, build_on_run=True)
    prefs.devices.cpp_standalone.openmp_threads = 0
    prefs.codegen.cpp.extra_compile_args_gcc = STRICT
    prefs.core.default_float_dtype = np.float64
    defaultclock.dt = 0.1 * ms
    r = bc.adjoint_network()
    if device_name == "b200":
        out = os.path.join(HERE, "jobs", "adjoint_forward")
        shutil.rmtree(out, ignore_errors=True)
        shutil.copytree(device.b200_job_dir, out)
        print("job ->", out)
        return
    spk = r["spikes"]
    ts = np.round(np.asarray(spk.t_[:]) / 1e-4).astype(np.int32)
    vo = np.asarray(r["readout"].v_[:]).T.copy()  # [steps, n_o]
    np.savez_compressed(os.path.join(HERE, "adjoint_forward_f64.npz"), spk_i=np.asarray(spk.i[:], dtype=np.int32),
                        spk_ts=ts, vo=vo, v=np.asarray(r["P"].v_[:]), I=np.asarray(r["P"].I_[:]))
    meta = dict(case="adjoint_forward_f64", n_spikes=int(len(ts)), n_steps=int(vo.shape[0]),
                run_time_s=float(device._last_run_time), float_dtype="float64")
    with open(os.path.join(HERE, "adjoint_forward_f64.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("fixture:", meta)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--one"]:
        one(sys.argv[2])
        sys.exit(0)
    os.makedirs(BUILD, exist_ok=True)
    for dev in ("cpp_standalone", "b200"):
        subprocess.run([sys.executable, os.path.abspath(__file__), "--one", dev], check=True)
