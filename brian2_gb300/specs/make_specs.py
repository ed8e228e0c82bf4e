"""Regenerates the committed network specs from the Brian2 scripts.

Each spec is what ``set_device('b200')`` extracts from the corresponding script
in ``oracle/brian_configs.py`` (Brian's own equations -> abstract code ->
``B200CodeGenerator`` snippets).  They are committed so that machines without
Brian2 (the GPU hosts) can build the same models.  Needs an importable brian2::

    PYTHONPATH=oracle/_ref/pyenv python brian2_gb300/specs/make_specs.py [--check]
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# spec name -> (builder in oracle/brian_configs.py, float dtype, builder kwargs)
SPECS = {
    "cuba_f64": ("cuba", "float64", dict(N=100)),
    "cuba_f32": ("cuba", "float32", dict(N=100)),
    "cobahh_f64": ("cobahh", "float64", dict(N=100)),
    "cobahh_f32": ("cobahh", "float32", dict(N=100)),
    "delays_f64": ("cuba_delays", "float64", dict(N=200, K=20)),
    "delays_f32": ("cuba_delays", "float32", dict(N=200, K=20)),
}


def generate(name):
    """One spec per process (a standalone device builds one network)."""
    code = f"""
import json, sys
sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {os.path.join(ROOT, 'oracle')!r})
import numpy as np
from brian2 import set_device, prefs, device
import brian2_gb300.brian_device as bd
import brian_configs as bc
builder, fdt, kw = {SPECS[name]!r}
set_device('b200', directory=None, build_on_run=False)
prefs.devices.cpp_standalone.openmp_threads = 0
prefs.core.default_float_dtype = getattr(np, fdt)
getattr(bc, builder)(duration_ms=1.0, **kw)
spec = bd.B200Device.public_spec(device.b200_runs[0]['spec'])
spec['name'] = {name!r}
print(json.dumps(spec, indent=1, sort_keys=True))
"""
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    if r.returncode:
        raise RuntimeError(r.stderr[-3000:])
    return json.loads(r.stdout[r.stdout.index("{"):])


if __name__ == "__main__":
    check = "--check" in sys.argv
    bad = 0
    for name in SPECS:
        spec = generate(name)
        path = os.path.join(HERE, name + ".json")
        if check:
            with open(path) as f:
                same = json.load(f) == spec
            print(name, "up to date" if same else "DIFFERS")
            bad += not same
        else:
            with open(path, "w") as f:
                json.dump(spec, f, indent=1, sort_keys=True)
                f.write("\n")
            print("wrote", path)
    sys.exit(1 if bad else 0)
