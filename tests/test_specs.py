"""Committed specs: structure, code generation, and (where Brian2 is
importable) equality with what the b200 device extracts from the scripts."""
import json
import os
import subprocess
import sys

import pytest

from brian2_gb300 import codegen, workloads
from conftest import ROOT, brian_importable

NAMES = sorted(f[:-5] for f in os.listdir(workloads.SPECS) if f.endswith(".json"))


@pytest.mark.parametrize("name", NAMES)
def test_spec_renders(name):
    spec = workloads.load_spec(name)
    src = codegen.render_model(spec)
    assert "b200_step_kernel" in src and '#include "b200_host.h"' in src
    for g in spec["groups"]:
        for blk in ("update", "threshold"):
            assert g.get(blk), f"{name}: group without {blk}"
    for p in spec["pathways"]:
        assert "_b200_atomic_add" in p["on_pre"]["vector_device"]
        assert "_b200_atomic_add" not in p["on_pre"]["vector"]


def test_scalar_outputs_parse():
    code = "const double dt = _ptr_array_defaultclock_dt[0];\nconst float _lio_1 = exp(1.0f*(- dt)/taue);\ndouble x;"
    assert codegen.scalar_outputs(code) == [("double", "dt"), ("float", "_lio_1"), ("double", "x")]


@pytest.mark.skipif(not brian_importable(), reason="brian2 not importable here")
def test_specs_are_what_the_device_extracts():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "brian2_gb300", "specs", "make_specs.py"), "--check"],
                       capture_output=True, text=True, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
