"""Every committed spec compiles for sm_103a (nvcc cross-compiles without a GPU)."""
import os
from concurrent.futures import ThreadPoolExecutor

from brian2_gb300 import native, workloads


def test_all_model_libraries_build():
    names = sorted(f[:-5] for f in os.listdir(workloads.SPECS) if f.endswith(".json"))
    with ThreadPoolExecutor(max_workers=8) as ex:
        paths = list(ex.map(lambda n: native.build_model(workloads.load_spec(n)), names))
    assert all(os.path.exists(p) for p in paths)


def test_construction_libraries_build():
    assert os.path.exists(native.build_construct())
    assert os.path.exists(native.build_scale())
