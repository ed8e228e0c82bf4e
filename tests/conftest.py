import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np

    def load(name):
        with open(os.path.join(GOLDEN, name + ".json")) as f:
            meta = json.load(f)
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        return meta, {k: z[k] for k in z.files}
    return load


def brian_importable():
    try:
        import brian2  # noqa: F401
        return True
    except Exception:
        return False
