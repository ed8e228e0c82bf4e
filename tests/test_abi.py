"""The C-ABI libraries load and export every symbol their headers declare
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

from brian2_gb300 import native, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(b200[sap]?_\w+)\s*\(", text)))


def exported(path):
    lib = ctypes.CDLL(path)
    return lib


@pytest.mark.parametrize("spec_name", ["cuba_f64"])
def test_model_library_exports_abi(spec_name):
    lib = exported(native.build_model(workloads.load_spec(spec_name)))
    names = declared("b200.h")
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_construct_library_exports_abi():
    lib = exported(native.build_construct())
    missing = [n for n in declared("b200_construct.h") if not hasattr(lib, n)]
    assert not missing, missing


def test_scale_library_exports_abi():
    lib = exported(native.build_scale())
    missing = [n for n in declared("b200_scale.h") if not hasattr(lib, n)]
    assert not missing, missing


def test_adjoint_library_exports_abi():
    lib = exported(native.build_adjoint())
    names = declared("b200_adjoint.h")
    assert len(names) == 7
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_model_name_without_device():
    lib = exported(native.build_model(workloads.load_spec("cuba_f64")))
    buf = ctypes.create_string_buffer(64)
    assert lib.b200_model_name(buf, 64) == 0
    assert buf.value == b"cuba_f64"


def test_peaks_library_exports_abi():
    lib = exported(native.build_peaks())
    names = declared("b200_peaks.h")
    assert names == ["b200p_fma_peak", "b200p_last_error"]
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
