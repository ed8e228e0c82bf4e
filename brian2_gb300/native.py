"""Building and loading the native libraries (in-tree, for sm_103a).

* model libraries: one per network spec, rendered by :mod:`brian2_gb300.codegen`
  and compiled by nvcc into ``brian2_gb300/_build/models/<name>_<hash>.so``;
* ``libb200_construct.so``: host construction with Brian's random stream (g++);
* ``libb200_scale.so``: device-side construction for networks too large for the
  host path (nvcc).

Nothing here falls back to a CPU implementation: if a library cannot be built
or loaded, the caller gets an exception.
"""
from __future__ import annotations

import ctypes
import fcntl
import hashlib
import os
import shutil
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

_lock = threading.Lock()
_loaded: dict[str, ctypes.CDLL] = {}


def nvcc_path() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the b200 device needs the CUDA toolkit")
    return p


def nvcc_flags(exact: bool = True, single: bool = False) -> list[str]:
    """exact: IEEE division and square root, no contraction into FMAs (the
    float64 models' bit-exactness with the reference needs all three).
    single (float32 models): no contraction either -- Brian's float32
    expressions keep their rounding order -- but the fast division and square
    root; float32 results are held to a stated error against the float64
    reference, not to bit-exactness."""
    flags = [ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xptxas", "-dlcm=cg",
             "-diag-suppress", "177,550,2361", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
             "-shared", f"-I{CSRC}"]
    if exact and single:
        flags += ["--fmad=false", "-prec-div=false", "-prec-sqrt=false"]
    elif exact:
        flags += ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"]
    return flags


def _sources_digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:12]


def _run(cmd, what):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building {what} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _locked_build(out: str, build_fn):
    """Builds `out` once across processes (file lock), atomically renamed."""
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if os.path.exists(out):
        return out
    lockf = out + ".lock"
    with open(lockf, "w") as lf:
        fcntl.flock(lf, fcntl.LOCK_EX)
        try:
            if not os.path.exists(out):
                tmp = out + f".tmp{os.getpid()}"
                build_fn(tmp)
                os.replace(tmp, out)
        finally:
            fcntl.flock(lf, fcntl.LOCK_UN)
    return out


def model_library_path(spec: dict) -> str:
    from .codegen import spec_hash
    deps = [os.path.join(CSRC, f) for f in ("b200_device.cuh", "b200_host.h")]
    tag = spec_hash(spec) + _sources_digest(deps + [os.path.join(HERE, "codegen.py"), os.path.abspath(__file__)])
    return os.path.join(BUILD, "models", f"{spec['name']}_{tag}.so")


def build_model(spec: dict) -> str:
    """Renders and compiles the model library of a spec; returns its path."""
    from .codegen import render_model
    out = model_library_path(spec)

    def _build(tmp):
        src = out[:-3] + ".cu"
        with open(src, "w") as f:
            f.write(render_model(spec))
        exact = not spec.get("fast_math", False)
        single = spec.get("float", "double") == "float"
        _run([nvcc_path()] + nvcc_flags(exact, single) + [src, "-o", tmp], f"model {spec['name']}")

    return _locked_build(out, _build)


def build_construct() -> str:
    src = os.path.join(CSRC, "b200_construct.cpp")
    out = os.path.join(BUILD, f"libb200_construct_{_sources_digest([src])}.so")
    cxx = shutil.which("g++") or "g++"
    return _locked_build(out, lambda tmp: _run(
        [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", src, "-o", tmp],
        "libb200_construct"))


def build_scale() -> str:
    src = os.path.join(CSRC, "b200_scale.cu")
    hdr = os.path.join(INCLUDE, "b200_scale.h")
    out = os.path.join(BUILD, f"libb200_scale_{_sources_digest([src, hdr, os.path.join(CSRC, 'b200_device.cuh')])}.so")
    return _locked_build(out, lambda tmp: _run(
        [nvcc_path()] + nvcc_flags(True) + [f"-I{INCLUDE}", src, "-o", tmp], "libb200_scale"))


def build_peaks() -> str:
    """libb200_peaks: the measured FMA throughput (the ALU roofline's peaks)."""
    src = os.path.join(CSRC, "b200_peaks.cu")
    hdr = os.path.join(INCLUDE, "b200_peaks.h")
    out = os.path.join(BUILD, f"libb200_peaks_{_sources_digest([src, hdr])}.so")
    return _locked_build(out, lambda tmp: _run(
        [nvcc_path(), ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", f"-I{INCLUDE}", src, "-o", tmp],
        "libb200_peaks"))


def build_adjoint() -> str:
    src = os.path.join(CSRC, "b200_adjoint.cu")
    out = os.path.join(BUILD, f"libb200_adjoint_{_sources_digest([src])}.so")
    return _locked_build(out, lambda tmp: _run(
        [nvcc_path()] + nvcc_flags(True) + [src, "-o", tmp], "libb200_adjoint"))


def load(path: str) -> ctypes.CDLL:
    with _lock:
        lib = _loaded.get(path)
        if lib is None:
            lib = ctypes.CDLL(path)
            _loaded[path] = lib
        return lib


def loaded_paths() -> list[str]:
    return sorted(_loaded)
