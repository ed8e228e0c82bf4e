"""Compiles and times the reference's generated ``cpp_standalone`` project.

Test infrastructure only: the timed CPU baseline beside the GPU numbers (the
reference's own OpenMP step loop on the host cores).  The projects under
``oracle/_ref/standalone_delays_t<threads>/`` are written by
``make_ref_standalone.py`` from the reference's code generator, one per OpenMP
thread count; this module compiles them with the
reference's default GCC options for this architecture
(``brian2/codegen/cpp_prefs.py:109-116``) minus ``-march=native`` (kept
portable), plus ``-fopenmp``, and runs it.  The run time is the reference's own
measurement of its step loop (``Network::_last_run_time``, written to
``results/last_run_info.txt`` by ``templates/objects.cpp:364-371``), so
construction and file output are outside it.  Synaptic events are counted from
the run's own results: the out-degree of every spiking source, from the
synapses' presynaptic index arrays.
"""
from __future__ import annotations

import json
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
FLAGS = ["-w", "-O3", "-ffast-math", "-fno-finite-math-only", "-std=c++17", "-fopenmp"]


def project(threads: int) -> str:
    return os.path.join(REF, f"standalone_delays_t{threads}")


def variants() -> list[int]:
    """OpenMP thread counts of the generated projects present here."""
    out = []
    if os.path.isdir(REF):
        for d in os.listdir(REF):
            if d.startswith("standalone_delays_t") and os.path.exists(os.path.join(REF, d, "manifest.json")):
                out.append(int(d.rsplit("_t", 1)[1]))
    return sorted(out)


def available() -> bool:
    return bool(variants())


def all_threads() -> int:
    """The largest generated thread count this host has cores for (the
    smallest one when it has fewer cores than any)."""
    v = variants()
    fit = [t for t in v if t <= (os.cpu_count() or 1)]
    return max(fit) if fit else min(v)


def manifest(threads: int) -> dict:
    with open(os.path.join(project(threads), "manifest.json")) as f:
        return json.load(f)


def binary_path(threads: int) -> str:
    return os.path.join(project(threads), f"main_{platform.machine()}")


def build_all() -> list[str]:
    return [build(t) for t in variants()]


def build(threads: int, jobs: int = 0) -> str:
    """Compiles one project (one g++ per source file, in parallel); returns the
    binary's path.  Rebuilds only when the binary is missing."""
    out = binary_path(threads)
    if os.path.exists(out):
        return out
    PROJECT = project(threads)
    man = manifest(threads)
    cxx = shutil.which("g++") or "g++"
    objdir = os.path.join(PROJECT, f"_obj_{platform.machine()}")
    os.makedirs(objdir, exist_ok=True)

    def one(src):
        obj = os.path.join(objdir, src.replace("/", "__") + ".o")
        lang = ["-x", "c++"] if src.endswith(".c") else []
        r = subprocess.run([cxx] + FLAGS + ["-I", PROJECT, "-c"] + lang + [os.path.join(PROJECT, src), "-o", obj],
                           capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compiling {src} failed:\n{r.stderr[-2000:]}")
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, man["sources"]))
    tmp = out + f".tmp{os.getpid()}"
    r = subprocess.run([cxx] + objs + ["-fopenmp", "-o", tmp], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"linking the reference project failed:\n{r.stderr[-2000:]}")
    os.replace(tmp, out)
    return out


def run(threads: int, timeout: float = 600.0) -> dict:
    """Runs one compiled project once; returns its step-loop time, simulated
    steps, spikes and synaptic events."""
    man = manifest(threads)
    PROJECT = project(threads)
    res = os.path.join(PROJECT, "results")
    os.makedirs(res, exist_ok=True)
    r = subprocess.run([binary_path(threads)], cwd=PROJECT, capture_output=True, text=True, timeout=timeout)
    if r.returncode:
        raise RuntimeError(f"reference project exited with {r.returncode}:\n{r.stdout[-1000:]}{r.stderr[-1000:]}")
    with open(os.path.join(res, "last_run_info.txt")) as f:
        run_time, frac = (float(x) for x in f.read().split())
    spk = np.fromfile(os.path.join(res, man["spike_i"]), dtype=np.int32)
    N = man["N"]
    outdeg = np.zeros(N, np.int64)
    for k, fname in man["pre"].items():
        pre = np.fromfile(os.path.join(res, fname), dtype=np.int32)
        outdeg += np.bincount(pre, minlength=N)
    steps = int(round(man["duration_ms"] * 1e-3 / man["dt"] * frac))
    shutil.rmtree(res, ignore_errors=True)  # every array of the run: hundreds of MB
    return dict(run_time_s=run_time, steps=steps, spikes=int(spk.size), events=int(outdeg[spk].sum()),
                threads=man["threads"], sim_s=steps * man["dt"])
