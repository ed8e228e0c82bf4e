"""Compiles and times the reference's generated ``cpp_standalone`` projects.

Test infrastructure only: the timed CPU baseline beside the GPU numbers (the
reference's own OpenMP step loop on the host cores).  The projects under
``oracle/_ref/standalone_<workload>_t<threads>/`` are written by
``make_ref_standalone.py`` from the reference's code generator, one per
workload and OpenMP thread count; this module compiles them with the
reference's default GCC options for this architecture
(``brian2/codegen/cpp_prefs.py:109-116``) minus ``-march=native`` (kept
portable), plus ``-fopenmp``, and runs them.  The run time is the reference's
own measurement of its step loop: ``Network::_last_run_time`` (written to
``results/last_run_info.txt`` by ``templates/objects.cpp:364-371``) for the
whole run, and for a run that reports its progress the elapsed times its report
function prints (the same ``elapsed_realtime``,
``templates/network.cpp:59-121``); construction and file output are outside
it.  Synaptic events are counted from the run's own results: the out-degree of
every spiking source, from the synapses' presynaptic index arrays, and for a
run that reports its progress the spikes of each interval between reports from
the monitor's spike times.
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


def project(threads: int, workload: str = "delays") -> str:
    return os.path.join(REF, f"standalone_{workload}_t{threads}")


def variants(workload: str = "delays") -> list[int]:
    """OpenMP thread counts of the generated projects of a workload present here."""
    out = []
    pre = f"standalone_{workload}_t"
    if os.path.isdir(REF):
        for d in os.listdir(REF):
            if d.startswith(pre) and d[len(pre):].isdigit() and os.path.exists(os.path.join(REF, d, "manifest.json")):
                out.append(int(d[len(pre):]))
    return sorted(out)


def workloads() -> list[tuple[str, int]]:
    """(workload, threads) of every generated project present here."""
    out = []
    if os.path.isdir(REF):
        for d in sorted(os.listdir(REF)):
            if d.startswith("standalone_") and os.path.exists(os.path.join(REF, d, "manifest.json")):
                w, t = d[len("standalone_"):].rsplit("_t", 1)
                out.append((w, int(t)))
    return out


def available(workload: str = "delays") -> bool:
    return bool(variants(workload))


def all_threads(workload: str = "delays") -> int:
    """The largest generated thread count this host has cores for (the
    smallest one when it has fewer cores than any)."""
    v = variants(workload)
    fit = [t for t in v if t <= (os.cpu_count() or 1)]
    return max(fit) if fit else min(v)


def manifest(threads: int, workload: str = "delays") -> dict:
    with open(os.path.join(project(threads, workload), "manifest.json")) as f:
        return json.load(f)


def binary_path(threads: int, workload: str = "delays") -> str:
    return os.path.join(project(threads, workload), f"main_{platform.machine()}")


def build_all(jobs: int = 0) -> list[str]:
    """Compiles every generated project present here, all source files of all
    projects in one pool of g++ processes; returns the binaries' paths."""
    todo = [(w, t) for w, t in workloads() if not os.path.exists(binary_path(t, w))]
    units = [(w, t, src) for w, t in todo for src in manifest(t, w)["sources"]]
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(project(u[1], u[0]), u[2]), units))
    for w, t in todo:
        _link(binary_path(t, w), [o for (w2, t2, _), o in zip(units, objs) if (w2, t2) == (w, t)])
    return [binary_path(t, w) for w, t in workloads()]


def _compile(PROJECT, src):
    cxx = shutil.which("g++") or "g++"
    objdir = os.path.join(PROJECT, f"_obj_{platform.machine()}")
    os.makedirs(objdir, exist_ok=True)
    obj = os.path.join(objdir, src.replace("/", "__") + ".o")
    lang = ["-x", "c++"] if src.endswith(".c") else []
    r = subprocess.run([cxx] + FLAGS + ["-I", PROJECT, "-c"] + lang + [os.path.join(PROJECT, src), "-o", obj],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"compiling {src} failed:\n{r.stderr[-2000:]}")
    return obj


def _link(out, objs):
    cxx = shutil.which("g++") or "g++"
    tmp = out + f".tmp{os.getpid()}"
    r = subprocess.run([cxx] + objs + ["-fopenmp", "-o", tmp], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"linking the reference project failed:\n{r.stderr[-2000:]}")
    os.replace(tmp, out)


def build(threads: int, jobs: int = 0, workload: str = "delays") -> str:
    """Compiles one project (one g++ per source file, in parallel); returns the
    binary's path.  Rebuilds only when the binary is missing."""
    out = binary_path(threads, workload)
    if os.path.exists(out):
        return out
    PROJECT = project(threads, workload)
    srcs = manifest(threads, workload)["sources"]
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda src: _compile(PROJECT, src), srcs))
    _link(out, objs)
    return out


def run(threads: int, timeout: float = 1200.0, workload: str = "delays") -> dict:
    """Runs one compiled project once; returns its step-loop time, simulated
    steps, spikes and synaptic events -- over its (last) run, and, for a
    project whose run reports its progress, per interval between consecutive
    reports (``samples``; the report function is called with the run's
    elapsed time and completed fraction, ``templates/network.cpp:59-121``)."""
    man = manifest(threads, workload)
    PROJECT = project(threads, workload)
    res = os.path.join(PROJECT, "results")
    os.makedirs(res, exist_ok=True)
    try:
        r = subprocess.run([binary_path(threads, workload)], cwd=PROJECT, capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode:
            raise RuntimeError(f"reference project exited with {r.returncode}:\n{r.stdout[-1000:]}{r.stderr[-1000:]}")
        if man.get("networks"):
            return _run_networks(man, res, r.stdout)
        with open(os.path.join(res, "last_run_info.txt")) as f:
            last_time, frac = (float(x) for x in f.read().split())
        N, dt = man["N"], man["dt"]
        spk = np.fromfile(os.path.join(res, man["spike_i"]), dtype=np.int32)
        outdeg = np.zeros(N, np.int64)
        for k, fname in man["pre"].items():
            pre = np.fromfile(os.path.join(res, fname), dtype=np.int32)
            outdeg += np.bincount(pre, minlength=N)
            del pre
        ev = outdeg[spk]
        n_run = int(round(man["duration_ms"] * 1e-3 / dt))
        done = int(round(n_run * frac))
        samples = []
        if man.get("spike_t"):
            step = np.rint(np.fromfile(os.path.join(res, man["spike_t"]), dtype=np.float64) / dt).astype(np.int64)
        else:  # (a project of one run from its start)
            step = None
        s0 = int(round(man.get("warmup_ms", 0.0) * 1e-3 / dt))  # first step of the reported run
        if step is not None:
            in_run = (step >= s0) & (step < s0 + done)
            total = dict(run_time_s=last_time, steps=done, spikes=int(in_run.sum()), events=int(ev[in_run].sum()))
        else:
            total = dict(run_time_s=last_time, steps=done, spikes=int(spk.size), events=int(ev.sum()))
        if man.get("run_mark") and step is not None:
            rep = [(float(a), float(b)) for ln in r.stdout.splitlines() if ln.startswith(man["run_mark"] + " ")
                   for a, b in [ln.split()[1:3]]]
            for (e0, c0), (e1, c1) in zip(rep, rep[1:]):
                a, b = s0 + int(round(c0 * n_run)), s0 + int(round(c1 * n_run))
                if b > a and e1 > e0:
                    m = (step >= a) & (step < b)
                    samples.append(dict(run_time_s=e1 - e0, steps=b - a, spikes=int(m.sum()),
                                        events=int(ev[m].sum())))
    finally:
        shutil.rmtree(res, ignore_errors=True)  # every array of the run: up to many GB
    return dict(total, threads=man["threads"], sim_s=total["steps"] * dt, samples=samples, N=man["N"],
                K=man.get("K"), float_dtype=man.get("float_dtype", "float64"))


def _run_networks(man, res, stdout):
    """A project of several networks run one after another: each run's own
    time is the elapsed time its report function got at the end of the run
    (completed fraction 1; the call at its start has fraction 0,
    ``templates/network.cpp:51-52, 119-120``)."""
    ends = [float(ln.split()[1]) for ln in stdout.splitlines()
            if ln.startswith(man["run_mark"] + " ") and float(ln.split()[2]) >= 1.0]
    nets = man["networks"]
    if len(ends) != len(nets):
        raise RuntimeError(f"expected {len(nets)} end-of-run reports, found {len(ends)}")
    steps = int(round(man["duration_ms"] * 1e-3 / man["dt"]))
    per = []
    for n, t in zip(nets, ends):
        spk = np.fromfile(os.path.join(res, n["spike_i"]), dtype=np.int32)
        outdeg = np.zeros(n["N"], np.int64)
        for fname in n["pre"].values():
            outdeg += np.bincount(np.fromfile(os.path.join(res, fname), dtype=np.int32), minlength=n["N"])
        per.append(dict(N=n["N"], run_time_s=t, steps=steps, spikes=int(spk.size), events=int(outdeg[spk].sum())))
    return dict(run_time_s=float(sum(p["run_time_s"] for p in per)), steps=steps * len(per),
                spikes=sum(p["spikes"] for p in per), events=sum(p["events"] for p in per),
                threads=man["threads"], networks=per, sweep_networks=man.get("sweep_networks"),
                sweep_indices=man.get("sweep_indices"), float_dtype=man.get("float_dtype", "float64"))
