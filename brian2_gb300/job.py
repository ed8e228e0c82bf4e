"""A network run as a self-contained job directory (no Brian2 needed).

``set_device('b200')`` (:mod:`brian2_gb300.brian_device`) writes, after
Brian's standalone ``main`` has built the network, a job directory:

* ``spec.json``: the network spec (groups, variables, Brian's generated code
  snippets, pathways, monitors, namespace constants);
* ``init.npz``: the initial state written by ``main`` (group variables,
  spike generators' time bins, neuron indices, period and cursor, synapse indices, quantised delays and synaptic variables, monitor ranges and
  recorded indices, the clock's time step);
* ``job.json``: dt, the step counts of the recorded ``run()`` calls and the
  launch options.

:func:`run_job` executes it on the GPU through the C ABI and writes ``out.npz``
(final state, synaptic variables, monitor contents, device time); the plugin
turns that into the standalone results files.  The split is the reference's
own: ``device.build`` writes a project, the project runs where it is compiled,
and results come back as files (``brian2/devices/cpp_standalone/device.py:
1184-1351``).  So a network built where Brian2 is installed can run on a GPU
host that only has this package::

    python -m brian2_gb300.job <job directory> [--threads T] [--ctas C]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np


def write_job(directory, spec, init, runs, dt, options=None, actions=None):
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "spec.json"), "w") as f:
        json.dump(spec, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(directory, "init.npz"), **init)
    job = dict(dt=float(dt), runs=[int(r) for r in runs], options=dict(options or {}))
    if actions:
        job["actions"] = list(actions)
    with open(os.path.join(directory, "job.json"), "w") as f:
        json.dump(job, f, indent=1)


def apply_actions(job, init, after, download, upload):
    """The script's assignments after run `after` (job["actions"]: a group's
    state variable or a pathway's synaptic variable, all of it or at indices):
    download(kind, obj, var) -> array, upload(kind, obj, var, array)."""
    for j, a in enumerate(job.get("actions", [])):
        if a["after"] != after:
            continue
        cur = download(a["kind"], a["obj"], a["var"])
        vals = np.asarray(init[f"act{j}_values"])
        if a["indexed"]:
            cur[np.asarray(init[f"act{j}_index"], np.int64)] = vals.astype(cur.dtype)
        else:
            cur[...] = np.broadcast_to(vals.astype(cur.dtype), cur.shape)
        upload(a["kind"], a["obj"], a["var"], cur)


def _format_time(seconds):
    """The reference's progress-report time format (d h m s, or "< 1s")."""
    remaining, parts = float(seconds), []
    for div, letter in ((86400, "d"), (3600, "h"), (60, "m"), (1, "s")):
        k = int(remaining / div)
        remaining -= k * div
        if k > 0 or parts:
            parts.append(f"{k}{letter}")
    return " ".join(parts) if parts else "< 1s"


def _report(stream, elapsed, completed, start, duration):
    """A progress line as the reference's standard report function prints it
    (brian2/devices/cpp_standalone/device.py:1843-1887), to stdout or stderr."""
    out = sys.stderr if stream == "stderr" else sys.stdout
    if completed == 0.0:
        print(f"Starting simulation at t={start:g} s for duration {duration:g} s", file=out, flush=True)
        return
    line = f"{completed * duration:g} s ({int(completed * 100.0)}%) simulated in {_format_time(elapsed)}"
    if completed < 1.0:
        line += f", estimated {_format_time(int((1 - completed) / completed * elapsed + 0.5))} remaining."
    print(line, file=out, flush=True)


def load_job(directory):
    with open(os.path.join(directory, "spec.json")) as f:
        spec = json.load(f)
    with open(os.path.join(directory, "job.json")) as f:
        job = json.load(f)
    with np.load(os.path.join(directory, "init.npz")) as z:
        init = {k: z[k] for k in z.files}
    return spec, init, job


def run_job(directory, threads=None, ctas_per_inst=None, write=True, owner=None, profile=None, push=None):
    """Runs a job on the GPU; returns (and writes as out.npz) its outputs.
    `owner`, `push`: delivery modes (True, False, "auto"; None keeps the default);
    `profile`: record the device profile (None: as the job's options say, set
    by run(profile=True)) -- its slots' SM cycles in prof_names/prof_cycles."""
    from .runtime import Model, Network
    spec, init, job = load_job(directory)
    opts = dict(job.get("options", {}))
    dt = job["dt"]
    model = Model.get(spec)
    sizes = [int(init[f"g{gi}_N"]) for gi in range(len(spec["groups"]))]
    net = Network(model, [sizes], dt)
    threads = threads or opts.get("threads") or (1024 if max(sizes) <= 8192 else 256)
    ctas = ctas_per_inst or opts.get("ctas_per_inst") or 1
    net.configure(threads=threads, ctas_per_inst=ctas)
    if owner is not None:
        net.set_owner(owner)
    if push is not None:
        net.set_push(push)
    for gi, g in enumerate(spec["groups"]):
        for v in g["vars"] if g.get("alias_of") is None else []:  # (a custom event's group shares them)
            net.upload(0, gi, v["name"], init[f"g{gi}_{v['name']}"])
        if g.get("generator"):
            net.set_generator(0, gi, init[f"g{gi}_gen_bins"], init[f"g{gi}_gen_index"],
                              int(init[f"g{gi}_gen_period"]), int(init[f"g{gi}_gen_last"]))
    for pi, p in enumerate(spec.get("pathways", [])):
        steps = init[f"p{pi}_delay_steps"] if f"p{pi}_delay_steps" in init else None
        net.set_synapses(0, pi, init[f"p{pi}_pre"], init[f"p{pi}_post"], steps, int(init[f"p{pi}_scalar_delay"]),
                         tuple(int(x) for x in init[f"p{pi}_src_range"]),
                         tuple(int(x) for x in init[f"p{pi}_tgt_range"]))
        for v in p.get("vars", []) if p.get("alias", -1) < 0 else []:  # (an alias shares its owner's)
            net.upload_synapse_var(0, pi, v["name"], init[f"p{pi}_{v['name']}"])
    for mi in range(len(spec.get("spike_monitors", []))):
        net.set_spikemon_range(0, mi, *(int(x) for x in init[f"sm{mi}_range"]))
    for mi in range(len(spec.get("rate_monitors", []))):
        net.set_ratemon_range(0, mi, *(int(x) for x in init[f"rm{mi}_range"]))
    for mi, m in enumerate(spec.get("state_monitors", [])):
        net.set_statemon(0, mi, init[f"stm{mi}_idx"], list(init[f"stm{mi}_vars"]))
    ts0 = int(init["ts0"])
    net.set_step(0, ts0)
    if spec.get("draws"):  # the reference's generator, where the step loop starts drawing
        net.set_rng(0, init["rng_words"], int(init["rng_position"]), init.get("rng_gauss"))
    net.reset_monitors(0)
    profile = bool(opts.get("profile")) if profile is None else bool(profile)
    if profile:  # per-phase SM cycles of the step kernel (run(profile=True))
        net.set_profiling(True)
    total_ms, kernel_ms, t0 = 0.0, 0.0, time.time()
    def download(kind, obj, var):
        return net.download(0, obj, var) if kind == "group" else net.download_synapse_var(0, obj, var)

    def upload(kind, obj, var, arr):
        (net.upload if kind == "group" else net.upload_synapse_var)(0, obj, var, arr)

    reports = opts.get("reports") or [None] * len(job["runs"])
    periods = opts.get("report_periods") or [10.0] * len(job["runs"])
    for k, n in enumerate(job["runs"]):
        if reports[k]:
            _report(reports[k], 0.0, 0.0, net.step(0) * dt, int(n) * dt)
        t_run = time.time()
        done = 0
        while done < int(n):  # (a run reporting its progress: pieces of about one report period)
            piece = int(n) - done
            if reports[k]:
                piece = min(piece, 1000)
            net.run(piece)
            done += piece
            total_ms += net.last_run_ms()
            kernel_ms += net.last_kernel_ms()
            if reports[k] and done < int(n) and time.time() - t_run > periods[k]:
                _report(reports[k], time.time() - t_run, done / int(n), (net.step(0) - done) * dt, int(n) * dt)
        if reports[k]:
            _report(reports[k], time.time() - t_run, 1.0, (net.step(0) - int(n)) * dt, int(n) * dt)
        apply_actions(job, init, k, download, upload)  # the script's assignments after this run
    out = dict(device_ms=np.float64(total_ms), wall_s=np.float64(time.time() - t0), ts_end=np.int64(net.step(0)),
               ts0=np.int64(ts0), owner=np.int64(net.owner_active()), kernel_ms=np.float64(kernel_ms),
               push=np.int64(net.push_active()))
    if profile:
        prof = net.profile(0)
        out["prof_names"] = np.array(list(prof), dtype=str)
        out["prof_cycles"] = np.array(list(prof.values()), dtype=np.float64)
    for gi, g in enumerate(spec["groups"]):
        for v in g["vars"] if g.get("alias_of") is None else []:
            out[f"g{gi}_{v['name']}"] = net.download(0, gi, v["name"])
        if g.get("generator"):
            out[f"g{gi}_gen_last"] = np.int64(net.generator_cursor(0, gi))
    for pi, p in enumerate(spec.get("pathways", [])):
        for v in p.get("vars", []) if p.get("alias", -1) < 0 else []:
            out[f"p{pi}_{v['name']}"] = net.download_synapse_var(0, pi, v["name"])
    for mi, m in enumerate(spec.get("spike_monitors", [])):
        i, ts, cnt = net.spikes(0, mi)
        out[f"sm{mi}_i"], out[f"sm{mi}_ts"], out[f"sm{mi}_count"] = i, ts, cnt
        if m.get("vars"):
            out[f"sm{mi}_vals"] = net.spike_values(0, mi)
    for mi in range(len(spec.get("rate_monitors", []))):
        out[f"rm{mi}_counts"] = net.rate_counts(0, mi)
    for mi in range(len(spec.get("state_monitors", []))):
        out[f"stm{mi}_trace"] = net.state_trace(0, mi)
    net.close()
    if write:
        np.savez(os.path.join(directory, "out.npz"), **out)
    return out


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="run a b200 job directory on the GPU")
    ap.add_argument("directory")
    ap.add_argument("--threads", type=int, default=None)
    ap.add_argument("--ctas", type=int, default=None)
    a = ap.parse_args(argv)
    out = run_job(a.directory, a.threads, a.ctas)
    print(f"{a.directory}: steps {int(out['ts0'])}..{int(out['ts_end'])}, {float(out['device_ms']):.2f} ms on the device")


if __name__ == "__main__":
    sys.exit(main())
