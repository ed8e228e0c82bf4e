"""Benchmark of the clock-driven step loop on one GB300 (or N replicas).

Workload (default): the large CUBA network with delays -- 1,000,000 LIF neurons
(80/20 E/I), fixed in-degree 1000 (800 E + 200 I sources, 1e9 synapses),
per-synapse float32 weights, per-synapse delays uniform in 0.1-5.0 ms quantised
to dt = 0.1 ms, float32 state, exact-linear integration.  Synthetic data: the
network is constructed on the device from a seed.  One bench step = 1000 clock
steps (100 ms simulated), continuing the same simulation.

Printed (rank 0, one JSON line): synaptic events/s over the timed steps
(events = sum over emitted spikes of the source's out-degree), simulated
seconds per wall second, an end-to-end figure through the public API with host
buffers (state uploaded from pinned memory and the step's spikes read back every
step), the step kernel's roofline, and a CPU baseline: the reference's own
generated cpp_standalone project (OpenMP) of the 10,000-neuron subnetwork of
identical construction, a bounded sample that fits the default run (where that
project was not generated, the oracle instead).  On one GPU the line also
carries the other workloads, each measured in this run: CUBA 4000 (float64),
COBAHH 4000 (float64 and float32), the 256-network batched sweep against the
same networks run one after another, and the adjoint's forward+adjoint /
forward cost ratio; beside each, the reference's own generated project of the
same network timed on the host cores at 1 thread and at all cores
(``cpu_reference``).

--impl reference runs the reference's own step loop on the headline network
itself (1e6 neurons, 1e9 synapses, float32, its generated cpp_standalone
project with OpenMP on all host cores) and prints the same metric and config;
each of its steps is one progress-report interval of that run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_NEURONS = 1_000_000
K_IN = 1000
STEPS_PER_BENCH_STEP = 1000  # 100 ms simulated
WORKLOAD = "cuba_delays_1e6_k1000_f32"
METRIC = "synaptic_events_per_s"
UNIT = "events/s"


def reduce_ranks(dist, seconds, events):
    """Whole-job figures of a timed region run on every rank: the slowest rank's
    time and the events of all ranks (weak scaling: every rank simulates its
    own network)."""
    if dist is None:
        return float(seconds), float(events)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e = torch.tensor([float(events)], dtype=torch.float64)
    dist.all_reduce(e, op=dist.ReduceOp.SUM)
    return float(t.item()), float(e.item())


def sync_all(dist):
    """Barrier over the ranks and a device synchronisation on both sides of a
    timed region."""
    import torch
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 3 + k and s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def ncu_traffic(K, kernel="b200_step_kernel"):
    """DRAM bytes per launch (1000 clock steps of the 1e6-neuron network) of the
    step kernel (b200_step_kernel: classic delivery; b200_push_kernel: push
    mode) at in-degree K, from the committed ncu captures at in-degree 250 and
    500 (profiles/<kernel>_cuba_delays.json; the full-size network is too large
    for a capture), extrapolated linearly in K; or None."""
    name = {"b200_step_kernel": "step_kernel_cuba_delays.json",
            "b200_push_kernel": "push_kernel_cuba_delays.json"}.get(kernel, "")
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            d = json.load(f)
        fit = d["fit"]
        return fit["bytes_per_launch_at_in_degree_0"] + fit["bytes_per_launch_per_in_degree"] * K
    except Exception:
        return None


def cpu_baseline(max_seconds=20.0):
    """The reference's CPU step loop on a bounded sample of the same workload:
    the 10,000-neuron network of identical construction (in-degree 1000, delays
    0.1-5 ms), float64, 1 s simulated.  The reference's own generated
    cpp_standalone project (OpenMP) where it is present, else the oracle."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_standalone
    if ref_standalone.available():
        T = ref_standalone.all_threads()
        ref_standalone.build(T)
        r = ref_standalone.run(T)
        return {"value": r["events"] / r["run_time_s"], "unit": UNIT, "cores": r["threads"], "kind": "reference",
                "sample": f"reference cpp_standalone project (generated by the reference, g++ -O3 -ffast-math "
                          f"-fopenmp, {r['threads']} OpenMP threads) on the 10,000-neuron subnetwork of identical "
                          f"construction: {r['steps']} clock steps ({r['sim_s']:.2f} s simulated), "
                          f"{r['spikes']} spikes, {r['events']} events, step loop {r['run_time_s']:.2f} s",
                "sim_s_per_wall_s": r["sim_s"] / r["run_time_s"], "host_cpus": os.cpu_count(),
                "single_thread": _reference_single_thread(ref_standalone, T)}
    return cpu_baseline_port(max_seconds)


def _reference_single_thread(ref_standalone, T):
    """The same reference project without OpenMP parallelism (1 thread)."""
    if T == 1 or 1 not in ref_standalone.variants():
        return None
    ref_standalone.build(1)
    r = ref_standalone.run(1)
    return {"value": r["events"] / r["run_time_s"], "cores": 1, "step_loop_s": r["run_time_s"],
            "sim_s_per_wall_s": r["sim_s"] / r["run_time_s"]}


def cpu_baseline_port(max_seconds=20.0):
    """The oracle (single-threaded CPU restatement of the reference's step loop)
    on the same sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import oracle_from_built
    from brian2_gb300 import workloads as W
    spec = W.load_spec("delays_f64")
    b = W.build_delays(spec, N=10_000, K=K_IN, seed=1234)
    outdeg = np.zeros(10_000, np.int64)
    for s in b.synapses.values():
        outdeg += np.bincount(s["pre"] + s["src"][0], minlength=10_000)
    o = oracle_from_built(spec, b)
    o.run(500)  # warm-up: fill the delay ring
    i0 = len(o.spikes(0)[0])
    t0 = time.perf_counter()
    steps = 0
    while steps < 20000 and time.perf_counter() - t0 < max_seconds:
        o.run(500)
        steps += 500
        if time.perf_counter() - t0 > max_seconds / 2 and steps >= 2000:
            break
    dt = time.perf_counter() - t0
    i, ts, _ = o.spikes(0)
    ev = int(outdeg[i[i0:]].sum())
    return {"value": ev / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle (C++ restatement, float64) on the 10,000-neuron subnetwork of identical "
                      f"construction, {steps} clock steps ({steps * 1e-4:.2f} s simulated) in {dt:.2f} s wall",
            "sim_s_per_wall_s": steps * 1e-4 / dt}


def _outdegree(b, n):
    out = np.zeros(n, np.int64)
    for syn in b.synapses.values():
        out += np.bincount(syn["pre"] + syn["src"][0], minlength=n)
    return out


def extra_plain(name, builder, steps=10_000):
    """One plain network (1 s simulated) with the autotuned launch shape."""
    from brian2_gb300 import autotune, workloads as W
    spec = W.load_spec(name)
    b = builder(spec)
    n = sum(b.sizes)
    shape = autotune.tune(spec, [b])
    net = W.instantiate(spec, [b], threads=shape["threads"], ctas_per_inst=shape["ctas_per_inst"])
    net.run(steps)
    ms = net.last_kernel_ms()
    i, _, _ = net.spikes(0, 0)
    ev = int(_outdegree(b, n)[i].sum())
    net.close()
    return {"neurons": n, "clock_steps": steps, "device_ms": ms, "sim_s_per_wall_s": steps * 1e-4 / (ms * 1e-3),
            "events_per_s": ev / (ms * 1e-3), "spikes": int(len(i)), "us_per_clock_step": ms * 1e3 / steps,
            "launch_shape": {k: shape[k] for k in ("threads", "ctas_per_inst")}}


def extra_batched(steps=5000):
    """256 CUBA networks of uneven size (float32, 500 ms): one persistent
    graph-replayed launch (autotuned block size) against the same networks run
    one after another on the plain path, both at one fixed shape (512 threads,
    one CTA) and each at the autotuned shape of its size class."""
    from brian2_gb300 import autotune, batched, workloads as W
    spec = W.load_spec("cuba_f32")
    t0 = time.perf_counter()
    builts = batched.build_sweep(spec, batched.sweep_parameters(256))
    t_build = time.perf_counter() - t0
    shape = autotune.tune(spec, builts)
    r = batched.compare(spec, builts, steps, threads=shape["threads"])
    r.update(instances=len(builts), neurons=int(sum(sum(b.sizes) for b in builts)), clock_steps=steps,
             threads=shape["threads"], host_build_s=round(t_build, 2))
    return r


def extra_adjoint(reps=5):
    """Adjoint workload (float32): forward alone vs forward+adjoint (the loss's
    forward through the autograd function and its backward), median of reps."""
    import torch
    from brian2_gb300.adjoint import AdjointConfig, AdjointProblem, forward_trace
    P = AdjointProblem(AdjointConfig(), dtype=torch.float32)
    Wt, Wo, tm = P.params()
    fw, fb = [], []
    for rep in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.no_grad():
            forward_trace(P.ctx, Wt.detach(), Wo.detach(), float(tm.detach()))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        P.loss(Wt, Wo, tm).backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        Wt.grad = Wo.grad = tm.grad = None
        if rep:
            fw.append(t1 - t0)
            fb.append(t2 - t1)
    f, b = float(np.median(fw)), float(np.median(fb))
    return {"forward_ms": f * 1e3, "forward_adjoint_ms": b * 1e3, "ratio": b / f, "dtype": "f32",
            "clock_steps": P.cfg.steps, "hidden": P.cfg.n_h, "inputs": P.cfg.n_in, "readout": P.cfg.n_o}


def alu_roofline(entry, spec_name, fp64, peaks_cache={}):
    """ALU roofline of a compute-bound plain run (Hodgkin-Huxley): the update's
    arithmetic operators per neuron-step counted from its generated code, over
    the run's device time, against the FMA throughput measured on this device
    in the same precision (libb200_peaks)."""
    from brian2_gb300 import roofline, workloads as W
    ops = roofline.update_ops(W.load_spec(spec_name))
    if fp64 not in peaks_cache:
        peaks_cache[fp64] = roofline.fma_peak_gflops(fp64)
    peak = peaks_cache[fp64]
    achieved = ops["flops"] * entry["neurons"] * entry["clock_steps"] / (entry["device_ms"] * 1e-3) / 1e9
    return {"bound": "fp64 alu" if fp64 else "fp32 alu", "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
            "frac": achieved / peak, "peak_kind": "measured (FMA loop on every SM, libb200_peaks)",
            "flops_per_neuron_step": ops["flops"], "calls_per_neuron_step": ops["calls"],
            "note": "counted arithmetic of the generated update; each exp/expm1/pow call is many more "
                    "instructions, so this is a lower bound of the executed work"}


def extras():
    from brian2_gb300 import workloads as W
    out = {}
    jobs = [("cuba_4000_f64", lambda: extra_plain("cuba_f64", lambda s: W.build_cuba(s, N=4000, seed=1234))),
            ("cobahh_4000_f64", lambda: extra_plain("cobahh_f64", lambda s: W.build_cobahh(s, N=4000, seed=1234))),
            ("cobahh_4000_f32", lambda: extra_plain("cobahh_f32", lambda s: W.build_cobahh(s, N=4000, seed=1234))),
            ("batched_sweep_256_f32", extra_batched),
            ("adjoint_f32", extra_adjoint)]
    for name, fn in jobs:
        try:
            out[name] = fn()
        except Exception as e:  # reported, not fatal: the headline line still prints
            out[name] = {"error": f"{type(e).__name__}: {e}"[:300]}
    for name, spec_name, fp64 in (("cobahh_4000_f64", "cobahh_f64", True), ("cobahh_4000_f32", "cobahh_f32", False)):
        if "error" not in out.get(name, {"error": 1}):
            try:
                out[name]["roofline"] = alu_roofline(out[name], spec_name, fp64)
            except Exception as e:
                out[name]["roofline"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return out


# other workloads -> the reference's generated project of the same network
REFERENCE_OF = {"cuba_4000_f64": "cuba", "cobahh_4000_f64": "cobahh", "cobahh_4000_f32": "cobahh32",
                "batched_sweep_256_f32": "sweep8", "adjoint_f32": "adjoint"}


def reference_of_others(other):
    """The reference's CPU step loop beside each other workload: its generated
    cpp_standalone project of the same network (same script, seed and
    precision), at 1 OpenMP thread and at the largest generated count the host
    has cores for, timed by its own step-loop clock.  The sweep is sampled: 8
    of the 256 networks, the middle one of each size stratum of 32, run one
    after another; the 256-network time is the stratified estimate (32 x the
    sample).  Adds ``cpu_reference`` to each entry of ``other`` (in place)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_standalone
    for name, wl in REFERENCE_OF.items():
        if name not in other or "error" in other[name] or not ref_standalone.available(wl):
            continue
        entry = {"kind": "reference", "host_cpus": os.cpu_count()}
        try:
            for T in sorted({1, ref_standalone.all_threads(wl)}):
                if T not in ref_standalone.variants(wl):
                    continue
                ref_standalone.build(T, workload=wl)
                r = ref_standalone.run(T, workload=wl)
                d = {"threads": T, "step_loop_s": r["run_time_s"], "spikes": r["spikes"], "events": r["events"]}
                if r.get("networks"):
                    per = len(r["networks"])
                    scale = r["sweep_networks"] / per
                    d.update(sample_networks=[n["N"] for n in r["networks"]],
                             projected_all_s=r["run_time_s"] * scale,
                             events_per_s=r["events"] / r["run_time_s"])
                elif wl == "adjoint":  # forward time is the figure; its event count would miss the inputs'
                    del d["events"]
                    d.update(sim_s_per_wall_s=r["sim_s"] / r["run_time_s"])
                else:
                    d.update(sim_s_per_wall_s=r["sim_s"] / r["run_time_s"], events_per_s=r["events"] / r["run_time_s"])
                entry[f"threads_{T}"] = d
            runs = [v for k, v in entry.items() if k.startswith("threads_")]
            if not runs:
                continue
            best = min(runs, key=lambda v: v.get("projected_all_s", v["step_loop_s"]))
            o = other[name]
            if name == "batched_sweep_256_f32":
                entry["sample"] = ("8 of the 256 networks (sizes sorted, the middle one of each stratum of 32), "
                                   "500 ms each, run one after another; projected_all_s = 32 x the sample")
                entry["speedup_batched_vs_best"] = best["projected_all_s"] / (o["batched_ms"] * 1e-3)
            elif name == "adjoint_f32":
                entry["sample"] = "forward pass only (the reference has no gradient code), 5000 steps"
                entry["speedup_forward_vs_best"] = best["step_loop_s"] / (o["forward_ms"] * 1e-3)
            else:
                entry["sample"] = "the whole run: 1 s simulated, 10000 clock steps"
                entry["speedup_vs_best"] = best["step_loop_s"] / (o["device_ms"] * 1e-3)
            o["cpu_reference"] = entry
        except Exception as e:  # reported, not fatal
            other[name]["cpu_reference"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return other


def workload_config(N, K):
    """The workload both arms of the benchmark run (the reference arm prints
    the same dictionary)."""
    return {"workload": WORKLOAD if (N, K) == (N_NEURONS, K_IN) else f"cuba_delays_n{N}_k{K}_f32",
            "neurons": N, "in_degree": K, "synapses": N * K, "delays_ms": [0.1, 5.0], "dt_ms": 0.1,
            "state": "float32", "l2": "inputs larger than L2 (synapse arrays 8 GB per GPU)"}


def reference_headline(steps, warmup):
    """The reference's own step loop on the headline network itself: its
    generated cpp_standalone project of the 1,000,000-neuron network (float32,
    OpenMP on all host cores) runs once -- construction, a 50 ms run, then a
    100 ms run whose progress reports (about every 0.5 s of wall time) are the
    samples; the first `warmup` samples are discarded, the next `steps` timed.
    None when the project was not generated."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_standalone
    if not ref_standalone.available("delays1e6"):
        return None
    T = ref_standalone.all_threads("delays1e6")
    ref_standalone.build(T, workload="delays1e6")
    t0 = time.perf_counter()
    r = ref_standalone.run(T, workload="delays1e6", timeout=1500)
    wall = time.perf_counter() - t0
    smp = r["samples"]
    use = smp[warmup:warmup + steps] if len(smp) > warmup else smp
    if not use:
        return None
    ev = sum(x["events"] for x in use)
    sec = sum(x["run_time_s"] for x in use)
    st = sum(x["steps"] for x in use)
    return {"value": ev / sec, "unit": UNIT, "cores": r["threads"], "kind": "reference",
            "sample": f"reference cpp_standalone project of this network (generated by the reference, "
                      f"g++ -O3 -ffast-math -fopenmp, {r['threads']} OpenMP threads, float32): one execution "
                      f"(construction, 50 ms run, 100 ms reported run; {wall:.0f} s wall in all), "
                      f"{len(use)} progress-report intervals after {min(warmup, len(smp))} discarded: "
                      f"{st} clock steps, {sum(x['spikes'] for x in use)} spikes, {ev} events, "
                      f"step loop {sec:.2f} s",
            "sim_s_per_wall_s": st * 1e-4 / sec, "samples_used": len(use), "samples_available": len(smp),
            "per_sample": [round(x["events"] / x["run_time_s"], 1) for x in use]}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path for this workload -- its
    generated cpp_standalone project of the same network with OpenMP -- on the
    same metric and config; every step is one progress-report interval of the
    reference's own run.  Where that project was not generated: the
    10,000-neuron subnetwork project, else the oracle port, each stated."""
    if rank != 0:
        return
    r = reference_headline(args.steps, args.warmup) if args.reference_sample == "headline" else None
    if r is not None:
        config = workload_config(N_NEURONS, K_IN)
        dtype = "f32"
    else:
        vals = []
        for _ in range(min(args.warmup, 1)):
            cpu_baseline(max_seconds=5.0)
        for _ in range(args.steps):
            vals.append(cpu_baseline(max_seconds=10.0))
        r = dict(vals[0], value=float(np.median([x["value"] for x in vals])))
        config = dict(workload_config(N_NEURONS, K_IN), sample="10,000-neuron subnetwork, same construction, float64")
        dtype = "f64"
    v = r["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded construction)",
            "config": config,
            "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample") if k in r},
            "sim_s_per_wall_s": r.get("sim_s_per_wall_s"),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if "per_sample" in r:
        line["per_sample"] = r["per_sample"]
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--neurons", type=int, default=N_NEURONS)
    ap.add_argument("--in-degree", type=int, default=K_IN,
                    help="synapses per neuron and pathway group (smaller networks for profiling)")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--ctas", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-sample", default="headline", choices=["headline", "subnetwork"],
                    help="--impl reference: the headline network itself (default) or its 10,000-neuron "
                         "subnetwork (a quick check)")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--chunk-steps", type=int, default=0,
                    help="clock steps per kernel launch (default: one launch per bench step)")
    ap.add_argument("--push", default="auto", choices=["auto", "on", "off"],
                    help="push-mode delivery (auto: the library's choice)")
    ap.add_argument("--owner", default="auto", choices=["auto", "on", "off"],
                    help="owner-mode delivery (auto: the library's choice)")
    args = ap.parse_args()
    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local)) if world > 1 else None
    from brian2_gb300 import workloads as W
    from brian2_gb300.scale import build_delays_scale
    spec = W.load_spec("delays_f32")
    N = args.neurons
    seed = 1234 + rank  # weak scaling: every rank simulates its own network
    t_build = time.perf_counter()
    # two 256-thread CTAs per SM (128 registers each): one CTA's barrier waits
    # overlap the other's work, and each thread keeps four events' loads in flight
    threads = args.threads or 256
    ctas = args.ctas or 304
    K = args.in_degree
    net, _ = build_delays_scale(spec, N=N, K=K, seed=seed, threads=threads, ctas_per_inst=ctas)
    if args.chunk_steps:
        net.configure(threads=threads, ctas_per_inst=ctas, queue_mode=False, chunk_steps=args.chunk_steps,
                      use_graph=False)
    net.set_owner({"auto": "auto", "on": True, "off": False}[args.owner])
    net.set_push({"auto": "auto", "on": True, "off": False}[args.push])
    t_build = time.perf_counter() - t_build
    outdeg = net.outdegree
    plan = net.launch_plan()
    net_owner = net.owner_active()
    net_mode = net.delivery_mode()

    def bench_step():
        net.run(STEPS_PER_BENCH_STEP)
        return net.last_kernel_ms()

    for _ in range(args.warmup):
        bench_step()
    n_before = int(net.spikes(0, 0)[0].size)
    launches0 = net.launches()
    clocks = Clocks(local)
    clocks.start()
    sync_all(dist)
    t0 = time.perf_counter()
    kernel_ms = []
    for _ in range(args.steps):
        kernel_ms.append(bench_step())   # CUDA events around each launch
    sync_all(dist)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = net.launches() - launches0
    i, ts, _ = net.spikes(0, 0)
    i = i[n_before:]
    events = int(outdeg[i].sum())
    sim_s = args.steps * STEPS_PER_BENCH_STEP * 1e-4
    # value: device time of the timed launches (CUDA events), slowest rank
    device_s, events_all = reduce_ranks(dist, sum(kernel_ms) * 1e-3, events)
    wall, _ = reduce_ranks(dist, wall, 0)
    value = events_all / device_s

    # roofline of the step kernel: algorithmic bytes per launch (one launch = one
    # bench step of 1000 clock steps): 24 B per neuron-step (v, ge, gi read and
    # written, float32) + 8 B per synaptic event (target index + weight)
    launch_ms = float(np.mean(kernel_ms))
    alg_bytes = 24.0 * N * STEPS_PER_BENCH_STEP + 8.0 * events / args.steps
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    peaks, peak_kind = measured_peaks()
    kernel_name = {"push": "b200_push_kernel", "owner": "b200_owner_kernel"}.get(net_mode, "b200_step_kernel")
    traffic = ncu_traffic(K, kernel_name) if N == N_NEURONS else None  # (captured on the 1e6-neuron network)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_kind": peak_kind,
                "traffic": traffic,
                "dram_gbs": traffic / (launch_ms * 1e-3) / 1e9 if traffic else None,
                "dram_frac": traffic / (launch_ms * 1e-3) / 1e9 / peaks["hbm_gbs"] if traffic else None,
                "traffic_note": "ncu DRAM bytes at in-degree 250 and 500, extrapolated linearly to this in-degree; "
                                "the neuron state mostly stays in L2, so DRAM traffic is below the algorithmic bytes",
                "kernel": kernel_name, "ms_per_launch": launch_ms,
                "algorithmic_bytes_per_launch": alg_bytes}

    # end to end through the public API: every step uploads the state from
    # pinned host memory, runs, and reads the step's spikes back
    import torch
    host = {v: torch.empty(N, dtype=torch.float32).pin_memory() for v in ("v", "ge", "gi")}
    for v in host:
        host[v].numpy()[:] = net.download(0, "neurongroup", v)
    # the step's raster is read into pinned host buffers (one pair per step, so
    # the events are counted from them after the timed region)
    cap = 4 * max(1, len(i) // max(args.steps, 1)) + 4096
    rasters = [(torch.empty(cap, dtype=torch.int32).pin_memory().numpy(),
                torch.empty(cap, dtype=torch.int32).pin_memory().numpy()) for _ in range(args.steps)]
    e2e_events, h2d, d2h, got = 0, 0, 0, []
    sync_all(dist)
    t1 = time.perf_counter()
    for k in range(args.steps):
        for v, buf in host.items():
            net.upload(0, "neurongroup", v, buf.numpy())
            h2d += buf.numel() * 4
        net.reset_monitors(0)
        net.run(STEPS_PER_BENCH_STEP)
        si, sts, _ = net.spikes(0, 0, counts=False, out=rasters[k])
        d2h += si.nbytes + sts.nbytes
        got.append(si)
    sync_all(dist)
    e2e_wall = time.perf_counter() - t1
    e2e_events = sum(int(outdeg[si].sum()) for si in got)
    e2e_wall, e2e_events = reduce_ranks(dist, e2e_wall, e2e_events)

    other = None
    if rank == 0 and world == 1 and not args.no_extras:
        net.close()  # frees the 1e9-synapse network before the other workloads
        other = extras()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline()
        if other:
            reference_of_others(other)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": device_s / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: network constructed on the device from a seed",
            "config": workload_config(N, K),
            "launch": {"clock_steps_per_step": STEPS_PER_BENCH_STEP, "threads": threads, "ctas": ctas,
                       "launch_plan": plan, "build_s": round(t_build, 2), "owner_mode": net_owner,
                       "delivery": net_mode},
            "sim_s_per_wall_s": sim_s / device_s,
            "wall_ms_per_step": wall / args.steps * 1e3,
            "spikes_per_step": float(len(i)) / args.steps,
            "e2e": {"value": e2e_events / e2e_wall, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps},
            "roofline": roofline,
            "gpu_launches": int(launches),
            "clocks": clk,
            "cpu_baseline": cpu,
            "other_workloads": other,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
