"""Benchmark networks built without Brian2 installed.

Each builder loads a committed spec (``brian2_gb300/specs/<name>.json``, produced
by the ``b200`` device from the Brian2 script of the same network) and
constructs the network's initial state and synapses with the native host
construction, consuming Brian's random stream in the order the Brian2 script
does, so the result is the network the reference builds for the same seed.
The Brian2 scripts are the ``oracle/brian_configs.py`` functions of the same
name.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field

import numpy as np

from .construct import BrianRandom, quantise_delays
from .runtime import Model, Network

SPECS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "specs")
DT = 1e-4  # 0.1 ms


def load_spec(name: str) -> dict:
    with open(os.path.join(SPECS, name + ".json")) as f:
        return json.load(f)


def const(spec, name):
    for c in spec["consts"]:
        if c["name"] == name:
            return c["value"]
    raise KeyError(name)


@dataclass
class Built:
    """Host-side description of one constructed network instance."""
    sizes: list
    group_init: dict = field(default_factory=dict)        # (group, var) -> array
    synapses: dict = field(default_factory=dict)          # pathway -> dict(pre, post, delay_steps, src, tgt, vars)
    consts: dict = field(default_factory=dict)
    spikemon_ranges: dict = field(default_factory=dict)
    ratemon_ranges: dict = field(default_factory=dict)


def _ftype(spec):
    return np.float64 if spec.get("float", "double") == "double" else np.float32


def _defaults(spec, b: Built, group="neurongroup"):
    """Brian's initial values for the variables a script does not set:
    zeros, the index array ``i``, and the refractoriness state
    (``lastspike = -1e4 s``, ``not_refractory = True``,
    brian2/groups/neurongroup.py:689-692)."""
    g = next(x for x in spec["groups"] if x["name"] == group)
    N = b.sizes[[x["name"] for x in spec["groups"]].index(group)]
    for v in g["vars"]:
        key = (group, v["name"])
        if key in b.group_init:
            continue
        if v["name"] == "i":
            b.group_init[key] = np.arange(N, dtype=np.int32)
        elif v["name"] == "lastspike":
            b.group_init[key] = np.full(N, -1e4, np.float64)
        elif v["name"] == "not_refractory":
            b.group_init[key] = np.ones(N, np.int8)
        else:
            b.group_init[key] = np.zeros(N, np.float64 if v["ctype"] == "double" else
                                         np.float32 if v["ctype"] == "float" else np.int32)


def build_cuba(spec, N=4000, seed=1234, ne_frac=0.8, p=0.02, consts=None) -> Built:
    """CUBA (``oracle/brian_configs.py:cuba``): v0 = Vr + rand()*(Vt-Vr), then
    Ce.connect('i<Ne and i!=j', p), Ci.connect('i>=Ne and i!=j', p)."""
    c = {x["name"]: x["value"] for x in spec["consts"]}
    if consts:
        c.update(consts)
    r = BrianRandom(seed)
    Ne = int(N * ne_frac)
    b = Built(sizes=[N], consts=dict(consts or {}))
    v0 = r.affine_rand(c["Vr"], c["Vt"] - c["Vr"], N)
    b.group_init[("neurongroup", "v")] = v0.astype(_ftype(spec))
    _defaults(spec, b)
    pe, qe = r.connect_bernoulli(N, N, p, (0, Ne), no_self=True)
    pi, qi = r.connect_bernoulli(N, N, p, (Ne, N), no_self=True)
    b.synapses["synapses_pre"] = dict(pre=pe, post=qe, src=(0, N), tgt=(0, N))
    b.synapses["synapses_1_pre"] = dict(pre=pi, post=qi, src=(0, N), tgt=(0, N))
    return b


def build_cobahh(spec, N=4000, seed=1234, ne_frac=0.8, p=0.02) -> Built:
    """COBAHH (``oracle/brian_configs.py:cobahh``): Ce.connect('i<Ne', p) and
    Ci.connect('i>=Ne', p) (conditions on i only: rejected sources draw no
    random numbers), then v0 = El + (randn()*5 - 5)*mV."""
    r = BrianRandom(seed)
    Ne = int(N * ne_frac)
    b = Built(sizes=[N])
    pe, qe = r.connect_bernoulli(N, N, p, (0, Ne), no_self=False, cond_uses_j=False)
    pi, qi = r.connect_bernoulli(N, N, p, (Ne, N), no_self=False, cond_uses_j=False)
    El, mV = -60 * 1e-3, 1e-3
    # Brian evaluates ``El + (randn()*5 - 5)*mV`` as El + (mV * ((-5.0) + (5.0 * randn())))
    v0 = r.affine_randn(El, mV, -5.0, 5.0, N)
    b.group_init[("neurongroup", "v")] = v0.astype(_ftype(spec))
    _defaults(spec, b)
    b.synapses["synapses_pre"] = dict(pre=pe, post=qe, src=(0, N), tgt=(0, N))
    b.synapses["synapses_1_pre"] = dict(pre=pi, post=qi, src=(0, N), tgt=(0, N))
    return b


def delay_constants(wscale=1.0 / 50, dmin_ms=0.1, dmax_ms=5.0):
    """The weight and delay constants of ``oracle/brian_configs.py:cuba_delays``,
    evaluated with the same float operations as the script."""
    mV, ms = 1e-3, 1e-3
    we = (60 * 0.27 / 10) * mV * wscale
    wi = (-20 * 4.5 / 10) * mV * wscale
    return we, wi, dmin_ms * ms, (dmax_ms - dmin_ms) * ms


def build_delays(spec, N=10000, K=1000, seed=1234, ne_frac=0.8, wscale=1.0 / 50, dmin_ms=0.1,
                 dmax_ms=5.0) -> Built:
    """Fixed in-degree CUBA with delays (``oracle/brian_configs.py:cuba_delays``):
    v0, then Ce/Ci ``connect(i='k for k in sample(N_pre, size=K)')`` from the
    E and I subgroups, w constant per pathway, delay = dmin + rand()*dspan."""
    c = {x["name"]: x["value"] for x in spec["consts"]}
    r = BrianRandom(seed)
    Ne = int(N * ne_frac)
    Ke = int(K * ne_frac)
    Ki = K - Ke
    b = Built(sizes=[N])
    ft = _ftype(spec)
    b.group_init[("neurongroup", "v")] = r.affine_rand(c["Vr"], c["Vt"] - c["Vr"], N).astype(ft)
    _defaults(spec, b)
    pe, qe = r.connect_fixed_indegree(Ne, N, Ke)
    pi, qi = r.connect_fixed_indegree(N - Ne, N, Ki)
    we, wi, dmin, dspan = delay_constants(wscale, dmin_ms, dmax_ms)
    de = r.affine_rand(dmin, dspan, len(pe))
    di = r.affine_rand(dmin, dspan, len(pi))
    if ft == np.float32:
        de, di = de.astype(np.float32), di.astype(np.float32)
    b.synapses["synapses_pre"] = dict(pre=pe, post=qe, src=(0, Ne), tgt=(0, N),
                                      delay_steps=quantise_delays(de, DT),
                                      vars={"w": np.full(len(pe), we, ft)}, delay=de)
    b.synapses["synapses_1_pre"] = dict(pre=pi, post=qi, src=(Ne, N), tgt=(0, N),
                                        delay_steps=quantise_delays(di, DT),
                                        vars={"w": np.full(len(pi), wi, ft)}, delay=di)
    return b


def instantiate(spec, builts, threads=256, ctas_per_inst=1, queue_mode=False, chunk_steps=0) -> Network:
    """Creates the device network for a list of built instances."""
    model = Model.get(spec)
    net = Network(model, [b.sizes for b in builts], DT)
    net.configure(threads=threads, ctas_per_inst=ctas_per_inst, queue_mode=queue_mode, chunk_steps=chunk_steps)
    for k, b in enumerate(builts):
        if b.consts:
            net.set_consts(k, b.consts)
        for (g, v), arr in b.group_init.items():
            net.upload(k, g, v, arr)
        for pw, s in b.synapses.items():
            net.set_synapses(k, pw, s["pre"], s["post"], s.get("delay_steps"), s.get("scalar_delay", 0),
                             s.get("src"), s.get("tgt"))
            for var, arr in s.get("vars", {}).items():
                net.upload_synapse_var(k, pw, var, arr)
        for m, (lo, hi) in b.spikemon_ranges.items():
            net.set_spikemon_range(k, m, lo, hi)
        for m, (lo, hi) in b.ratemon_ranges.items():
            net.set_ratemon_range(k, m, lo, hi)
    return net
