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


def build_cuba(spec, N=4000, seed=1234, ne_frac=0.8, p=0.02, consts=None) -> Built:
    """CUBA (``oracle/brian_configs.py:cuba``): v0 = Vr + rand()*(Vt-Vr), then
    Ce.connect('i<Ne and i!=j', p), Ci.connect('i>=Ne and i!=j', p)."""
    c = {x["name"]: x["value"] for x in spec["consts"]}
    if consts:
        c.update(consts)
    r = BrianRandom(seed)
    Ne = int(N * ne_frac)
    b = Built(sizes=[N], consts=dict(consts or {}))
    ftype = np.float64 if spec.get("float", "double") == "double" else np.float32
    v0 = r.affine_rand(c["Vr"], c["Vt"] - c["Vr"], N)
    b.group_init[("neurongroup", "v")] = v0.astype(ftype)
    b.group_init[("neurongroup", "ge")] = np.zeros(N, ftype)
    b.group_init[("neurongroup", "gi")] = np.zeros(N, ftype)
    pe, qe = r.connect_bernoulli(N, N, p, (0, Ne), no_self=True)
    pi, qi = r.connect_bernoulli(N, N, p, (Ne, N), no_self=True)
    b.synapses["synapses_pre"] = dict(pre=pe, post=qe, src=(0, N), tgt=(0, N))
    b.synapses["synapses_1_pre"] = dict(pre=pi, post=qi, src=(0, N), tgt=(0, N))
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
