"""The draws of the step loop, site by site, on a model built to reach every
branch of the walk of the reference's stream (brian2/devices/cpp_standalone/
templates/objects.cpp:426-478, brian2/input/binomial.py:93-141):

* site 0: rand() once per neuron of a 333-neuron group;
* site 1: randn() twice per neuron of a 777-neuron group (a kept value at the
  start is the first one used);
* site 2: a binomial sampler whose bound is passed by one draw in ten, so
  the count starts over with a new number (in the reference's order);
* site 3: the normal approximation over 401 neurons (an odd count: the kept
  value passes to the next step's site 1).

Each state variable accumulates its site's draws, so the final state holds
every draw of the run.  The oracle is checked against an independent walk in
Python (numpy's MT19937 gives the outputs of std::mt19937 from the same
state; Python's floats are IEEE doubles and math.log is the C library's), the
CUDA path against the oracle: bit-exact for rand() and the binomial counts;
normal values within the last bits (the device's log is CUDA's)."""
import math

import numpy as np
import pytest

from oracle import OracleNet

N_G, N_H, STEPS = 777, 333, 40
BIN = dict(qn="0.3", bound="1.5", n=3, p="0.4", q="0.6", reverse=False)
NORM = dict(scale="2.5", loc="10.0")


def make_spec():
    clock = {"dt": "_ptr_array_defaultclock_dt", "t": "_ptr_array_defaultclock_t",
             "timestep": "_ptr_array_defaultclock_timestep"}
    gvars = [dict(name=n, ctype="double", ptr=f"_ptr_array_g_{n}") for n in ("a", "b", "c", "d")]
    g = dict(name="g", vars=gvars, threshold=None, reset=None, update=dict(scalar="", draw=1, vector="\n".join([
        "double a = _ptr_array_g_a[_idx];", "double b = _ptr_array_g_b[_idx];",
        "a = a + _b200_draw_1_0(_vectorisation_idx);", "b = b + _b200_draw_1_1(_vectorisation_idx);",
        "_ptr_array_g_a[_idx] = a;", "_ptr_array_g_b[_idx] = b;"])))
    h = dict(name="h", vars=[dict(name="u", ctype="double", ptr="_ptr_array_h_u")], threshold=None, reset=None,
             update=dict(scalar="", draw=0, vector="\n".join([
                 "double u = _ptr_array_h_u[_idx];", "u = u + _b200_draw_0_0(_vectorisation_idx);",
                 "_ptr_array_h_u[_idx] = u;"])))
    inputs = [dict(name="in_c", group=0, lo=0, hi=-1, draw=2, code=dict(scalar="", vector="\n".join([
                  "double c = _ptr_array_g_c[_idx];", "c += 1.0 * _b200_draw_2_0(_vectorisation_idx);",
                  "_ptr_array_g_c[_idx] = c;"]))),
              dict(name="in_d", group=0, lo=100, hi=501, draw=3, code=dict(scalar="", vector="\n".join([
                  "const int32_t _sub_idx = _b200_abs_idx;", "double d = _ptr_array_g_d[_sub_idx];",
                  "d += 1.0 * _b200_draw_3_0(_vectorisation_idx);", "_ptr_array_g_d[_sub_idx] = d;"])))]
    draws = [dict(name="h_update", kind="rand", group=1, lo=0, hi=-1, calls=1),
             dict(name="g_update", kind="randn", group=0, lo=0, hi=-1, calls=2),
             dict(name="in_c", kind="binomial", group=0, lo=0, hi=-1, calls=1, binom=dict(BIN)),
             dict(name="in_d", kind="binormal", group=0, lo=100, hi=501, calls=1, binom=dict(NORM))]
    return dict(name="draw_sites", float="double", consts=[], clock_ptrs=clock, groups=[g, h], pathways=[],
                spike_monitors=[], rate_monitors=[], state_monitors=[], draws=draws, inputs=inputs)


def start_state(seed=11):
    st = np.random.MT19937(seed).state["state"]
    return np.asarray(st["key"], np.uint32), int(st["pos"]), (1, 0.123)


class Walk:
    """The reference's RandomGenerator restated over numpy's MT19937."""

    def __init__(self, words, pos, gauss):
        self.bg = np.random.MT19937()
        s = self.bg.state
        s["state"] = {"key": np.asarray(words, np.uint32), "pos": int(pos)}
        self.bg.state = s
        self.has, self.kept = bool(gauss[0]), float(gauss[1])
        self.restarts = 0

    def word(self):
        return int(self.bg.random_raw())

    def rand(self):
        a = self.word() >> 5
        b = self.word() >> 6
        return (a * 67108864.0 + b) / 9007199254740992.0

    def randn(self):
        if self.has:
            self.has = False
            return self.kept
        while True:
            x1 = 2.0 * self.rand() - 1.0
            x2 = 2.0 * self.rand() - 1.0
            r2 = x1 * x1 + x2 * x2
            if not (r2 >= 1.0 or r2 == 0.0):
                break
        f = math.sqrt(-2.0 * math.log(r2) / r2)
        self.kept, self.has = f * x1, True
        return f * x2

    def binomial(self, qn, bound, n, p, q, reverse):
        X, px, U = 0, qn, self.rand()
        while U > px:
            X += 1
            if X > bound:
                X, px, U = 0, qn, self.rand()
                self.restarts += 1
            else:
                U -= px
                px = ((n - X + 1) * p * px) / (X * q)
        return n - X if reverse else X


def walk_state(steps):
    """The final state: every variable the sum of its site's draws."""
    words, pos, gauss = start_state()
    w = Walk(words, pos, gauss)
    u, a, b, c, d = np.zeros(N_H), np.zeros(N_G), np.zeros(N_G), np.zeros(N_G), np.zeros(N_G)
    bn = (float(BIN["qn"]), float(BIN["bound"]), BIN["n"], float(BIN["p"]), float(BIN["q"]), BIN["reverse"])
    scale, loc = float(NORM["scale"]), float(NORM["loc"])
    for _ in range(steps):
        for i in range(N_H):
            u[i] = u[i] + w.rand()
        for i in range(N_G):
            a[i] = a[i] + w.randn()
            b[i] = b[i] + w.randn()
        for i in range(N_G):
            c[i] += 1.0 * w.binomial(*bn)
        for i in range(100, 501):
            d[i] += 1.0 * float(np.float32(w.randn() * scale + loc))
    return dict(u=u, a=a, b=b, c=c, d=d), w


def oracle_state(steps):
    spec = make_spec()
    o = OracleNet(spec, [N_G, N_H], 1e-4)
    words, pos, gauss = start_state()
    o.set_rng(words, pos, gauss)
    o.run(steps)
    return {v: o.download("h" if v == "u" else "g", v) for v in "uabcd"}


def test_oracle_follows_the_reference_walk():
    ref, w = walk_state(STEPS)
    assert w.restarts > 1000  # the binomial's start-over branch is exercised
    out = oracle_state(STEPS)
    for v in "uabcd":
        np.testing.assert_array_equal(out[v], ref[v], err_msg=v)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [dict(threads=256), dict(threads=128, ctas_per_inst=4),
                                   dict(threads=256, ctas_per_inst=20), dict(threads=1024, chunk_steps=7)])
def test_device_draws_match_oracle(shape):
    from brian2_gb300.runtime import Model, Network
    spec = make_spec()
    net = Network(Model.get(spec), [[N_G, N_H]], 1e-4)
    net.configure(**shape)
    words, pos, gauss = start_state()
    net.set_rng(0, words, pos, gauss)
    for chunk in (1, 12, STEPS - 13):  # launches that stop with draws made ahead
        net.run(chunk)
    ref = oracle_state(STEPS)
    got = {v: net.download(0, "h" if v == "u" else "g", v) for v in "uabcd"}
    for v in "uc":  # rand() and the binomial counts (with their starts over): exact
        np.testing.assert_array_equal(got[v], ref[v], err_msg=v)
    for v in "abd":  # normal values: CUDA's log against the C library's
        np.testing.assert_allclose(got[v], ref[v], rtol=1e-13, atol=1e-13, err_msg=v)
    exact = np.mean(got["a"] == ref["a"])
    print(f"\nnormal sums bit-exact: {exact:.4f}; binormal sums bit-exact: {np.mean(got['d'] == ref['d']):.4f}")
