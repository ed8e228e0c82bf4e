"""THE ORACLE -- test infrastructure only (tests/, smoke(), bench.py cpu_baseline).

A CPU restatement of the reference's clock-driven step loop, used to check the
CUDA path.  It is generated per network spec, like Brian2's ``cpp_standalone``
code objects, and executes the spec's *plain* C++ snippets (Brian's own
``CPPCodeGenerator`` output) inside loops that restate the reference templates:

* ``Network::run``: per step, every code object in schedule order, then the
  clock tick ``t = timestep*dt``
  (brian2/devices/cpp_standalone/templates/network.cpp:67-104,
  brianlib/clocks.h:34-38; schedule brian2/core/network.py:42-50);
* state update over all neurons (templates/stateupdate.cpp:5-21);
* threshold with sequential ascending compaction into the spike space and the
  refractory bookkeeping (templates/threshold.cpp:18-31);
* spike generators: the entries from the cursor whose time bin is <= the
  step's (modulo the period, with the cursor reset after a wrap), in array
  order (templates/spikegenerator.cpp:5-31);
* spike monitor append of (i, t) and per-neuron counts
  (templates/spikemonitor.cpp:13-48);
* per pathway ``advance()`` then ``push()`` into a ring of synapse-index
  vectors, ``peek()`` and ``on_pre`` for each queued synapse in queue order
  (templates/synapses_push_spikes.cpp:24-28, synapses/spikequeue.h:146-205,
  templates/synapses.cpp:20-49);
* reset for each spike (templates/reset.cpp:16-22);
* rand() in thresholds (PoissonGroup): the reference's generator,
  std::mt19937 continued from the state the standalone program had at the
  run, rand() = (a*2^26 + b)/2^53 of two outputs (templates/objects.cpp:
  426-453), drawing groups in schedule order and neurons in index order;
* Poisson inputs (PoissonInput, input/poissoninput.py:20-141): after the
  on_pre pathways and before the on_post ones, every target neuron adds a
  binomial count drawn by inversion (input/binomial.py:93-141, including the
  redraw past the bound) from the same generator;
* summed variables: the target range zeroed, then the expression of every
  synapse in creation order added to its target (templates/summed_variable.cpp:
  11-25), after the state monitors and before the state updates;
* rate monitor count per step (templates/ratemonitor.cpp:7-35);
* state monitor record at the start of the step (templates/statemonitor.cpp);
* operations (Group.run_regularly): the start slot's before the state
  monitors, the end slot's after the resets, on the steps of their clock.

A spec with ``"push_order": true`` gives the oracle of the device's push-mode
delivery: every on_pre of a step adds into a per-variable accumulator (zero at
the start of the step) instead of its target, and after the last pathway each
target neuron adds its accumulator -- the one change push mode makes to the
reference's arithmetic (the order of the additions into a target).  For models
whose increments into one variable are equal within a step, the device's
push mode reproduces this oracle bit for bit whatever order its atomics take.

Scalar blocks are evaluated every step, as the reference does.  The library is
built with ``g++ -O2 -ffp-contract=off -fno-fast-math`` (the reference's strict
build).  It is pinned against fixtures produced by running Brian2 itself
(tests/golden/make_golden.py) and must never be used by the product path.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)

_CT_NP = {"double": np.float64, "float": np.float32, "int32_t": np.int32, "char": np.int8,
          "int8_t": np.int8, "int64_t": np.int64}


def _ind(code, n):
    return "\n".join(" " * n + ln if ln.strip() else "" for ln in code.splitlines())


def render_oracle(spec: dict) -> str:
    groups = spec["groups"]
    paths = spec.get("pathways", [])
    spkmons = spec.get("spike_monitors", [])
    ratemons = spec.get("rate_monitors", [])
    statemons = spec.get("state_monitors", [])
    consts = spec.get("consts", [])
    clock = spec.get("clock_ptrs", {"dt": "_ptr_array_defaultclock_dt", "t": "_ptr_array_defaultclock_t",
                                     "timestep": "_ptr_array_defaultclock_timestep"})
    # push order: the variables the pathways deliver into (group, variable)
    PUSH_ORDER = bool(spec.get("push_order"))
    ACC = sorted({(gi, vi) for p in paths for _, (gi, vi) in p.get("group_ptrs", {}).items() if gi == p["tgt"]}) \
        if PUSH_ORDER else []
    o = []
    w = o.append
    w("// oracle for model '%s' (generated; test infrastructure)" % spec["name"])
    w("#include <cmath>\n#include <cstdint>\n#include <cstring>\n#include <vector>\n#include <algorithm>")
    # Brian's code objects see ``using namespace std`` (brian2/synapses/spikequeue.h:10,
    # included through objects.h), so exp(float) is std::exp(float); _exprel and
    # _brian_pow keep the reference's definitions (double-only _exprel, pow macro)
    # (brian2/codegen/generators/cpp_generator.py:90-197, 567-618)
    w("using namespace std;")
    w("static inline double _exprel(double x) { if (fabs(x) < 1e-16) return 1.0; if (x > 717) return INFINITY; return expm1(x)/x; }")
    w("template <typename T> static inline T _clip(const T v, const double a, const double b) { if (v < a) return a; if (v > b) return b; return v; }")
    w("#define _brian_pow(x, y) (pow((x), (y)))")
    w("template <typename T1, typename T2> static inline double _brian_mod(T1 x, T2 y) { return x - y * floor(1.0 * x / y); }")
    w("template <typename T1, typename T2> static inline double _brian_floordiv(T1 x, T2 y) { return floor(1.0 * x / y); }")
    w("template <typename T> static inline int int_(T v) { return (int)v; }")
    w("static inline int64_t _timestep(double t, double dt) { return (int64_t)((t + 1e-3 * dt) / dt); }")
    w("#define _brian_abs fabs")
    INPUTS = spec.get("inputs", [])
    SITES = spec.get("draws", [])
    DRAWS = bool(SITES)
    if DRAWS:
        w("#include <random>\n#include <sstream>\n#include <string>")
        w("static std::mt19937* _b200_gen = nullptr;")
        w("static bool* _b200_has = nullptr; static double* _b200_kept = nullptr;")
        w("static inline double _rand(int64_t) {")
        w("  const long a = (long)((*_b200_gen)() >> 5);")
        w("  const long b = (long)((*_b200_gen)() >> 6);")
        w("  return (a * 67108864.0 + b) / 9007199254740992.0;")
        w("}")
        # the polar method, keeping the second value for the next call
        w("static inline double _randn(int64_t i) {")
        w("  if (*_b200_has) { *_b200_has = false; return *_b200_kept; }")
        w("  double x1, x2, r2;")
        w("  do { x1 = 2.0 * _rand(i) - 1.0; x2 = 2.0 * _rand(i) - 1.0; r2 = x1 * x1 + x2 * x2; } while (r2 >= 1.0 || r2 == 0.0);")
        w("  const double f = sqrt(-2.0 * log(r2) / r2);")
        w("  *_b200_kept = f * x1; *_b200_has = true;")
        w("  return f * x2;")
        w("}")
    for si, d in enumerate(SITES):
        bn = d.get("binom") or {}
        if d["kind"] in ("rand", "randn"):
            for c in range(d["calls"]):
                w(f"#define _b200_draw_{si}_{c}(i) _{d['kind']}(i)")
        elif d["kind"] == "binomial":
            w(f"static inline long _b200_draw_{si}_0(int64_t _vidx) {{  // inversion, with the reference's constants")
            w(f"  long X = 0; double px = {bn['qn']}; double U = _rand(_vidx);")
            w("  while (U > px) {")
            w("    X++;")
            w(f"    if (X > {bn['bound']}) {{ X = 0; px = {bn['qn']}; U = _rand(_vidx); }}  // start over with a new draw")
            w(f"    else {{ U -= px; px = (({bn['n']} - X + 1) * {bn['p']} * px) / (X * {bn['q']}); }}")
            w("  }")
            w(f"  return {str(bn['n']) + ' - X' if bn['reverse'] else 'X'};")
            w("}")
        else:  # normal approximation
            w(f"static inline float _b200_draw_{si}_0(int64_t _vidx) {{ return _randn(_vidx) * {bn['scale']} + {bn['loc']}; }}")
    # blocks that draw run in the order of their sites (the schedule's order)
    site_of = {}
    for si, d in enumerate(SITES):
        if d["kind"] in ("rand", "randn"):
            blk = next(b for b in ("update", "threshold") if (groups[d["group"]].get(b) or {}).get("draw") == si)
            site_of[(d["group"], blk)] = si

    def block_order(blk):
        plain = [gi for gi in range(len(groups)) if (gi, blk) not in site_of]
        return plain + sorted((gi for gi in range(len(groups)) if (gi, blk) in site_of),
                              key=lambda gi: site_of[(gi, blk)])
    w("struct Net {")
    w("  double dt; int64_t ts = 0;")
    if DRAWS:
        w("  std::mt19937 gen; bool has = false; double kept = 0.0;")
    w("  std::vector<double> c;")
    for gi, g in enumerate(groups):
        w(f"  int32_t N{gi} = 0;")
        for v in g["vars"]:
            w(f"  std::vector<{v['ctype']}> g{gi}_{v['name']};")
        w(f"  std::vector<int32_t> spk{gi};")
        if g.get("generator"):
            w(f"  std::vector<int32_t> gen{gi}_bins, gen{gi}_index; int32_t gen{gi}_period = 0, gen{gi}_last = 0;")
    for pi, p in enumerate(paths):
        w(f"  int32_t p{pi}_src_lo = 0, p{pi}_src_hi = 0, p{pi}_tgt_lo = 0, p{pi}_tgt_hi = 0; std::vector<int32_t> p{pi}_pre, p{pi}_post, p{pi}_delay;")
        for v in p.get("vars", []):
            w(f"  std::vector<{v['ctype']}> p{pi}_{v['name']};")
        w(f"  std::vector<std::vector<int32_t>> p{pi}_queue = std::vector<std::vector<int32_t>>(1); int p{pi}_offset = 0;")
        w(f"  std::vector<std::vector<int32_t>> p{pi}_syn;")
    for mi, m in enumerate(spkmons):
        w(f"  int32_t sm{mi}_lo = 0, sm{mi}_hi = 0; std::vector<int32_t> sm{mi}_i, sm{mi}_ts, sm{mi}_count;")
        w(f"  std::vector<double> sm{mi}_vals;  // recorded variables, one row per spike")
    for mi, m in enumerate(ratemons):
        w(f"  int32_t rm{mi}_lo = 0, rm{mi}_hi = 0; std::vector<int32_t> rm{mi}_cnt;")
    for mi, m in enumerate(statemons):
        w(f"  std::vector<int32_t> st{mi}_idx, st{mi}_vars; std::vector<double> st{mi}_data; int64_t st{mi}_n = 0;")
    for gi, vi in ACC:
        v = groups[gi]["vars"][vi]
        w(f"  std::vector<{v['ctype']}> acc_g{gi}_{v['name']};  // push order: the step's deliveries")
    w("};")
    w('extern "C" {')
    w("Net* oracle_create(const int32_t* sizes, double dt) {")
    w("  Net* n = new Net(); n->dt = dt;")
    w("  n->c = {" + ", ".join(repr(float(c["value"])) for c in consts) + "};")
    for gi, g in enumerate(groups):
        w(f"  n->N{gi} = sizes[{gi}];")
        for v in g["vars"]:
            w(f"  n->g{gi}_{v['name']}.assign(sizes[{gi}], 0);")
    for gi, vi in ACC:
        w(f"  n->acc_g{gi}_{groups[gi]['vars'][vi]['name']}.assign(sizes[{gi}], 0);")
    for pi, p in enumerate(paths):
        w(f"  n->p{pi}_src_hi = sizes[{p['src']}];")
    for mi, m in enumerate(spkmons):
        w(f"  n->sm{mi}_hi = sizes[{m['group']}]; n->sm{mi}_count.assign(sizes[{m['group']}], 0);")
    for mi, m in enumerate(ratemons):
        w(f"  n->rm{mi}_hi = sizes[{m['group']}];")
    w("  return n;")
    w("}")
    w("void oracle_destroy(Net* n) { delete n; }")
    w("void oracle_set_consts(Net* n, const double* v, int32_t k) { n->c.assign(v, v + k); }")
    # uploads / downloads through a switch over (group, var)
    w("void* oracle_var(Net* n, int32_t kind, int32_t obj, int32_t var) {")
    for gi, g in enumerate(groups):
        src = gi if g.get("alias_of") is None else g["alias_of"]
        for vi, v in enumerate(g["vars"]):
            w(f"  if (kind == 0 && obj == {gi} && var == {vi}) return n->g{src}_{v['name']}.data();")
    for pi, p in enumerate(paths):
        for vi, v in enumerate(p.get("vars", [])):
            w(f"  if (kind == 1 && obj == {pi} && var == {vi}) return n->p{pi}_{v['name']}.data();")
    w("  return nullptr;")
    w("}")
    # synapses: pre/post relative to the source/target range; stored absolute
    w("int oracle_set_synapses(Net* n, int32_t pw, const int32_t* pre, const int32_t* post, const int32_t* delay, int32_t tgt_hi,")
    w("                        int32_t scalar_delay, int64_t n_syn, int32_t src_lo, int32_t src_hi, int32_t tgt_lo) {")
    for pi, p in enumerate(paths):
        w(f"  if (pw == {pi}) {{")
        w(f"    n->p{pi}_src_lo = src_lo; n->p{pi}_src_hi = src_hi; n->p{pi}_tgt_lo = tgt_lo; n->p{pi}_tgt_hi = tgt_hi;")
        w(f"    n->p{pi}_pre.resize(n_syn); n->p{pi}_post.resize(n_syn); n->p{pi}_delay.resize(n_syn);")
        w(f"    for (int64_t k = 0; k < n_syn; ++k) {{ n->p{pi}_pre[k] = pre[k] + src_lo; n->p{pi}_post[k] = post[k] + tgt_lo;")
        w(f"      n->p{pi}_delay[k] = delay ? delay[k] : scalar_delay; }}")
        for v in p.get("vars", []):
            w(f"    n->p{pi}_{v['name']}.assign(n_syn, 0);")
        # CSpikeQueue::prepare: per-source synapse lists, ring size max_delay+1 (spikequeue.h:45-105)
        w(f"    n->p{pi}_syn.assign(src_hi - src_lo, std::vector<int32_t>());")
        w(f"    int32_t md = 0; for (int64_t k = 0; k < n_syn; ++k) {{ n->p{pi}_syn[pre[k]].push_back((int32_t)k); md = std::max(md, n->p{pi}_delay[k]); }}")
        w(f"    if ((int)n->p{pi}_queue.size() < md + 1) {{")
        w(f"      std::rotate(n->p{pi}_queue.begin(), n->p{pi}_queue.begin() + n->p{pi}_offset, n->p{pi}_queue.end());")
        w(f"      n->p{pi}_offset = 0; n->p{pi}_queue.resize(md + 1); }}")
        w("    return 0;")
        w("  }")
    w("  return 1;")
    w("}")
    w("void oracle_set_generator(Net* n, int32_t g, const int32_t* bins, const int32_t* index, int64_t count,")
    w("                          int32_t period, int32_t last) {")
    for gi, g in enumerate(groups):
        if g.get("generator"):
            w(f"  if (g == {gi}) {{ n->gen{gi}_bins.assign(bins, bins + count); n->gen{gi}_index.assign(index, index + count);")
            w(f"    n->gen{gi}_period = period; n->gen{gi}_last = last; }}")
    w("}")
    w("int32_t oracle_get_generator(Net* n, int32_t g) {")
    for gi, g in enumerate(groups):
        if g.get("generator"):
            w(f"  if (g == {gi}) return n->gen{gi}_last;")
    w("  return -1;")
    w("}")
    w("void oracle_set_step(Net* n, int64_t ts) { n->ts = ts; }")
    w("void oracle_set_rng(Net* n, const uint32_t* words, int32_t pos) {")
    if DRAWS:  # (the C++ library's text form of the state: the 624 words, then the position)
        w("  std::ostringstream o; for (int k = 0; k < 624; ++k) o << words[k] << ' '; o << pos;")
        w("  std::istringstream in(o.str()); in >> n->gen;")
        w("  n->has = false;")
    else:
        w("  (void)n; (void)words; (void)pos;")
    w("}")
    w("void oracle_set_gauss(Net* n, int32_t has, double value) {")
    w("  n->has = has != 0; n->kept = value;" if DRAWS else "  (void)n; (void)has; (void)value;")
    w("}")
    w("void oracle_set_range(Net* n, int32_t kind, int32_t mon, int32_t lo, int32_t hi) {")
    for mi, m in enumerate(spkmons):
        w(f"  if (kind == 0 && mon == {mi}) {{ n->sm{mi}_lo = lo; n->sm{mi}_hi = hi; n->sm{mi}_count.assign(hi - lo, 0); }}")
    for mi, m in enumerate(ratemons):
        w(f"  if (kind == 1 && mon == {mi}) {{ n->rm{mi}_lo = lo; n->rm{mi}_hi = hi; }}")
    w("}")
    w("void oracle_set_statemon(Net* n, int32_t mon, const int32_t* idx, int32_t nr, const int32_t* vars, int32_t nv) {")
    for mi, m in enumerate(statemons):
        w(f"  if (mon == {mi}) {{ n->st{mi}_idx.assign(idx, idx + nr); n->st{mi}_vars.assign(vars, vars + nv); }}")
    w("}")

    # ---- the step loop
    w("void oracle_run(Net* n, int64_t n_steps) {")
    if DRAWS:
        w("  _b200_gen = &n->gen; _b200_has = &n->has; _b200_kept = &n->kept;")
    for k, cst in enumerate(consts):
        w(f"  const {cst['ctype']} {cst['name']} = ({cst['ctype']})n->c[{k}]; (void){cst['name']};")
    w("  const double _dt_v = n->dt;")
    w(f"  const double* const {clock['dt']} = &_dt_v;")
    w("  for (int64_t _s = 0; _s < n_steps; ++_s) {")
    w("    const int64_t _ts_v = n->ts;")
    w("    const double _t_v = (double)n->ts * n->dt;")
    w(f"    const double* const {clock['t']} = &_t_v; (void){clock['t']};")
    w(f"    const int64_t* const {clock['timestep']} = &_ts_v; (void){clock['timestep']};")

    def gptrs(gi, indent):
        g = groups[gi]
        src = gi if g.get("alias_of") is None else g["alias_of"]  # (a custom event's group: its parent's state)
        return _ind("\n".join(f"{v['ctype']}* const {v['ptr']} = n->g{src}_{v['name']}.data(); (void){v['ptr']};"
                              for v in g["vars"]), indent)

    def extra(block, indent):
        lines = []
        for ptr, (kind, obj, var) in sorted((block or {}).get("extra_ptrs", {}).items()):
            v = groups[obj]["vars"][var]
            lines.append(f"{v['ctype']}* const {ptr} = n->g{obj}_{v['name']}.data(); (void){ptr};")
        return _ind("\n".join(lines), indent)

    def emit_ops(when):
        """Operations (run_regularly) of the slot, on the steps of their clock."""
        for gi, g in enumerate(groups):
            for op in g.get("ops", []):
                if op["when"] != when:
                    continue
                w(f"    if (n->ts % {op['every']} == 0) {{  // operation '{op['name']}'")
                w(gptrs(gi, 6))
                w(f"      const int32_t N = n->N{gi}; (void)N;")
                w("      {")
                w(_ind(op["code"]["scalar"], 8))
                w(f"        const int32_t _lo = {op['lo']}, _hi = {op['hi'] if op['hi'] >= 0 else 'N'};")
                w("        for (int32_t _b200_abs_idx = _lo; _b200_abs_idx < _hi; ++_b200_abs_idx) {")
                w("          const int32_t _idx = _b200_abs_idx - _lo;")
                w("          const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
                w(_ind(op["code"]["vector"], 10))
                w("        }")
                w("      }")
                w("    }")

    def emit_statemons(when):
        for mi, m in enumerate(statemons):
            if m.get("when", "start") != when or m.get("syn", -1) >= 0:
                continue
            emit_statemon(mi, m)

    def emit_syn(when):
        """Per-synapse code (clock-driven synaptic equations, run_regularly of a
        Synapses object; templates/stateupdate.cpp over the synapses) and state
        monitors of synaptic variables in the slot, in schedule order, over the
        synapses in creation order."""
        items = [("op", op) for op in spec.get("syn_ops", []) if op["when"] == when] + \
                [("mon", (mi, m)) for mi, m in enumerate(statemons) if m.get("syn", -1) >= 0 and
                 m.get("when", "start") == when]
        items.sort(key=lambda x: (x[1] if x[0] == "op" else x[1][1]).get("pos", 0))
        for kind, it in items:
            if kind == "mon":
                mi, m = it
                pi = m["syn"]
                w(f"    if (n->ts % {int(m.get('every', 1))} == 0) {{  // synaptic state monitor '{m['name']}'")
                w(f"      for (size_t v = 0; v < n->st{mi}_vars.size(); ++v) for (size_t r = 0; r < n->st{mi}_idx.size(); ++r) {{")
                w("        double val = 0;")
                for vi, v in enumerate(paths[pi].get("vars", [])):
                    w(f"        if (n->st{mi}_vars[v] == {vi}) val = (double)n->p{pi}_{v['name']}[n->st{mi}_idx[r]];")
                w(f"        n->st{mi}_data.push_back(val);")
                w("      }")
                w(f"      n->st{mi}_n++;")
                w("    }")
                continue
            pi = it["pathway"]
            p = paths[pi]
            w(f"    if (n->ts % {it['every']} == 0) {{  // per-synapse code '{it['name']}'")
            for v in p.get("vars", []):
                w(f"      {v['ctype']}* const {v['ptr']} = n->p{pi}_{v['name']}.data(); (void){v['ptr']};")
            w(f"      int32_t* const {p['pre_ptr']} = n->p{pi}_pre.data(); (void){p['pre_ptr']};")
            w(f"      int32_t* const {p['post_ptr']} = n->p{pi}_post.data(); (void){p['post_ptr']};")
            w("      {")
            w(_ind(it["code"]["scalar"], 8))
            w(f"        for (int64_t _idx = 0; _idx < (int64_t)n->p{pi}_pre.size(); ++_idx) {{")
            w("          const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            w(_ind(it["code"]["vector"], 10))
            w("        }")
            w("      }")
            w("    }")

    def emit_statemon(mi, m):
        gi = m["group"]
        w(f"    if (n->ts % {int(m.get('every', 1))} == 0) {{  // (a monitor on a slower clock: its steps)")
        w(gptrs(gi, 6))
        w(f"      for (size_t v = 0; v < n->st{mi}_vars.size(); ++v) for (size_t r = 0; r < n->st{mi}_idx.size(); ++r) {{")
        w("        double val = 0;")
        for vi, v in enumerate(groups[gi]["vars"]):
            w(f"        if (n->st{mi}_vars[v] == {vi}) val = (double)n->g{gi}_{v['name']}[n->st{mi}_idx[r]];")
        w(f"        n->st{mi}_data.push_back(val);")
        w("      }")
        w(f"      n->st{mi}_n++;")
        w("    }")

    # operations of the start slot, then the state monitors (start of the step)
    emit_ops("start")
    emit_statemons("start")
    emit_syn("start")
    emit_syn("groups")
    # summed variables (groups slot, before the groups' updates)
    for si, sm in enumerate(spec.get("summed", [])):
        pi, gi = sm["pathway"], sm["tgt_group"]
        p = paths[pi]
        tv = groups[gi]["vars"][sm["tgt_var"]]
        w(f"    {{  // summed variable {sm['name']}")
        w(f"      int32_t* const {p['pre_ptr']} = n->p{pi}_pre.data(); (void){p['pre_ptr']};")
        w(f"      int32_t* const {p['post_ptr']} = n->p{pi}_post.data(); (void){p['post_ptr']};")
        for v in p.get("vars", []):
            w(f"      {v['ctype']}* const {v['ptr']} = n->p{pi}_{v['name']}.data(); (void){v['ptr']};")
        for ptr, (gidx, vidx) in sorted(sm.get("group_ptrs", {}).items()):
            v = groups[gidx]["vars"][vidx]
            w(f"      {v['ctype']}* const {ptr} = n->g{gidx}_{v['name']}.data(); (void){ptr};")
        w(f"      {tv['ctype']}* const _tgt = n->g{gi}_{tv['name']}.data();")
        idx = f"n->p{pi}_post" if sm["index_post"] else f"n->p{pi}_pre"
        lo, hi = (f"n->p{pi}_tgt_lo", f"n->p{pi}_tgt_hi") if sm["index_post"] else (f"n->p{pi}_src_lo", f"n->p{pi}_src_hi")
        w(f"      for (int32_t _t = {lo}; _t < {hi}; ++_t) _tgt[_t] = 0;")
        w("      {")
        w(_ind(sm["code"]["scalar"], 8))
        w(f"        for (int64_t _idx = 0; _idx < (int64_t){idx}.size(); ++_idx) {{")
        w("          const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        w(_ind(sm["code"]["vector"], 10))
        w(f"          _tgt[{idx}[_idx]] += _synaptic_var;")
        w("        }")
        w("      }")
        w("    }")
    # state updaters of all groups (those drawing random numbers last, in the
    # schedule's order)
    for gi in block_order("update"):
        g = groups[gi]
        if not g.get("update"):
            continue
        w("    {")
        w(gptrs(gi, 6))
        w(f"      const int32_t N = n->N{gi}; (void)N;")
        w("      {")
        w(_ind(g["update"]["scalar"], 8))
        w(extra(g.get("update"), 8))
        w("        for (int32_t _idx = 0; _idx < N; ++_idx) {")
        w("          const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        w(_ind(g["update"]["vector"], 10))
        w("        }")
        w("      }")
        w("    }")
    # thresholders (those drawing random numbers last, in the schedule's order)
    for gi in block_order("threshold"):
        g = groups[gi]
        w("    {")
        w(gptrs(gi, 6))
        w(f"      const int32_t N = n->N{gi}; (void)N;")
        w(f"      n->spk{gi}.clear();")
        if g.get("generator"):
            w(f"      int32_t tb = (int32_t)n->ts; int32_t& last = n->gen{gi}_last;")
            w(f"      if (n->gen{gi}_period > 0) {{")
            w(f"        tb %= n->gen{gi}_period;")
            w(f"        if (last > 0 && n->gen{gi}_bins[last - 1] >= tb) last = 0;")
            w("      }")
            w(f"      for (size_t k = last; k < n->gen{gi}_bins.size(); ++k) {{")
            w(f"        if (n->gen{gi}_bins[k] > tb) break;")
            w(f"        n->spk{gi}.push_back(n->gen{gi}_index[k]);")
            w("      }")
            w(f"      last += (int32_t)n->spk{gi}.size();")
        if g.get("threshold"):
            w("      {")
            w(_ind(g["threshold"]["scalar"], 8))
            w(extra(g.get("threshold"), 8))
            w("        for (int32_t _idx = 0; _idx < N; ++_idx) {")
            w("          const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            w(_ind(g["threshold"]["vector"], 10))
            w("          if (_cond) {")
            w(f"            n->spk{gi}.push_back(_idx);")
            if g["threshold"].get("refractory"):
                nr = next(v["ptr"] for v in g["vars"] if v["name"] == "not_refractory")
                ls = next(v["ptr"] for v in g["vars"] if v["name"] == "lastspike")
                w(f"            {nr}[_idx] = false; {ls}[_idx] = _t_v;")
            w("          }")
            w("        }")
            w("      }")
        w("    }")
    # spike monitors
    for mi, m in enumerate(spkmons):
        gi = m["group"]
        w("    {")
        w(f"      const std::vector<int32_t>& sp = n->spk{gi};")
        w(f"      for (int32_t idx : sp) if (idx >= n->sm{mi}_lo && idx < n->sm{mi}_hi) {{")
        w(f"        n->sm{mi}_i.push_back(idx - n->sm{mi}_lo); n->sm{mi}_ts.push_back((int32_t)n->ts); n->sm{mi}_count[idx - n->sm{mi}_lo]++;")
        src = gi if groups[gi].get("alias_of") is None else groups[gi]["alias_of"]  # (an event monitor: the group's state)
        for k in m.get("vars", []):  # (spikemonitor.cpp:37-47: _source_<var>[idx] after the thresholder)
            w(f"        n->sm{mi}_vals.push_back((double)n->g{src}_{groups[gi]['vars'][k]['name']}[idx]);")
        w("      }")
        w("    }")
    def emit_inputs():
        for k, inp in enumerate(INPUTS):
            gi = inp["group"]
            w(f"    {{  // Poisson input {k} '{inp['name']}'")
            w(gptrs(gi, 6))
            w(f"      const int32_t N = n->N{gi}; (void)N;")
            w("      {")
            w(_ind(inp["code"]["scalar"], 8))
            w(f"        const int32_t _lo = {inp['lo']}, _hi = {inp['hi'] if inp['hi'] >= 0 else 'N'};")
            w("        for (int32_t _b200_abs_idx = _lo; _b200_abs_idx < _hi; ++_b200_abs_idx) {")
            w("          const int32_t _idx = _b200_abs_idx - _lo;")
            w("          const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            w(_ind(inp["code"]["vector"], 10))
            w("        }")
            w("      }")
            w("    }")

    # pathways: advance, push, peek, on_pre; the Poisson inputs between the
    # on_pre (order -1) and on_post (order +1) pathways
    inputs_done = False
    for pi, p in enumerate(paths):
        sg = p["src"]
        if p.get("prepost") == "post" and not inputs_done:
            emit_inputs()
            inputs_done = True
        w("    {")
        w(f"      std::vector<std::vector<int32_t>>& Q = n->p{pi}_queue; int& off = n->p{pi}_offset;")
        w("      Q[off].clear(); off = (off + 1) % (int)Q.size();")
        w(f"      const std::vector<int32_t>& sp = n->spk{sg};")
        w(f"      const int a = (int)(std::lower_bound(sp.begin(), sp.end(), n->p{pi}_src_lo) - sp.begin());")
        w(f"      const int b = (int)(std::upper_bound(sp.begin(), sp.end(), n->p{pi}_src_hi - 1) - sp.begin());")
        w("      for (int s = a; s < b; ++s) {")
        w(f"        const std::vector<int32_t>& syn = n->p{pi}_syn[sp[s] - n->p{pi}_src_lo];")
        w(f"        for (int32_t k : syn) Q[(off + n->p{pi}_delay[k]) % Q.size()].push_back(k);")
        w("      }")
        # the on_post pathway of a Synapses object shares the synapses (creation
        # order) and the synaptic variables of its on_pre pathway
        own = p.get("alias", -1) if p.get("alias", -1) >= 0 else pi
        # a pathway keeps its spiking side as `pre`: swapped for an on_post pathway
        sw = paths[own].get("prepost") == "post"
        w(f"      int32_t* const {p['pre_ptr']} = n->p{own}_{'post' if sw else 'pre'}.data(); (void){p['pre_ptr']};")
        w(f"      int32_t* const {p['post_ptr']} = n->p{own}_{'pre' if sw else 'post'}.data(); (void){p['post_ptr']};")
        for v in p.get("vars", []):
            w(f"      {v['ctype']}* const {v['ptr']} = n->p{own}_{v['name']}.data(); (void){v['ptr']};")
        for ptr, (gidx, vidx) in sorted(p.get("group_ptrs", {}).items()):
            v = groups[gidx]["vars"][vidx]
            arr = "acc_g" if (gidx, vidx) in ACC else "g"
            w(f"      {v['ctype']}* const {ptr} = n->{arr}{gidx}_{v['name']}.data(); (void){ptr};")
        w("      {")
        w(_ind(p["on_pre"]["scalar"], 8))
        w("        const std::vector<int32_t>& q = Q[off];")
        w("        for (size_t _q = 0; _q < q.size(); ++_q) {")
        w("          const int64_t _idx = q[_q];")
        w("          const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        w(_ind(p["on_pre"]["vector"], 10))
        w("        }")
        w("      }")
        w("    }")
    for gi, vi in ACC:  # push order: the step's deliveries reach their targets
        nm = groups[gi]["vars"][vi]["name"]
        w(f"    for (int32_t i = 0; i < n->N{gi}; ++i) {{ n->g{gi}_{nm}[i] += n->acc_g{gi}_{nm}[i]; n->acc_g{gi}_{nm}[i] = 0; }}")
    if not inputs_done:
        emit_inputs()
    # resets (a group's and its custom events' in the schedule's order)
    reset_seq = []
    for gi, g in enumerate(groups):
        if g.get("alias_of") is None:
            reset_seq += g.get("reset_order") or [gi]
    for gi in reset_seq:
        g = groups[gi]
        if not g.get("reset"):
            continue
        w("    {")
        w(gptrs(gi, 6))
        w(f"      const int32_t N = n->N{gi}; (void)N;")
        w("      {")
        w(_ind(g["reset"]["scalar"], 8))
        w(extra(g.get("reset"), 8))
        w(f"        for (int32_t _idx : n->spk{gi}) {{")
        w("          const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        w(_ind(g["reset"]["vector"], 10))
        w("        }")
        w("      }")
        w("    }")
    for mi, m in enumerate(ratemons):
        gi = m["group"]
        w(f"    {{ int c = 0; for (int32_t idx : n->spk{gi}) if (idx >= n->rm{mi}_lo && idx < n->rm{mi}_hi) ++c; n->rm{mi}_cnt.push_back(c); }}")
    emit_ops("end")  # (the rate monitors count spikes, which the operations do not change)
    emit_statemons("end")
    emit_syn("end")
    w("    n->ts += 1;")
    w("  }")
    w("}")
    for mi, _ in enumerate(spkmons):
        w(f"int64_t oracle_spikemon_size_{mi}(Net* n) {{ return (int64_t)n->sm{mi}_i.size(); }}")
        w(f"void oracle_spikemon_get_{mi}(Net* n, int32_t* i, int32_t* ts, int32_t* cnt) {{")
        w(f"  std::copy(n->sm{mi}_i.begin(), n->sm{mi}_i.end(), i); std::copy(n->sm{mi}_ts.begin(), n->sm{mi}_ts.end(), ts);")
        w(f"  std::copy(n->sm{mi}_count.begin(), n->sm{mi}_count.end(), cnt); }}")
        w(f"void oracle_spikemon_values_{mi}(Net* n, double* vals) {{ std::copy(n->sm{mi}_vals.begin(), n->sm{mi}_vals.end(), vals); }}")
    for mi, _ in enumerate(ratemons):
        w(f"int64_t oracle_ratemon_size_{mi}(Net* n) {{ return (int64_t)n->rm{mi}_cnt.size(); }}")
        w(f"void oracle_ratemon_get_{mi}(Net* n, int32_t* c) {{ std::copy(n->rm{mi}_cnt.begin(), n->rm{mi}_cnt.end(), c); }}")
    for mi, _ in enumerate(statemons):
        w(f"int64_t oracle_statemon_size_{mi}(Net* n) {{ return n->st{mi}_n; }}")
        w(f"void oracle_statemon_get_{mi}(Net* n, double* d) {{ std::copy(n->st{mi}_data.begin(), n->st{mi}_data.end(), d); }}")
    w("}  // extern C")
    return "\n".join(o) + "\n"


def _build(spec):
    src_text = render_oracle(spec)
    tag = hashlib.sha256(src_text.encode()).hexdigest()[:16]
    out = os.path.join(BUILD, f"oracle_{spec['name']}_{tag}.so")
    if not os.path.exists(out):
        os.makedirs(BUILD, exist_ok=True)
        src = out[:-3] + ".cpp"
        with open(src, "w") as f:
            f.write(src_text)
        tmp = out + f".tmp{os.getpid()}"
        cxx = shutil.which("g++") or "g++"
        r = subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                            "-w", src, "-o", tmp], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("oracle build failed:\n" + r.stderr[-4000:])
        os.replace(tmp, out)
    return out


class OracleNet:
    """Same interface subset as brian2_gb300.runtime.Network, on the CPU."""

    _libs = {}

    def __init__(self, spec, sizes, dt):
        self.spec = spec
        path = _build(spec)
        lib = self._libs.get(path)
        if lib is None:
            lib = self._libs[path] = C.CDLL(path)
            lib.oracle_create.restype = C.c_void_p
            lib.oracle_create.argtypes = [_i32p, C.c_double]
            lib.oracle_destroy.argtypes = [C.c_void_p]
            lib.oracle_var.restype = C.c_void_p
            lib.oracle_var.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
            lib.oracle_set_consts.argtypes = [C.c_void_p, _f64p, C.c_int32]
            lib.oracle_set_synapses.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, _i32p, C.c_int32, C.c_int32, C.c_int64,
                                                C.c_int32, C.c_int32, C.c_int32]
            lib.oracle_set_range.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
            lib.oracle_set_statemon.argtypes = [C.c_void_p, C.c_int32, _i32p, C.c_int32, _i32p, C.c_int32]
            lib.oracle_run.argtypes = [C.c_void_p, C.c_int64]
            lib.oracle_set_generator.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, C.c_int64, C.c_int32,
                                                 C.c_int32]
            lib.oracle_get_generator.argtypes = [C.c_void_p, C.c_int32]
            lib.oracle_get_generator.restype = C.c_int32
            lib.oracle_set_step.argtypes = [C.c_void_p, C.c_int64]
            lib.oracle_set_rng.argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.c_int32]
            lib.oracle_set_gauss.argtypes = [C.c_void_p, C.c_int32, C.c_double]
        self.lib = lib
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32).reshape(-1)
        self.h = lib.oracle_create(self.sizes.ctypes.data_as(_i32p), float(dt))
        self.n_syn = {}
        self._stm = {}

    def __del__(self):
        try:
            self.lib.oracle_destroy(self.h)
        except Exception:
            pass

    def _gv(self, group, var):
        gs = self.spec["groups"]
        g = group if isinstance(group, int) else [x["name"] for x in gs].index(group)
        names = [v["name"] for v in gs[g]["vars"]]
        v = var if isinstance(var, int) else names.index(var)
        return g, v, _CT_NP[gs[g]["vars"][v]["ctype"]]

    def set_consts(self, values: dict):
        cur = {c["name"]: c["value"] for c in self.spec.get("consts", [])}
        cur.update(values)
        a = np.array([float(cur[c["name"]]) for c in self.spec.get("consts", [])], np.float64)
        self.lib.oracle_set_consts(self.h, a.ctypes.data_as(_f64p), a.size)

    def upload(self, group, var, values):
        g, v, dt = self._gv(group, var)
        a = np.ascontiguousarray(values, dtype=dt)
        assert a.size == self.sizes[g]
        C.memmove(self.lib.oracle_var(self.h, 0, g, v), a.ctypes.data, a.nbytes)

    def download(self, group, var):
        g, v, dt = self._gv(group, var)
        a = np.empty(int(self.sizes[g]), dt)
        C.memmove(a.ctypes.data, self.lib.oracle_var(self.h, 0, g, v), a.nbytes)
        return a

    def _pv(self, pathway, var):
        ps = self.spec["pathways"]
        p = pathway if isinstance(pathway, int) else [x["name"] for x in ps].index(pathway)
        if ps[p].get("alias", -1) >= 0:
            p = ps[p]["alias"]  # shared synaptic variables
        names = [v["name"] for v in ps[p].get("vars", [])]
        v = var if isinstance(var, int) else names.index(var)
        return p, v, _CT_NP[ps[p]["vars"][v]["ctype"]]

    def set_synapses(self, pathway, pre, post, delay_steps=None, scalar_delay=0, src_range=None, tgt_range=None):
        ps = self.spec["pathways"]
        p = pathway if isinstance(pathway, int) else [x["name"] for x in ps].index(pathway)
        s0, s1 = src_range if src_range is not None else (0, int(self.sizes[ps[p]["src"]]))
        t0, t1 = tgt_range if tgt_range is not None else (0, int(self.sizes[ps[p]["tgt"]]))
        pre = np.ascontiguousarray(pre, np.int32)
        post = np.ascontiguousarray(post, np.int32)
        d = None if delay_steps is None else np.ascontiguousarray(delay_steps, np.int32)
        r = self.lib.oracle_set_synapses(self.h, p, pre.ctypes.data_as(_i32p), post.ctypes.data_as(_i32p),
                                         None if d is None else d.ctypes.data_as(_i32p), int(t1), int(scalar_delay),
                                         pre.size, s0, s1, t0)
        assert r == 0
        self.n_syn[p] = pre.size

    def upload_synapse_var(self, pathway, var, values):
        p, v, dt = self._pv(pathway, var)
        a = np.ascontiguousarray(values, dtype=dt)
        assert a.size == self.n_syn[p]
        C.memmove(self.lib.oracle_var(self.h, 1, p, v), a.ctypes.data, a.nbytes)

    def download_synapse_var(self, pathway, var):
        p, v, dt = self._pv(pathway, var)
        a = np.empty(self.n_syn[p], dt)
        C.memmove(a.ctypes.data, self.lib.oracle_var(self.h, 1, p, v), a.nbytes)
        return a

    def set_spikemon_range(self, mon, lo, hi):
        self.lib.oracle_set_range(self.h, 0, int(mon), int(lo), int(hi))

    def set_ratemon_range(self, mon, lo, hi):
        self.lib.oracle_set_range(self.h, 1, int(mon), int(lo), int(hi))

    def set_statemon(self, mon, indices, variables):
        sm = self.spec["state_monitors"][mon]
        if sm.get("syn", -1) >= 0:  # a Synapses object's monitor: its pathway's variables
            names = [v["name"] for v in self.spec["pathways"][sm["syn"]]["vars"]]
        else:
            names = [v["name"] for v in self.spec["groups"][sm["group"]]["vars"]]
        idx = np.ascontiguousarray(indices, np.int32)
        vs = np.ascontiguousarray([v if isinstance(v, int) else names.index(v) for v in variables], np.int32)
        self.lib.oracle_set_statemon(self.h, int(mon), idx.ctypes.data_as(_i32p), idx.size,
                                     vs.ctypes.data_as(_i32p), vs.size)
        self._stm[mon] = (vs.size, idx.size)

    def set_generator(self, group, timebins, indices, period_bins=0, last=0):
        b = np.ascontiguousarray(timebins, np.int32)
        i = np.ascontiguousarray(indices, np.int32)
        self.lib.oracle_set_generator(self.h, int(group), b.ctypes.data_as(_i32p), i.ctypes.data_as(_i32p), b.size,
                                      int(period_bins), int(last))

    def generator_cursor(self, group):
        return int(self.lib.oracle_get_generator(self.h, int(group)))

    def set_step(self, ts):
        self.lib.oracle_set_step(self.h, int(ts))

    def set_rng(self, words, position, gauss=None):
        w = np.ascontiguousarray(words, np.uint32)
        self.lib.oracle_set_rng(self.h, w.ctypes.data_as(C.POINTER(C.c_uint32)), int(position))
        if gauss is not None:  # randn()'s kept value: (has, value)
            self.lib.oracle_set_gauss(self.h, int(gauss[0]), float(gauss[1]))

    def run(self, n_steps):
        self.lib.oracle_run(self.h, int(n_steps))

    def spikes(self, mon=0):
        f = getattr(self.lib, f"oracle_spikemon_size_{mon}")
        f.restype = C.c_int64
        f.argtypes = [C.c_void_p]
        n = f(self.h)
        i = np.empty(n, np.int32)
        ts = np.empty(n, np.int32)
        g = self.spec["spike_monitors"][mon]["group"]
        cnt = np.empty(int(self.sizes[g]), np.int32)
        getattr(self.lib, f"oracle_spikemon_get_{mon}")(C.c_void_p(self.h), i.ctypes.data_as(_i32p),
                                                         ts.ctypes.data_as(_i32p), cnt.ctypes.data_as(_i32p))
        return i, ts, cnt

    def spike_values(self, mon=0):
        """[spikes, n_vars] values of the monitor's recorded variables."""
        nv = len(self.spec["spike_monitors"][mon].get("vars", []))
        f = getattr(self.lib, f"oracle_spikemon_size_{mon}")
        f.restype = C.c_int64
        f.argtypes = [C.c_void_p]
        n = f(self.h)
        a = np.empty((n, nv), np.float64)
        if nv and n:
            getattr(self.lib, f"oracle_spikemon_values_{mon}")(C.c_void_p(self.h), a.ctypes.data_as(C.POINTER(C.c_double)))
        return a

    def rate_counts(self, mon=0):
        f = getattr(self.lib, f"oracle_ratemon_size_{mon}")
        f.restype = C.c_int64
        f.argtypes = [C.c_void_p]
        n = f(self.h)
        a = np.empty(n, np.int32)
        getattr(self.lib, f"oracle_ratemon_get_{mon}")(C.c_void_p(self.h), a.ctypes.data_as(_i32p))
        return a

    def state_trace(self, mon=0):
        f = getattr(self.lib, f"oracle_statemon_size_{mon}")
        f.restype = C.c_int64
        f.argtypes = [C.c_void_p]
        n = f(self.h)
        nv, nr = self._stm[mon]
        a = np.empty((n, nv, nr), np.float64)
        getattr(self.lib, f"oracle_statemon_get_{mon}")(C.c_void_p(self.h), a.ctypes.data_as(_f64p))
        return a


def oracle_from_built(spec, built, dt=1e-4):
    """An OracleNet holding the same network as a brian2_gb300.workloads.Built."""
    o = OracleNet(spec, built.sizes, dt)
    if built.consts:
        o.set_consts(built.consts)
    for (g, v), arr in built.group_init.items():
        o.upload(g, v, arr)
    for pw, s in built.synapses.items():
        o.set_synapses(pw, s["pre"], s["post"], s.get("delay_steps"), s.get("scalar_delay", 0), s.get("src"),
                       s.get("tgt"))
        for var, arr in s.get("vars", {}).items():
            o.upload_synapse_var(pw, var, arr)
    for m, (lo, hi) in built.spikemon_ranges.items():
        o.set_spikemon_range(m if isinstance(m, int) else 0, lo, hi)
    for m, (lo, hi) in built.ratemon_ranges.items():
        o.set_ratemon_range(m if isinstance(m, int) else 0, lo, hi)
    return o


def run_job_on_oracle(directory, push_order=False):
    """Runs a job directory (brian2_gb300/job.py's format) on the oracle; the
    returned dict has run_job's keys for state, monitors and generator cursors.
    push_order: the oracle of the device's push-mode delivery."""
    import json as _json
    with open(os.path.join(directory, "spec.json")) as f:
        spec = _json.load(f)
    if push_order:
        spec = dict(spec, push_order=True)
    with open(os.path.join(directory, "job.json")) as f:
        job = _json.load(f)
    with np.load(os.path.join(directory, "init.npz")) as z:
        init = {k: z[k] for k in z.files}
    sizes = [int(init[f"g{gi}_N"]) for gi in range(len(spec["groups"]))]
    o = OracleNet(spec, sizes, job["dt"])
    for gi, g in enumerate(spec["groups"]):
        for v in g["vars"] if g.get("alias_of") is None else []:  # (a custom event's group shares them)
            o.upload(gi, v["name"], init[f"g{gi}_{v['name']}"])
        if g.get("generator"):
            o.set_generator(gi, init[f"g{gi}_gen_bins"], init[f"g{gi}_gen_index"], int(init[f"g{gi}_gen_period"]),
                            int(init[f"g{gi}_gen_last"]))
    for pi, p in enumerate(spec.get("pathways", [])):
        steps = init.get(f"p{pi}_delay_steps")
        o.set_synapses(pi, init[f"p{pi}_pre"], init[f"p{pi}_post"], steps, int(init[f"p{pi}_scalar_delay"]),
                       tuple(int(x) for x in init[f"p{pi}_src_range"]), tuple(int(x) for x in init[f"p{pi}_tgt_range"]))
        for v in p.get("vars", []) if p.get("alias", -1) < 0 else []:
            o.upload_synapse_var(pi, v["name"], init[f"p{pi}_{v['name']}"])
    for mi in range(len(spec.get("spike_monitors", []))):
        o.set_spikemon_range(mi, *(int(x) for x in init[f"sm{mi}_range"]))
    for mi in range(len(spec.get("rate_monitors", []))):
        o.set_ratemon_range(mi, *(int(x) for x in init[f"rm{mi}_range"]))
    for mi in range(len(spec.get("state_monitors", []))):
        o.set_statemon(mi, init[f"stm{mi}_idx"], list(init[f"stm{mi}_vars"]))
    o.set_step(int(init["ts0"]))
    if spec.get("draws"):
        o.set_rng(init["rng_words"], int(init["rng_position"]), init.get("rng_gauss"))
    from brian2_gb300.job import apply_actions  # (the job format's own helper)

    def download(kind, obj, var):
        return o.download(obj, var) if kind == "group" else o.download_synapse_var(obj, var)

    def upload(kind, obj, var, arr):
        (o.upload if kind == "group" else o.upload_synapse_var)(obj, var, arr)

    for k, n in enumerate(job["runs"]):
        o.run(int(n))
        apply_actions(job, init, k, download, upload)
    out = {}
    for gi, g in enumerate(spec["groups"]):
        for v in g["vars"] if g.get("alias_of") is None else []:
            out[f"g{gi}_{v['name']}"] = o.download(gi, v["name"])
        if g.get("generator"):
            out[f"g{gi}_gen_last"] = np.int64(o.generator_cursor(gi))
    for pi, p in enumerate(spec.get("pathways", [])):
        for v in p.get("vars", []) if p.get("alias", -1) < 0 else []:
            out[f"p{pi}_{v['name']}"] = o.download_synapse_var(pi, v["name"])
    for mi, m in enumerate(spec.get("spike_monitors", [])):
        out[f"sm{mi}_i"], out[f"sm{mi}_ts"], out[f"sm{mi}_count"] = o.spikes(mi)
        if m.get("vars"):
            out[f"sm{mi}_vals"] = o.spike_values(mi)
    for mi in range(len(spec.get("rate_monitors", []))):
        out[f"rm{mi}_counts"] = o.rate_counts(mi)
    for mi in range(len(spec.get("state_monitors", []))):
        out[f"stm{mi}_trace"] = o.state_trace(mi)
    return out
