"""Renders a network *spec* into one CUDA source file for sm_103a.

A spec is plain data (JSON-serialisable dict) describing one Brian2 network
model: its neuron groups with their state variables and the scalar/vector C++
snippets of the ``stateupdate``, ``threshold`` and ``reset`` code objects, its
synaptic pathways with the ``on_pre`` snippets, and its monitors.  The snippets
are produced by :class:`brian2_gb300.brian_device.B200CodeGenerator`, a subclass
of Brian's ``CPPCodeGenerator`` (``brian2/codegen/generators/cpp_generator.py:200``),
so the arithmetic is Brian's own; this module only places them into the fused
persistent step kernel and the host-side scalar evaluator.

The per-step schedule reproduced by the kernel is Brian's default schedule
(``brian2/core/network.py:42-50``): state update -> threshold -> spike monitor
-> synaptic propagation (push + on_pre) -> reset -> rate monitor, with the
clock tick ``t = timestep*dt`` (``brianlib/clocks.h:34-38``).  The reset is
applied at the start of the following step (or at the end of the launch), which
is equivalent because nothing reads the state in between.
"""
from __future__ import annotations

import hashlib
import json
import re

CTYPE_KIND = {"double": 0, "float": 1, "int32_t": 2, "char": 3, "int8_t": 3, "int64_t": 4}
KIND_NP = {0: "float64", 1: "float32", 2: "int32", 3: "int8", 4: "int64"}

_DECL_RE = re.compile(
    r"^\s*(?:const\s+)?(double|float|int32_t|int64_t|char|bool|int|long|size_t|uint32_t|uint64_t)\s+"
    r"([A-Za-z_]\w*)\s*(=|;)")


def spec_hash(spec: dict) -> str:
    return hashlib.sha256(json.dumps(spec, sort_keys=True).encode()).hexdigest()[:16]


def c_literal(value: float, ctype: str) -> str:
    if ctype in ("double", "float"):
        v = float(value)
        if v != v:
            return "NAN"
        if v in (float("inf"), float("-inf")):
            return "INFINITY" if v > 0 else "-INFINITY"
        return f"{v.hex()}"
    return str(int(value))


def scalar_outputs(code: str):
    """(ctype, name) of every variable declared by a scalar block, in order."""
    out = []
    for line in code.splitlines():
        m = _DECL_RE.match(line)
        if m:
            out.append((m.group(1), m.group(2)))
    return out


_FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def _single_precision(code: str) -> str:
    """Device code of a float32 network stays in single precision.

    Brian's float32 code objects keep namespace constants and literals in
    double (``const double Vt``, ``1.0f*(- 4.0)/ms``), which on the host costs
    nothing but on GB300 puts every such operation on the FP64 pipe (about
    1/64 of the FP32 rate).  Here double literals become float literals;
    constants and loop-invariant scalars are loaded as float (see
    ``_Tables.device_loads``).  The clock time and ``lastspike`` stay double.
    This is a deliberate difference from the reference's float32 mode, whose
    results the float32 device path matches within the stated tolerance, not
    bit for bit.
    """
    return _FLOAT_LIT.sub(lambda m: m.group(1) + "f", code)


def _indent(code: str, n: int) -> str:
    pad = " " * n
    return "\n".join(pad + ln if ln.strip() else "" for ln in code.splitlines())


def _block(spec_block):
    if not spec_block:
        return None
    return {"scalar": spec_block.get("scalar", "") or "", "vector": spec_block.get("vector", "") or "",
            "vector_device": spec_block.get("vector_device"), "refractory": spec_block.get("refractory", False)}


def split_time_dependent(code: str, clock_ptrs):
    """Brian's scalar blocks hold what is invariant over neurons, not over
    steps: a declaration that reads the clock's t or timestep (or a name
    declared from them) changes every step.  Returns (step-invariant lines,
    time-dependent lines)."""
    fixed, moving, names = [], [], set()
    for line in (code or "").splitlines():
        dep = any(p in line for p in clock_ptrs) or any(re.search(r"\b%s\b" % re.escape(n), line) for n in names)
        if dep:
            moving.append(line)
            m = _DECL_RE.match(line)
            if m:
                names.add(m.group(2))
        else:
            fixed.append(line)
    return "\n".join(fixed), "\n".join(moving)


class _Tables:
    """Scalar-table layout of one group or pathway: [constants | block scalars...].
    Block scalars that depend on the clock's time are not in the table: they
    are evaluated on the device every step (``time_code``)."""

    def __init__(self, consts, blocks, clock_ptrs=()):
        self.consts = consts
        self.entries = [(c["ctype"], c["name"]) for c in consts]
        self.block_ranges = {}
        self.fixed_code, self.moving_code = {}, {}
        for name, blk in blocks:
            if blk is None:
                continue
            fixed, moving = split_time_dependent(blk["scalar"], clock_ptrs)
            self.fixed_code[name], self.moving_code[name] = fixed, moving
            outs = scalar_outputs(fixed)
            self.block_ranges[name] = (len(self.entries), outs)
            self.entries += outs

    @property
    def size(self):
        return len(self.entries)

    def _load(self, ct, nm, k, single):
        et = "float" if (single and ct == "double") else ct
        src = {"double": "_b200_S", "float": "_b200_Sf"}.get(et, "_b200_Si")
        return f"const {et} {nm} = ({et}){src}[{k}];"

    def const_loads(self, single=False):
        """The namespace constants (the same values in every table of a model)."""
        return "\n".join(self._load(ct, nm, k, single) for k, (ct, nm) in enumerate(self.entries[:len(self.consts)]))

    def scalar_loads(self, name, single=False):
        """The loop-invariant scalars of one block (no constants)."""
        if name not in self.block_ranges:
            return ""
        off, outs = self.block_ranges[name]
        return "\n".join(self._load(ct, nm, off + k, single) for k, (ct, nm) in enumerate(outs))

    def time_code(self, name):
        """Device lines of the block's time-dependent scalars (clock reads as in
        the block: the caller maps them to the step's registers)."""
        return self.moving_code.get(name, "")

    def scalar_names(self, name):
        return [nm for _, nm in self.block_ranges.get(name, (0, []))[1]]

    def device_loads(self, name, single=False):
        """Declarations reading the constants and this block's scalars from the
        typed shared copies of S (_b200_S double, _b200_Sf float, _b200_Si
        integer), so no conversion runs per use (float instead of double when
        `single`)."""
        def load(ct, nm, k):
            et = "float" if (single and ct == "double") else ct
            src = {"double": "_b200_S", "float": "_b200_Sf"}.get(et, "_b200_Si")
            return f"const {et} {nm} = ({et}){src}[{k}];"
        lines = [load(ct, nm, k) for k, (ct, nm) in enumerate(self.entries[:len(self.consts)])]
        if name in self.block_ranges:
            off, outs = self.block_ranges[name]
            lines += [load(ct, nm, off + k) for k, (ct, nm) in enumerate(outs)]
        lines.append("(void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
        return "\n".join(lines)

    def host_eval(self, blocks):
        """Host code that evaluates the scalar blocks and fills _out."""
        lines = []
        for k, (ct, nm) in enumerate(self.entries[:len(self.consts)]):
            lines.append(f"_out[{k}] = (double){nm};")
        for name, blk in blocks:
            if blk is None or name not in self.block_ranges:
                continue
            off, outs = self.block_ranges[name]
            lines.append("{")
            lines.append(_indent(self.fixed_code[name], 2))
            for k, (ct, nm) in enumerate(outs):
                lines.append(f"  _out[{off + k}] = (double){nm};")
            lines.append("}")
        return "\n".join(lines)


# state words (4-byte) a thread keeps in flight in phase A's prefetch, in the
# kernel variants with more than 64 registers
PF_WORDS = 12
# events per thread whose loads are issued before any is applied (variants
# with more than 64 registers)
EVENT_BATCH = 4

_LOAD_RE = re.compile(r"^\s*(?:const\s+)?(\w+)\s+(\w+)\s*=\s*(_ptr_array_\w+)\[_idx\];\s*$")


def split_loads(code: str):
    """Brian's vector code starts with one load per variable it reads
    (``T x = _ptr_array_...[_idx];``).  Returns [(ctype, name, ptr)] of those
    leading loads and the code that follows them."""
    lines = (code or "").split("\n")
    loads, k = [], 0
    while k < len(lines):
        ln = lines[k]
        if not ln.strip():
            k += 1
            continue
        m = _LOAD_RE.match(ln)
        if not m:
            break
        loads.append((m.group(1), m.group(2), m.group(3)))
        k += 1
    return loads, "\n".join(lines[k:])


def stored_ptrs(code: str):
    return set(re.findall(r"(_ptr_array_\w+)\[_idx\]\s*=[^=]", code or ""))


def render_model(spec: dict) -> str:
    """Returns the complete .cu text for a spec."""
    groups = spec["groups"]
    paths = spec.get("pathways", [])
    spkmons = spec.get("spike_monitors", [])
    ratemons = spec.get("rate_monitors", [])
    statemons = spec.get("state_monitors", [])
    consts = spec.get("consts", [])
    clock = spec.get("clock_ptrs", {"dt": "_ptr_array_defaultclock_dt", "t": "_ptr_array_defaultclock_t",
                                     "timestep": "_ptr_array_defaultclock_timestep"})
    NG, NP = len(groups), len(paths)
    # device code reads the clock from registers, not through pointers to locals
    def _clockless(code):
        if not code:
            return code
        for key, var in (("t", "_b200_t"), ("dt", "_b200_dt"), ("timestep", "_b200_ts")):
            code = re.sub(re.escape(clock[key]) + r"\s*\[\s*0\s*\]", var, code)
        return code
    f32 = spec.get("float", "double") == "float"

    def _device(code):
        code = _clockless(code)
        return _single_precision(code) if (f32 and code) else code
    groups = [dict(g) for g in groups]
    for g in groups:
        for blk in ("update", "threshold", "reset"):
            if g.get(blk):
                g[blk] = dict(g[blk], vector=_device(g[blk].get("vector")))
        g["ops"] = [dict(op, code=dict(op["code"], vector=_device(op["code"]["vector"]))) for op in g.get("ops", [])]
    paths = [dict(p, on_pre=dict(p["on_pre"], vector=_device(p["on_pre"].get("vector")),
                                 vector_device=_device(p["on_pre"].get("vector_device"))))
             for p in paths]
    assert 1 <= NG <= 4 and NP <= 8 and len(spkmons) <= 4 and len(ratemons) <= 4 and len(statemons) <= 4

    o = []
    w = o.append
    w(f"// Generated by brian2_gb300.codegen for model '{spec['name']}' ({spec_hash(spec)}); do not edit.")
    w('#include "b200_device.cuh"')
    w("")
    # ------------------------------------------------------------- constants
    w("static const char* const b200_const_names[] = {" + ", ".join(f'"{c["name"]}"' for c in consts) + ("" if consts else '""') + "};")
    w("static const double b200_const_defaults[] = {" + ", ".join(c_literal(c["value"], "double") for c in consts) + ("" if consts else "0.0") + "};")
    w("")
    # Poisson inputs (PoissonInput), in schedule order: their scalar code sits in
    # their target group's table, their vector code runs over the group's neurons
    INPUTS = [dict(inp, code=dict(inp["code"], vector=_device(inp["code"]["vector"])))
              for inp in spec.get("inputs", [])]
    assert len(INPUTS) <= 8
    gtables, ptables = [], []
    for gi, g in enumerate(groups):
        blocks = [("update", _block(g.get("update"))), ("threshold", _block(g.get("threshold"))),
                  ("reset", _block(g.get("reset")))]
        blocks += [(f"input{k}", _block(inp["code"])) for k, inp in enumerate(INPUTS) if inp["group"] == gi]
        blocks += [(f"op{j}", _block(op["code"])) for j, op in enumerate(g["ops"])]
        gtables.append((_Tables(consts, blocks, (clock["t"], clock["timestep"])), blocks))
    SUMMED = spec.get("summed", [])
    # code objects drawing from the reference's generator, in the order of the draws
    DRAWS = spec.get("draws", [])
    assert len(DRAWS) <= 8

    def draw_macros(si, tsexpr):
        """Declarations reading draw site si's values of step `tsexpr` (drawn
        ahead by b200_variates_kernel): the c-th call of the site's code for
        neuron i is _b200_draw_<si>_<c>(i).  Returns (lines, undef lines)."""
        d = DRAWS[si]
        calls = d["calls"]
        cast = {"binomial": "(long long)", "binormal": "(float)"}.get(d["kind"], "")
        lines = [f"const double* const _b200_rv{si} = I.rng_vals + (({tsexpr}) - I.rng_ts0) * I.rng_per_step + I.draw_off[{si}];"]
        undef = []
        for c in range(calls):
            lines.append(f"#define _b200_draw_{si}_{c}(i) ({cast}_b200_rv{si}[(int64_t)(i) * {calls} + {c}])")
            undef.append(f"#undef _b200_draw_{si}_{c}")
        return lines, undef
    # per-synapse code of a Synapses object (clock-driven equations, run_regularly)
    # and state monitors of its variables, over its synapses in CSR order
    SYNOPS = spec.get("syn_ops", [])
    SYNMONS = [(mi, m) for mi, m in enumerate(statemons) if m.get("syn", -1) >= 0]
    for pi, p in enumerate(paths):
        blocks = [("on_pre", _block(p.get("on_pre")))]
        blocks += [(f"summed{si}", _block(sm["code"])) for si, sm in enumerate(SUMMED) if sm["pathway"] == pi]
        blocks += [(f"synop{j}", _block(op["code"])) for j, op in enumerate(SYNOPS) if op["pathway"] == pi]
        ptables.append((_Tables(consts, blocks, (clock["t"], clock["timestep"])), blocks))

    SIZE = {"double": 8, "int64_t": 8, "float": 4, "int32_t": 4, "char": 1, "int8_t": 1}

    def used_vars(gi):
        """Variables of group gi that the step code touches (cached in smem)."""
        g = groups[gi]
        text = ""
        for blk in ("update", "threshold", "reset"):
            if g.get(blk):
                text += g[blk].get("vector", "") + "\n" + json.dumps(g[blk].get("extra_ptrs", {}))
        for inp in INPUTS:
            if inp["group"] == gi:
                text += inp["code"]["vector"] + "\n"
        for op in g.get("ops", []):
            text += op["code"]["vector"] + "\n"
        for p in paths:
            text += (p["on_pre"].get("vector_device") or p["on_pre"].get("vector", "")) + json.dumps(p.get("group_ptrs", {}))
        for sm in SUMMED:
            text += sm["code"].get("vector", "") + json.dumps(sm["group_ptrs"])
            if sm["tgt_group"] == gi:
                text += " " + g["vars"][sm["tgt_var"]]["ptr"] + " "
            for gg in groups:
                for blk in ("update", "threshold", "reset"):
                    if gg.get(blk):
                        text += json.dumps(gg[blk].get("extra_ptrs", {}))
        used = []
        for k, v in enumerate(g["vars"]):
            if re.search(r"\b%s\b" % re.escape(v["ptr"]), text):
                used.append(k)
            elif v["name"] in ("not_refractory", "lastspike") and g.get("threshold") and g["threshold"].get("refractory"):
                used.append(k)
        # pack 8-byte variables first so every cached array stays aligned
        return sorted(used, key=lambda k: -SIZE[g["vars"][k]["ctype"]])

    # a custom event's group (alias_of: the group whose events they are) has no
    # state of its own: its pointers are its parent's, cached with the parent's
    ALIAS = [g.get("alias_of") for g in groups]
    USED = [used_vars(gi) if ALIAS[gi] is None else [] for gi in range(NG)]

    def private_vars(gi):
        """Used variables of group gi that only the CTA owning a neuron touches:
        no pathway's on_pre and no other block's pointers name them (so a
        multi-CTA classic instance may keep them in shared memory)."""
        g = groups[gi]
        if g.get("generator"):
            return []
        text = ""
        for p in paths:
            text += json.dumps(p.get("on_pre", {})) + json.dumps(p.get("group_ptrs", {}))
        for sm in SUMMED:  # (a summed expression reads other neurons' variables)
            text += json.dumps(sm["code"]) + json.dumps(sm["group_ptrs"])
        for gg in groups:
            for blk in ("update", "threshold", "reset"):
                if gg.get(blk):
                    text += json.dumps(gg[blk].get("extra_ptrs", {}))
        return [k for k in USED[gi] if not re.search(r"\b%s\b" % re.escape(g["vars"][k]["ptr"]), text)]

    PRIV = [private_vars(gi) if ALIAS[gi] is None else [] for gi in range(NG)]

    def syn_arr(pi, which):
        """Device array holding Brian's _synaptic_pre ('pre') or _synaptic_post
        ('post') for pathway pi: a pathway stores its spiking side as `pre`, so
        an on_post pathway that owns its synapses has them swapped."""
        if paths[pi].get("prepost") == "post":
            return {"pre": "post", "post": "pre"}[which]
        return which

    def owner_payloads():
        """Owner mode applies when every on_pre only adds, into variables of its
        target neuron, values computed from synaptic variables and constants.
        Returns, per pathway, the synaptic variables an event carries (indices
        into the pathway's variables), or None for the whole model."""
        if not paths or SUMMED or SYNOPS or SYNMONS or \
                any(p.get("alias", -1) >= 0 or not p.get("events", True) for p in paths):
            return None
        for g in groups:
            for blk in ("update", "threshold", "reset"):
                if g.get(blk) and g[blk].get("extra_ptrs"):
                    return None
        out = []
        for p in paths:
            code = p["on_pre"].get("vector_device") or p["on_pre"].get("vector") or ""
            loads, rest = split_loads(code)
            varptr = {v["ptr"]: k for k, v in enumerate(p.get("vars", []))}
            pay, has_post = [], False
            for ct, nm, ptr in loads:
                if ptr == p["post_ptr"] and nm == "_postsynaptic_idx":
                    has_post = True
                elif ptr in varptr and SIZE.get(ct) in (4, 8):
                    pay.append(varptr[ptr])
                else:
                    return None
            if not has_post or len(pay) > 4:
                return None
            tgt_ptrs = {ptr for ptr, (gi, vi) in p.get("group_ptrs", {}).items() if gi == p["tgt"]}
            for ln in rest.split("\n"):
                ln = ln.strip()
                if not ln:
                    continue
                m = re.match(r"^_b200_atomic_add\(&(\w+)\[_postsynaptic_idx\],\s*(.*)\);$", ln)
                if not m or m.group(1) not in tgt_ptrs or "_ptr_array" in m.group(2) or "[" in m.group(2):
                    return None
            out.append(pay)
        return out

    PAYLOAD = owner_payloads()
    OWNER = PAYLOAD is not None
    # device profile slots: classic kernel A, barrier A, lists, one per pathway,
    # barrier B; owner kernel update, barrier, lists, push pass 1, batch table +
    # pass 2, delivery
    # classic kernel, after those: per group update, threshold, reset; per group
    # the copy of its spikes into the delay ring; per spike / rate monitor its
    # recording (the code objects of profile_slots())
    NSM, NRM = len(spkmons), len(ratemons)
    PH_UPD = lambda gi: 6 + NP + 3 * gi
    PH_THR = lambda gi: 7 + NP + 3 * gi
    PH_RST = lambda gi: 8 + NP + 3 * gi
    PH_RING = lambda gi: 6 + NP + 3 * NG + gi
    PH_SPKMON = lambda m: 6 + NP + 4 * NG + m
    PH_RATEMON = lambda m: 6 + NP + 4 * NG + NSM + m
    NPH = 6 + NP + 4 * NG + NSM + NRM
    MAXV = max(len(g["vars"]) for g in groups)

    # ------------------------------------------------------------- model tables
    for gi, g in enumerate(groups):
        w(f"static const char* const b200_g{gi}_vars[] = {{" + ", ".join(f'"{v["name"]}"' for v in g["vars"]) + "};")
        w(f"static const int b200_g{gi}_kinds[] = {{" + ", ".join(str(CTYPE_KIND[v["ctype"]]) for v in g["vars"]) + "};")
        w(f"static const int b200_g{gi}_used[] = {{" + ", ".join("1" if k in USED[gi] else "0" for k in range(len(g["vars"]))) + "};")
        w(f"static const int b200_g{gi}_priv[] = {{" + ", ".join("1" if k in PRIV[gi] else "0" for k in range(len(g["vars"]))) + "};")
    for pi, p in enumerate(paths):
        pv = p.get("vars", [])
        w(f"static const char* const b200_p{pi}_vars[] = {{" + ", ".join(f'"{v["name"]}"' for v in pv) + ('' if pv else '""') + "};")
        w(f"static const int b200_p{pi}_kinds[] = {{" + ", ".join(str(CTYPE_KIND[v["ctype"]]) for v in pv) + ('' if pv else '0') + "};")
    w("static const b200_group_info b200_groups[] = {" + ", ".join(
        f'{{"{g["name"]}", {len(g["vars"])}, b200_g{gi}_vars, b200_g{gi}_kinds, {gtables[gi][0].size}, b200_g{gi}_used, '
        f'{1 if g.get("generator") else 0}, b200_g{gi}_priv, {-1 if ALIAS[gi] is None else ALIAS[gi]}}}'
        for gi, g in enumerate(groups)) + "};")
    for pi, p in enumerate(paths):
        pay = PAYLOAD[pi] if OWNER else []
        w(f"static const int b200_p{pi}_payload[] = {{" + (", ".join(str(k) for k in pay) if pay else "0") + "};")
    if paths:
        w("static const b200_pathway_info b200_pathways[] = {" + ", ".join(
            f'{{"{p["name"]}", {p["src"]}, {p["tgt"]}, {len(p.get("vars", []))}, b200_p{pi}_vars, b200_p{pi}_kinds, '
            f'{ptables[pi][0].size}, {len(PAYLOAD[pi]) if OWNER else 0}, b200_p{pi}_payload, {p.get("alias", -1)}}}'
            for pi, p in enumerate(paths)) + "};")
    else:
        w("static const b200_pathway_info* const b200_pathways = nullptr;")
    for nm, mons in (("spkmon", spkmons), ("ratemon", ratemons), ("statemon", statemons)):
        if mons:
            w(f"static const b200_mon_info b200_{nm}[] = {{" + ", ".join(
                f'{{"{m["name"]}", {m["group"]}, {m.get("every", 1)}, {len(m.get("vars", [])) if nm == "spkmon" else 0}, '
                f'{m.get("syn", -1)}}}' for m in mons) + "};")
        else:
            w(f"static const b200_mon_info* const b200_{nm} = nullptr;")
    w("")

    # ------------------------------------------------------------- host scalars
    w("// Host evaluation of the scalar (loop-invariant) blocks.  Compiled by the host")
    w("// compiler with IEEE semantics (-ffp-contract=off), so values equal those of")
    w("// Brian's C++ code objects, which evaluate the same expressions per call.")
    w("static void b200_eval_scalars(int _kind, int _id, const double* _c, double _b200_dt, double* _out) {")
    for k, c in enumerate(consts):
        w(f"  const {c['ctype']} {c['name']} = ({c['ctype']})_c[{k}];")
    w(f"  const double* const {clock['dt']} = &_b200_dt;")
    w(f"  const double _b200_t0 = 0.0; const double* const {clock['t']} = &_b200_t0;")
    w(f"  const int64_t _b200_ts0 = 0; const int64_t* const {clock['timestep']} = &_b200_ts0;")
    w(f"  (void){clock['dt']}; (void){clock['t']}; (void){clock['timestep']}; (void)_c;")
    for k, c in enumerate(consts):
        w(f"  (void){c['name']};")
    for gi, (tab, blocks) in enumerate(gtables):
        w(f"  if (_kind == 0 && _id == {gi}) {{")
        w(_indent(tab.host_eval(blocks), 4))
        w("  }")
    for pi, (tab, blocks) in enumerate(ptables):
        w(f"  if (_kind == 1 && _id == {pi}) {{")
        w(_indent(tab.host_eval(blocks), 4))
        w("  }")
    w("}")
    w("")

    # ------------------------------------------------------------- kernel
    def gptr_decls(gi, indent, restrict):
        g = groups[gi]
        r = " __restrict__" if restrict else ""
        lines = [f"{v['ctype']}*{r} const {v['ptr']} = ({v['ctype']}*)s_gv[{gi}][{k}]; (void){v['ptr']};"
                 for k, v in enumerate(g["vars"])]
        return _indent("\n".join(lines), indent)

    def snap_code(gi, idx):
        """The recorded variables of the spike monitors of group gi for the
        spiking neuron `idx`, taken when the thresholder runs (after the
        update, before the step's deliveries and its reset)."""
        out = []
        for mi, m in enumerate(spkmons):
            if m["group"] == gi:
                for v, k in enumerate(m.get("vars", [])):
                    ptr = groups[gi]["vars"][k]["ptr"]
                    out.append(f"I.sm[{mi}].snap[(size_t){v} * I.g[{gi}].N + ({idx})] = (double){ptr}[{idx}];")
        return " ".join(out)

    def value_rows(mi, gi, pos, idx):
        """The recorded variables of spike monitor mi into its row `pos`."""
        m = spkmons[mi]
        nv = len(m.get("vars", []))
        return " ".join(f"SM.vals[({pos}) * {nv} + {v}] = SM.snap[(size_t){v} * I.g[{gi}].N + ({idx})];"
                        for v in range(nv))

    def extra_ptrs(block_spec, indent):
        lines = []
        for ptr, (kind, obj, var) in sorted((block_spec or {}).get("extra_ptrs", {}).items()):
            if kind == "group":
                v = groups[obj]["vars"][var]
                lines.append(f"{v['ctype']}* const {ptr} = ({v['ctype']}*)s_gv[{obj}][{var}]; (void){ptr};")
        return _indent("\n".join(lines), indent)

    def owner_list(gi, tsexpr):
        """Owner mode: spike list and tile counts of step `tsexpr` in the ring."""
        return (f"I.g[{gi}].ring + (int64_t)(({tsexpr}) % B200_OWNER_RING) * I.g[{gi}].N",
                f"I.g[{gi}].ring_prefix + (int64_t)(({tsexpr}) % B200_OWNER_RING) * (I.g[{gi}].n_tiles + 1)")

    def reset_block(gi, indent, tsexpr, owner=False):
        """Reset of the spikes of step `tsexpr` in this CTA's tiles."""
        tab, blocks = gtables[gi]
        bd = dict(blocks)
        if bd["reset"] is None:
            return ""
        g = groups[gi]
        scr_e, tc_e = owner_list(gi, tsexpr) if owner else (f"s_oscr[{gi}]", f"s_otc[{gi}]")
        L = ["{",
             f"  const double _b200_t = (double)({tsexpr}) * _b200_dt; (void)_b200_t;  // the step of the reset",
             f"  const int64_t _b200_ts = {tsexpr}; (void)_b200_ts;",
             f"  const int32_t* const scr = {scr_e}; const int32_t* const tcnt = {tc_e};",
             f"  const int* const tst = s_tst + {gi} * max_tiles1;",
             f"  const int32_t N = I.g[{gi}].N; (void)N;",
             f"  const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;",
             gptr_decls(gi, 2, False),
             f"  for (int u = s_ut[{gi}][0]; u < s_ut[{gi}][1]; ++u) {{",
             "    const int cnt = tcnt[u], base = tst[u];",
             "    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {",
             "      const int32_t _idx = scr[base + j];",
             "      const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;",
             "      {",
             _indent(tab.device_loads("reset", f32), 8),
             _indent(_device(tab.time_code("reset")), 8),
             extra_ptrs(g.get("reset"), 8),
             _indent(bd["reset"]["vector"], 8),
             "      }",
             "    }",
             "  }",
             "}"]
        return _indent("\n".join(L), indent)

    def input_block(gi, indent, tsexpr):
        """The Poisson inputs into group gi of step `tsexpr`, over this CTA's
        neurons: the reference runs them in the synapses slot, after every
        on_pre delivery of the step and before the resets
        (brian2/input/poissoninput.py:126-135, templates/stateupdate.cpp:5-21)."""
        ins = [(k, inp) for k, inp in enumerate(INPUTS) if inp["group"] == gi]
        if not ins:
            return ""
        tab, _ = gtables[gi]
        L = ["{",
             f"  const double _b200_t = (double)({tsexpr}) * _b200_dt; (void)_b200_t;  // the step of the inputs",
             f"  const int64_t _b200_ts = {tsexpr}; (void)_b200_ts;",
             f"  const int32_t N = I.g[{gi}].N; (void)N;",
             f"  const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;",
             gptr_decls(gi, 2, False),
             f"  const int _own0 = s_tst[{gi} * max_tiles1 + s_ut[{gi}][0]], _own1 = s_tst[{gi} * max_tiles1 + s_ut[{gi}][1]];"]
        for q, (k, inp) in enumerate(ins):
            hi = str(inp["hi"]) if inp["hi"] >= 0 else "N"
            if q:
                L.append("  __syncthreads();  // (inputs into one variable add in schedule order)")
            dl, du = draw_macros(inp["draw"], tsexpr)
            L += [f"  {{  // Poisson input {k} '{inp['name']}'",
                  f"    const int _lo = {inp['lo']}, _hi = {hi};",
                  _indent("\n".join(dl), 4),
                  _indent(tab.device_loads(f"input{k}", f32), 4),
                  _indent(_device(tab.time_code(f"input{k}")), 4),
                  "    const int _a = _own0 > _lo ? _own0 : _lo, _b = _own1 < _hi ? _own1 : _hi;",
                  "    for (int _b200_abs_idx = _a + (int)threadIdx.x; _b200_abs_idx < _b; _b200_abs_idx += (int)blockDim.x) {",
                  "      const int32_t _idx = _b200_abs_idx - _lo;",
                  "      const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;",
                  "      {",
                  _indent(inp["code"]["vector"], 8),
                  "      }",
                  "    }",
                  "\n".join(du),
                  "  }"]
        L += ["}"]
        return _indent("\n".join(L), indent)

    def op_block(gi, indent, tsexpr, when):
        """The operations (run_regularly) of group gi in slot `when` of step
        `tsexpr`, over this CTA's neurons, each on the steps of its clock."""
        ops = [(j, op) for j, op in enumerate(groups[gi].get("ops", [])) if op["when"] == when]
        if not ops:
            return ""
        tab, _ = gtables[gi]
        L = ["{",
             f"  const double _b200_t = (double)({tsexpr}) * _b200_dt; (void)_b200_t;  // the step of the operations",
             f"  const int64_t _b200_ts = {tsexpr}; (void)_b200_ts;",
             f"  const int32_t N = I.g[{gi}].N; (void)N;",
             f"  const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;",
             gptr_decls(gi, 2, False),
             f"  const int _own0 = s_tst[{gi} * max_tiles1 + s_ut[{gi}][0]], _own1 = s_tst[{gi} * max_tiles1 + s_ut[{gi}][1]];"]
        for q, (j, op) in enumerate(ops):
            hi = str(op["hi"]) if op["hi"] >= 0 else "N"
            if q:
                L.append("  __syncthreads();  // (operations on one variable run in schedule order)")
            L += [f"  if (_b200_ts % {op['every']} == 0) {{  // operation '{op['name']}'",
                  f"    const int _lo = {op['lo']}, _hi = {hi};",
                  _indent(tab.device_loads(f"op{j}", f32), 4),
                  _indent(_device(tab.time_code(f"op{j}")), 4),
                  "    const int _a = _own0 > _lo ? _own0 : _lo, _b = _own1 < _hi ? _own1 : _hi;",
                  "    for (int _b200_abs_idx = _a + (int)threadIdx.x; _b200_abs_idx < _b; _b200_abs_idx += (int)blockDim.x) {",
                  "      const int32_t _idx = _b200_abs_idx - _lo;",
                  "      const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;",
                  "      {",
                  _indent(op["code"]["vector"], 8),
                  "      }",
                  "    }",
                  "  }"]
        L.append("}")
        return _indent("\n".join(L), indent)

    def syn_text(indent, tsexpr, when):
        """The per-synapse code and the synaptic state monitors of slot `when`
        of step `tsexpr`, in schedule order, over this CTA's share of each
        Synapses object's synapses (a contiguous range of CSR positions); each
        on the steps of its clock.  Ends with a barrier of the CTA."""
        items = [("op", j, op) for j, op in enumerate(SYNOPS) if op["when"] == when] + \
                [("mon", mi, m) for mi, m in SYNMONS if m.get("when", "start") == when]
        if not items:
            return ""
        items.sort(key=lambda x: x[2].get("pos", 0))
        L = ["{",
             f"  const double _b200_t = (double)({tsexpr}) * _b200_dt; (void)_b200_t;",
             f"  const int64_t _b200_ts = {tsexpr}; (void)_b200_ts;"]
        for kind, j, it in items:
            pi = it["pathway"] if kind == "op" else it["syn"]
            p = paths[pi]
            every = int(it.get("every", 1))
            L += [f"  if (_b200_ts % {every} == 0) {{  // {'code' if kind == 'op' else 'state monitor'} '{it['name']}'",
                  f"    const b200_pathway_d& PQ = I.p[{pi}];",
                  "    const int64_t _q0 = PQ.n_syn * rank / I.n_cta, _q1 = PQ.n_syn * (rank + 1) / I.n_cta;"]
            if kind == "op":
                tab = ptables[pi][0]
                L += [f"    const double* const _b200_S = s_Sp{pi}; const float* const _b200_Sf = s_Sp{pi}f; "
                      f"const long long* const _b200_Si = s_Sp{pi}i;",
                      "    (void)_b200_S; (void)_b200_Sf; (void)_b200_Si;"]
                for k, v in enumerate(p.get("vars", [])):
                    L.append(f"    {v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)PQ.var[{k}]; (void){v['ptr']};")
                L += [f"    const int32_t* __restrict__ const {p['pre_ptr']} = PQ.pre; (void){p['pre_ptr']};",
                      f"    const int32_t* __restrict__ const {p['post_ptr']} = PQ.post; (void){p['post_ptr']};",
                      _indent(tab.device_loads(f"synop{j}", f32), 4),
                      _indent(_device(tab.time_code(f"synop{j}")), 4),
                      "    for (int64_t _idx = _q0 + threadIdx.x; _idx < _q1; _idx += blockDim.x) {",
                      "      const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;",
                      "      {",
                      _indent(it["code"]["vector"], 8),
                      "      }",
                      "    }"]
            else:
                rec = ("_b200_ts - SM.step0" if every == 1 else
                       f"_b200_ts / {every} - (SM.step0 + {every - 1}) / {every}")
                L += [f"    const b200_statemon_d& SM = I.stm[{j}];",
                      f"    const int64_t rec = {rec};  // row of this step",
                      "    double* const row = SM.data + (size_t)rec * SM.n_vars * SM.n_rec;",
                      "    for (int k = threadIdx.x; k < SM.n_rec * SM.n_vars; k += blockDim.x) {",
                      "      const int r = k % SM.n_rec, v = k / SM.n_rec;",
                      "      const int64_t pos = SM.idx[r];  // the synapse's CSR position",
                      "      if (pos >= _q0 && pos < _q1) {",
                      "        double val = 0.0;",
                      "        switch (SM.var_id[v]) {"]
                for k, v in enumerate(p.get("vars", [])):
                    L.append(f"          case {k}: val = (double)(({v['ctype']}*)PQ.var[{k}])[pos]; break;")
                L += ["        }",
                      "        row[k] = val;",
                      "      }",
                      "    }",
                      f"    if (threadIdx.x == 0) s_stm_n[{j}] = rec + 1;"]
            L += ["  }", "  __syncthreads();"]
        L.append("}")
        return _indent("\n".join(L), indent)

    def deferred_block(gi, indent, tsexpr, owner=False):
        """What the reference runs after the deliveries of step `tsexpr`: the
        Poisson inputs, the reset, the end-slot operations and state monitors
        (this CTA's neurons)."""
        if ALIAS[gi] is not None:
            return ""  # (its reset runs in its parent's block)
        resets = [reset_block(k, indent, tsexpr, owner) for k in (groups[gi].get("reset_order") or [gi])]
        parts = [x for x in [input_block(gi, indent, tsexpr)] + resets +
                 [op_block(gi, indent, tsexpr, "end"), statemon_text(gi, indent, tsexpr, "end")] if x]
        return ("\n" + " " * indent + "__syncthreads();\n").join(parts)

    def emit_generator(gi, owner):
        """A spike generator group's step (templates/spikegenerator.cpp:5-31):
        the entries from the cursor whose time bin is <= the step's (modulo
        the period), compacted per tile in array order (the entries of a bin
        are sorted by neuron index, input/spikegeneratorgroup.py:356)."""
        if owner:
            scr_e, tc_e = owner_list(gi, "ts")
        else:
            scr_e, tc_e = f"s_scr[{gi}]", f"s_tc[{gi}]"
        w(f"      {{  // ---- group {gi} '{groups[gi]['name']}': spike generator")
        w(f"        const b200_group_d& GG = I.g[{gi}];")
        w(f"        int32_t* const scr = {scr_e}; int32_t* const tcnt = {tc_e};")
        if not owner:
            w(f"        int32_t* const oscr = s_oscr[{gi}]; int32_t* const otc = s_otc[{gi}];")
        w(f"        const int* const tst = s_tst + {gi} * max_tiles1;")
        w("        if (threadIdx.x == 0) {")
        w(f"          long long tb = ts; int lo = s_glast[{gi}];")
        w("          if (GG.gen_period > 0) {")
        w("            tb %= GG.gen_period;")
        w("            if (lo > 0 && GG.gen_bins[lo - 1] >= tb) lo = 0;")
        w("          }")
        w("          int a = lo, b = (int)GG.gen_n;  // first entry after the step's bin")
        w("          while (a < b) { const int m = (a + b) >> 1; if (GG.gen_bins[m] <= tb) a = m + 1; else b = m; }")
        w(f"          s_gen_lo = lo; s_gen_hi = a; s_glast[{gi}] = a;")
        w("        }")
        w("        __syncthreads();")
        w("        const int glo = s_gen_lo, ghi = s_gen_hi;")
        w(f"        for (int u = s_ut[{gi}][0]; u < s_ut[{gi}][1]; ++u) {{")
        w("          const int t0 = tst[u], t1 = tst[u + 1];")
        w("          int cnt = 0;")
        w("          for (int j0 = glo; j0 < ghi; j0 += blockDim.x) {")
        w("            const int j = j0 + threadIdx.x;")
        w("            const int idx = j < ghi ? GG.gen_index[j] : -1;")
        w("            const bool f = idx >= t0 && idx < t1;")
        w("            int tot;")
        w("            const int rk = b200_block_compact(f, s_wsum, &tot);")
        w("            if (f && t0 + cnt + rk < t1) {")
        w("              scr[t0 + cnt + rk] = idx;")
        if not owner:
            w("              oscr[t0 + cnt + rk] = idx;")
        w("            }")
        w("            cnt += tot;")
        w("          }")
        w("          if (cnt > t1 - t0) cnt = t1 - t0;")
        w("          if (threadIdx.x == 0) { tcnt[u] = cnt;" + ("" if owner else " otc[u] = cnt;") + " }")
        w("        }")
        w("        __syncthreads();")
        w("      }")

    QUADV = {"float": ("float4", 4), "int32_t": ("int4", 4), "char": ("char4", 1), "int8_t": ("char4", 1)}

    def emit_quad(gi, g, bd, tab, hoist_sc):
        """Update + threshold four neurons per thread with 16-byte (4-byte for
        1-byte variables) loads and stores, when every variable the update and
        threshold load or store is one of this group's 4- or 1-byte state
        variables; the CTA takes this path when its state pointers are aligned
        for it (s_quad), else the per-neuron path that follows.  Opens the
        `if (s_quad) { ... } else {` that the caller closes.  Same order of
        spikes (ascending) and the same arithmetic per neuron."""
        upd_v = bd["update"]["vector"] if bd["update"] is not None else ""
        thr_v = bd["threshold"]["vector"] if bd["threshold"] is not None else ""
        upd_loads, upd_rest = split_loads(upd_v)
        thr_loads, thr_rest = split_loads(thr_v)
        upd_st = stored_ptrs(upd_v)
        own = {v["ptr"]: v for v in g["vars"]}
        pf = {}
        for ct, nm, ptr in upd_loads + [x for x in thr_loads if x[2] not in upd_st]:
            pf.setdefault(ptr, ct)
        st_lines = {}
        rest_lines = []
        for ln in upd_rest.split("\n"):
            m = re.match(r"^\s*(_ptr_array_\w+)\[_idx\]\s*=\s*([^=;][^;]*);\s*$", ln)
            if m and m.group(1) in upd_st:
                st_lines.setdefault(m.group(1), True)
                rest_lines.append((m.group(1), m.group(2)))
            else:
                rest_lines.append((None, ln))
        ptrs = set(pf) | set(upd_st)
        if not ptrs or any(p_ not in own or own[p_]["ctype"] not in QUADV for p_ in ptrs):
            return False
        if "_idx]" in "\n".join(ln for p_, ln in rest_lines if p_ is None).replace("_idx] =", ""):
            return False  # other indexed accesses in the update code
        if bd["threshold"] is not None and re.search(r"_ptr_array_\w+\[", thr_rest):
            return False
        nbytes = sum(QUADV[own[p_]["ctype"]][1] for p_ in pf)  # bytes per neuron prefetched
        pfq_big = max(1, min(8, (2 * PF_WORDS) // max(nbytes, 1)))  # quads in flight per thread
        pfi = {ptr: j for j, ptr in enumerate(sorted(pf))}
        sti = {ptr: j for j, ptr in enumerate(sorted(upd_st))}
        vt = lambda ptr: QUADV[own[ptr]["ctype"]][0]
        w(f"        if ((MAXT * MINB < 1024) && s_quad[{gi}]) {{  // four neurons per thread, 16-byte accesses")
        w("          // (not in the variants capped at 64 registers, where it spills)")
        w(f"          for (int u = s_ut[{gi}][0]; u < s_ut[{gi}][1]; ++u) {{")
        w("            const int start = tst[u], end = tst[u + 1];")
        w("            int cnt = 0;")
        w("            const int q0 = start >> 2, q1 = (end + 3) >> 2;  // quads touching the tile")
        w("            for (int qb = q0; qb < q1; qb += 8 * (int)blockDim.x) {")
        w("              const int qe = (q1 - qb < 8 * (int)blockDim.x) ? q1 : qb + 8 * (int)blockDim.x;")
        w("              const int E = (qe - qb + blockDim.x - 1) / blockDim.x;  // <= 8 slices of quads")
        w(f"              constexpr int PFQ = (MAXT * MINB < 1024) ? {pfq_big} : 1;")
        w("              unsigned flags = 0u;  // 4 bits per slice")
        w("              for (int k0 = 0; k0 < E; k0 += PFQ) {")
        for ptr, j in pfi.items():
            w(f"                {vt(ptr)} _qf{j}[PFQ];")
        w("#pragma unroll")
        w("                for (int kq = 0; kq < PFQ; ++kq) {")
        w("                  const int q = qb + (k0 + kq) * (int)blockDim.x + (int)threadIdx.x;")
        w("                  if (k0 + kq < E && q < qe) {")
        for ptr, j in pfi.items():
            w(f"                    _qf{j}[kq] = *(const {vt(ptr)}*)({ptr} + 4 * (size_t)q);")
        w("                  }")
        w("                }")
        w("#pragma unroll")
        w("                for (int kq = 0; kq < PFQ; ++kq) {")
        w("                  const int k = k0 + kq;")
        w("                  const int q = qb + k * (int)blockDim.x + (int)threadIdx.x;")
        w("                  if (k < E && q < qe) {")
        for ptr, j in sti.items():
            w(f"                    {vt(ptr)} _qs{j};")
        w("#pragma unroll")
        w("                    for (int e = 0; e < 4; ++e) {")
        w("                      const int32_t _idx = 4 * q + e;")
        w("                      if (_idx >= start && _idx < end) {")
        w("                        const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        if bd["update"] is not None:
            w("                        {")
            if not hoist_sc:
                w(_indent(tab.scalar_loads("update", f32), 26))
                w(_indent(_device(tab.time_code("update")), 26))
            for ct, nm, ptr in upd_loads:
                w(f"                          {ct} {nm} = (({ct}*)&_qf{pfi[ptr]}[kq])[e];")
            for p_, ln in rest_lines:
                if p_ is None:
                    w(_indent(ln, 26) if ln.strip() else "")
                else:
                    ct = own[p_]["ctype"]
                    w(f"                          (({ct}*)&_qs{sti[p_]})[e] = {ln};")
            w("                        }")
        if bd["threshold"] is not None:
            w("                        {")
            if not hoist_sc:
                w(_indent(tab.scalar_loads("threshold", f32), 26))
                w(_indent(_device(tab.time_code("threshold")), 26))
            for ct, nm, ptr in thr_loads:
                if ptr in upd_st:
                    w(f"                          {ct} {nm} = (({own[ptr]['ctype']}*)&_qs{sti[ptr]})[e];")
                else:
                    w(f"                          {ct} {nm} = (({own[ptr]['ctype']}*)&_qf{pfi[ptr]}[kq])[e];")
            w(_indent(thr_rest, 26))
            w("                          if (_cond) flags |= 1u << (4 * k + e);")
            if bd["threshold"].get("refractory"):
                nr = next(v["ptr"] for v in g["vars"] if v["name"] == "not_refractory")
                ls = next(v["ptr"] for v in g["vars"] if v["name"] == "lastspike")
                # a variable the update stores is written back from its register
                # copy after this loop: the refractory writes go to that copy
                def ref_store(ptr, val):
                    if ptr in sti:
                        return f"(({own[ptr]['ctype']}*)&_qs{sti[ptr]})[e] = {val};"
                    return f"{ptr}[_idx] = {val};"
                w("                          if (_cond) {")
                w("                            " + ref_store(nr, "false"))
                w("                            " + ref_store(ls, "_b200_t"))
                w("                          }")
            w("                        }")
        w("                      }")
        w("                    }")
        if sti:
            w("                    if (4 * q >= start && 4 * q + 4 <= end) {")
            for ptr, j in sti.items():
                w(f"                      *({vt(ptr)}*)({ptr} + 4 * (size_t)q) = _qs{j};")
            w("                    } else {")
            w("#pragma unroll")
            w("                      for (int e = 0; e < 4; ++e)")
            w("                        if (4 * q + e >= start && 4 * q + e < end) {")
            for ptr, j in sti.items():
                ct = own[ptr]["ctype"]
                w(f"                          {ptr}[4 * q + e] = (({ct}*)&_qs{j})[e];")
            w("                        }")
            w("                    }")
        w("                  }")
        w("                }")
        w("              }")
        w(f"              B200_PHASE({PH_UPD(gi)});  // update + threshold condition")
        w("              // order-preserving compaction: ascending = slice, warp, lane, element")
        w("              for (int k = 0; k < E; ++k) {")
        w("                int c = 0;")
        w("#pragma unroll")
        w("                for (int e = 0; e < 4; ++e) c += __popc(__ballot_sync(0xffffffffu, (flags >> (4 * k + e)) & 1u));")
        w("                if (lane == 0) s_cnt[k * NW + wid] = c;")
        w("              }")
        w("              __syncthreads();")
        w("              int tot;")
        w("              const int x = (int)threadIdx.x < E * NW ? s_cnt[threadIdx.x] : 0;")
        w("              const int ex = b200_block_exscan(x, s_wsum, &tot);")
        w("              if ((int)threadIdx.x < E * NW) s_cnt[threadIdx.x] = ex;")
        w("              __syncthreads();")
        w("              const unsigned lt = b200_lanemask_lt();")
        w("              for (int k = 0; k < E; ++k) {")
        w("                int below = 0;  // set elements of the lower lanes")
        w("#pragma unroll")
        w("                for (int e = 0; e < 4; ++e) below += __popc(__ballot_sync(0xffffffffu, (flags >> (4 * k + e)) & 1u) & lt);")
        w("                const unsigned mine = (flags >> (4 * k)) & 15u;")
        w("                if (mine) {")
        w("                  int p = start + cnt + s_cnt[k * NW + wid] + below;")
        w("                  const int nb = 4 * (qb + k * (int)blockDim.x + (int)threadIdx.x);")
        w("#pragma unroll")
        w("                  for (int e = 0; e < 4; ++e)")
        w("                    if ((mine >> e) & 1u) { scr[p] = nb + e; oscr[p] = nb + e; " + snap_code(gi, "nb + e") + " ++p; }")
        w("                }")
        w("              }")
        w("              cnt += tot;")
        w("              __syncthreads();")
        w(f"              B200_PHASE({PH_THR(gi)});  // spike list (threshold)")
        w("            }")
        w("            if (threadIdx.x == 0) { tcnt[u] = cnt; otc[u] = cnt; }")
        w("          }")
        w("        } else {")
        return True

    def statemon_text(gi, indent, tsexpr, when):
        """State monitors of group gi in slot `when` (start: values at the start
        of step `tsexpr`; end: after its resets), this CTA's recorded neurons
        (templates/statemonitor.cpp).  Ends with a barrier of the CTA: the code
        that follows overwrites what other threads record."""
        g = groups[gi]
        mons = [(mi, m) for mi, m in enumerate(statemons) if m["group"] == gi and m.get("when", "start") == when]
        if not mons:
            return ""
        L = []
        for mi, m in mons:
            every = int(m.get("every", 1))
            L.append("{")
            L.append(f"  const int64_t _b200_sts = {tsexpr};  // the step recorded")
            if every == 1:
                L.append(f"  {{  // state monitor {mi}")
                L.append(f"    const b200_statemon_d& SM = I.stm[{mi}];")
                L.append("    const int64_t rec = _b200_sts - SM.step0;  // row of this step")
            else:  # a slower clock: the steps that are multiples of its dt
                L.append(f"  if (_b200_sts % {every} == 0) {{  // state monitor {mi}: every {every}th step")
                L.append(f"    const b200_statemon_d& SM = I.stm[{mi}];")
                L.append(f"    const int64_t rec = _b200_sts / {every} - (SM.step0 + {every - 1}) / {every};  // row of this step")
            L.append(f"    const int lo = s_tst[{gi} * max_tiles1 + s_ut[{gi}][0]], hi = s_tst[{gi} * max_tiles1 + s_ut[{gi}][1]];")
            L.append("    double* const row = SM.data + (size_t)rec * SM.n_vars * SM.n_rec;")
            L.append("    for (int k = threadIdx.x; k < SM.n_rec * SM.n_vars; k += blockDim.x) {")
            L.append("      const int r = k % SM.n_rec, v = k / SM.n_rec;")
            L.append("      const int idx = SM.idx[r];")
            L.append("      if (idx >= lo && idx < hi) {")
            L.append("        double val = 0.0;")
            L.append("        switch (SM.var_id[v]) {")
            for k, v in enumerate(g["vars"]):
                L.append(f"          case {k}: val = (double)(({v['ctype']}*)s_gv[{gi}][{k}])[idx]; break;")
            L.append("        }")
            L.append("        row[k] = val;")
            L.append("      }")
            L.append("    }")
            L.append(f"    if (threadIdx.x == 0) s_stm_n[{mi}] = rec + 1;")
            L.append("  }")
            L.append("}")
        L.append("__syncthreads();")
        return _indent("\n".join(L), indent)

    def emit_statemons(gi):
        """The start-slot state monitors of group gi at step ts."""
        txt = statemon_text(gi, 8, "ts", "start")
        if txt:
            w(txt)

    def emit_summed(si):
        """Summed variable si (templates/summed_variable.cpp:11-25): each of
        this CTA's target neurons sums the expression over its synapses in
        creation order, from zero."""
        sm = SUMMED[si]
        pi, gi = sm["pathway"], sm["tgt_group"]
        p = paths[pi]
        tab, blocks = ptables[pi]
        bname = f"summed{si}"
        tv = groups[gi]["vars"][sm["tgt_var"]]
        blk = dict(blocks)[bname]
        w(f"      {{  // summed variable {sm['name']}")
        w(f"        const b200_pathway_d& PQ = I.p[{pi}]; (void)PQ;")
        w(f"        const double* const _b200_S = s_Sp{pi}; const float* const _b200_Sf = s_Sp{pi}f; const long long* const _b200_Si = s_Sp{pi}i;")
        w("        (void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
        for k, v in enumerate(p.get("vars", [])):
            w(f"        {v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)PQ.var[{k}]; (void){v['ptr']};")
        w(f"        const int32_t* __restrict__ const {p['post_ptr']} = PQ.{syn_arr(pi, 'post')}; (void){p['post_ptr']};")
        w(f"        const int32_t* __restrict__ const {p['pre_ptr']} = PQ.{syn_arr(pi, 'pre')}; (void){p['pre_ptr']};")
        for ptr, (gidx, vidx) in sorted(sm.get("group_ptrs", {}).items()):
            v = groups[gidx]["vars"][vidx]
            w(f"        {v['ctype']}* __restrict__ const {ptr} = ({v['ctype']}*)s_gv[{gidx}][{vidx}]; (void){ptr};")
        w(_indent(tab.const_loads(f32), 8))
        w(_indent(tab.scalar_loads(bname, f32), 8))
        w(_indent(_device(tab.time_code(bname)), 8))
        w(f"        {tv['ctype']}* const _b200_tgt = ({tv['ctype']}*)s_gv[{gi}][{sm['tgt_var']}];")
        w(f"        const b200_summed_d& SD = I.sum[{si}];")
        w(f"        const int o0 = s_tst[{gi} * max_tiles1 + s_ut[{gi}][0]], o1 = s_tst[{gi} * max_tiles1 + s_ut[{gi}][1]];")
        w("        for (int j = o0 + (int)threadIdx.x; j < o1; j += blockDim.x) {")
        w("          if (j < SD.lo || j >= SD.hi) continue;")
        w(f"          {tv['ctype']} _b200_acc = 0;")
        w("          for (int64_t k = SD.seg[j - SD.lo]; k < SD.seg[j - SD.lo + 1]; ++k) {")
        w("            const int64_t _idx = SD.syn[k];")
        w("            const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        w("            {")
        w(_indent(blk["vector"], 14))
        w("              _b200_acc += _synaptic_var;")
        w("            }")
        w("          }")
        w("          _b200_tgt[j] = _b200_acc;")
        w("        }")
        w("      }")

    def emit_phase_a(owner):
        """Reset of the previous step, state monitors, update + threshold with
        ordered compaction of this CTA's tiles."""
        # ---- Phase A
        if not owner and (SYNOPS or SYNMONS):
            # per-synapse code and synaptic monitors: after the previous step's
            # deliveries (its end slot), then this step's start and groups slots;
            # the step's deliveries follow the barrier
            end = syn_text(8, "ts - 1", "end")
            if end:
                w("      if (ts > ts0) {")
                w(end)
                w("      }")
            for when in ("start", "groups"):
                txt = syn_text(6, "ts", when)
                if txt:
                    w(txt)
        for gi, g in enumerate(groups):
            tab, blocks = gtables[gi]
            bd = dict(blocks)
            if g.get("generator"):
                emit_generator(gi, owner)
                continue
            w(f"      // ---- group {gi} '{g['name']}': phase A (reset of step ts-1, monitors, update + threshold)")
            dfr = deferred_block(gi, 8, "ts - 1", owner)
            if not owner:
                w("      B200_PHASE(0);")
            if dfr and not SUMMED:  # (with summed variables: before the sums)
                w("      if (ts > ts0) {")
                w(dfr)
                w("        __syncthreads();")
                w("      }")
                if not owner:
                    w(f"      B200_PHASE({PH_RST(gi)});  // reset of the previous step")
            sop = op_block(gi, 6, "ts", "start")
            if sop and not SUMMED:  # the start-slot operations of this step
                w(sop)
                w("      __syncthreads();")
            w("      {")
            w(f"        const int32_t N = I.g[{gi}].N; (void)N;")
            w(f"        const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;")
            w(gptr_decls(gi, 8, True))
            if owner:
                scr_e, tc_e = owner_list(gi, "ts")
                w(f"        int32_t* const scr = {scr_e}; int32_t* const tcnt = {tc_e};")
            else:
                w(f"        int32_t* const scr = s_scr[{gi}]; int32_t* const tcnt = s_tc[{gi}];")
                w(f"        int32_t* const oscr = s_oscr[{gi}]; int32_t* const otc = s_otc[{gi}];")
            w(f"        const int* const tst = s_tst + {gi} * max_tiles1;")
            # rand() / randn() in the update or threshold: the step's draws of the
            # site, `calls` per neuron in index order (the reference's order)
            rng_undef = []
            for blk_name in ("update", "threshold"):
                if g.get(blk_name) and g[blk_name].get("draw") is not None:
                    dl, du = draw_macros(g[blk_name]["draw"], "ts")
                    w(_indent("\n".join(dl), 8))
                    rng_undef += du
            rng = bool(rng_undef)
            if not SUMMED:  # (with summed variables the monitors record before those are summed)
                emit_statemons(gi)
            # constants and block scalars are loaded once per step, not per neuron
            upd_sc = {nm for _, nm in scalar_outputs(bd["update"]["scalar"])} if bd["update"] is not None else set()
            thr_sc = {nm for _, nm in scalar_outputs(bd["threshold"]["scalar"])} if bd["threshold"] is not None else set()
            hoist_sc = not (upd_sc & thr_sc)
            w(_indent(tab.const_loads(f32), 8))
            if hoist_sc:
                for blk_name in ("update", "threshold"):
                    if bd[blk_name] is not None:
                        w(_indent(tab.scalar_loads(blk_name, f32), 8))
                        w(_indent(_device(tab.time_code(blk_name)), 8))
            quad = (not owner) and not rng and emit_quad(gi, g, bd, tab, hoist_sc)
            w(f"        for (int u = s_ut[{gi}][0]; u < s_ut[{gi}][1]; ++u) {{")
            w("          const int start = tst[u], end = tst[u + 1];")
            w("          int cnt = 0;")
            w("          for (int pb = start; pb < end; pb += 32 * (int)blockDim.x) {")
            w("            const int pe = (end - pb < 32 * (int)blockDim.x) ? end : pb + 32 * (int)blockDim.x;")
            w("            const int E = (pe - pb + blockDim.x - 1) / blockDim.x;")
            # the state loads of up to PF slices are issued before any of them is
            # computed (each slice is one L2 round trip otherwise)
            upd_v = bd["update"]["vector"] if bd["update"] is not None else ""
            thr_v = bd["threshold"]["vector"] if bd["threshold"] is not None else ""
            upd_loads, upd_rest = split_loads(upd_v)
            thr_loads, thr_rest = split_loads(thr_v)
            upd_st = stored_ptrs(upd_v)
            pf = {}
            for ct, nm, ptr in upd_loads + [x for x in thr_loads if x[2] not in upd_st]:
                pf.setdefault(ptr, ct)
            pfi = {ptr: j for j, ptr in enumerate(pf)}
            words = sum(max(1, SIZE.get(ct, 8) // 4) for ct in pf.values())
            # 16 words of loads in flight per thread in the variants capped at 64
            # registers, PF_WORDS in the others
            pf_small = max(1, min(4, 16 // max(words, 1)))
            pf_big = max(1, min(32, PF_WORDS // max(words, 1)))
            w(f"            constexpr int PF = (MAXT * MINB < 1024) ? {pf_big} : {pf_small};")
            w("            unsigned flags = 0u;")
            w("            for (int k0 = 0; k0 < E; k0 += PF) {")
            for ptr, j in pfi.items():
                w(f"              {pf[ptr]} _pf{j}[PF];")
            w("#pragma unroll")
            w("              for (int kq = 0; kq < PF; ++kq) {")
            w("                const int32_t _idx = pb + (k0 + kq) * (int)blockDim.x + threadIdx.x;")
            w("                if (k0 + kq < E && _idx < pe) {")
            for ptr, j in pfi.items():
                w(f"                  _pf{j}[kq] = {ptr}[_idx];")
            w("                }")
            w("              }")
            w("#pragma unroll")
            w("              for (int kq = 0; kq < PF; ++kq) {")
            w("              const int k = k0 + kq;")
            w("              const int32_t _idx = pb + k * (int)blockDim.x + threadIdx.x;")
            w("              if (k < E && _idx < pe) {")
            w("                const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            if bd["update"] is not None:
                w("                {")
                if not hoist_sc:
                    w(_indent(tab.scalar_loads("update", f32), 18))
                    w(_indent(_device(tab.time_code("update")), 18))
                w(extra_ptrs(g.get("update"), 18))
                for ct, nm, ptr in upd_loads:
                    w(f"                  {ct} {nm} = _pf{pfi[ptr]}[kq];")
                w(_indent(upd_rest, 18))
                w("                }")
            if bd["threshold"] is not None:
                w("                {")
                if not hoist_sc:
                    w(_indent(tab.scalar_loads("threshold", f32), 18))
                    w(_indent(_device(tab.time_code("threshold")), 18))
                w(extra_ptrs(g.get("threshold"), 18))
                for ct, nm, ptr in thr_loads:
                    w(f"                  {ct} {nm} = " + (f"_pf{pfi[ptr]}[kq];" if ptr not in upd_st else f"{ptr}[_idx];"))
                w(_indent(thr_rest, 18))
                w("                  if (_cond) flags |= 1u << k;")
                if bd["threshold"].get("refractory"):
                    nr = next(v["ptr"] for v in g["vars"] if v["name"] == "not_refractory")
                    ls = next(v["ptr"] for v in g["vars"] if v["name"] == "lastspike")
                    w("                  if (_cond) {")
                    w(f"                    {nr}[_idx] = false;")
                    w(f"                    {ls}[_idx] = _b200_t;")
                    w("                  }")
                w("                }")
            w("              }")
            w("              }")
            w("            }")
            if not owner:
                w(f"            B200_PHASE({PH_UPD(gi)});  // update + threshold condition")
            w("            // order-preserving compaction: counts per (slice k, warp), one block scan")
            w("            for (int k = 0; k < E; ++k) {")
            w("              const unsigned m = __ballot_sync(0xffffffffu, (flags >> k) & 1u);")
            w("              if (lane == 0) s_cnt[k * NW + wid] = __popc(m);")
            w("            }")
            w("            __syncthreads();")
            w("            int tot;")
            w("            const int x = (int)threadIdx.x < E * NW ? s_cnt[threadIdx.x] : 0;")
            w("            const int ex = b200_block_exscan(x, s_wsum, &tot);")
            w("            if ((int)threadIdx.x < E * NW) s_cnt[threadIdx.x] = ex;")
            w("            __syncthreads();")
            w("            for (int k = 0; k < E; ++k) {")
            w("              const unsigned m = __ballot_sync(0xffffffffu, (flags >> k) & 1u);")
            w("              if ((flags >> k) & 1u)")
            w("                {")
            w("                  const int _p = start + cnt + s_cnt[k * NW + wid] + __popc(m & b200_lanemask_lt());")
            w("                  const int _sn = pb + k * (int)blockDim.x + threadIdx.x;  // the spiking neuron")
            w("                  scr[_p] = _sn;")
            if not owner:
                w("                  oscr[_p] = _sn;  // this CTA's copy")
            sc = snap_code(gi, "_sn")
            if sc:
                w("                  " + sc)
            w("                }")
            w("            }")
            w("            cnt += tot;")
            w("            __syncthreads();")
            if not owner:
                w(f"            B200_PHASE({PH_THR(gi)});  // spike list (threshold)")
            w("          }")
            w("          if (threadIdx.x == 0) tcnt[u] = cnt;" if owner else "          if (threadIdx.x == 0) { tcnt[u] = cnt; otc[u] = cnt; }")
            w("        }")
            if quad:
                w("        }  // scalar path")
            if rng:
                w("\n".join(rng_undef))
            w("      }")

    w("__device__ __forceinline__ int b200_upper_bound(const int* a, int n, int x) {")
    w("  int lo = 0, hi = n;")
    w("  while (lo < hi) { const int m = (lo + hi) >> 1; if (a[m] <= x) lo = m + 1; else hi = m; }")
    w("  return lo;")
    w("}")
    w("")
    w(f"#define B200_NG {NG}")
    w("#define B200_LIST_RUN 4  // tile counts a thread loads at once in the spike-list prefix")
    w(f"#define B200_EVENT_BATCH {EVENT_BATCH}  // events whose loads a thread issues before applying them")
    w(f"#define B200_WR_SLOTS {max(16, min(128, 1024 // max(NP, 1)))}  // ring slots whose spike bounds a CTA keeps in shared memory")
    w(f"#define B200_MAXV {MAXV}")
    w("// dynamic shared memory: [state cache | item seg | item off | item src | item pathway | prefix |")
    w("//                         tile starts | delays]")
    w("static size_t b200_dyn_smem(int threads, int max_tiles1, int max_w, int state_bytes) {")
    w("  return (size_t)state_bytes + (size_t)threads * 8 + (size_t)(threads + 1) * 4 + (size_t)threads * 8 +")
    w("         (size_t)2 * B200_NG * max_tiles1 * 4 + (size_t)(3 * max_w + 1) * 4 + 16;")
    w("}")
    w("")
    w("template <int MAXT, int MINB>")
    w("__global__ void __launch_bounds__(MAXT, MINB) b200_step_kernel(")
    w("    const b200_inst_d* __restrict__ insts, const int2* __restrict__ cta_map, int n_inst,")
    w("    int queue_mode, int* work, int64_t max_steps, uint64_t limit_ns, int max_tiles1, int max_w,")
    w("    int fault_rank, int state_bytes, unsigned long long* __restrict__ prof, int cluster) {")
    w("  extern __shared__ __align__(16) unsigned char b200_dyn[];")
    w("  unsigned char* const s_state = b200_dyn;")
    w("  int64_t* const s_item_seg = (int64_t*)(b200_dyn + state_bytes);")
    w("  int* const s_item_off = (int*)(s_item_seg + blockDim.x);")
    w("  int* const s_item_src = s_item_off + blockDim.x + 1;")
    w("  int* const s_item_q = s_item_src + blockDim.x;")
    w("  int* const s_pref_all = s_item_q + blockDim.x;")
    w("  int* const s_tst = s_pref_all + B200_NG * max_tiles1;")
    w("  int* const s_nd = s_tst + B200_NG * max_tiles1;")
    w("  int* const s_base = s_nd + max_w;")
    w("  int* const s_ndoff = s_base + max_w;")
    w("  __shared__ __align__(16) b200_inst_d I;")
    w("  __shared__ int s_wsum[B200_MAX_WARPS + 1];")
    w("  __shared__ int s_cnt[B200_MAX_THREADS];")
    w("  __shared__ int s_unit, s_rank, s_flag, s_cache;")
    w("  __shared__ long long s_mon_n[B200_MAX_SPKMON];")
    w("  __shared__ long long s_stm_n[B200_MAX_STATEMON];")
    w("  __shared__ void* s_gv[B200_NG][B200_MAXV];")
    w("  __shared__ int32_t* s_scr[B200_NG];")
    w("  __shared__ int32_t* s_tc[B200_NG];")
    w("  __shared__ int32_t* s_oscr[B200_NG];  // this CTA's own spike lists / tile counts (shared copy")
    w("  __shared__ int32_t* s_otc[B200_NG];   //  when there is room, else the global lists)")
    w("  __shared__ int s_ut[B200_NG][2];")
    w("  __shared__ int s_glast[B200_NG], s_gen_lo, s_gen_hi;  // spike generator cursors")
    w("  (void)s_glast; (void)s_gen_lo; (void)s_gen_hi;")
    w("  __shared__ int s_pcache, s_pown[B200_NG][2];  // private-variable cache: on, own neuron range")
    w("  __shared__ int s_quad[B200_NG];  // 1: the group's state pointers allow 4-neuron accesses")
    w(f"  __shared__ int s_wr[{max(NP, 1)} * B200_WR_SLOTS * 2];  // per pathway and ring slot: bounds of the slot's spikes")
    w(f"  __shared__ int s_wr_ok[{max(NP, 1)}];                   // 1: the ring fits B200_WR_SLOTS")
    w("  (void)s_pown;")
    for gi in range(NG):
        n_ = max(gtables[gi][0].size, 1)
        w(f"  __shared__ double s_Sg{gi}[{n_}]; __shared__ float s_Sg{gi}f[{n_}]; __shared__ long long s_Sg{gi}i[{n_}];")
    for pi in range(NP):
        n_ = max(ptables[pi][0].size, 1)
        w(f"  __shared__ double s_Sp{pi}[{n_}]; __shared__ float s_Sp{pi}f[{n_}]; __shared__ long long s_Sp{pi}i[{n_}];")
    w("  unsigned gen = 0;")
    w("  (void)s_nd; (void)s_base; (void)s_ndoff; (void)s_item_seg; (void)s_item_off; (void)s_item_src; (void)s_item_q;")
    w("  (void)s_state;")
    w("  for (int pass = 0;; ++pass) {")
    w("    if (threadIdx.x == 0) {")
    w("      if (queue_mode) { s_unit = atomicAdd(work, 1); s_rank = 0; }")
    w("      else if (pass == 0) { const int2 m = cta_map[blockIdx.x]; s_unit = m.x; s_rank = m.y; }")
    w("      else s_unit = n_inst;")
    w("    }")
    w("    __syncthreads();")
    w("    const int unit = s_unit, rank = s_rank;")
    w("    if (unit >= n_inst) break;")
    w("    {")
    w("      const long long* src = (const long long*)&insts[unit];")
    w("      long long* dst = (long long*)&I;")
    w("      for (int k = threadIdx.x; k < (int)(sizeof(b200_inst_d) / 8); k += blockDim.x) dst[k] = src[k];")
    w("    }")
    w("    __syncthreads();")
    # pointer table and smem cache
    w("    if (threadIdx.x == 0) {")
    w("      gen = b200_ld_acquire(&I.bar[1]);")
    for m in range(len(spkmons)):
        w(f"      s_mon_n[{m}] = *((volatile long long*)I.sm[{m}].n);")
    for m in range(len(statemons)):
        w(f"      s_stm_n[{m}] = *((volatile long long*)I.stm[{m}].n);")
    w("      const int cache = (I.n_cta == 1 && I.cache_bytes > 0 && I.cache_bytes <= state_bytes) ? 1 : 0;")
    w("      s_cache = cache;")
    w("      size_t off = 0;")
    for gi, g in enumerate(groups):
        for k in range(len(g["vars"])):
            w(f"      s_gv[{gi}][{k}] = I.g[{gi}].var[{k}];")
        w(f"      s_scr[{gi}] = I.g[{gi}].scratch; s_tc[{gi}] = I.g[{gi}].tile_cnt;")
        w("      if (cache) {")
        for k in USED[gi]:
            sz = SIZE[g["vars"][k]["ctype"]]
            w(f"        s_gv[{gi}][{k}] = s_state + off; off += ((size_t)I.g[{gi}].N * {sz} + 15) & ~(size_t)15;")
        w("        if (I.cache_lists) {")
        w(f"          s_scr[{gi}] = (int32_t*)(s_state + off); off += ((size_t)I.g[{gi}].N * 4 + 15) & ~(size_t)15;")
        w(f"          s_tc[{gi}] = (int32_t*)(s_state + off); off += ((size_t)I.g[{gi}].n_tiles * 4 + 15) & ~(size_t)15;")
        w("        }")
        w("      }")
        w(f"      s_ut[{gi}][0] = I.g[{gi}].cta_tile[rank]; s_ut[{gi}][1] = I.g[{gi}].cta_tile[rank + 1];")
        w(f"      s_oscr[{gi}] = s_scr[{gi}]; s_otc[{gi}] = s_tc[{gi}];")
        if g.get("generator"):
            w(f"      s_glast[{gi}] = *((volatile int32_t*)I.g[{gi}].gen_last);")
        w(f"      if (!cache && I.g[{gi}].own_off >= 0) {{  // offset so that global positions address them")
        w(f"        s_oscr[{gi}] = (int32_t*)(s_state + I.g[{gi}].own_off) - I.g[{gi}].tile_start[s_ut[{gi}][0]];")
        w(f"        s_otc[{gi}] = (int32_t*)(s_state + I.g[{gi}].own_off + (((size_t)I.g[{gi}].own_cap * 4 + 15) & ~(size_t)15)) - s_ut[{gi}][0];")
        w("      }")
    # private variables of a multi-CTA instance: this CTA's neurons in shared
    # memory for the launch, addressed by global index
    w("      const int pcache = (!cache && I.priv_bytes > 0 && I.priv_bytes <= state_bytes) ? 1 : 0;")
    w("      s_pcache = pcache;")
    if any(PRIV):
        w("      if (pcache) {")
        w("        size_t poff = 0;")
        for gi, g in enumerate(groups):
            if not PRIV[gi]:
                continue
            w(f"        s_pown[{gi}][0] = I.g[{gi}].tile_start[s_ut[{gi}][0]]; s_pown[{gi}][1] = I.g[{gi}].tile_start[s_ut[{gi}][1]];")
            for k in PRIV[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"        s_gv[{gi}][{k}] = s_state + poff - (size_t)s_pown[{gi}][0] * {sz}; "
                  f"poff += ((size_t)(s_pown[{gi}][1] - s_pown[{gi}][0]) * {sz} + 15) & ~(size_t)15;")
        w("      }")
    w("    }")
    # quad accesses need every state pointer aligned to 4 elements (shared
    # memory copies are offset by the CTA's first neuron)
    w("    if (threadIdx.x == 0) {")
    for gi, g in enumerate(groups):
        if ALIAS[gi] is not None:
            for k in range(len(g["vars"])):
                w(f"      s_gv[{gi}][{k}] = s_gv[{ALIAS[gi]}][{k}];  // a custom event of group {ALIAS[gi]}")
    for gi, g in enumerate(groups):
        conds = []
        for k, v in enumerate(g["vars"]):
            if v["ctype"] in QUADV:
                conds.append(f"(((uintptr_t)s_gv[{gi}][{k}]) % {4 * SIZE[v['ctype']]} == 0)")
        w(f"      s_quad[{gi}] = {' && '.join(conds) if conds else '0'};")
    w("    }")
    w("    __syncthreads();")
    if any(PRIV):
        w("    if (s_pcache) {")
        for gi, g in enumerate(groups):
            for k in PRIV[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"      b200_copy_bytes((char*)s_gv[{gi}][{k}] + (size_t)s_pown[{gi}][0] * {sz}, "
                  f"(const char*)I.g[{gi}].var[{k}] + (size_t)s_pown[{gi}][0] * {sz}, "
                  f"(size_t)(s_pown[{gi}][1] - s_pown[{gi}][0]) * {sz});")
        w("    }")
    for gi, g in enumerate(groups):
        w(f"    for (int u = threadIdx.x; u <= I.g[{gi}].n_tiles; u += blockDim.x) s_tst[{gi} * max_tiles1 + u] = I.g[{gi}].tile_start[u];")
    # loop-invariant scalars: one shared copy per CTA (all threads read the same words)
    for gi in range(NG):
        w(f"    for (int k = threadIdx.x; k < {gtables[gi][0].size}; k += blockDim.x) {{")
        w(f"      const double x = I.g[{gi}].S[k]; s_Sg{gi}[k] = x; s_Sg{gi}f[k] = (float)x; s_Sg{gi}i[k] = (long long)x;")
        w("    }")
    for pi in range(NP):
        w(f"    for (int k = threadIdx.x; k < {ptables[pi][0].size}; k += blockDim.x) {{")
        w(f"      const double x = I.p[{pi}].S[k]; s_Sp{pi}[k] = x; s_Sp{pi}f[k] = (float)x; s_Sp{pi}i[k] = (long long)x;")
        w("    }")
    # the spike bounds of the ring slots written by earlier launches
    for pi, p in enumerate(paths):
        sg = p["src"]
        w("    {")
        w(f"      const b200_group_d& G = I.g[{sg}];")
        w(f"      const int okw = G.R > 1 && G.R <= B200_WR_SLOTS;")
        w(f"      if (threadIdx.x == 0) s_wr_ok[{pi}] = okw;")
        w("      if (okw)")
        w("        for (int sl = threadIdx.x; sl < G.R; sl += blockDim.x) {")
        w("          const int32_t* rp = G.ring_prefix + (int64_t)sl * (G.n_tiles + 1);")
        w(f"          s_wr[({pi} * B200_WR_SLOTS + sl) * 2] = rp[I.p[{pi}].tile_lo];")
        w(f"          s_wr[({pi} * B200_WR_SLOTS + sl) * 2 + 1] = rp[I.p[{pi}].tile_hi];")
        w("        }")
        w("    }")
    w("    if (s_cache) {  // state of a single-CTA instance lives in shared memory for the launch")
    for gi, g in enumerate(groups):
        for k in USED[gi]:
            sz = SIZE[g["vars"][k]["ctype"]]
            w(f"      b200_copy_bytes(s_gv[{gi}][{k}], I.g[{gi}].var[{k}], (size_t)I.g[{gi}].N * {sz});")
    w("    }")
    w("    __syncthreads();")
    w("    const int64_t ts0 = I.ts;")
    w("    const int64_t ts_stop = (I.ts_end < ts0 + max_steps) ? I.ts_end : ts0 + max_steps;")
    w("    const double _b200_dt = I.dt;")
    w("    int64_t ts = ts0;")
    w("    bool ok = true;")
    # deliveries read no spikes of their own step; not in the variants capped at
    # 64 registers (their code would spill; they serve single-CTA instances)
    w(f"    const bool lagm = (MAXT * MINB < 1024) && I.lag && I.n_cta > 1{' && false' if SYNOPS else ''};")
    w("    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, NW = blockDim.x >> 5;")
    w(f"    // per-phase device profile (thread 0 of each CTA; phases: A, barrier A, spike lists,")
    w(f"    // {NP} pathway(s), barrier B)")
    # (in shared memory, written by thread 0 only: no registers held across the steps)
    w(f"    __shared__ unsigned long long _pt, _pacc[{NPH}];")
    w(f"    if (threadIdx.x == 0) {{ _pt = 0; for (int q = 0; q < {NPH}; ++q) _pacc[q] = 0; }}")
    w("#define B200_PHASE(q) do { if (prof && threadIdx.x == 0) { const unsigned long long _c = clock64(); _pacc[q] += _c - _pt; _pt = _c; } } while (0)")
    w("    for (; ts < ts_stop; ++ts) {")
    w("      if (threadIdx.x == 0) {")
    w("        int st = 0;")
    for m in range(len(spkmons)):
        w(f"        if (s_mon_n[{m}] + (I.sm[{m}].hi - I.sm[{m}].lo) > I.sm[{m}].cap) st = 1;")
    w("        s_flag = st;")
    w("      }")
    w("      __syncthreads();")
    w("      if (s_flag) break;")
    w("      const double _b200_t = (double)ts * _b200_dt;")
    w("      const int64_t _b200_ts = ts;")
    w("      if (prof && threadIdx.x == 0) _pt = clock64();")
    if SUMMED:
        # the reference's schedule: resets of the previous step (after its
        # deliveries), state monitors (start), then the summed variables (groups
        # slot, before the groups' updates).  The sums read other CTAs' neurons:
        # every CTA has applied its resets before any sums, and finishes its sums
        # before any update
        for gi in range(NG):
            dfr = deferred_block(gi, 8, "ts - 1")
            if dfr:
                w("      if (ts > ts0) {")
                w(dfr)
                w("      }")
            sop = op_block(gi, 6, "ts", "start")
            if sop:
                w("      __syncthreads();")
                w(sop)
        w("      if (!b200_inst_barrier(I, gen, limit_ns, cluster, rank)) { ok = false; break; }")
        for gi in range(NG):
            emit_statemons(gi)
        for si in range(len(SUMMED)):
            emit_summed(si)
        w("      if (!b200_inst_barrier(I, gen, limit_ns, cluster, rank)) { ok = false; break; }")

    emit_phase_a(False)
    w("      B200_PHASE(0);")
    w("      // test hook: CTA `fault_rank` leaves without arriving, the others must time out")
    w("      if (rank == fault_rank && ts == ts0) { ok = false; break; }")
    def emit_preload(ind):
        """Lag mode, right after barrier A: the step's tile counts, loaded now
        so that their round trip overlaps the deliveries."""
        sp = " " * ind
        w(sp + "lc_ok = true;")
        for gi in range(NG):
            w(sp + "{")
            w(sp + f"  const int nt = I.g[{gi}].n_tiles;")
            w(sp + "  const int per = (nt + (int)blockDim.x - 1) / (int)blockDim.x;")
            w(sp + "  const int u0r = threadIdx.x * per;")
            w(sp + f"  const int32_t* const tcnt = s_tc[{gi}];")
            w(sp + "  if (per > B200_LIST_RUN) lc_ok = false;")
            w("#pragma unroll")
            w(sp + f"  for (int r = 0; r < B200_LIST_RUN; ++r) _lc{gi}[r] = (r < per && u0r + r < nt) ? tcnt[u0r + r] : 0;")
            w(sp + "}")

    # ---- Phase B: prefix of tile counts, ring, monitors
    def emit_lists():
        for gi, g in enumerate(groups):
            w(f"      // ---- group {gi}: phase B (spike lists)")
            w("      {")
            w(f"        b200_group_d& GD = I.g[{gi}];")
            w(f"        int* const pref = s_pref_all + {gi} * max_tiles1;")
            w(f"        const int* const tst = s_tst + {gi} * max_tiles1;")
            w(f"        const int32_t* const tcnt = s_tc[{gi}];")
            w(f"        const int32_t* const oscr = s_oscr[{gi}];  // this CTA's own lists")
            w("        const int nt = GD.n_tiles;")
            # every thread loads its run of consecutive tile counts at once (one
            # round trip), then one block scan of the run totals
            w("        {")
            w("          const int per = (nt + (int)blockDim.x - 1) / (int)blockDim.x;")
            w("          const int u0r = threadIdx.x * per;")
            w("          int c[B200_LIST_RUN];")
            w("          int sum = 0;")
            w("          if (per <= B200_LIST_RUN) {")
            w("#pragma unroll")
            w(f"            for (int r = 0; r < B200_LIST_RUN; ++r) c[r] = lc_ok ? _lc{gi}[r] : "
              "((r < per && u0r + r < nt) ? tcnt[u0r + r] : 0);")
            w("#pragma unroll")
            w("            for (int r = 0; r < B200_LIST_RUN; ++r) sum += c[r];")
            w("          } else {")
            w("            for (int r = 0; r < per; ++r) sum += (u0r + r < nt) ? tcnt[u0r + r] : 0;")
            w("          }")
            w("          int tot;")
            w("          int ex = b200_block_exscan(sum, s_wsum, &tot);")
            w("          if (per <= B200_LIST_RUN) {")
            w("#pragma unroll")
            w("            for (int r = 0; r < B200_LIST_RUN; ++r) if (r < per && u0r + r < nt) { pref[u0r + r] = ex; ex += c[r]; }")
            w("          } else {")
            w("            for (int r = 0; r < per; ++r) if (u0r + r < nt) { pref[u0r + r] = ex; ex += tcnt[u0r + r]; }")
            w("          }")
            w("          if (threadIdx.x == 0) pref[nt] = tot;")
            w("        }")
            w("        __syncthreads();")
            w(f"        B200_PHASE({PH_THR(gi)});  // the step's spike list (threshold)")
            w(f"        const int u0 = s_ut[{gi}][0], u1 = s_ut[{gi}][1];")
            src_of = [pi for pi, p in enumerate(paths) if p["src"] == gi]
            if src_of:
                w("        if (GD.R > 1 && threadIdx.x == 0) {  // the slot's spike bounds per pathway, for later steps")
                w("          const int slot = (int)(ts % GD.R);")
                for pi in src_of:
                    w(f"          if (s_wr_ok[{pi}]) {{ s_wr[({pi} * B200_WR_SLOTS + slot) * 2] = pref[I.p[{pi}].tile_lo]; "
                      f"s_wr[({pi} * B200_WR_SLOTS + slot) * 2 + 1] = pref[I.p[{pi}].tile_hi]; }}")
                w("        }")
            w("        if (GD.R > 1) {")
            w("          const int slot = (int)(ts % GD.R);")
            w("          int32_t* const ring = GD.ring + (int64_t)slot * GD.N;")
            w("          for (int u = u0; u < u1; ++u) {")
            w("            const int cnt = pref[u + 1] - pref[u], base = tst[u];")
            w("            for (int j = threadIdx.x; j < cnt; j += blockDim.x) ring[pref[u] + j] = oscr[base + j];")
            w("          }")
            w("          if (rank == 0) {")
            w("            for (int u = threadIdx.x; u <= nt; u += blockDim.x) GD.ring_prefix[(int64_t)slot * (nt + 1) + u] = pref[u];")
            w("            if (threadIdx.x == 0) GD.ring_total[slot] = pref[nt];")
            w("          }")
            w("        }")
            w(f"        B200_PHASE({PH_RING(gi)});  // spikes into the delay ring (push)")
            for mi, m in enumerate(spkmons):
                if m["group"] != gi:
                    continue
                w(f"        {{  // spike monitor {mi}")
                w(f"          const b200_spkmon_d& SM = I.sm[{mi}];")
                w(f"          const long long mbase = s_mon_n[{mi}] - pref[SM.tile_lo];")
                w("          const int a = u0 > SM.tile_lo ? u0 : SM.tile_lo, b = u1 < SM.tile_hi ? u1 : SM.tile_hi;")
                w("          for (int u = a; u < b; ++u) {")
                w("            const int cnt = pref[u + 1] - pref[u], base = tst[u];")
                w("            for (int j = threadIdx.x; j < cnt; j += blockDim.x) {")
                w("              const int idx = oscr[base + j];")
                w("              const long long pos = mbase + pref[u] + j;")
                w("              SM.i[pos] = idx - SM.lo;")
                w("              SM.ts[pos] = (int32_t)ts;")
                if m.get("vars"):
                    w("              " + value_rows(mi, gi, "pos", "idx"))
                w("              atomicAdd(&SM.count[idx - SM.lo], 1);  // no read round trip (own neurons: uncontended)")
                w("            }")
                w("          }")
                w("          __syncthreads();")
                w(f"          if (threadIdx.x == 0) s_mon_n[{mi}] += pref[SM.tile_hi] - pref[SM.tile_lo];")
                w("        }")
                w(f"        B200_PHASE({PH_SPKMON(mi)});  // spike monitor")
            for mi, m in enumerate(ratemons):
                if m["group"] != gi:
                    continue
                w(f"        if (rank == 0 && threadIdx.x == 0) {{  // rate monitor {mi}")
                w(f"          const b200_ratemon_d& RM = I.rm[{mi}];")
                w("          RM.cnt[ts - RM.step0] = pref[RM.tile_hi] - pref[RM.tile_lo];")
                w("        }")
                w(f"        B200_PHASE({PH_RATEMON(mi)});  // rate monitor")
            w("      }")

        if NP:
            w("      __syncthreads();  // the slot bounds recorded above")
        w("      B200_PHASE(2);")
    w("      unsigned bar_old = 0u;")
    w("      bool pend = false;  // lag mode: barrier A arrived, not yet waited for")
    w("      bool lc_ok = false;  // lag mode: the tile counts were loaded right after the wait")
    w("      bool lists_due = lagm;  // lag mode: the step's spike lists are still to do")
    for gi in range(NG):
        w(f"      int _lc{gi}[B200_LIST_RUN]; (void)_lc{gi};")
    w("      bool arrive_due = false;")
    w("      if (lagm) {")
    w("        arrive_due = true;  // arrive after the delivery windows (the arrival's fence overlaps the item loads)")
    w("      } else {")
    w("        if (!b200_inst_barrier(I, gen, limit_ns, cluster, rank)) { ok = false; break; }")
    w("        B200_PHASE(1);")
    emit_lists()
    w("      }")
    # ---- Phase B: synaptic propagation, one pass per source group: the items
    # (delay slot, spike) of all its pathways form one list, so the dependent
    # loads (ring -> segment bounds -> synapses) of the pathways overlap
    # consecutive pathways from the same source whose on_pre code touches
    # disjoint neuron variables: running them interleaved cannot change what
    # any of them reads, so the reference's pathway-by-pathway order is kept
    merged = delivery_passes(paths)
    seen_svars = set()
    for sg, pis, _ in merged:
        L = len(pis)
        svars = {v["ptr"] for q in pis for v in paths[q].get("vars", [])}
        if svars & seen_svars:
            # synaptic variables shared with an earlier pathway of this step (the
            # on_pre and on_post pathways of one Synapses object): all of the
            # earlier pathway's events come first, as in the reference's schedule
            w("      if (arrive_due) { b200_inst_arrive(I, cluster, rank, bar_old); arrive_due = false; pend = true; }")
            w("      if (pend) {")
            w("        if (!b200_inst_wait(I, gen, limit_ns, cluster, rank, bar_old)) ok = false;")
            w("        pend = false;")
            emit_preload(8)
            w("      }")
            w("      if (!ok) break;")
            w("      if (!b200_inst_barrier(I, gen, limit_ns, cluster, rank)) { ok = false; break; }")
        seen_svars |= svars

        def which(kexpr, ind):
            """q (index into pis) and the local window index kk of item window k."""
            out = [f"int q = 0, kk = {kexpr};"]
            for q in range(1, L):
                out.append(f"if (q == {q - 1} && kk >= W{q - 1}) {{ kk -= W{q - 1}; q = {q}; }}")
            pexpr = "0"
            for q in reversed(range(L)):
                pexpr = f"{pis[q]}" if q == L - 1 else f"(q == {q} ? {pis[q]} : {pexpr})"
            out.append(f"const int pw = {pexpr}; (void)pw;")
            out.append("const b200_pathway_d& PD = I.p[pw];")
            return _indent("\n".join(out), ind)

        def emit_wait(ind, prefetch=False):
            """Lag mode: wait for barrier A before the first atomic of the step."""
            sp = " " * ind
            w(sp + "if (pend) {")
            if prefetch:
                # the synapses of the later event batches: into L2 while the barrier completes
                w(sp + "  for (int jj = threadIdx.x; jj < nitems; jj += blockDim.x) {")
                w(sp + "    const int o0 = s_item_off[jj], o1 = (jj + 1 < nitems) ? s_item_off[jj + 1] : E;")
                w(sp + "    if (o1 <= B200_EVENT_BATCH * (int)blockDim.x || o1 <= o0) continue;")
                w(sp + "    const int64_t sg0 = s_item_seg[jj]; const int ln = o1 - o0; const int q = s_item_q[jj];")
                for q, pi in enumerate(pis):
                    lds, _ = split_loads(dict(ptables[pi][1])["on_pre"]["vector_device"] or
                                         dict(ptables[pi][1])["on_pre"]["vector"])
                    arrs = []
                    p = paths[pi]
                    for ct, nm, ptr in lds:
                        if ptr == p["post_ptr"]:
                            arrs.append((f"I.p[{pi}].post", 4))
                        elif ptr == p["pre_ptr"]:
                            arrs.append((f"I.p[{pi}].pre", 4))
                        else:
                            k = next(k for k, v in enumerate(p.get("vars", [])) if v["ptr"] == ptr)
                            arrs.append((f"(const char*)I.p[{pi}].var[{k}]", SIZE[ct]))
                    w(sp + f"    if (q == {q}) {{")
                    for a, sz in arrs:
                        w(sp + f"      for (int ob = 0; ob < ln * {sz}; ob += 128) b200_prefetch_l2((const char*)({a}) + sg0 * {sz} + ob);")
                    w(sp + "    }")
                w(sp + "  }")
            w(sp + f"  B200_PHASE({5 + NP});")
            w(sp + "  if (!b200_inst_wait(I, gen, limit_ns, cluster, rank, bar_old)) ok = false;")
            w(sp + "  pend = false;")
            emit_preload(ind + 2)
            w(sp + "  B200_PHASE(1);")
            w(sp + "}")
        w(f"      // ---- pathways {', '.join(paths[q]['name'] for q in pis)}: propagation")
        w("      {")
        w(f"        const double* const _b200_S = s_Sp{pis[0]}; const float* const _b200_Sf = s_Sp{pis[0]}f; const long long* const _b200_Si = s_Sp{pis[0]}i;")
        w("        (void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
        w(_indent(ptables[pis[0]][0].const_loads(f32), 8))
        w(f"        const b200_group_d& SGD = I.g[{sg}];")
        w(f"        const int* const pref = s_pref_all + {sg} * max_tiles1;")
        w(f"        const int* const tst = s_tst + {sg} * max_tiles1;")
        w(f"        const int32_t* const scr = s_scr[{sg}];")
        for q, pi in enumerate(pis):
            w(f"        const int W{q} = I.p[{pi}].D - I.p[{pi}].dmin + 1; (void)W{q};")
        w(f"        const int WT = {' + '.join(f'W{q}' for q in range(L))};")
        w("        for (int k = threadIdx.x; k < WT; k += blockDim.x) {")
        w(which("k", 10))
        w("          const int d = PD.dmin + kk;")
        w("          const int64_t s = ts - d;")
        w("          int n = 0, b = 0;")
        w("          if (s >= 0) {")
        w("            if (d == 0) {  // (lag mode: only pathways without synapses have delay 0)")
        w("              if (!lagm) { b = pref[PD.tile_lo]; n = pref[PD.tile_hi] - b; }")
        w("            }")
        w("            else if (s_wr_ok[pw]) {  // this CTA's shared copy of the slot's bounds")
        w("              const int* wr = s_wr + (pw * B200_WR_SLOTS + (int)(s % SGD.R)) * 2;")
        w("              b = wr[0]; n = wr[1] - b;")
        w("            } else {")
        w("              const int32_t* rp = SGD.ring_prefix + (int64_t)(s % SGD.R) * (SGD.n_tiles + 1);")
        w("              b = rp[PD.tile_lo]; n = rp[PD.tile_hi] - b;")
        w("            }")
        w("          }")
        w("          s_nd[k] = n; s_base[k] = b;")
        w("        }")
        w("        __syncthreads();")
        w("        {")
        w("          int carry = 0;")
        w("          for (int c0 = 0; c0 < WT; c0 += blockDim.x) {")
        w("            const int k = c0 + threadIdx.x;")
        w("            const int x = k < WT ? s_nd[k] : 0;")
        w("            int tot;")
        w("            const int ex = b200_block_exscan(x, s_wsum, &tot);")
        w("            if (k < WT) s_ndoff[k] = carry + ex;")
        w("            carry += tot;")
        w("          }")
        w("          if (threadIdx.x == 0) s_ndoff[WT] = carry;")
        w("          __syncthreads();")
        w("        }")
        w(f"        B200_PHASE({4 + NP});  // windows")
        w("        if (arrive_due) { b200_inst_arrive(I, cluster, rank, bar_old); arrive_due = false; pend = true; }")
        w("        const int Wtot = s_ndoff[WT];")
        w("        const int i0 = (int)((int64_t)Wtot * rank / I.n_cta);")
        w("        const int i1 = (int)((int64_t)Wtot * (rank + 1) / I.n_cta);")
        w("        for (int cb = i0; cb < i1; cb += blockDim.x) {")
        w("          const int it = cb + threadIdx.x;")
        w("          int len = 0;")
        w("          if (it < i1) {")
        w("            const int k = b200_upper_bound(s_ndoff, WT + 1, it) - 1;")
        w(which("k - 0", 12))
        w("            const int W = PD.D - PD.dmin + 1;")
        w("            const int d = PD.dmin + kk, r = it - s_ndoff[k];")
        w("            int32_t src;")
        w("            if (d == 0) {")
        w("              const int pos = s_base[k] + r;")
        w("              const int u = b200_upper_bound(pref, SGD.n_tiles + 1, pos) - 1;")
        w("              src = scr[tst[u] + pos - pref[u]];")
        w("            } else {")
        w("              src = SGD.ring[(int64_t)((ts - d) % SGD.R) * SGD.N + s_base[k] + r];")
        w("            }")
        w("            const int64_t seg = (int64_t)(src - PD.src_lo) * W + kk;")
        w("            const int64_t lo = PD.segptr[seg];")
        w("            len = (int)(PD.segptr[seg + 1] - lo);")
        w("            s_item_seg[threadIdx.x] = lo;")
        w("            s_item_src[threadIdx.x] = src;")
        w("            s_item_q[threadIdx.x] = q;")
        w("          }")
        w("          int E;")
        w("          const int off = b200_block_exscan(len, s_wsum, &E);")
        w("          s_item_off[threadIdx.x] = off;")
        w("          __syncthreads();")
        w(f"          B200_PHASE({5 + NP});  // items")
        w("          const int nitems = (i1 - cb) < (int)blockDim.x ? (i1 - cb) : (int)blockDim.x;")
        # events: when every pathway of the group starts its on_pre with loads of
        # the same types, a thread first issues the loads of its four events,
        # then applies them (the loads no longer wait behind the atomics)
        sigs = []
        for pi in pis:
            lds, _ = split_loads(dict(ptables[pi][1])["on_pre"]["vector_device"] or
                                 dict(ptables[pi][1])["on_pre"]["vector"])
            sigs.append([ct for ct, _, _ in lds])
        two_phase = all(sg_ == sigs[0] for sg_ in sigs) and len(sigs[0]) > 0
        if two_phase:
            # (the variants capped at 64 registers keep the one-phase loop: the
            # loads of four events in flight would spill there)
            w("          if constexpr (MAXT * MINB < 1024) {")
            NL = len(sigs[0])

            def load_expr(pi, ptr, ct):
                p = paths[pi]
                own = p.get("alias", -1) if p.get("alias", -1) >= 0 else pi  # shared synapses: the owner's arrays
                if ptr == p["post_ptr"]:
                    return f"I.p[{own}].{syn_arr(own, 'post')}[_idx]"
                if ptr == p["pre_ptr"]:
                    return f"I.p[{own}].{syn_arr(own, 'pre')}[_idx]"
                k = next(k for k, v in enumerate(p.get("vars", [])) if v["ptr"] == ptr)
                return f"(({ct}*)I.p[{pi}].var[{k}])[_idx]"

            w("          for (int b0 = 0; b0 < E; b0 += B200_EVENT_BATCH * (int)blockDim.x) {  // block-uniform")
            w("            int _q4[B200_EVENT_BATCH]; int32_t _pre4[B200_EVENT_BATCH]; int64_t _ix4[B200_EVENT_BATCH];")
            for li, ct in enumerate(sigs[0]):
                w(f"            {ct} _ld{li}[B200_EVENT_BATCH];")
            w("#pragma unroll")
            w("            for (int qq = 0; qq < B200_EVENT_BATCH; ++qq) {")
            w("              const int e = b0 + qq * (int)blockDim.x + (int)threadIdx.x;")
            w("              _q4[qq] = -1;")
            w("              if (e < E) {")
            w("                const int j = b200_upper_bound(s_item_off, nitems, e) - 1;")
            w("                const int64_t _idx = s_item_seg[j] + (e - s_item_off[j]);")
            w("                const int q = s_item_q[j];")
            w("                _q4[qq] = q; _pre4[qq] = s_item_src[j]; _ix4[qq] = _idx;")
            for q, pi in enumerate(pis):
                lds, _ = split_loads(dict(ptables[pi][1])["on_pre"]["vector_device"] or
                                     dict(ptables[pi][1])["on_pre"]["vector"])
                w(("                if" if q == 0 else "                else if") + f" (q == {q}) {{")
                if paths[pi].get("alias", -1) >= 0:  # the synapse's position in the owning pathway
                    w(f"                  const int64_t _idx = I.p[{pi}].sidx[_ix4[qq]]; _ix4[qq] = _idx;")
                for li, (ct, nm, ptr) in enumerate(lds):
                    w(f"                  _ld{li}[qq] = {load_expr(pi, ptr, ct)};")
                w("                }")
            w("              }")
            w("            }")
            emit_wait(12, prefetch=not any(paths[q].get("alias", -1) >= 0 for q in pis))
            w("#pragma unroll")
            w("            for (int qq = 0; qq < B200_EVENT_BATCH; ++qq) {")
            w("              if (_q4[qq] >= 0) {")
            w("                const int q = _q4[qq];")
            w("                const int64_t _idx = _ix4[qq]; (void)_idx;")
            w("                const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            w("                const int32_t _b200_pre = _pre4[qq]; (void)_b200_pre;")
            for q, pi in enumerate(pis):
                p = paths[pi]
                tab, blocks = ptables[pi]
                blk = dict(blocks)["on_pre"]
                lds, rest = split_loads(blk["vector_device"] or blk["vector"])
                w(("                if" if q == 0 else "                else if") + f" (q == {q}) {{  // {p['name']}")
                w(f"                  const b200_pathway_d& PQ = I.p[{pi}]; (void)PQ;")
                w(f"                  const double* const _b200_S = s_Sp{pi}; const float* const _b200_Sf = s_Sp{pi}f; const long long* const _b200_Si = s_Sp{pi}i;")
                for ptr, (gidx, vidx) in sorted(p.get("group_ptrs", {}).items()):
                    v = groups[gidx]["vars"][vidx]
                    w(f"                  {v['ctype']}* __restrict__ const {ptr} = ({v['ctype']}*)s_gv[{gidx}][{vidx}]; (void){ptr};")
                for k, v in enumerate(p.get("vars", [])):
                    w(f"                  {v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)PQ.var[{k}]; (void){v['ptr']};")
                own = p.get("alias", -1) if p.get("alias", -1) >= 0 else pi
                w(f"                  const int32_t* __restrict__ const {p['post_ptr']} = I.p[{own}].{syn_arr(own, 'post')}; (void){p['post_ptr']};")
                w(f"                  const int32_t* __restrict__ const {p['pre_ptr']} = I.p[{own}].{syn_arr(own, 'pre')}; (void){p['pre_ptr']};")
                w(_indent(tab.scalar_loads("on_pre", f32), 18))
                w(_indent(_device(tab.time_code("on_pre")), 18))
                w("                  {  // (Brian's vector code may redeclare the clock's names)")
                for li, (ct, nm, ptr) in enumerate(lds):
                    w(f"                  {ct} {nm} = _ld{li}[qq];")
                w(_indent(rest, 18))
                w("                  }")
                w("                }")
            w("              }")
            w("            }")
            if (sg, pis) == (merged[0][0], merged[0][1]):
                # lag mode: this step's spike lists while the first batch's atomics drain
                w("            if (lists_due) {")
                w("              lists_due = false;")
                emit_lists()
                w("            }")
            w("          }")
            w("          } else {")
        if True:  # the one-phase loop (always emitted; the only one without a common load signature)
            emit_wait(10)
            w("          for (int e0 = threadIdx.x; e0 < E; e0 += 4 * (int)blockDim.x) {")
            w("#pragma unroll")
            w("            for (int qq = 0; qq < 4; ++qq) {")
            w("              const int e = e0 + qq * (int)blockDim.x;")
            w("              if (e < E) {")
            w("                const int j = b200_upper_bound(s_item_off, nitems, e) - 1;")
            w("                const int64_t _idx = s_item_seg[j] + (e - s_item_off[j]);")
            w("                const int32_t _b200_pre = s_item_src[j]; (void)_b200_pre;")
            w("                const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            w("                const int q = s_item_q[j]; (void)q;")
            for q, pi in enumerate(pis):
                p = paths[pi]
                tab, blocks = ptables[pi]
                blk = dict(blocks)["on_pre"]
                w(("                if" if q == 0 else "                else if") + f" (q == {q}) {{  // {p['name']}")
                w(f"                  const b200_pathway_d& PQ = I.p[{pi}]; (void)PQ;")
                w(f"                  const double* const _b200_S = s_Sp{pi}; const float* const _b200_Sf = s_Sp{pi}f; const long long* const _b200_Si = s_Sp{pi}i;")
                for k, v in enumerate(p.get("vars", [])):
                    w(f"                  {v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)PQ.var[{k}]; (void){v['ptr']};")
                own = p.get("alias", -1) if p.get("alias", -1) >= 0 else pi
                w(f"                  const int32_t* __restrict__ const {p['post_ptr']} = I.p[{own}].{syn_arr(own, 'post')}; (void){p['post_ptr']};")
                w(f"                  const int32_t* __restrict__ const {p['pre_ptr']} = I.p[{own}].{syn_arr(own, 'pre')}; (void){p['pre_ptr']};")
                for ptr, (gidx, vidx) in sorted(p.get("group_ptrs", {}).items()):
                    v = groups[gidx]["vars"][vidx]
                    w(f"                  {v['ctype']}* __restrict__ const {ptr} = ({v['ctype']}*)s_gv[{gidx}][{vidx}]; (void){ptr};")
                w(_indent(tab.scalar_loads("on_pre", f32), 18))
                w(_indent(_device(tab.time_code("on_pre")), 18))
                if own != pi:  # the synapse's position in the owning pathway
                    w("                  const int64_t _idx_csr = _idx;")
                w("                  {  // (Brian's vector code may redeclare the clock's names)")
                if own != pi:
                    w(f"                  const int64_t _idx = I.p[{pi}].sidx[_idx_csr];")
                    w("                  const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
                w(_indent(blk["vector_device"] if blk.get("vector_device") else blk["vector"], 18))
                w("                  }")
                w("                }")
            w("              }")
            w("            }")
        w("          }")
        if two_phase:
            w("          }  // if constexpr")
        w("          __syncthreads();")
        w(f"          B200_PHASE({3 + pis[0]});  // events")
        w("        }")
        w("      }")
        w(f"      B200_PHASE({3 + pis[0]});")
    w("      if (arrive_due) { b200_inst_arrive(I, cluster, rank, bar_old); arrive_due = false; pend = true; }")
    w("      if (pend) {  // no events this step")
    w("        if (!b200_inst_wait(I, gen, limit_ns, cluster, rank, bar_old)) ok = false;")
    w("        pend = false;")
    emit_preload(8)
    w("        B200_PHASE(1);")
    w("      }")
    w("      if (!ok) break;")
    w("      if (lagm && lists_due) {")
    emit_lists()
    w("      }")
    w("      if (!b200_inst_barrier(I, gen, limit_ns, cluster, rank)) { ok = false; break; }")
    w(f"      B200_PHASE({3 + NP});")
    w("    }  // steps")
    w(f"    if (prof && threadIdx.x == 0)")
    w(f"      for (int q = 0; q < {NPH}; ++q) atomicAdd(&prof[(size_t)unit * {NPH} + q], _pacc[q]);")
    w("#undef B200_PHASE")

    # ---- end of launch: apply the reset of the last executed step, write back the cache
    w("    if (ok && ts > ts0) {")
    w("      const double _b200_t = (double)(ts - 1) * _b200_dt; (void)_b200_t;")
    w("      const int64_t _b200_ts = ts - 1;")
    for gi in range(NG):
        rb = deferred_block(gi, 6, "ts - 1")
        if rb:
            w(rb)
    end = syn_text(6, "ts - 1", "end")
    if end:
        w(end)
    w("    }")
    w("    __syncthreads();")
    w("    if (s_cache) {")
    for gi, g in enumerate(groups):
        for k in USED[gi]:
            sz = SIZE[g["vars"][k]["ctype"]]
            w(f"      b200_copy_bytes(I.g[{gi}].var[{k}], s_gv[{gi}][{k}], (size_t)I.g[{gi}].N * {sz});")
    w("    }")
    if any(PRIV):
        w("    if (s_pcache) {")
        for gi, g in enumerate(groups):
            for k in PRIV[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"      b200_copy_bytes((char*)I.g[{gi}].var[{k}] + (size_t)s_pown[{gi}][0] * {sz}, "
                  f"(const char*)s_gv[{gi}][{k}] + (size_t)s_pown[{gi}][0] * {sz}, "
                  f"(size_t)(s_pown[{gi}][1] - s_pown[{gi}][0]) * {sz});")
        w("    }")
    w("    if (threadIdx.x == 0 && rank == 0) {")
    w("      *I.ts_done = ts;")
    for gi, g in enumerate(groups):
        if g.get("generator"):
            w(f"      *I.g[{gi}].gen_last = s_glast[{gi}];")
    for m in range(len(spkmons)):
        w(f"      *I.sm[{m}].n = s_mon_n[{m}];")
    for m in range(len(statemons)):
        w(f"      *I.stm[{m}].n = s_stm_n[{m}];")
    w("    }")
    w("    __syncthreads();")
    w("  }")
    w("}")
    w("")

    # ------------------------------------------------------------- owner-mode kernel
    def emit_owner_kernel():
        """Owner mode: each CTA of an instance owns the target neurons of its
        tiles and is the only one to deliver into them.  A step is
        update+threshold (own tiles, spike list published in the ring) -> split
        barrier -> push of the spikes of step ts-lag into per-CTA event FIFOs
        (delay 0: applied at once) -> delivery of the events due at ts."""
        merged = []
        for pi, p in enumerate(paths):
            touched = set(p.get("group_ptrs", {}))
            last = merged[-1] if merged else None
            if last and last[0] == p["src"] and not (last[2] & touched):
                last[1].append(pi)
                last[2].update(touched)
            else:
                merged.append((p["src"], [pi], set(touched)))

        def body_decls(pi, ind):
            """Declarations the on_pre body of pathway pi needs (owner arrays)."""
            p = paths[pi]
            L = [f"const b200_pathway_d& PQ = I.p[{pi}]; (void)PQ;",
                 f"const double* const _b200_S = s_Sp{pi}; const float* const _b200_Sf = s_Sp{pi}f; const long long* const _b200_Si = s_Sp{pi}i;"]
            for k, v in enumerate(p.get("vars", [])):
                L.append(f"{v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)PQ.var[{k}]; (void){v['ptr']};")
            L.append(f"const int32_t* __restrict__ const {p['post_ptr']} = PQ.post; (void){p['post_ptr']};")
            for ptr, (gidx, vidx) in sorted(p.get("group_ptrs", {}).items()):
                v = groups[gidx]["vars"][vidx]
                L.append(f"{v['ctype']}* const {ptr} = ({v['ctype']}*)s_gv[{gidx}][{vidx}]; (void){ptr};")
            tab, blocks = ptables[pi]
            L.append(tab.scalar_loads("on_pre", f32))
            L.append(_device(tab.time_code("on_pre")))
            L.append("(void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
            return _indent("\n".join(L), ind)

        def body_code(pi):
            p = paths[pi]
            blk = dict(ptables[pi][1])["on_pre"]
            return blk["vector_device"] if blk.get("vector_device") else blk["vector"]

        def fifo_body(pi, ind):
            """on_pre applied to the FIFO record `rec` (loads bound to the record)."""
            p = paths[pi]
            loads, rest = split_loads(body_code(pi))
            varptr = {v["ptr"]: k for k, v in enumerate(p.get("vars", []))}
            L = []
            for ct, nm, ptr in loads:
                if ptr == p["post_ptr"]:
                    L.append(f"const {ct} {nm} = ({ct})PQ.ev.tgt[rbase + rec];")
                else:
                    m = PAYLOAD[pi].index(varptr[ptr])
                    L.append(f"const {ct} {nm} = (({ct}*)PQ.ev.pay[{m}])[rbase + rec];")
            L.append(rest)
            return _indent("\n".join(L), ind)

        def fifo_store(pi, ind):
            """pass 2: the record of synapse `syn` at FIFO position `rec`."""
            p = paths[pi]
            L = ["PQ.ev.tgt[rbase + rec] = PQ.post[syn];"]
            for m, k in enumerate(PAYLOAD[pi]):
                ct = p["vars"][k]["ctype"]
                L.append(f"(({ct}*)PQ.ev.pay[{m}])[rbase + rec] = (({ct}*)PQ.var[{k}])[syn];")
            return _indent("\n".join(L), ind)

        def qdispatch(pis, ind, fn):
            """if (q == 0) { fn(pi0) } else if ... over the pathways of a group."""
            L = []
            for q, pi in enumerate(pis):
                L.append(("if" if q == 0 else "else if") + f" (q == {q}) {{  // {paths[pi]['name']}")
                L.append(fn(pi))
                L.append("}")
            return _indent("\n".join(L), ind)

        w("static size_t b200_dyn_smem_owner(int threads, int max_tiles1, int max_w, int state_bytes) {")
        w("  return b200_dyn_smem(threads, max_tiles1, max_w, state_bytes) + (size_t)max_w * 8 + (size_t)(max_w + 1) * 4;")
        w("}")
        w("")
        w("template <int MAXT, int MINB>")
        w("__global__ void __launch_bounds__(MAXT, MINB) b200_owner_kernel(")
        w("    const b200_inst_d* __restrict__ insts, const int2* __restrict__ cta_map, int n_inst,")
        w("    int queue_mode, int* work, int64_t max_steps, uint64_t limit_ns, int max_tiles1, int max_w,")
        w("    int fault_rank, int state_bytes, unsigned long long* __restrict__ prof, int cluster) {")
        w("  (void)queue_mode; (void)work;")
        w("  extern __shared__ __align__(16) unsigned char b200_dyn[];")
        w("  unsigned char* const s_state = b200_dyn;")
        w("  int64_t* const s_item_seg = (int64_t*)(b200_dyn + state_bytes);  // [threads]")
        w("  int64_t* const s_wbase = s_item_seg + blockDim.x;                   // [max_w] first record of each window")
        w("  int* const s_item_off = (int*)(s_wbase + max_w);                    // [threads + 1]")
        w("  int* const s_item_src = s_item_off + blockDim.x + 1;                // [threads]")
        w("  int* const s_item_q = s_item_src + blockDim.x;                      // [threads]")
        w("  int* const s_pref_all = s_item_q + blockDim.x;                      // [NG * max_tiles1]")
        w("  int* const s_tst = s_pref_all + B200_NG * max_tiles1;               // [NG * max_tiles1]")
        w("  int* const s_nd = s_tst + B200_NG * max_tiles1;                     // [max_w] per-delay counts")
        w("  int* const s_base = s_nd + max_w;                                   // [max_w + 1] batch offsets")
        w("  int* const s_ndoff = s_base + max_w + 1;                            // [max_w + 1] window offsets")
        w("  __shared__ __align__(16) b200_inst_d I;")
        w("  __shared__ int s_wsum[B200_MAX_WARPS + 1];")
        w("  __shared__ int s_cnt[B200_MAX_THREADS];")
        w("  __shared__ int s_unit, s_rank, s_flag, s_cache;")
        w("  __shared__ long long s_mon_n[B200_MAX_SPKMON];")
        w("  __shared__ long long s_stm_n[B200_MAX_STATEMON];")
        w("  __shared__ void* s_gv[B200_NG][B200_MAXV];")
        w("  __shared__ int s_ut[B200_NG][2];")
        w("  __shared__ int s_own[B200_NG][2];")
        w("  __shared__ int s_glast[B200_NG], s_gen_lo, s_gen_hi;  // spike generator cursors")
        w("  (void)s_glast; (void)s_gen_lo; (void)s_gen_hi;")
        w(f"  __shared__ long long s_head[{max(NP, 1)}], s_tail[{max(NP, 1)}];")
        w(f"  __shared__ int s_qoff[{max(NP, 1) + 1}], s_skip[{max(NP, 1)}];")
        w(f"  __shared__ int32_t* s_toff[{max(NP, 1)}];        // this CTA's batch table: per-delay offsets,")
        w(f"  __shared__ long long* s_tbase[{max(NP, 1)}];     // first record and step of each batch")
        w(f"  __shared__ long long* s_ttag[{max(NP, 1)}];      // (shared memory or global)")
        for gi in range(NG):
            n_ = max(gtables[gi][0].size, 1)
            w(f"  __shared__ double s_Sg{gi}[{n_}]; __shared__ float s_Sg{gi}f[{n_}]; __shared__ long long s_Sg{gi}i[{n_}];")
        for pi in range(NP):
            n_ = max(ptables[pi][0].size, 1)
            w(f"  __shared__ double s_Sp{pi}[{n_}]; __shared__ float s_Sp{pi}f[{n_}]; __shared__ long long s_Sp{pi}i[{n_}];")
        w("  (void)s_item_src; (void)s_state;")
        w("  for (int pass = 0;; ++pass) {")
        w("    if (threadIdx.x == 0) {")
        w("      if (pass == 0) { const int2 m = cta_map[blockIdx.x]; s_unit = m.x; s_rank = m.y; }")
        w("      else s_unit = n_inst;")
        w("    }")
        w("    __syncthreads();")
        w("    const int unit = s_unit, rank = s_rank;")
        w("    if (unit >= n_inst) break;")
        w("    {")
        w("      const long long* src = (const long long*)&insts[unit];")
        w("      long long* dst = (long long*)&I;")
        w("      for (int k = threadIdx.x; k < (int)(sizeof(b200_inst_d) / 8); k += blockDim.x) dst[k] = src[k];")
        w("    }")
        w("    __syncthreads();")
        w("    if (threadIdx.x == 0) {")
        for m in range(len(spkmons)):
            w(f"      s_mon_n[{m}] = *((volatile long long*)I.sm[{m}].n);")
        for m in range(len(statemons)):
            w(f"      s_stm_n[{m}] = *((volatile long long*)I.stm[{m}].n);")
        w("      const int cache = (I.cache_bytes > 0 && I.cache_bytes <= state_bytes) ? 1 : 0;")
        w("      s_cache = cache;")
        w("      size_t off = 0;")
        for gi, g in enumerate(groups):
            w(f"      s_ut[{gi}][0] = I.g[{gi}].cta_tile[rank]; s_ut[{gi}][1] = I.g[{gi}].cta_tile[rank + 1];")
            w(f"      s_own[{gi}][0] = I.g[{gi}].tile_start[s_ut[{gi}][0]]; s_own[{gi}][1] = I.g[{gi}].tile_start[s_ut[{gi}][1]];")
            if g.get("generator"):
                w(f"      s_glast[{gi}] = *((volatile int32_t*)I.g[{gi}].gen_last);")
            for k in range(len(g["vars"])):
                w(f"      s_gv[{gi}][{k}] = I.g[{gi}].var[{k}];")
            w("      if (cache) {  // own neurons only: pointers offset so that global indices address them")
            for k in USED[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"        s_gv[{gi}][{k}] = (void*)(s_state + off - (size_t)s_own[{gi}][0] * {sz});")
                w(f"        off += ((size_t)(s_own[{gi}][1] - s_own[{gi}][0]) * {sz} + 15) & ~(size_t)15;")
            w("      }")
        for pi in range(NP):
            w(f"      if (I.p[{pi}].D > 0) {{")
            w(f"        const b200_fifo_d& F = I.p[{pi}].ev;")
            w(f"        s_head[{pi}] = F.state[2 * rank]; s_tail[{pi}] = F.state[2 * rank + 1];")
            w("        if (I.tab_smem) {")
            w(f"          s_toff[{pi}] = (int32_t*)(s_state + F.tab_off);")
            w(f"          s_tbase[{pi}] = (long long*)(s_state + F.tab_off + (((size_t)F.RB * (F.W + 1) * 4 + 15) & ~(size_t)15));")
            w(f"          s_ttag[{pi}] = s_tbase[{pi}] + F.RB;")
            w("        } else {")
            w(f"          s_toff[{pi}] = F.off + (size_t)rank * F.RB * (F.W + 1);")
            w(f"          s_tbase[{pi}] = (long long*)F.base + (size_t)rank * F.RB;")
            w(f"          s_ttag[{pi}] = (long long*)F.tag + (size_t)rank * F.RB;")
            w("        }")
            w("      }")
        for gi, g in enumerate(groups):
            if ALIAS[gi] is not None:
                for k in range(len(g["vars"])):
                    w(f"      s_gv[{gi}][{k}] = s_gv[{ALIAS[gi]}][{k}];  // a custom event of group {ALIAS[gi]}")
        w("    }")
        w("    __syncthreads();")
        w("    if (I.tab_smem) {  // this CTA's batch tables live in shared memory for the launch")
        for pi in range(NP):
            w(f"      if (I.p[{pi}].D > 0) {{")
            w(f"        const b200_fifo_d& F = I.p[{pi}].ev;")
            w(f"        b200_copy_bytes(s_toff[{pi}], F.off + (size_t)rank * F.RB * (F.W + 1), (size_t)F.RB * (F.W + 1) * 4);")
            w(f"        b200_copy_bytes(s_tbase[{pi}], F.base + (size_t)rank * F.RB, (size_t)F.RB * 8);")
            w(f"        b200_copy_bytes(s_ttag[{pi}], F.tag + (size_t)rank * F.RB, (size_t)F.RB * 8);")
            w("      }")
        w("    }")
        for gi in range(NG):
            w(f"    for (int u = threadIdx.x; u <= I.g[{gi}].n_tiles; u += blockDim.x) s_tst[{gi} * max_tiles1 + u] = I.g[{gi}].tile_start[u];")
        for gi in range(NG):
            w(f"    for (int k = threadIdx.x; k < {gtables[gi][0].size}; k += blockDim.x) {{")
            w(f"      const double x = I.g[{gi}].S[k]; s_Sg{gi}[k] = x; s_Sg{gi}f[k] = (float)x; s_Sg{gi}i[k] = (long long)x;")
            w("    }")
        for pi in range(NP):
            w(f"    for (int k = threadIdx.x; k < {ptables[pi][0].size}; k += blockDim.x) {{")
            w(f"      const double x = I.p[{pi}].S[k]; s_Sp{pi}[k] = x; s_Sp{pi}f[k] = (float)x; s_Sp{pi}i[k] = (long long)x;")
            w("    }")
        w("    if (s_cache) {  // the owned neurons' state lives in shared memory for the launch")
        for gi, g in enumerate(groups):
            for k in USED[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"      b200_copy_bytes((char*)s_gv[{gi}][{k}] + (size_t)s_own[{gi}][0] * {sz}, (const char*)I.g[{gi}].var[{k}] + (size_t)s_own[{gi}][0] * {sz},")
                w(f"                      (size_t)(s_own[{gi}][1] - s_own[{gi}][0]) * {sz});")
        w("    }")
        w("    __syncthreads();")
        w("    const int64_t ts0 = I.ts;")
        w("    const int64_t ts_stop = (I.ts_end < ts0 + max_steps) ? I.ts_end : ts0 + max_steps;")
        w("    const double _b200_dt = I.dt;")
        w("    int64_t ts = ts0;")
        w("    bool ok = true, pend = false;")
        w("    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, NW = blockDim.x >> 5;")
        w("    (void)lane; (void)wid; (void)NW;")
        w(f"    __shared__ unsigned long long _pt, _pacc[{NPH}];")
        w(f"    if (threadIdx.x == 0) {{ _pt = 0; for (int q = 0; q < {NPH}; ++q) _pacc[q] = 0; }}")
        w("#define B200_PHASE(q) do { if (prof && threadIdx.x == 0) { const unsigned long long _c = clock64(); _pacc[q] += _c - _pt; _pt = _c; } } while (0)")

        def emit_lists(tsexpr, record_mon, ind):
            """Tile prefix of the spikes of step `tsexpr` for every group, and
            (if `record_mon`) the spike and rate monitors of that step."""
            sp = " " * ind
            for gi, g in enumerate(groups):
                scr_e, tc_e = owner_list(gi, tsexpr)
                w(sp + "{")
                w(sp + f"  const int32_t* const lst = {scr_e}; const int32_t* const tcnt = {tc_e};")
                w(sp + f"  int* const pref = s_pref_all + {gi} * max_tiles1;")
                w(sp + f"  const int* const tst = s_tst + {gi} * max_tiles1;")
                w(sp + f"  const int nt = I.g[{gi}].n_tiles;")
                w(sp + "  int carry = 0;")
                w(sp + "  for (int c0 = 0; c0 < nt; c0 += blockDim.x) {")
                w(sp + "    const int u = c0 + threadIdx.x;")
                w(sp + "    const int x = u < nt ? tcnt[u] : 0;")
                w(sp + "    int tot;")
                w(sp + "    const int ex = b200_block_exscan(x, s_wsum, &tot);")
                w(sp + "    if (u < nt) pref[u] = carry + ex;")
                w(sp + "    carry += tot;")
                w(sp + "  }")
                w(sp + "  if (threadIdx.x == 0) pref[nt] = carry;")
                w(sp + "  __syncthreads();")
                w(sp + "  (void)lst; (void)tst;")
                for mi, m in enumerate(spkmons):
                    if m["group"] != gi:
                        continue
                    w(sp + f"  if ({record_mon}) {{  // spike monitor {mi}")
                    w(sp + f"    const b200_spkmon_d& SM = I.sm[{mi}];")
                    w(sp + f"    const long long mbase = s_mon_n[{mi}] - pref[SM.tile_lo];")
                    w(sp + f"    const int a = s_ut[{gi}][0] > SM.tile_lo ? s_ut[{gi}][0] : SM.tile_lo;")
                    w(sp + f"    const int b = s_ut[{gi}][1] < SM.tile_hi ? s_ut[{gi}][1] : SM.tile_hi;")
                    w(sp + "    for (int u = a; u < b; ++u) {")
                    w(sp + "      const int cnt = pref[u + 1] - pref[u], base = tst[u];")
                    w(sp + "      for (int j = threadIdx.x; j < cnt; j += blockDim.x) {")
                    w(sp + "        const int idx = lst[base + j];")
                    w(sp + "        const long long pos = mbase + pref[u] + j;")
                    w(sp + "        SM.i[pos] = idx - SM.lo;")
                    w(sp + f"        SM.ts[pos] = (int32_t)({tsexpr});")
                    if m.get("vars"):
                        w(sp + "        " + value_rows(mi, gi, "pos", "idx"))
                    w(sp + "        SM.count[idx - SM.lo] += 1;")
                    w(sp + "      }")
                    w(sp + "    }")
                    w(sp + "    __syncthreads();")
                    w(sp + f"    if (threadIdx.x == 0) s_mon_n[{mi}] += pref[SM.tile_hi] - pref[SM.tile_lo];")
                    w(sp + "  }")
                for mi, m in enumerate(ratemons):
                    if m["group"] != gi:
                        continue
                    w(sp + f"  if (({record_mon}) && rank == 0 && threadIdx.x == 0) {{  // rate monitor {mi}")
                    w(sp + f"    const b200_ratemon_d& RM = I.rm[{mi}];")
                    w(sp + f"    RM.cnt[({tsexpr}) - RM.step0] = pref[RM.tile_hi] - pref[RM.tile_lo];")
                    w(sp + "  }")
                w(sp + "}")
            w(sp + "__syncthreads();")

        w("    for (; ts < ts_stop; ++ts) {")
        w("      if (threadIdx.x == 0) {")
        w("        int st = 0;")
        for m in range(len(spkmons)):
            w(f"        if (s_mon_n[{m}] + 2 * (long long)(I.sm[{m}].hi - I.sm[{m}].lo) > I.sm[{m}].cap) st = 1;")
        w("        s_flag = st;")
        w("      }")
        w("      __syncthreads();")
        w("      if (s_flag) break;")
        w("      const double _b200_t = (double)ts * _b200_dt;")
        w("      const int64_t _b200_ts = ts;")
        w("      if (prof && threadIdx.x == 0) _pt = clock64();")
        emit_phase_a(True)
        w("      B200_PHASE(0);")
        w("      // test hook: CTA `fault_rank` leaves without arriving, the others must time out")
        w("      if (rank == fault_rank && ts == ts0) { ok = false; pend = false; break; }")
        w("      // split barrier: lag 1 waits for the previous step's spikes (arrived long ago)")
        w("      if (I.lag) {")
        w("        if (pend && !b200_owner_wait(I, ts - 1, limit_ns, cluster)) { ok = false; pend = false; break; }")
        w("        b200_owner_arrive(I, cluster);")
        w("        pend = true;")
        w("      } else {")
        w("        b200_owner_arrive(I, cluster);")
        w("        if (!b200_owner_wait(I, ts, limit_ns, cluster)) { ok = false; break; }")
        w("      }")
        w("      B200_PHASE(1);")
        w("      const int64_t s_step = ts - I.lag;  // the step whose spikes are pushed now")
        w("      if (s_step >= 0) {")
        emit_lists("s_step", "s_step >= ts0", 8)
        w("      }")
        w("      B200_PHASE(2);")
        for sg, pis, _ in merged:
            L = len(pis)
            w(f"      // ---- pathways {', '.join(paths[q]['name'] for q in pis)}: push and delivery")
            w("      {")
            w(f"        const double* const _b200_S = s_Sp{pis[0]}; const float* const _b200_Sf = s_Sp{pis[0]}f; const long long* const _b200_Si = s_Sp{pis[0]}i;")
            w("        (void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
            w(_indent(ptables[pis[0]][0].const_loads(f32), 8))
            w(f"        const b200_group_d& SGD = I.g[{sg}];")
            w(f"        const int* const pref = s_pref_all + {sg} * max_tiles1;")
            w(f"        const int* const tst = s_tst + {sg} * max_tiles1;")
            w(f"        const int32_t* const lst = SGD.ring + (int64_t)((s_step >= 0 ? s_step : 0) % B200_OWNER_RING) * SGD.N;")
            for q, pi in enumerate(pis):
                w(f"        const int W{q} = I.p[{pi}].D > 0 ? I.p[{pi}].D - I.p[{pi}].dmin + 1 : 0;")
            w(f"        const int WT = {' + '.join(f'W{q}' for q in range(L))};")
            w("        if (threadIdx.x == 0) {")
            w("          int acc = 0;")
            for q, pi in enumerate(pis):
                w(f"          s_qoff[{q}] = acc;")
                w(f"          if (s_step >= 0) acc += pref[I.p[{pi}].tile_hi] - pref[I.p[{pi}].tile_lo];")
            w(f"          s_qoff[{L}] = acc;")
            w("        }")
            w("        for (int k = threadIdx.x; k < WT; k += blockDim.x) s_nd[k] = 0;")
            w("        __syncthreads();")
            w(f"        const int NI = s_qoff[{L}];")

            def window_of(kexpr, ind):
                """q and kk (delay index) of FIFO window k (pathways with D > 0)."""
                out = [f"int q = 0, kk = {kexpr};"]
                for q in range(1, L):
                    out.append(f"if (q == {q - 1} && kk >= W{q - 1}) {{ kk -= W{q - 1}; q = {q}; }}")
                return _indent("\n".join(out), ind)

            koff = " + ".join(["0"] + [f"W{q}" for q in range(L)])

            def koff_of(q):
                return "(" + " + ".join(["0"] + [f"W{x}" for x in range(q)]) + ")"

            def traverse(pass_no):
                """Items (spike of step s_step, pathway) -> owner segments -> events."""
                w("        for (int cb = 0; cb < NI; cb += blockDim.x) {")
                w("          const int it = cb + threadIdx.x;")
                w("          int len = 0;")
                w("          if (it < NI) {")
                w("            int q = 0;")
                for q in range(1, L):
                    w(f"            if (it >= s_qoff[{q}]) q = {q};")
                pexpr = f"{pis[L - 1]}"
                for q in reversed(range(L - 1)):
                    pexpr = f"(q == {q} ? {pis[q]} : {pexpr})"
                w(f"            const b200_pathway_d& PD = I.p[{pexpr}];")
                w("            const int pos = it - s_qoff[q] + pref[PD.tile_lo];")
                w(f"            const int u = b200_upper_bound(pref, I.g[{sg}].n_tiles + 1, pos) - 1;")
                w("            const int32_t src = lst[tst[u] + pos - pref[u]];")
                w("            const int64_t sg_ = (int64_t)(src - PD.src_lo) * I.n_cta + rank;")
                w("            const int64_t lo = PD.segptr[sg_];")
                w("            len = (int)(PD.segptr[sg_ + 1] - lo);")
                w("            s_item_seg[threadIdx.x] = lo;")
                w("            s_item_q[threadIdx.x] = q;")
                w("          }")
                w("          int E;")
                w("          const int eoff = b200_block_exscan(len, s_wsum, &E);")
                w("          s_item_off[threadIdx.x] = eoff;")
                w("          __syncthreads();")
                w("          const int nitems = (NI - cb) < (int)blockDim.x ? (NI - cb) : (int)blockDim.x;")
                w("          for (int e0 = threadIdx.x; e0 < E; e0 += 4 * (int)blockDim.x) {")
                w("#pragma unroll")
                w("            for (int qq = 0; qq < 4; ++qq) {")
                w("              const int e = e0 + qq * (int)blockDim.x;")
                w("              if (e < E) {")
                w("                const int j = b200_upper_bound(s_item_off, nitems, e) - 1;")
                w("                const int64_t syn = s_item_seg[j] + (e - s_item_off[j]);")
                w("                const int q = s_item_q[j];")
                for q, pi in enumerate(pis):
                    w(("                if" if q == 0 else "                else if") + f" (q == {q}) {{  // {paths[pi]['name']}")
                    if pass_no == 1:
                        w(f"                  if (I.p[{pi}].D == 0) {{  // no delay: applied now")
                        w("                    const int64_t _idx = syn; const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
                        w(body_decls(pi, 20))
                        w(_indent(body_code(pi), 20))
                        w("                  } else {")
                        w(f"                    atomicAdd(&s_nd[{koff_of(q)} + (int)I.p[{pi}].odelay[syn] - I.p[{pi}].dmin], 1);")
                        w("                  }")
                    else:
                        w(f"                  if (I.p[{pi}].D > 0 && !s_skip[{pi}]) {{")
                        w(f"                    const b200_pathway_d& PQ = I.p[{pi}];")
                        w(f"                    const int k = {koff_of(q)} + (int)PQ.odelay[syn] - PQ.dmin;")
                        w(f"                    const int64_t p_ = (int64_t)(s_base[k] - s_base[{koff_of(q)}]) + atomicAdd(&s_nd[k], 1);")
                        w("                    const int64_t rec = (s_head[" + str(pi) + "] + p_) & (PQ.ev.cap - 1);")
                        w("                    const int64_t rbase = (int64_t)rank * PQ.ev.cap;")
                        w(fifo_store(pi, 20))
                        w("                  }")
                    w("                }")
                w("              }")
                w("            }")
                w("          }")
                w("          __syncthreads();")
                w("        }")

            # ---- staging area (events of this step, in shared memory) for this group
            cs = []
            for pi in pis:
                for m, k in enumerate(PAYLOAD[pi]):
                    sz = SIZE[paths[pi]["vars"][k]["ctype"]]
                    if m >= len(cs):
                        cs.append(sz)
                    else:
                        cs[m] = max(cs[m], sz)
            group_ev_bytes.append(8 + sum(cs))
            w("        int* const st_k = (int*)(s_state + I.stage_off);          // window of the event (-1: none)")
            w("        int* const st_tgt = st_k + I.stage_cap;                     // target neuron")
            for m in range(len(cs)):
                base = "(unsigned char*)(st_tgt + I.stage_cap)" if m == 0 else f"st_col{m - 1} + (size_t){cs[m - 1]} * I.stage_cap"
                w(f"        unsigned char* const st_col{m} = {base};  // payload column {m}")
            w("        (void)st_k; (void)st_tgt;")

            def stage_store(pi, q, ind):
                p = paths[pi]
                L = [f"const int k = {koff_of(q)} + (int)PQ.odelay[syn] - PQ.dmin;",
                     "st_k[e] = k;",
                     "st_tgt[e] = PQ.post[syn];"]
                for m, k in enumerate(PAYLOAD[pi]):
                    ct = p["vars"][k]["ctype"]
                    L.append(f"*({ct}*)(st_col{m} + (size_t)e * {cs[m]}) = (({ct}*)PQ.var[{k}])[syn];")
                L.append("atomicAdd(&s_nd[k], 1);")
                return _indent("\n".join(L), ind)

            def stage_apply(pi, ind):
                """on_pre applied from staged event e (due now)."""
                p = paths[pi]
                loads, rest = split_loads(body_code(pi))
                varptr = {v["ptr"]: k for k, v in enumerate(p.get("vars", []))}
                L = []
                for ct, nm, ptr in loads:
                    if ptr == p["post_ptr"]:
                        L.append(f"const {ct} {nm} = ({ct})st_tgt[e];")
                    else:
                        m = PAYLOAD[pi].index(varptr[ptr])
                        L.append(f"const {ct} {nm} = *({ct}*)(st_col{m} + (size_t)e * {cs[m]});")
                L.append(rest)
                return _indent("\n".join(L), ind)

            def stage_to_fifo(pi, ind):
                p = paths[pi]
                L = ["PQ.ev.tgt[rbase + rec] = st_tgt[e];"]
                for m, k in enumerate(PAYLOAD[pi]):
                    ct = p["vars"][k]["ctype"]
                    L.append(f"(({ct}*)PQ.ev.pay[{m}])[rbase + rec] = *({ct}*)(st_col{m} + (size_t)e * {cs[m]});")
                return _indent("\n".join(L), ind)

            w("        // one pass when the step's events fit the staging area: every synapse is")
            w("        // read once, events without delay are applied, the others staged and counted")
            w("        if (threadIdx.x == 0) s_flag = 0;")
            w("        __syncthreads();")
            w("        int E1 = 0;")
            w("        if (I.stage_cap > 0 && NI > 0 && NI <= (int)blockDim.x) {")
            w("          const int it = threadIdx.x;")
            w("          int len = 0;")
            w("          if (it < NI) {")
            w("            int q = 0;")
            for q in range(1, L):
                w(f"            if (it >= s_qoff[{q}]) q = {q};")
            pexpr = f"{pis[L - 1]}"
            for q in reversed(range(L - 1)):
                pexpr = f"(q == {q} ? {pis[q]} : {pexpr})"
            w(f"            const b200_pathway_d& PD = I.p[{pexpr}];")
            w("            const int pos = it - s_qoff[q] + pref[PD.tile_lo];")
            w(f"            const int u = b200_upper_bound(pref, I.g[{sg}].n_tiles + 1, pos) - 1;")
            w("            const int32_t src = lst[tst[u] + pos - pref[u]];")
            w("            const int64_t sg_ = (int64_t)(src - PD.src_lo) * I.n_cta + rank;")
            w("            const int64_t lo = PD.segptr[sg_];")
            w("            len = (int)(PD.segptr[sg_ + 1] - lo);")
            w("            s_item_seg[threadIdx.x] = lo;")
            w("            s_item_q[threadIdx.x] = q;")
            w("          }")
            w("          const int eoff = b200_block_exscan(len, s_wsum, &E1);")
            w("          s_item_off[threadIdx.x] = eoff;")
            w("          __syncthreads();")
            w("          if (E1 <= I.stage_cap) {")
            w("            for (int e0 = threadIdx.x; e0 < E1; e0 += 4 * (int)blockDim.x) {")
            w("#pragma unroll")
            w("              for (int qq = 0; qq < 4; ++qq) {")
            w("                const int e = e0 + qq * (int)blockDim.x;")
            w("                if (e < E1) {")
            w("                  const int j = b200_upper_bound(s_item_off, NI, e) - 1;")
            w("                  const int64_t syn = s_item_seg[j] + (e - s_item_off[j]);")
            w("                  const int q = s_item_q[j];")
            for q, pi in enumerate(pis):
                w(("                  if" if q == 0 else "                  else if") + f" (q == {q}) {{  // {paths[pi]['name']}")
                w(f"                    if (I.p[{pi}].D == 0) {{  // no delay: applied now")
                w("                      st_k[e] = -1;")
                w("                      const int64_t _idx = syn; const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
                w(body_decls(pi, 22))
                w(_indent(body_code(pi), 22))
                w("                    } else {")
                w(f"                      const b200_pathway_d& PQ = I.p[{pi}];")
                w(stage_store(pi, q, 22))
                w("                    }")
                w("                  }")
            w("                }")
            w("              }")
            w("            }")
            w("            if (threadIdx.x == 0) s_flag = 1;")
            w("          }")
            w("          __syncthreads();")
            w("        }")
            w("        const bool staged = s_flag != 0;")
            w("        if (!staged) {")
            w("          // pass 1 over global memory: events without delay applied, the others counted")
            traverse(1)
            w("        }")
            w("        B200_PHASE(3);")
            w("        if (WT > 0) {")
            w("          // batch offsets (exclusive, per pathway) and the FIFO capacity check")
            w("          int carry = 0;")
            w("          for (int c0 = 0; c0 < WT; c0 += blockDim.x) {")
            w("            const int k = c0 + threadIdx.x;")
            w("            const int x = k < WT ? s_nd[k] : 0;")
            w("            int tot;")
            w("            const int ex = b200_block_exscan(x, s_wsum, &tot);")
            w("            if (k < WT) s_base[k] = carry + ex;")
            w("            carry += tot;")
            w("          }")
            w("          if (threadIdx.x == 0) s_base[WT] = carry;")
            w("          __syncthreads();")
            w("          // a batch that does not fit is dropped and the instance status set: every")
            w("          // CTA keeps the same barrier sequence, the host reports the error")
            w("          if (threadIdx.x == 0) {")
            for q, pi in enumerate(pis):
                w(f"            if (I.p[{pi}].D > 0) {{")
                w(f"              const long long nq = s_base[{koff_of(q)} + W{q}] - s_base[{koff_of(q)}];")
                w(f"              s_skip[{pi}] = s_step < 0 ? 1 : 0;")
                w(f"              if (s_step >= 0 && s_head[{pi}] + nq - s_tail[{pi}] > I.p[{pi}].ev.cap) {{")
                w(f"                atomicCAS(I.status, 0, B200_ERR_EVENT_OVERFLOW); s_skip[{pi}] = 1;")
                w("              }")
                w("            }")
            w("          }")
            w("          __syncthreads();")
            w("          if (s_step >= 0) {")
            for q, pi in enumerate(pis):
                w(f"            if (I.p[{pi}].D > 0) {{  // batch table entry of step s_step")
                w(f"              const int b = (int)(s_step % I.p[{pi}].ev.RB);")
                w(f"              for (int kk = threadIdx.x; kk <= W{q}; kk += blockDim.x)")
                w(f"                s_toff[{pi}][b * (W{q} + 1) + kk] = s_skip[{pi}] ? 0 : s_base[{koff_of(q)} + kk] - s_base[{koff_of(q)}];")
                w(f"              if (threadIdx.x == 0) {{ s_tbase[{pi}][b] = s_head[{pi}]; s_ttag[{pi}][b] = s_step; }}")
                w("            }")
            w("          }")
            w("          for (int k = threadIdx.x; k < WT; k += blockDim.x) s_nd[k] = 0;")
            w("          __syncthreads();")
            w("          if (staged) {")
            w("            // records from the staging area; the events due now are applied at once")
            w("            for (int e = threadIdx.x; e < E1; e += blockDim.x) {")
            w("              const int k = st_k[e];")
            w("              if (k >= 0) {")
            w(window_of("k", 16))
            for q, pi in enumerate(pis):
                w(("                if" if q == 0 else "                else if") + f" (q == {q} && !s_skip[{pi}]) {{  // {paths[pi]['name']}")
                w(body_decls(pi, 18))
                w("                  if (s_step + PQ.dmin + kk == ts) {")
                w(stage_apply(pi, 20))
                w("                  } else {")
                w(f"                    const int64_t p_ = (int64_t)(s_base[k] - s_base[{koff_of(q)}]) + atomicAdd(&s_nd[k], 1);")
                w(f"                    const int64_t rec = (s_head[{pi}] + p_) & (PQ.ev.cap - 1);")
                w("                    const int64_t rbase = (int64_t)rank * PQ.ev.cap;")
                w(stage_to_fifo(pi, 20))
                w("                  }")
                w("                }")
            w("              }")
            w("            }")
            w("            __syncthreads();")
            w("          } else {")
            w("            // pass 2 over global memory: the records, in delay order, at the FIFO head")
            traverse(2)
            w("          }")
            w("          if (threadIdx.x == 0 && s_step >= 0) {")
            for q, pi in enumerate(pis):
                w(f"            if (I.p[{pi}].D > 0 && !s_skip[{pi}]) s_head[{pi}] += s_base[{koff_of(q)} + W{q}] - s_base[{koff_of(q)}];")
            w("          }")
            w("          B200_PHASE(4);")
            w("          // delivery of the events due at ts: window (pathway, delay d) is the part")
            w("          // of the batch of step ts - d with that delay (already applied when staged)")
            w("          for (int k = threadIdx.x; k < WT; k += blockDim.x) {")
            w(window_of("k", 12))
            w("            int n = 0;")
            w("            int64_t lo = 0;")
            for q, pi in enumerate(pis):
                w(("            if" if q == 0 else "            else if") + f" (q == {q}) {{")
                w(f"              const int64_t sb = ts - (I.p[{pi}].dmin + kk);")
                w("              if (sb >= 0 && !(staged && sb == s_step)) {")
                w(f"                const int b = (int)(sb % I.p[{pi}].ev.RB);")
                w(f"                if (s_ttag[{pi}][b] == sb) {{")
                w(f"                  const int32_t* o = s_toff[{pi}] + b * (W{q} + 1);")
                w(f"                  lo = s_tbase[{pi}][b] + o[kk];")
                w("                  n = o[kk + 1] - o[kk];")
                w("                }")
                w("              }")
                w("            }")
            w("            s_nd[k] = n; s_wbase[k] = lo;")
            w("          }")
            w("          __syncthreads();")
            w("          {")
            w("            int carry2 = 0;")
            w("            for (int c0 = 0; c0 < WT; c0 += blockDim.x) {")
            w("              const int k = c0 + threadIdx.x;")
            w("              const int x = k < WT ? s_nd[k] : 0;")
            w("              int tot;")
            w("              const int ex = b200_block_exscan(x, s_wsum, &tot);")
            w("              if (k < WT) s_ndoff[k] = carry2 + ex;")
            w("              carry2 += tot;")
            w("            }")
            w("            if (threadIdx.x == 0) s_ndoff[WT] = carry2;")
            w("            __syncthreads();")
            w("          }")
            w("          const int ED = s_ndoff[WT];")
            w("          for (int e0 = threadIdx.x; e0 < ED; e0 += 4 * (int)blockDim.x) {")
            w("#pragma unroll")
            w("            for (int qq = 0; qq < 4; ++qq) {")
            w("              const int e = e0 + qq * (int)blockDim.x;")
            w("              if (e < ED) {")
            w("                const int k = b200_upper_bound(s_ndoff, WT + 1, e) - 1;")
            w(window_of("k", 16))
            w("                (void)kk;")
            for q, pi in enumerate(pis):
                w(("                if" if q == 0 else "                else if") + f" (q == {q}) {{  // {paths[pi]['name']}")
                w(body_decls(pi, 18))
                w("                  const int64_t rbase = (int64_t)rank * PQ.ev.cap;")
                w("                  const int64_t rec = (s_wbase[k] + (e - s_ndoff[k])) & (PQ.ev.cap - 1);")
                w(fifo_body(pi, 18))
                w("                }")
            w("              }")
            w("            }")
            w("          }")
            w("          __syncthreads();")
            w("          // retire the batches whose largest delay was due now")
            w("          if (threadIdx.x == 0) {")
            for q, pi in enumerate(pis):
                w(f"            if (I.p[{pi}].D > 0) {{")
                w(f"              const int64_t sb = ts - I.p[{pi}].D;")
                w("              if (sb >= 0) {")
                w(f"                const int b = (int)(sb % I.p[{pi}].ev.RB);")
                w(f"                if (s_ttag[{pi}][b] == sb) s_tail[{pi}] = s_tbase[{pi}][b] + s_toff[{pi}][b * (W{q} + 1) + W{q}];")
                w("              }")
                w("            }")
            w("          }")
            w("          __syncthreads();")
            w("        }")
            w("      }")
            w("      B200_PHASE(5);")
        w("    }  // steps")
        w(f"    if (prof && threadIdx.x == 0)")
        w(f"      for (int q = 0; q < {NPH}; ++q) atomicAdd(&prof[(size_t)unit * {NPH} + q], _pacc[q]);")
        w("#undef B200_PHASE")
        w("    // the last step's arrival: wait for it, then record its spikes in the monitors")
        w("    if (pend) {")
        w("      if (!b200_owner_wait(I, ts - 1, limit_ns, cluster)) ok = false;")
        w("      else {")
        w("        const int64_t s_step = ts - 1;")
        emit_lists("s_step", "true", 8)
        w("      }")
        w("    }")
        w("    if (ok && ts > ts0) {")
        w("      const double _b200_t = (double)(ts - 1) * _b200_dt; (void)_b200_t;")
        w("      const int64_t _b200_ts = ts - 1;")
        for gi in range(NG):
            rb = deferred_block(gi, 6, "ts - 1", True)
            if rb:
                w(rb)
        w("    }")
        w("    __syncthreads();")
        w("    if (s_cache) {")
        for gi, g in enumerate(groups):
            for k in USED[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"      b200_copy_bytes((char*)I.g[{gi}].var[{k}] + (size_t)s_own[{gi}][0] * {sz}, (const char*)s_gv[{gi}][{k}] + (size_t)s_own[{gi}][0] * {sz},")
                w(f"                      (size_t)(s_own[{gi}][1] - s_own[{gi}][0]) * {sz});")
        w("    }")
        w("    if (I.tab_smem) {")
        for pi in range(NP):
            w(f"      if (I.p[{pi}].D > 0) {{")
            w(f"        const b200_fifo_d& F = I.p[{pi}].ev;")
            w(f"        b200_copy_bytes(F.off + (size_t)rank * F.RB * (F.W + 1), s_toff[{pi}], (size_t)F.RB * (F.W + 1) * 4);")
            w(f"        b200_copy_bytes(F.base + (size_t)rank * F.RB, s_tbase[{pi}], (size_t)F.RB * 8);")
            w(f"        b200_copy_bytes(F.tag + (size_t)rank * F.RB, s_ttag[{pi}], (size_t)F.RB * 8);")
            w("      }")
        w("    }")
        w("    if (threadIdx.x == 0) {")
        for pi in range(NP):
            w(f"      if (I.p[{pi}].D > 0) {{ I.p[{pi}].ev.state[2 * rank] = s_head[{pi}]; I.p[{pi}].ev.state[2 * rank + 1] = s_tail[{pi}]; }}")
        w("      if (rank == 0) {")
        w("        *I.ts_done = ts;")
        for gi, g in enumerate(groups):
            if g.get("generator"):
                w(f"        *I.g[{gi}].gen_last = s_glast[{gi}];")
        for m in range(len(spkmons)):
            w(f"        *I.sm[{m}].n = s_mon_n[{m}];")
        for m in range(len(statemons)):
            w(f"        *I.stm[{m}].n = s_stm_n[{m}];")
        w("      }")
        w("    }")
        w("    __syncthreads();")
        w("  }")
        w("}")
        w("")

    group_ev_bytes = []
    if OWNER:
        emit_owner_kernel()
    OWNER_EV_BYTES = max(group_ev_bytes) if group_ev_bytes else 8

    # ------------------------------------------------------------- launch glue
    w("// `tcode` = threads | (min CTAs per SM - 1) << 16: the (512, 2) variant caps")
    w("// registers so that two CTAs fit on an SM (sweeps with more instances than SMs)")
    w("static const void* b200_kernel_for(int tcode) {")
    w("  const int threads = tcode & 0xffff, minb = ((tcode >> 16) & 0xf) + 1;")
    if OWNER:
        w("  if (tcode & B200_TCODE_OWNER) {  // owner mode: one CTA per SM")
        w("    if (threads <= 256) return (const void*)b200_owner_kernel<256, 1>;")
        w("    if (threads <= 512) return (const void*)b200_owner_kernel<512, 1>;")
        w("    return (const void*)b200_owner_kernel<1024, 1>;")
        w("  }")
    w("  if (threads <= 256) return minb >= 2 ? (const void*)b200_step_kernel<256, 2> : (const void*)b200_step_kernel<256, 1>;")
    w("  if (threads <= 512) return minb >= 2 ? (const void*)b200_step_kernel<512, 2> : (const void*)b200_step_kernel<512, 1>;")
    w("  return (const void*)b200_step_kernel<1024, 1>;")
    w("}")
    w("static size_t b200_smem_for(int tcode, int max_tiles1, int max_w, int state_bytes) {")
    w("  const int threads = tcode & 0xffff;")
    if OWNER:
        w("  if (tcode & B200_TCODE_OWNER) return b200_dyn_smem_owner(threads, max_tiles1, max_w, state_bytes);")
    w("  return b200_dyn_smem(threads, max_tiles1, max_w, state_bytes);")
    w("}")
    w("static int b200_max_active(int tcode, int max_tiles1, int max_w, int state_bytes) {")
    w("  const void* k = b200_kernel_for(tcode);")
    w("  const int threads = tcode & 0xffff;")
    w("  const size_t smem = b200_smem_for(tcode, max_tiles1, max_w, state_bytes);")
    w("  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;")
    w("  int n = 0;")
    w("  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, threads, smem) != cudaSuccess) return 0;")
    w("  return n;")
    w("}")
    w("static int b200_static_smem(int tcode) {")
    w("  cudaFuncAttributes a;")
    w("  if (cudaFuncGetAttributes(&a, b200_kernel_for(tcode)) != cudaSuccess) return 64 * 1024;")
    w("  return (int)a.sharedSizeBytes;")
    w("}")
    w("static cudaError_t b200_launch(b200_inst_d* insts, const int2* cta_map, int n_inst, int queue_mode,")
    w("                               int* work, int64_t max_steps, uint64_t limit_ns, int grid, int tcode,")
    w("                               int cooperative, int max_tiles1, int max_w, int fault_rank, int state_bytes,")
    w("                               unsigned long long* prof, int cluster, cudaStream_t s) {")
    w("  const void* k = b200_kernel_for(tcode);")
    w("  const int threads = tcode & 0xffff;")
    w("  const size_t smem = b200_smem_for(tcode, max_tiles1, max_w, state_bytes);")
    w("  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);")
    w("  if (e != cudaSuccess) return e;")
    w("  const b200_inst_d* ci = insts;")
    w("  void* args[] = {(void*)&ci, (void*)&cta_map, (void*)&n_inst, (void*)&queue_mode, (void*)&work,")
    w("                  (void*)&max_steps, (void*)&limit_ns, (void*)&max_tiles1, (void*)&max_w, (void*)&fault_rank,")
    w("                  (void*)&state_bytes, (void*)&prof, (void*)&cluster};")
    w("  if (cluster > 1) {  // one thread-block cluster per instance")
    w("    if (cluster > 8) {")
    w("      e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);")
    w("      if (e != cudaSuccess) return e;")
    w("    }")
    w("    cudaLaunchConfig_t cfg = {};")
    w("    cfg.gridDim = dim3(grid); cfg.blockDim = dim3(threads); cfg.dynamicSmemBytes = smem; cfg.stream = s;")
    w("    cudaLaunchAttribute at[1];")
    w("    at[0].id = cudaLaunchAttributeClusterDimension;")
    w("    at[0].val.clusterDim.x = cluster; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;")
    w("    cfg.attrs = at; cfg.numAttrs = 1;")
    w("    return cudaLaunchKernelExC(&cfg, k, args);")
    w("  }")
    w("  if (cooperative) return cudaLaunchCooperativeKernel(k, dim3(grid), dim3(threads), args, smem, s);")
    w("  return cudaLaunchKernel(k, dim3(grid), dim3(threads), args, smem, s);")
    w("}")
    w("static int b200_max_cluster(int tcode, int max_tiles1, int max_w, int state_bytes, int cluster) {")
    w("  const void* k = b200_kernel_for(tcode);")
    w("  const int threads = tcode & 0xffff;")
    w("  const size_t smem = b200_smem_for(tcode, max_tiles1, max_w, state_bytes);")
    w("  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;")
    w("  if (cluster > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return 0;")
    w("  cudaLaunchConfig_t cfg = {};")
    w("  cfg.gridDim = dim3(cluster); cfg.blockDim = dim3(threads); cfg.dynamicSmemBytes = smem;")
    w("  cudaLaunchAttribute at[1];")
    w("  at[0].id = cudaLaunchAttributeClusterDimension;")
    w("  at[0].val.clusterDim.x = cluster; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;")
    w("  cfg.attrs = at; cfg.numAttrs = 1;")
    w("  int n = 0;")
    w("  if (cudaOccupancyMaxPotentialClusterSize(&n, k, &cfg) != cudaSuccess) return 0;")
    w("  return n;")
    w("}")
    w("")
    if DRAWS:
        kinds = {"rand": "B200_DRAW_UNIFORM", "randn": "B200_DRAW_NORMAL", "binomial": "B200_DRAW_BINOMIAL",
                 "binormal": "B200_DRAW_BINORMAL"}
        rows = []
        for d in DRAWS:
            bn = d.get("binom") or {}
            rows.append(f'{{"{d["name"]}", {kinds[d["kind"]]}, {d["group"]}, {d["lo"]}, {d["hi"]}, {d["calls"]}, '
                        f'{bn.get("n", 0)}, {1 if bn.get("reverse") else 0}, {bn.get("qn", "0.0")}, {bn.get("bound", "0.0")}, '
                        f'{bn.get("p", "0.0")}, {bn.get("q", "0.0")}, {bn.get("scale", "0.0")}, {bn.get("loc", "0.0")}}}')
        w("static const b200_draw_info b200_draws[] = {" + ", ".join(rows) + "};")
    if SUMMED:
        w("static const b200_summed_info b200_summed[] = {" + ", ".join(
            f'{{"{sm["name"]}", {sm["pathway"]}, {sm["tgt_group"]}, {sm["tgt_var"]}, {1 if sm["index_post"] else 0}}}'
            for sm in SUMMED) + "};")
    w(f'static const b200_model_info B200_MODEL = {{"{spec["name"]}", {NG}, {NP}, {len(spkmons)}, {len(ratemons)}, {len(statemons)},')
    w("  b200_groups, b200_pathways, b200_spkmon, b200_ratemon, b200_statemon,")
    w(f"  {len(consts)}, b200_const_names, b200_const_defaults, b200_eval_scalars, b200_launch, b200_max_active,")
    w(f"  b200_static_smem, b200_max_cluster, {NPH}, {1 if OWNER else 0}, {OWNER_EV_BYTES},")
    w(f"  {len(SUMMED)}, {'b200_summed' if SUMMED else 'nullptr'}, {len(DRAWS)}, {'b200_draws' if DRAWS else 'nullptr'}}};")
    w("")
    w('#include "b200_host.h"')
    w("")
    return "\n".join(o) + "\n"


def delivery_passes(paths) -> list:
    """The classic kernel's delivery passes: (source group, [pathway indices],
    touched pointers).  Consecutive pathways from one source whose on_pre code
    touches disjoint neuron and synaptic variables share a pass (running them
    interleaved cannot change what any of them reads); a pass's events are
    profiled in the slot of its first pathway."""
    merged = []
    for pi, p in enumerate(paths):
        if not p.get("events", True):
            continue  # the synapses of a Synapses object without a delivering pathway
        # neuron variables and synaptic variables (shared by the pathways of one
        # Synapses object): pathways touching the same ones are not interleaved
        touched = set(p.get("group_ptrs", {})) | {v["ptr"] for v in p.get("vars", [])}
        last = merged[-1] if merged else None
        if last and last[0] == p["src"] and not (last[2] & touched):
            last[1].append(pi)
            last[2].update(touched)
        else:
            merged.append((p["src"], [pi], set(touched)))
    return merged


def profile_slots(spec: dict, owner: bool = False) -> list[str]:
    """Names of the device profile's slots (b200_get_profile), in order.
    Owner-mode kernel: update (update, threshold and reset of every group),
    barrier, spike lists, push counts, push into the event FIFOs, delivery.
    Classic kernel: the rest of the update phase, barrier A, the rest of the
    spike-list phase, one slot per pathway for its events, barrier B,
    delivery windows, delivery items; per group its update (with the threshold
    condition), its spike list (threshold), its reset; per group the copy of
    its spikes into the delay ring; one slot per spike and per rate monitor."""
    groups = spec["groups"]
    paths = spec.get("pathways", [])
    if owner:
        names = ["update_threshold_reset", "barrier", "spike_lists_monitors", "push_count", "push_fifo", "deliver"]
    else:
        names = ["other", "barrier_a", "lists_other"] + [f"events:{p['name']}" for p in paths] + \
                ["barrier_b", "delay_windows", "items"]
    n = 6 + len(paths) + 4 * len(groups) + len(spec.get("spike_monitors", [])) + len(spec.get("rate_monitors", []))
    if not owner:
        for g in groups:
            names += [f"update:{g['name']}", f"threshold:{g['name']}", f"reset:{g['name']}"]
        names += [f"ring:{g['name']}" for g in groups]
        names += [f"spikemon:{m['name']}" for m in spec.get("spike_monitors", [])]
        names += [f"ratemon:{m['name']}" for m in spec.get("rate_monitors", [])]
    names += [f"unused{k}" for k in range(len(names), n)]
    return names


def spec_tables(spec: dict) -> dict:
    """Variable tables the Python host uses to address arrays by name."""
    return {
        "groups": [[v["name"] for v in g["vars"]] for g in spec["groups"]],
        "group_kinds": [[CTYPE_KIND[v["ctype"]] for v in g["vars"]] for g in spec["groups"]],
        "pathways": [[v["name"] for v in p.get("vars", [])] for p in spec.get("pathways", [])],
        "pathway_kinds": [[CTYPE_KIND[v["ctype"]] for v in p.get("vars", [])] for p in spec.get("pathways", [])],
        "consts": [c["name"] for c in spec.get("consts", [])],
    }
