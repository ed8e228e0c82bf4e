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
PF_WORDS_PUSH = 12
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
    # push mode: owner mode's condition, and every group keeps its own spike lists
    # (no spike generator, no custom-event group), so that each CTA can deliver
    # its own neurons' spikes; ACC: the neuron variables that receive deliveries
    PUSH = OWNER and NP > 0 and not any(g.get("generator") or g.get("alias_of") is not None for g in groups)
    ACC = sorted({(gi, vi) for p in paths for _, (gi, vi) in p.get("group_ptrs", {}).items() if gi == p["tgt"]})
    if len(ACC) > 8:
        PUSH = False
    ACCI_ = {gv: k for k, gv in enumerate(ACC)}

    def _fusable(gi, vi):
        """A delivered variable whose deliveries can be added as the update
        loads it: the update reads it, and nothing that runs between the
        deliveries and the update (inputs, resets, operations, state monitors)
        names it, so adding them later changes no value that anything reads."""
        g = groups[gi]
        ptr = g["vars"][vi]["ptr"]
        if not g.get("update") or g["update"].get("vector") is None:
            return False
        if ptr not in {p_ for _, _, p_ in split_loads(g["update"]["vector"])[0]}:
            return False
        # (the code itself, not its JSON form: there a line break is the two
        # characters \\n, and a pointer starting a line would have no word boundary)
        codes = [(g.get("reset") or {}).get(k) or "" for k in ("scalar", "vector")]
        codes += [op["code"].get(k) or "" for op in g.get("ops", []) for k in ("scalar", "vector")]
        codes += [inp["code"].get(k) or "" for inp in INPUTS if inp["group"] == gi for k in ("scalar", "vector")]
        if any(re.search(r"(?<![A-Za-z0-9_])%s(?![A-Za-z0-9_])" % re.escape(ptr), c) for c in codes):
            return False
        if any(m["group"] == gi for m in statemons):
            return False  # (its recorded variables are chosen at run time)
        return True

    FUSED = {gv for gv in ACC if PUSH and _fusable(*gv)}

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

    def reset_block(gi, indent, tsexpr, owner=False, push=False):
        """Reset of the spikes of step `tsexpr` in this CTA's tiles (push: from
        the CTA's compact spike history)."""
        tab, blocks = gtables[gi]
        bd = dict(blocks)
        if bd["reset"] is None:
            return ""
        g = groups[gi]
        if push:
            L = ["{",
                 f"  const double _b200_t = (double)({tsexpr}) * _b200_dt; (void)_b200_t;  // the step of the reset",
                 f"  const int64_t _b200_ts = {tsexpr}; (void)_b200_ts;",
                 f"  const int _rsl = (int)(({tsexpr}) % I.g[{gi}].RH), _rcnt = s_hcnt[{gi}][_rsl], _rhc = I.g[{gi}].HCAP;",
                 f"  const int32_t* const _rhs = s_hist[{gi}] + _rsl * _rhc;",
                 f"  const int32_t* const _rhg = I.g[{gi}].hist + (int64_t)_rsl * I.g[{gi}].N + s_own[{gi}][0];",
                 f"  const int32_t N = I.g[{gi}].N; (void)N;",
                 f"  const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;",
                 gptr_decls(gi, 2, False),
                 "  for (int j = threadIdx.x; j < _rcnt; j += blockDim.x) {",
                 "    const int32_t _idx = j < _rhc ? _rhs[j] : _rhg[j];",
                 "    const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;",
                 "    {",
                 _indent(tab.device_loads("reset", f32), 6),
                 _indent(_device(tab.time_code("reset")), 6),
                 extra_ptrs(g.get("reset"), 6),
                 _indent(bd["reset"]["vector"], 6),
                 "    }",
                 "  }",
                 "}"]
            return _indent("\n".join(L), indent)
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

    def deferred_block(gi, indent, tsexpr, owner=False, push=False):
        """What the reference runs after the deliveries of step `tsexpr`: the
        Poisson inputs, the reset, the end-slot operations and state monitors
        (this CTA's neurons)."""
        if ALIAS[gi] is not None:
            return ""  # (its reset runs in its parent's block)
        resets = [reset_block(k, indent, tsexpr, owner, push) for k in (groups[gi].get("reset_order") or [gi])]
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

    def emit_phase_a(owner, push=False, only=None):
        """Reset of the previous step, state monitors, update + threshold with
        ordered compaction of this CTA's tiles.  `push`: the step's spikes are
        also appended to the CTA's compact spike history (shared memory for the
        first HCAP of the slot, global memory for all)."""
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
            if only is not None and gi not in only:
                continue
            tab, blocks = gtables[gi]
            bd = dict(blocks)
            if g.get("generator"):
                emit_generator(gi, owner)
                continue
            w(f"      // ---- group {gi} '{g['name']}': phase A (reset of step ts-1, monitors, update + threshold)")
            dfr = deferred_block(gi, 8, "ts - 1", owner, push)
            if not owner:
                w("      B200_PHASE(0);")
            if dfr and not SUMMED:  # (with summed variables: before the sums)
                w("      if (ts > ts0) {")
                w(dfr)
                w("        __syncthreads();")
                w("      }")
                if not owner or push:
                    w(f"      B200_PHASE({PH_RST(gi)});  // reset of the previous step")
            sop = op_block(gi, 6, "ts", "start")
            if sop and not SUMMED:  # the start-slot operations of this step
                w(sop)
                w("      __syncthreads();")
            w("      {")
            w(f"        const int32_t N = I.g[{gi}].N; (void)N;")
            w(f"        const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;")
            w(gptr_decls(gi, 8, True))
            if push:
                pass  # (the step's list goes to the compact history only)
            elif owner:
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
            if push:
                w("        int _hrun = 0;  // spikes of this CTA's earlier tiles this step")
                w(f"        const int _hslot = _hs{gi}, _hcap = I.g[{gi}].HCAP;")
                w(f"        int32_t* const _hsh = s_hist[{gi}] + _hslot * _hcap;")
                w(f"        int32_t* const _hgl = I.g[{gi}].hist + (int64_t)_hslot * I.g[{gi}].N + s_own[{gi}][0];")
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
            # push mode: the deliveries due at ts-1 of a fused variable are added as
            # the update loads it (buffer (ts-1) % 3; cleared in the compute loop,
            # since a store right behind the load of the same word would wait for it)
            fz = {v["ptr"]: ACCI_[(gi, k)] for k, v in enumerate(g["vars"])
                  if v["ptr"] in pf and (gi, k) in FUSED} if push else {}
            for ptr, a in fz.items():
                w(f"            {pf[ptr]}* const _facc{pfi[ptr]} = ({pf[ptr]}*)I.acc[{a}] + (size_t)((ts + 2) % B200_PUSH_BUFS) * I.g[{gi}].N;")

            words = sum(max(1, SIZE.get(ct, 8) // 4) for ct in pf.values())
            # 16 words of loads in flight per thread in the variants capped at 64
            # registers, PF_WORDS in the others
            pf_small = max(1, min(4, 16 // max(words, 1)))
            # (push mode with folded deliveries: the loads of more slices at once, the
            # deliveries' loads going to L2)
            pf_big = max(1, min(32, (PF_WORDS_PUSH if fz else PF_WORDS) // max(words, 1)))
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
                if ptr in fz:
                    w(f"                  _pf{j}[kq] = {ptr}[_idx] + __ldcg(_facc{j} + _idx);")
                else:
                    w(f"                  _pf{j}[kq] = {ptr}[_idx];")
            w("                }")
            w("              }")
            w("#pragma unroll")
            w("              for (int kq = 0; kq < PF; ++kq) {")
            w("              const int k = k0 + kq;")
            w("              const int32_t _idx = pb + k * (int)blockDim.x + threadIdx.x;")
            w("              if (k < E && _idx < pe) {")
            w("                const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            for ptr in fz:
                w(f"                __stcg(_facc{pfi[ptr]} + _idx, ({pf[ptr]})0);")
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
            if not owner or push:
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
            if not push:
                w("                  scr[_p] = _sn;")
            if not owner:
                w("                  oscr[_p] = _sn;  // this CTA's copy")
            if push:
                w("                  const int _h = _hrun + _p - start;  // position in the CTA's compact list")
                w("                  if (_h < _hcap) _hsh[_h] = _sn;")
                w("                  _hgl[_h] = _sn;")
            sc = snap_code(gi, "_sn")
            if sc:
                w("                  " + sc)
            w("                }")
            w("            }")
            w("            cnt += tot;")
            w("            __syncthreads();")
            if not owner or push:
                w(f"            B200_PHASE({PH_THR(gi)});  // spike list (threshold)")
            w("          }")
            if not push:
                w("          if (threadIdx.x == 0) tcnt[u] = cnt;" if owner else "          if (threadIdx.x == 0) { tcnt[u] = cnt; otc[u] = cnt; }")
            if push:
                w("          _hrun += cnt;")
            w("        }")
            if push:
                w("        if (threadIdx.x == 0) {")
                w(f"          s_hcnt[{gi}][_hslot] = _hrun;")
                w(f"          I.g[{gi}].hcnt[(int64_t)_hslot * I.n_cta + rank] = _hrun;")
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
                    w(sp + "        atomicAdd(&SM.count[idx - SM.lo], 1);  // (no read round trip)")
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


    def lean_ok(gi):
        """Push mode's lean phase A applies to group gi: no random draws in its
        update or threshold, no start-slot state monitors (the generic phase A
        handles those)."""
        g = groups[gi]
        if g.get("generator") or ALIAS[gi] is not None or not g.get("update") or not g.get("threshold"):
            return False
        for blk in ("update", "threshold"):
            if g[blk].get("draw") is not None:
                return False
        return not any(m["group"] == gi and m.get("when", "start") == "start" for m in statemons)

    def emit_lean_phase_a(gi):
        """Push mode, group gi: the reset of step ts-1 and the start-slot
        operations as in the generic phase A, then the update and threshold of
        this CTA's neurons with each warp on a contiguous run of them (32 per
        iteration, PFL iterations' loads issued at once), the deliveries of a
        folded variable added as it is loaded, the spikes appended to a per-warp
        list in neuron order, and one block scan placing the lists into the
        CTA's spike history.  Cached state is addressed through pointers derived
        from the dynamic shared memory, so its accesses are shared-memory ones."""
        g = groups[gi]
        tab, blocks = gtables[gi]
        bd = dict(blocks)
        w(f"      // ---- group {gi} '{g['name']}': push phase A")
        dfr = deferred_block(gi, 8, "ts - 1", True, True)
        if dfr:
            w("      if (ts > ts0) {")
            w(dfr)
            w("        __syncthreads();")
            w("      }")
            w(f"      B200_PHASE({PH_RST(gi)});  // reset of the previous step")
        sop = op_block(gi, 6, "ts", "start")
        if sop:
            w(sop)
            w("      __syncthreads();")
        upd_v = bd["update"]["vector"]
        thr_v = bd["threshold"]["vector"]
        upd_loads, upd_rest = split_loads(upd_v)
        thr_loads, thr_rest = split_loads(thr_v)
        upd_st = stored_ptrs(upd_v)
        pf = {}
        for ct, nm, ptr in upd_loads + [x for x in thr_loads if x[2] not in upd_st]:
            pf.setdefault(ptr, ct)
        pfi = {ptr: j for j, ptr in enumerate(pf)}
        words = sum(max(1, SIZE.get(ct, 8) // 4) for ct in pf.values())
        fz = {v["ptr"]: ACCI_[(gi, k)] for k, v in enumerate(g["vars"]) if v["ptr"] in pf and (gi, k) in FUSED}
        upd_sc = {nm for _, nm in scalar_outputs(bd["update"]["scalar"])}
        thr_sc = {nm for _, nm in scalar_outputs(bd["threshold"]["scalar"])}
        hoist_sc = not (upd_sc & thr_sc)

        def body(cached):
            """Slices of 32 consecutive neurons per warp (conflict-free shared
            memory, coalesced global memory); the deliveries of NS slices are
            loaded before any slice is computed (one L2 round trip per chunk)."""
            L = []
            if cached:
                # the cache's pointers as offsets from the dynamic shared memory base
                for k, v in enumerate(g["vars"]):
                    if k in USED[gi]:
                        L.append(f"{v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)(b200_dyn + ((const unsigned char*)s_gv[{gi}][{k}] - b200_dyn)); (void){v['ptr']};")
                    else:
                        L.append(f"{v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)s_gv[{gi}][{k}]; (void){v['ptr']};")
            else:
                L.append(gptr_decls(gi, 0, True))
            for ptr, a in fz.items():
                L.append(f"{pf[ptr]}* const _facc{pfi[ptr]} = ({pf[ptr]}*)I.acc[{a}] + (size_t)((ts + 2) % B200_PUSH_BUFS) * I.g[{gi}].N;")
            # (8: no register spills at 128 registers a thread, whose L1 traffic cost more
            # than the second round trip of a longer run)
            L.append("constexpr int NS = (MAXT * MINB < 1024) ? 8 : 4;  // slices per chunk")
            L.append("for (int _c0 = _a; _c0 < _b; _c0 += 32 * NS) {")
            for ptr in fz:
                L.append(f"  {pf[ptr]} _d{pfi[ptr]}[NS];")
            if fz:
                L.append("#pragma unroll")
                L.append("  for (int _s = 0; _s < NS; ++_s) {")
                L.append("    const int32_t _idx = _c0 + _s * 32 + lane;")
                for ptr in fz:
                    j = pfi[ptr]
                    L.append(f"    _d{j}[_s] = _idx < _b ? __ldcg(_facc{j} + _idx) : ({pf[ptr]})0;")
                L.append("  }")
            L.append("#pragma unroll")
            L.append("  for (int _s = 0; _s < NS; ++_s) {")
            L.append("    const int32_t _idx = _c0 + _s * 32 + lane;")
            L.append("    bool _sp = false;")
            L.append("    if (_idx < _b) {")
            L.append("      const int32_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
            for ptr, j in pfi.items():
                if ptr in fz:
                    L.append(f"      const {pf[ptr]} _pf{j} = {ptr}[_idx] + _d{j}[_s];")
                else:
                    L.append(f"      const {pf[ptr]} _pf{j} = {ptr}[_idx];")
            L.append("      {")
            if not hoist_sc:
                L.append(_indent(tab.scalar_loads("update", f32), 8))
                L.append(_indent(_device(tab.time_code("update")), 8))
            L.append(extra_ptrs(g.get("update"), 8))
            for ct, nm, ptr in upd_loads:
                L.append(f"        {ct} {nm} = _pf{pfi[ptr]};")
            L.append(_indent(upd_rest, 8))
            L.append("      }")
            L.append("      {")
            if not hoist_sc:
                L.append(_indent(tab.scalar_loads("threshold", f32), 8))
                L.append(_indent(_device(tab.time_code("threshold")), 8))
            L.append(extra_ptrs(g.get("threshold"), 8))
            for ct, nm, ptr in thr_loads:
                L.append(f"        {ct} {nm} = " + (f"_pf{pfi[ptr]};" if ptr not in upd_st else f"{ptr}[_idx];"))
            L.append(_indent(thr_rest, 8))
            L.append("        _sp = _cond;")
            if bd["threshold"].get("refractory"):
                nr = next(v["ptr"] for v in g["vars"] if v["name"] == "not_refractory")
                ls = next(v["ptr"] for v in g["vars"] if v["name"] == "lastspike")
                L.append("        if (_cond) {")
                L.append(f"          {nr}[_idx] = false;")
                L.append(f"          {ls}[_idx] = _b200_t;")
                L.append("        }")
            sc = snap_code(gi, "_idx")
            if sc:
                L.append("        if (_cond) { " + sc + " }")
            L.append("      }")
            L.append("    }")
            L.append("    const unsigned _m = __ballot_sync(0xffffffffu, _sp);")
            L.append("    if (_sp) _wl[_wcnt + __popc(_m & b200_lanemask_lt())] = _idx;")
            L.append("    _wcnt += __popc(_m);")
            L.append("  }")
            if fz:
                L.append("  {  // the chunk's folded deliveries cleared (16-byte stores where aligned)")
                L.append("    const int _z0 = _c0, _z1 = (_c0 + 32 * NS < _b) ? _c0 + 32 * NS : _b;")
                for ptr in fz:
                    j = pfi[ptr]
                    ct = pf[ptr]
                    L.append("    {")
                    L.append(f"      {ct}* const _z = _facc{j};")
                    if SIZE[ct] == 4:
                        L.append("      const int _n4 = ((((uintptr_t)(_z + _z0)) & 15) == 0) ? (_z1 - _z0) >> 2 : 0;")
                        L.append("      for (int _q = lane; _q < _n4; _q += 32) __stcg((float4*)(_z + _z0) + _q, make_float4(0.f, 0.f, 0.f, 0.f));")
                        L.append(f"      for (int _i = _z0 + 4 * _n4 + lane; _i < _z1; _i += 32) __stcg(_z + _i, ({ct})0);")
                    else:
                        L.append(f"      for (int _i = _z0 + lane; _i < _z1; _i += 32) __stcg(_z + _i, ({ct})0);")
                    L.append("    }")
                L.append("  }")
            L.append("}")
            return _indent("\n".join(L), 10)

        w("      {")
        w(f"        const int32_t N = I.g[{gi}].N; (void)N;")
        w(f"        const double* const _b200_S = s_Sg{gi}; const float* const _b200_Sf = s_Sg{gi}f; const long long* const _b200_Si = s_Sg{gi}i;")
        w("        (void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
        w(_indent(tab.const_loads(f32), 8))
        if hoist_sc:
            for blk_name in ("update", "threshold"):
                w(_indent(tab.scalar_loads(blk_name, f32), 8))
                w(_indent(_device(tab.time_code(blk_name)), 8))
        w(f"        const int _o0 = s_own[{gi}][0], _o1 = s_own[{gi}][1], _on = _o1 - _o0;")
        w("        const int _pw = (((_on + NW - 1) / NW) + 31) & ~31;  // neurons per warp")
        w("        const int _a = _o0 + wid * _pw, _b = (_a + _pw < _o1) ? _a + _pw : _o1;")
        w(f"        int32_t* const _wl = (int32_t*)(b200_dyn + I.g[{gi}].own_off) + wid * _pw;  // this warp's spikes")
        w("        int _wcnt = 0;")
        w("        if (s_cache) {")
        w(body(True))
        w("        } else {")
        w(body(False))
        w("        }")
        w(f"        B200_PHASE({PH_UPD(gi)});  // update + threshold condition")
        w("        int _tot;")
        w("        const int _wb = b200_block_exscan(lane == 0 ? _wcnt : 0, s_wsum, &_tot);")
        w("        const int _base = __shfl_sync(0xffffffffu, _wb, 0);")
        w(f"        const int _hslot = _hs{gi}, _hcap = I.g[{gi}].HCAP;")
        w(f"        int32_t* const _hsh = s_hist[{gi}] + _hslot * _hcap;")
        w(f"        int32_t* const _hgl = I.g[{gi}].hist + (int64_t)_hslot * I.g[{gi}].N + _o0;")
        w("        for (int j = lane; j < _wcnt; j += 32) {")
        w("          const int _h = _base + j;")
        w("          const int32_t _sn = _wl[j];")
        w("          if (_h < _hcap) _hsh[_h] = _sn;")
        w("          _hgl[_h] = _sn;")
        w("        }")
        w("        if (threadIdx.x == 0) {")
        w(f"          s_hcnt[{gi}][_hslot] = _tot;")
        w(f"          I.g[{gi}].hcnt[(int64_t)_hslot * I.n_cta + rank] = _tot;")
        w("        }")
        w(f"        B200_PHASE({PH_THR(gi)});  // spike list (threshold)")
        w("      }")

    def emit_push_kernel():
        """Push mode: each CTA owns the neurons of its tiles (their state lives in
        its shared memory for the launch) and delivers its own neurons' spikes.
        Every delay is >= 1 step, so the events due at step ts+1 come from spikes
        of steps <= ts: after arriving at step ts's barrier a CTA gathers them and
        adds them into accumulator buffer (ts+1) % 3 of each delivered variable;
        after the barrier of step ts+1 each owner adds buffer (ts+1) % 3 of its
        neurons to their state and clears it.  Three buffers, because a CTA
        starts the deliveries due at ts+2 before the slowest CTA has cleared the
        buffer of the deliveries due at ts.  A step is: wait for step ts-1 ->
        fold -> phase A (as the owner kernel: deferred reset, operations, state
        monitors, update, threshold) -> spike bounds and monitor counts of step
        ts -> arrive -> monitors of step ts-1 -> deliveries due at ts+1.  The
        only change against the reference's order is the order of the additions
        into a variable (the deliveries of a step are summed before they reach it)."""
        ACCI = {gv: k for k, gv in enumerate(ACC)}
        NSM_, NRM_ = len(spkmons), len(ratemons)
        # monitors of step ts-1 written after step ts's arrival (their counts, loaded
        # after the barrier, have arrived by then) unless a spike monitor records
        # variables: their per-neuron snapshot of step ts-1 is overwritten by step
        # ts's thresholder
        LATE = not any(m.get("vars") for m in spkmons)

        def pathway_window(kexpr, ind):
            """q (pathway index) and kk (delay index) of delivery window k."""
            out = [f"int q = 0, kk = {kexpr};"]
            for q in range(1, NP):
                out.append(f"if (q == {q - 1} && kk >= W{q - 1}) {{ kk -= W{q - 1}; q = {q}; }}")
            return _indent("\n".join(out), ind)

        def qsel(qexpr, attr):
            """I.p[q].attr for a runtime pathway index (small if-chain)."""
            e = f"I.p[{NP - 1}].{attr}"
            for q in reversed(range(NP - 1)):
                e = f"(({qexpr}) == {q} ? I.p[{q}].{attr} : {e})"
            return e

        def list_elem(gexpr, slot, k):
            return (f"(({k}) < I.g[{gexpr}].HCAP ? s_hist[{gexpr}][({slot}) * I.g[{gexpr}].HCAP + ({k})] : "
                    f"I.g[{gexpr}].hist[(int64_t)({slot}) * I.g[{gexpr}].N + s_own[{gexpr}][0] + ({k})])")

        # the pathways' source groups, as a runtime expression of q
        def src_of(qexpr):
            e = f"{paths[NP - 1]['src']}"
            for q in reversed(range(NP - 1)):
                e = f"(({qexpr}) == {q} ? {paths[q]['src']} : {e})"
            return e

        w("static size_t b200_dyn_smem_push(int threads, int max_tiles1, int max_w, int state_bytes) {")
        w("  (void)threads;")
        w("  return (size_t)state_bytes + (size_t)B200_NG * max_tiles1 * 8 + (size_t)(2 * max_w + 2) * 4 + 16;")
        w("}")
        w("")
        # a lower bound over a CTA's list of one slot (shared memory head, global tail)
        w("__device__ __forceinline__ int b200_push_lb(const int32_t* sh, const int32_t* gl, int hcap, int n, int x) {")
        w("  int lo = 0, hi = n;")
        w("  while (lo < hi) {")
        w("    const int m = (lo + hi) >> 1;")
        w("    const int v = m < hcap ? sh[m] : gl[m];")
        w("    if (v < x) lo = m + 1; else hi = m;")
        w("  }")
        w("  return lo;")
        w("}")
        w("")
        w("template <int MAXT, int MINB>")
        w("__global__ void __launch_bounds__(MAXT, MINB) b200_push_kernel(")
        w("    const b200_inst_d* __restrict__ insts, const int2* __restrict__ cta_map, int n_inst,")
        w("    int queue_mode, int* work, int64_t max_steps, uint64_t limit_ns, int max_tiles1, int max_w,")
        w("    int fault_rank, int state_bytes, unsigned long long* __restrict__ prof, int cluster) {")
        w("  (void)queue_mode; (void)work;")
        w("  extern __shared__ __align__(16) unsigned char b200_dyn[];")
        w("  unsigned char* const s_state = b200_dyn;")
        w("  int* const s_pref_all = (int*)(b200_dyn + state_bytes);              // [NG * max_tiles1]")
        w("  int* const s_tst = s_pref_all + B200_NG * max_tiles1;               // [NG * max_tiles1]")
        w("  int* const s_nd = s_tst + B200_NG * max_tiles1;                     // [max_w] events per window")
        w("  int* const s_ndoff = s_nd + max_w + 1;                              // [max_w + 1] window offsets")
        w("  (void)s_pref_all;")
        w("  __shared__ __align__(16) b200_inst_d I;")
        w("  __shared__ int s_wsum[B200_MAX_WARPS + 1];")
        w("  __shared__ int s_cnt[B200_MAX_THREADS];")
        w("  __shared__ int s_unit, s_rank, s_flag, s_cache;")
        w("  __shared__ long long s_mon_n[B200_MAX_SPKMON];")
        w("  __shared__ long long s_stm_n[B200_MAX_STATEMON];")
        w("  __shared__ void* s_gv[B200_NG][B200_MAXV];")
        w("  __shared__ int s_ut[B200_NG][2];")
        w("  __shared__ int s_own[B200_NG][2];")
        w("  __shared__ int s_glast[B200_NG], s_gen_lo, s_gen_hi;")
        w("  (void)s_glast; (void)s_gen_lo; (void)s_gen_hi;")
        w("  __shared__ int32_t* s_hist[B200_NG];   // this CTA's spike history (first HCAP of each slot)")
        w("  __shared__ int32_t* s_hcnt[B200_NG];   // its spikes per slot")
        w(f"  __shared__ int2* s_pb[{max(NP, 1)}];   // per slot, the bounds of the spikes in a pathway's source range")
        w(f"  __shared__ int s_mb[{max(NSM_, 1)}][2][2];   // per step parity: the recorded spikes not yet written")
        w(f"  __shared__ int s_red[2][{2 * max(NSM_ + NRM_, 1)}];  // monitors' block sums, by step parity")
        for gi in range(NG):
            n_ = max(gtables[gi][0].size, 1)
            w(f"  __shared__ double s_Sg{gi}[{n_}]; __shared__ float s_Sg{gi}f[{n_}]; __shared__ long long s_Sg{gi}i[{n_}];")
        for pi in range(NP):
            n_ = max(ptables[pi][0].size, 1)
            w(f"  __shared__ double s_Sp{pi}[{n_}]; __shared__ float s_Sp{pi}f[{n_}]; __shared__ long long s_Sp{pi}i[{n_}];")
        w("  (void)s_state; (void)s_red; (void)s_mb;")
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
            for k in range(len(g["vars"])):
                w(f"      s_gv[{gi}][{k}] = I.g[{gi}].var[{k}];")
            w("      if (cache) {  // own neurons only: pointers offset so that global indices address them")
            for k in USED[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"        s_gv[{gi}][{k}] = (void*)(s_state + off - (size_t)s_own[{gi}][0] * {sz});")
                w(f"        off += ((size_t)(s_own[{gi}][1] - s_own[{gi}][0]) * {sz} + 15) & ~(size_t)15;")
            w("      }")
            w(f"      s_hist[{gi}] = (int32_t*)(s_state + I.g[{gi}].hist_off);")
            w(f"      s_hcnt[{gi}] = (int32_t*)(s_state + I.g[{gi}].hcnt_off);")
        for pi in range(NP):
            w(f"      s_pb[{pi}] = (int2*)(s_state + I.p[{pi}].pb_off);")
        w("    }")
        w("    __syncthreads();")
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
        w("    // the spike history of the last RH steps: counts, then the head of each list")
        for gi in range(NG):
            w(f"    for (int sl = threadIdx.x; sl < I.g[{gi}].RH; sl += blockDim.x) s_hcnt[{gi}][sl] = I.g[{gi}].hcnt[(int64_t)sl * I.n_cta + rank];")
        w("    __syncthreads();")
        for gi in range(NG):
            w("    {")
            w(f"      const int hc = I.g[{gi}].HCAP, rh = I.g[{gi}].RH;")
            w("      for (int x = threadIdx.x; x < rh * hc; x += blockDim.x) {")
            w("        const int sl = x / hc, k = x - sl * hc;")
            w(f"        if (k < s_hcnt[{gi}][sl]) s_hist[{gi}][x] = I.g[{gi}].hist[(int64_t)sl * I.g[{gi}].N + s_own[{gi}][0] + k];")
            w("      }")
            w("    }")
        w("    __syncthreads();")
        for pi in range(NP):
            gi = paths[pi]["src"]
            w(f"    for (int sl = threadIdx.x; sl < I.g[{gi}].RH; sl += blockDim.x) {{  // pathway {pi}: bounds per slot")
            w(f"      const int nn = s_hcnt[{gi}][sl], hc = I.g[{gi}].HCAP;")
            w(f"      const int32_t* sh = s_hist[{gi}] + sl * hc;")
            w(f"      const int32_t* gl = I.g[{gi}].hist + (int64_t)sl * I.g[{gi}].N + s_own[{gi}][0];")
            w(f"      const int b = b200_push_lb(sh, gl, hc, nn, I.p[{pi}].src_lo), e = b200_push_lb(sh, gl, hc, nn, I.p[{pi}].src_hi);")
            w(f"      s_pb[{pi}][sl] = make_int2(b, e);")
            w("    }")
        w("    __syncthreads();")
        w("    const int64_t ts0 = I.ts;")
        w("    const int64_t ts_stop = (I.ts_end < ts0 + max_steps) ? I.ts_end : ts0 + max_steps;")
        w("    const double _b200_dt = I.dt;")
        w("    int64_t ts = ts0;")
        w("    bool ok = true;")
        w("    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, NW = blockDim.x >> 5;")
        w("    (void)lane; (void)wid; (void)NW;")
        w(f"    __shared__ unsigned long long _pt, _pacc[{NPH}];")
        w(f"    if (threadIdx.x == 0) {{ _pt = 0; for (int q = 0; q < {NPH}; ++q) _pacc[q] = 0; }}")
        w("#define B200_PHASE(q) do { if (prof && threadIdx.x == 0) { const unsigned long long _c = clock64(); _pacc[q] += _c - _pt; _pt = _c; } } while (0)")

        def emit_fold(sexpr, ind, all_vars=True):
            """Adds accumulator buffer (sexpr) % 3 of the own neurons to their
            state and clears it (the deliveries due at step sexpr).  The loads of
            every variable are issued before any is added (one L2 round trip):
            4-byte variables as float4/int4 groups of 4 neurons where aligned."""
            sp = " " * ind
            todo = [(kk, gv) for kk, gv in enumerate(ACC) if all_vars or gv not in FUSED]
            if not todo:
                return
            w(sp + "{")
            w(sp + f"  const int par = (int)(({sexpr}) % B200_PUSH_BUFS);")
            vec = [(kk, gi, vi) for kk, (gi, vi) in todo if SIZE[groups[gi]["vars"][vi]["ctype"]] == 4]
            sca = [(kk, gi, vi) for kk, (gi, vi) in todo if SIZE[groups[gi]["vars"][vi]["ctype"]] != 4]
            for kk, gi, vi in vec + sca:
                ct = groups[gi]["vars"][vi]["ctype"]
                w(sp + f"  {ct}* const _fa{kk} = ({ct}*)I.acc[{kk}] + (size_t)par * I.g[{gi}].N;")
                w(sp + f"  {ct}* const _fx{kk} = ({ct}*)s_gv[{gi}][{vi}];")
            if vec:
                # groups of 4 neurons from the (4-aligned) start of the CTA's range
                w(sp + "  bool _fv = true;")
                for kk, gi, vi in vec:
                    w(sp + f"  _fv = _fv && (((uintptr_t)(_fa{kk} + s_own[{gi}][0]) | (uintptr_t)(_fx{kk} + s_own[{gi}][0])) & 15) == 0;")
                gis = sorted({gi for _, gi, _ in vec})
                for gi in gis:
                    vs = [(kk, vi) for kk, g_, vi in vec if g_ == gi]
                    w(sp + "  {")
                    w(sp + f"    const int i0 = s_own[{gi}][0], i1 = s_own[{gi}][1];")
                    w(sp + "    const int n4 = _fv ? (i1 - i0) >> 2 : 0;  // whole groups of 4")
                    w(sp + "    for (int gb = (int)threadIdx.x; gb < n4; gb += 4 * (int)blockDim.x) {")
                    for kk, vi in vs:
                        w(sp + f"      float4 _d{kk}[4];")
                    w("#pragma unroll")
                    w(sp + "      for (int u = 0; u < 4; ++u) {")
                    w(sp + "        const int g4 = gb + u * (int)blockDim.x;")
                    w(sp + "        if (g4 < n4) {")
                    for kk, vi in vs:
                        w(sp + f"          _d{kk}[u] = __ldcg((const float4*)(_fa{kk} + i0) + g4);")
                    w(sp + "        }")
                    w(sp + "      }")
                    w("#pragma unroll")
                    w(sp + "      for (int u = 0; u < 4; ++u) {")
                    w(sp + "        const int g4 = gb + u * (int)blockDim.x;")
                    w(sp + "        if (g4 < n4) {")
                    for kk, vi in vs:
                        ct = groups[gi]["vars"][vi]["ctype"]
                        w(sp + f"          {{ {ct}* const xs = _fx{kk} + i0 + 4 * g4; const {ct}* const ds = ({ct}*)&_d{kk}[u];")
                        w(sp + "            xs[0] += ds[0]; xs[1] += ds[1]; xs[2] += ds[2]; xs[3] += ds[3]; }")
                        w(sp + f"          __stcg((float4*)(_fa{kk} + i0) + g4, make_float4(0.f, 0.f, 0.f, 0.f));")
                    w(sp + "        }")
                    w(sp + "      }")
                    w(sp + "    }")
                    w(sp + "    for (int i = i0 + 4 * n4 + (int)threadIdx.x; i < i1; i += (int)blockDim.x) {  // the rest, one by one")
                    for kk, vi in vs:
                        w(sp + f"      {{ const auto dd = __ldcg(_fa{kk} + i); _fx{kk}[i] += dd; _fa{kk}[i] = 0; }}")
                    w(sp + "    }")
                    w(sp + "  }")
            for kk, gi, vi in sca:
                ct = groups[gi]["vars"][vi]["ctype"]
                w(sp + "  {")
                w(sp + f"    const int i0 = s_own[{gi}][0], i1 = s_own[{gi}][1];")
                w(sp + "    for (int ib = i0 + (int)threadIdx.x; ib < i1; ib += 8 * (int)blockDim.x) {")
                w(sp + f"      {ct} d[8];")
                w("#pragma unroll")
                w(sp + f"      for (int u = 0; u < 8; ++u) {{ const int i = ib + u * (int)blockDim.x; d[u] = i < i1 ? __ldcg(_fa{kk} + i) : ({ct})0; }}")
                w("#pragma unroll")
                w(sp + "      for (int u = 0; u < 8; ++u) {")
                w(sp + "        const int i = ib + u * (int)blockDim.x;")
                w(sp + f"        if (i < i1) {{ _fx{kk}[i] += d[u]; __stcg(_fa{kk} + i, ({ct})0); }}")
                w(sp + "      }")
                w(sp + "    }")
                w(sp + "  }")
            w(sp + "}")
            w(sp + "__syncthreads();")

        NMON = NSM_ + NRM_

        def emit_monitor_raw_loads(sexpr, ind):
            """Late monitors: the counts of step sexpr loaded into registers (_xr,
            two per thread and monitor) and summed only when the monitors run, so
            the round trip overlaps the step; more CTAs than two per thread: summed
            at once."""
            sp = " " * ind
            if not NMON:
                return
            w(sp + "if (I.n_cta <= 2 * (int)blockDim.x) {")
            w(sp + f"  const int xb = (int)(({sexpr}) % 3) * I.n_cta;")
            w(sp + "#pragma unroll")
            w(sp + "  for (int u = 0; u < 2; ++u) {")
            w(sp + "    const int c = (int)threadIdx.x + u * (int)blockDim.x;")
            for mi in range(NSM_):
                w(sp + f"    _xr[{mi}][u] = c < I.n_cta ? I.sm[{mi}].xcnt[xb + c] : 0;")
            for ri in range(NRM_):
                w(sp + f"    _xr[{NSM_ + ri}][u] = c < I.n_cta ? I.rm[{ri}].xcnt[xb + c] : 0;")
            w(sp + "  }")
            w(sp + "} else {")
            emit_monitor_counts(sexpr, ind + 2)
            w(sp + "}")

        def emit_monitor_counts(sexpr, ind):
            """Each thread's share of all CTAs' counts of step sexpr (written
            before that step's barrier): into bf (CTAs before this one) and tt
            (all), declared by the caller."""
            sp = " " * ind
            if not NMON:
                return
            w(sp + "{")
            w(sp + f"  const int xb = (int)(({sexpr}) % 3) * I.n_cta;")
            w(sp + f"  for (int m = 0; m < {NMON}; ++m) {{ bf[m] = 0; tt[m] = 0; }}")
            w(sp + "  for (int c = threadIdx.x; c < I.n_cta; c += blockDim.x) {")
            for mi in range(NSM_):
                w(sp + f"    {{ const int x = I.sm[{mi}].xcnt[xb + c]; tt[{mi}] += x; if (c < rank) bf[{mi}] += x; }}")
            for ri in range(NRM_):
                w(sp + f"    {{ const int x = I.rm[{ri}].xcnt[xb + c]; tt[{NSM_ + ri}] += x; }}")
            w(sp + "  }")
            w(sp + "}")

        def emit_monitors(sexpr, ind, counts=True):
            """The spike and rate monitors of step sexpr: every CTA writes its own
            spikes after those of the CTAs before it (counts: load the counts
            here; otherwise emit_monitor_raw_loads loaded them earlier)."""
            sp = " " * ind
            if not NMON:
                return
            nmon = NMON
            if counts:
                emit_monitor_counts(sexpr, ind)
            else:
                w(sp + "if (I.n_cta <= 2 * (int)blockDim.x) {  // the counts loaded after the barrier")
                w(sp + f"  for (int m = 0; m < {NMON}; ++m) {{ bf[m] = 0; tt[m] = 0; }}")
                w(sp + "#pragma unroll")
                w(sp + "  for (int u = 0; u < 2; ++u) {")
                w(sp + "    const int c = (int)threadIdx.x + u * (int)blockDim.x;")
                w(sp + f"    for (int m = 0; m < {NMON}; ++m) {{ tt[m] += _xr[m][u]; if (c < rank) bf[m] += (m < {NSM_}) ? _xr[m][u] : 0; }}")
                w(sp + "  }")
                w(sp + "}")
            w(sp + "{")
            w(sp + f"  for (int m = 0; m < {nmon}; ++m) {{")
            w(sp + "#pragma unroll")
            w(sp + "    for (int o = 16; o >= 1; o >>= 1) { bf[m] += __shfl_down_sync(0xffffffffu, bf[m], o); tt[m] += __shfl_down_sync(0xffffffffu, tt[m], o); }")
            w(sp + "  }")
            # one block barrier: the sums of step parity p go to s_red[p], which the
            # previous step cleared (its readers are past a barrier by then)
            w(sp + f"  const int _rp = (int)(({sexpr}) & 1);")
            w(sp + f"  if (lane == 0) for (int m = 0; m < {nmon}; ++m) {{ atomicAdd(&s_red[_rp][2 * m], bf[m]); atomicAdd(&s_red[_rp][2 * m + 1], tt[m]); }}")
            w(sp + "  __syncthreads();")
            for mi, m in enumerate(spkmons):
                gi = m["group"]
                w(sp + f"  {{  // spike monitor {mi}")
                w(sp + f"    const b200_spkmon_d& SM = I.sm[{mi}];")
                w(sp + f"    const int sl = (int)(({sexpr}) % I.g[{gi}].RH);")
                w(sp + f"    const long long mbase = _mn[{mi}] + s_red[_rp][{2 * mi}];")
                w(sp + f"    const int mpar = (int)(({sexpr}) & 1);")
                w(sp + f"    for (int j = threadIdx.x; j < s_mb[{mi}][mpar][1]; j += blockDim.x) {{")
                w(sp + f"      const int idx = {list_elem(gi, 'sl', f's_mb[{mi}][mpar][0] + j')};")
                w(sp + "      const long long pos = mbase + j;")
                w(sp + "      SM.i[pos] = idx - SM.lo;")
                w(sp + f"      SM.ts[pos] = (int32_t)({sexpr});")
                if m.get("vars"):
                    w(sp + "      " + value_rows(mi, gi, "pos", "idx"))
                w(sp + "      atomicAdd(&SM.count[idx - SM.lo], 1);  // no read round trip (own neurons: uncontended)")
                w(sp + "    }")
                w(sp + "  }")
            for ri, m in enumerate(ratemons):
                w(sp + f"  if (rank == 0 && threadIdx.x == 0) I.rm[{ri}].cnt[({sexpr}) - I.rm[{ri}].step0] = s_red[_rp][{2 * (NSM_ + ri) + 1}];")
            # every thread keeps the spike monitors' running totals; thread 0 also in
            # shared memory (its capacity check and the write-back at the end)
            for mi in range(NSM_):
                w(sp + f"  _mn[{mi}] += s_red[_rp][{2 * mi + 1}];")
                w(sp + f"  if (threadIdx.x == 0) s_mon_n[{mi}] = _mn[{mi}];")
            w(sp + f"  if (threadIdx.x < {2 * nmon}) s_red[_rp ^ 1][threadIdx.x] = 0;  // for the next step")
            w(sp + "}")

        w(f"    int bf[{max(NMON, 1)}], tt[{max(NMON, 1)}];  // monitors: this thread's share of the CTAs' counts")
        w(f"    int _xr[{max(NMON, 1)}][2];  // (late monitors: the counts as loaded)")
        w("    (void)bf; (void)tt; (void)_xr;")
        w(f"    long long _mn[{max(NSM_, 1)}];  // the spike monitors' totals (every thread)")
        for mi in range(NSM_):
            w(f"    _mn[{mi}] = s_mon_n[{mi}];")
        w(f"    if (threadIdx.x < {4 * max(NSM_ + NRM_, 1)}) (&s_red[0][0])[threadIdx.x] = 0;")
        w("    __syncthreads();")
        w("    for (; ts < ts_stop; ++ts) {")
        w("      if (threadIdx.x == 0) {")
        w("        int st = 0;")
        for m in range(len(spkmons)):
            w(f"        if (s_mon_n[{m}] + 2 * (long long)(I.sm[{m}].hi - I.sm[{m}].lo) > I.sm[{m}].cap) st = 1;")
        w("        s_flag = st;")
        w("      }")
        w("      __syncthreads();")
        w("      if (s_flag) break;")
        w("      if (prof && threadIdx.x == 0) _pt = clock64();")
        w("      if (ts > ts0) {")
        w("        if (!b200_owner_wait(I, ts - 1, limit_ns, cluster)) { ok = false; break; }")
        w("        B200_PHASE(1);")
        if LATE:
            emit_monitor_raw_loads("ts - 1", 8)  # (their round trip overlaps the fold and the step)
        emit_fold("ts - 1", 8, all_vars=False)
        if not LATE:
            emit_monitors("ts - 1", 8)
        w("        B200_PHASE(3);")
        w("      }")
        w("      const double _b200_t = (double)ts * _b200_dt;")
        w("      const int64_t _b200_ts = ts;")
        for gi in range(NG):
            w(f"      const int _hs{gi} = (int)(ts % I.g[{gi}].RH);  // this step's history slot")
        w("      const int _x3 = (int)(ts % 3);")
        for gi in range(NG):
            if lean_ok(gi):
                emit_lean_phase_a(gi)
            else:
                emit_phase_a(True, push=True, only=[gi])
        w("      __syncthreads();")
        w("      B200_PHASE(0);")
        w("      // the step's spike bounds per pathway source range, and the monitors' counts")
        w("      {")
        w("        // job j (a pathway or monitor) on lane j / NW of warp j % NW: one per warp first")
        w("        const int t_ = lane < 16 ? lane * NW + wid : -1;")
        for pi in range(NP):
            gi = paths[pi]["src"]
            w(f"        if (t_ == {pi}) {{")
            w(f"          const int sl = _hs{gi}, nn = s_hcnt[{gi}][sl], hc = I.g[{gi}].HCAP;")
            w(f"          const int32_t* sh = s_hist[{gi}] + sl * hc;")
            w(f"          const int32_t* gl = I.g[{gi}].hist + (int64_t)sl * I.g[{gi}].N + s_own[{gi}][0];")
            w(f"          const bool all = I.p[{pi}].src_lo <= s_own[{gi}][0] && I.p[{pi}].src_hi >= s_own[{gi}][1];")
            w(f"          s_pb[{pi}][sl] = all ? make_int2(0, nn) : make_int2(b200_push_lb(sh, gl, hc, nn, I.p[{pi}].src_lo), b200_push_lb(sh, gl, hc, nn, I.p[{pi}].src_hi));")
            w("        }")
        for mi, m in enumerate(spkmons):
            gi = m["group"]
            w(f"        if (t_ == {NP + mi}) {{")
            w(f"          const int sl = _hs{gi}, nn = s_hcnt[{gi}][sl], hc = I.g[{gi}].HCAP;")
            w(f"          const int32_t* sh = s_hist[{gi}] + sl * hc;")
            w(f"          const int32_t* gl = I.g[{gi}].hist + (int64_t)sl * I.g[{gi}].N + s_own[{gi}][0];")
            w(f"          const bool all = I.sm[{mi}].lo <= s_own[{gi}][0] && I.sm[{mi}].hi >= s_own[{gi}][1];")
            w(f"          const int b = all ? 0 : b200_push_lb(sh, gl, hc, nn, I.sm[{mi}].lo), e = all ? nn : b200_push_lb(sh, gl, hc, nn, I.sm[{mi}].hi);")
            w(f"          s_mb[{mi}][ts & 1][0] = b; s_mb[{mi}][ts & 1][1] = e - b;")
            w(f"          I.sm[{mi}].xcnt[_x3 * I.n_cta + rank] = e - b;")
            w("        }")
        for ri, m in enumerate(ratemons):
            gi = m["group"]
            w(f"        if (t_ == {NP + NSM_ + ri}) {{")
            w(f"          const int sl = _hs{gi}, nn = s_hcnt[{gi}][sl], hc = I.g[{gi}].HCAP;")
            w(f"          const int32_t* sh = s_hist[{gi}] + sl * hc;")
            w(f"          const int32_t* gl = I.g[{gi}].hist + (int64_t)sl * I.g[{gi}].N + s_own[{gi}][0];")
            w(f"          const bool all = I.rm[{ri}].lo <= s_own[{gi}][0] && I.rm[{ri}].hi >= s_own[{gi}][1];")
            w(f"          I.rm[{ri}].xcnt[_x3 * I.n_cta + rank] = all ? nn : b200_push_lb(sh, gl, hc, nn, I.rm[{ri}].hi) - b200_push_lb(sh, gl, hc, nn, I.rm[{ri}].lo);")
            w("        }")
        w("      }")
        w("      B200_PHASE(6);")
        w("      // test hook: CTA `fault_rank` leaves without arriving, the others must time out")
        w("      if (rank == fault_rank && ts == ts0) { ok = false; break; }")
        w("      b200_owner_arrive(I, cluster);  // (its __syncthreads orders the bounds above)")
        w("      B200_PHASE(2);")
        if LATE:
            # right after the arrival: no atomics of this CTA are queued yet, so its
            # stores are not held behind them (after the deliveries they were)
            w("      if (ts > ts0) {  // the monitors of step ts-1")
            emit_monitors("ts - 1", 8, counts=False)
            w("      }")
            w("      B200_PHASE(5);")
        # ---------------------------------------------- deliveries due at ts + 1
        w("      {  // deliveries due at ts+1: this CTA's spikes of steps ts+1-d, d = dmin..D")
        w("        const int64_t tn = ts + 1;")
        w("        const double _b200_t = (double)tn * _b200_dt; (void)_b200_t;  // (on_pre runs at the due step)")
        w("        const int64_t _b200_ts = tn; (void)_b200_ts;")
        w("        const int _b200_apar = (int)(tn % B200_PUSH_BUFS);")
        for q in range(NP):
            w(f"        const int W{q} = I.p[{q}].D > 0 ? I.p[{q}].D - I.p[{q}].dmin + 1 : 0;")
        w(f"        const int WT = {' + '.join(f'W{q}' for q in range(NP))};")
        w("        for (int k = threadIdx.x; k < WT; k += blockDim.x) {")
        w(pathway_window("k", 10))
        w("          int n = 0;")
        for q in range(NP):
            gi = paths[q]["src"]
            w(("          if" if q == 0 else "          else if") + f" (q == {q}) {{")
            w(f"            const int dd = I.p[{q}].dmin + kk;  // spikes of step tn - dd, slot _hs + 1 - dd (mod RH)")
            w(f"            int sl = _hs{gi} + 1 - dd; if (sl < 0) sl += I.g[{gi}].RH;")
            w(f"            if (tn - dd >= 0) {{ const int2 bb = s_pb[{q}][sl]; n = bb.y - bb.x; }}")
            w("          }")
        w("          s_nd[k] = n;")
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
        w("        const int NI = s_ndoff[WT];")
        w("        // items (one spike at one delay) split evenly over the warps, at most 32")
        w("        // per warp and round; a warp's events are numbered across its items, each")
        w("        // lane finds its event's item by a binary search over the lanes")
        w("        const int per = NI < 32 * NW ? (NI + NW - 1) / NW : 32;")
        w("        for (int r0 = wid * per; r0 < NI; r0 += NW * per) {")
        w("          const int it = r0 + lane;")
        w("          int64_t ilo = 0; int len = 0, iq = 0;")
        w("          if (lane < per && it < NI) {")
        w("            const int k = b200_upper_bound(s_ndoff, WT + 1, it) - 1;")
        w(pathway_window("k", 12))
        for q in range(NP):
            gi = paths[q]["src"]
            w(("            if" if q == 0 else "            else if") + f" (q == {q}) {{")
            w(f"              const b200_pathway_d& PD = I.p[{q}];")
            w(f"              int sl = _hs{gi} + 1 - (PD.dmin + kk); if (sl < 0) sl += I.g[{gi}].RH;")
            w(f"              const int r = it - s_ndoff[k] + s_pb[{q}][sl].x;")
            w(f"              const int32_t src = {list_elem(gi, 'sl', 'r')};")
            w("              const int64_t sg = (int64_t)(src - PD.src_lo) * W" + str(q) + " + kk;")
            w("              ilo = PD.segptr[sg];")
            w("              len = (int)(PD.segptr[sg + 1] - ilo);")
            w("            }")
        w("            iq = q;")
        w("          }")
        w("          int inc = len;")
        w("#pragma unroll")
        w("          for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(0xffffffffu, inc, o); if (lane >= o) inc += y; }")
        w("          const int Ew = __shfl_sync(0xffffffffu, inc, 31);")
        w("          const int ioff = (lane < per && it < NI) ? inc - len : 0x7fffffff;")
        # event loop: two-phase loads when every pathway's on_pre starts with the same load types
        sigs = []
        for pi in range(NP):
            lds, _ = split_loads(dict(ptables[pi][1])["on_pre"]["vector_device"] or dict(ptables[pi][1])["on_pre"]["vector"])
            sigs.append([ct for ct, _, _ in lds])
        two = NP > 0 and all(sg_ == sigs[0] for sg_ in sigs)
        KB = "KBP"
        w("          constexpr int KBP = (MAXT * MINB <= 512) ? 8 : 2;  // events whose loads a lane issues at once")
        w(f"          for (int e0 = 0; e0 < Ew; e0 += 32 * {KB}) {{  // warp-uniform: every lane shuffles")
        w(f"            int _q[{KB}]; int64_t _ix[{KB}];")
        if two:
            for li, ct in enumerate(sigs[0]):
                w(f"            {ct} _ld{li}[{KB}];")
        w("#pragma unroll")
        w(f"            for (int _b200_kq = 0; _b200_kq < {KB}; ++_b200_kq) {{")
        w("              const int e = e0 + _b200_kq * 32 + lane;")
        w("              int j = 0;")
        w("#pragma unroll")
        w("              for (int st = 16; st >= 1; st >>= 1) { const int oj = __shfl_sync(0xffffffffu, ioff, j + st); if (oj <= e) j += st; }")
        w("              const int64_t lj = __shfl_sync(0xffffffffu, ilo, j);")
        w("              const int oj = __shfl_sync(0xffffffffu, ioff, j);")
        w("              const int qj = __shfl_sync(0xffffffffu, iq, j);")
        w("              _q[_b200_kq] = -1;")
        w("              if (e < Ew) {")
        w("                const int64_t _idx = lj + (e - oj);")
        w("                _q[_b200_kq] = qj; _ix[_b200_kq] = _idx;")
        if two:
            for q in range(NP):
                lds, _ = split_loads(dict(ptables[q][1])["on_pre"]["vector_device"] or dict(ptables[q][1])["on_pre"]["vector"])
                p = paths[q]
                w(("                if" if q == 0 else "                else if") + f" (qj == {q}) {{")
                for li, (ct, nm, ptr) in enumerate(lds):
                    if ptr == p["post_ptr"]:
                        ex = f"I.p[{q}].post[_idx]"
                    else:
                        kv = next(kk_ for kk_, v in enumerate(p.get("vars", [])) if v["ptr"] == ptr)
                        ex = f"(({ct}*)I.p[{q}].var[{kv}])[_idx]"
                    w(f"                  _ld{li}[_b200_kq] = {ex};")
                w("                }")
        w("              }")
        w("            }")
        w("#pragma unroll")
        w(f"            for (int _b200_kq = 0; _b200_kq < {KB}; ++_b200_kq) {{")
        w("              if (_q[_b200_kq] >= 0) {")
        w("                const int64_t _idx = _ix[_b200_kq]; (void)_idx;")
        w("                const int64_t _vectorisation_idx = _idx; (void)_vectorisation_idx;")
        for q in range(NP):
            p = paths[q]
            tab, blocks = ptables[q]
            blk = dict(blocks)["on_pre"]
            code = blk["vector_device"] if blk.get("vector_device") else blk["vector"]
            lds, rest = split_loads(code)
            w(("                if" if q == 0 else "                else if") + f" (_q[_b200_kq] == {q}) {{  // {p['name']}")
            w(f"                  const b200_pathway_d& PQ = I.p[{q}]; (void)PQ;")
            w(f"                  const double* const _b200_S = s_Sp{q}; const float* const _b200_Sf = s_Sp{q}f; const long long* const _b200_Si = s_Sp{q}i;")
            w("                  (void)_b200_S; (void)_b200_Sf; (void)_b200_Si;")
            w(_indent(tab.const_loads(f32), 18))
            for ptr, (gidx, vidx) in sorted(p.get("group_ptrs", {}).items()):
                v = groups[gidx]["vars"][vidx]
                w(f"                  {v['ctype']}* __restrict__ const {ptr} = ({v['ctype']}*)I.acc[{ACCI[(gidx, vidx)]}] + (size_t)_b200_apar * I.g[{gidx}].N; (void){ptr};")
            for kv, v in enumerate(p.get("vars", [])):
                w(f"                  {v['ctype']}* __restrict__ const {v['ptr']} = ({v['ctype']}*)PQ.var[{kv}]; (void){v['ptr']};")
            w(f"                  const int32_t* __restrict__ const {p['post_ptr']} = PQ.post; (void){p['post_ptr']};")
            w(_indent(tab.scalar_loads("on_pre", f32), 18))
            w(_indent(_device(tab.time_code("on_pre")), 18))
            w("                  {  // (Brian's vector code may redeclare the clock's names)")
            if two:
                for li, (ct, nm, ptr) in enumerate(lds):
                    w(f"                  {ct} {nm} = _ld{li}[_b200_kq];")
                w(_indent(rest, 18))
            else:
                w(_indent(code, 18))
            w("                  }")
            w("                }")
        w("              }")
        w("            }")
        w("          }")
        w("        }")
        w("      }")
        w("      B200_PHASE(4);")

        w("    }  // steps")
        w(f"    if (prof && threadIdx.x == 0)")
        w(f"      for (int q = 0; q < {NPH}; ++q) atomicAdd(&prof[(size_t)unit * {NPH} + q], _pacc[q]);")
        w("#undef B200_PHASE")
        w("    // the last step: wait for its arrivals, add its deliveries, record its spikes,")
        w("    // apply its reset; the deliveries due at the next step stay in their buffer")
        w("    if (ok && ts > ts0) {")
        w("      if (!b200_owner_wait(I, ts - 1, limit_ns, cluster)) ok = false;")
        w("      if (ok) {")
        emit_fold("ts - 1", 8)
        emit_monitors("ts - 1", 8)
        w("        const double _b200_t = (double)(ts - 1) * _b200_dt; (void)_b200_t;")
        w("        const int64_t _b200_ts = ts - 1;")
        for gi in range(NG):
            rb = deferred_block(gi, 8, "ts - 1", True, push=True)
            if rb:
                w(rb)
        w("      }")
        w("    }")
        w("    __syncthreads();")
        w("    if (s_cache) {")
        for gi, g in enumerate(groups):
            for k in USED[gi]:
                sz = SIZE[g["vars"][k]["ctype"]]
                w(f"      b200_copy_bytes((char*)I.g[{gi}].var[{k}] + (size_t)s_own[{gi}][0] * {sz}, (const char*)s_gv[{gi}][{k}] + (size_t)s_own[{gi}][0] * {sz},")
                w(f"                      (size_t)(s_own[{gi}][1] - s_own[{gi}][0]) * {sz});")
        w("    }")
        w("    if (threadIdx.x == 0 && rank == 0) {")
        w("      *I.ts_done = ts;")
        for m in range(len(spkmons)):
            w(f"      *I.sm[{m}].n = s_mon_n[{m}];")
        for m in range(len(statemons)):
            w(f"      *I.stm[{m}].n = s_stm_n[{m}];")
        w("    }")
        w("    __syncthreads();")
        w("  }")
        w("}")
        w("")

    group_ev_bytes = []
    if OWNER:
        emit_owner_kernel()
    if PUSH:
        emit_push_kernel()
    OWNER_EV_BYTES = max(group_ev_bytes) if group_ev_bytes else 8

    # ------------------------------------------------------------- launch glue
    w("// `tcode` = threads | (min CTAs per SM - 1) << 16: the (512, 2) variant caps")
    w("// registers so that two CTAs fit on an SM (sweeps with more instances than SMs)")
    w("static const void* b200_kernel_for(int tcode) {")
    w("  const int threads = tcode & 0xffff, minb = ((tcode >> 16) & 0xf) + 1;")
    if PUSH:
        w("  if (tcode & B200_TCODE_PUSH) {  // push mode")
        w("    if (threads <= 256) return minb >= 2 ? (const void*)b200_push_kernel<256, 2> : (const void*)b200_push_kernel<256, 1>;")
        w("    if (threads <= 512) return (const void*)b200_push_kernel<512, 1>;")
        w("    return (const void*)b200_push_kernel<1024, 1>;")
        w("  }")
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
    if PUSH:
        w("  if (tcode & B200_TCODE_PUSH) return b200_dyn_smem_push(threads, max_tiles1, max_w, state_bytes);")
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
    w("static const int b200_acc_vars[] = {" + (", ".join(f"{gi}, {vi}" for gi, vi in ACC) if ACC else "0") + "};")
    w(f'static const b200_model_info B200_MODEL = {{"{spec["name"]}", {NG}, {NP}, {len(spkmons)}, {len(ratemons)}, {len(statemons)},')
    w("  b200_groups, b200_pathways, b200_spkmon, b200_ratemon, b200_statemon,")
    w(f"  {len(consts)}, b200_const_names, b200_const_defaults, b200_eval_scalars, b200_launch, b200_max_active,")
    w(f"  b200_static_smem, b200_max_cluster, {NPH}, {1 if OWNER else 0}, {OWNER_EV_BYTES},")
    w(f"  {len(SUMMED)}, {'b200_summed' if SUMMED else 'nullptr'}, {len(DRAWS)}, {'b200_draws' if DRAWS else 'nullptr'},")
    w(f"  {1 if PUSH else 0}, {len(ACC)}, b200_acc_vars}};")
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


def profile_slots(spec: dict, owner: bool = False, push: bool = False) -> list[str]:
    """Names of the device profile's slots (b200_get_profile), in order.
    Owner-mode kernel: update (update, threshold and reset of every group),
    barrier, spike lists, push counts, push into the event FIFOs, delivery.
    Classic kernel: the rest of the update phase, barrier A, the rest of the
    spike-list phase, one slot per pathway for its events, barrier B,
    delivery windows, delivery items; per group its update (with the threshold
    condition), its spike list (threshold), its reset; per group the copy of
    its spikes into the delay ring; one slot per spike and per rate monitor.
    Push-mode kernel: update (update, threshold and reset of every group),
    barrier, spike bounds and arrival, accumulators added and monitors, delivery."""
    groups = spec["groups"]
    paths = spec.get("pathways", [])
    if push:
        # (phase A's per-group slots as in the classic layout)
        names = ["other", "barrier", "arrive", "fold", "deliver", "monitors", "bounds"]
        names += [f"unused{k}" for k in range(len(names), 6 + len(paths))]
        for g in groups:
            names += [f"update:{g['name']}", f"threshold:{g['name']}", f"reset:{g['name']}"]
        owner = True  # (no ring or monitor slots)
    elif owner:
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
