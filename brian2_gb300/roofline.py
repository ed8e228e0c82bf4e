"""ALU roofline of compute-bound step loops (Hodgkin-Huxley networks).

Their update is a chain of transcendental functions and divisions per neuron,
not a stream of bytes, so the bound is the arithmetic pipe of its precision.
The algorithmic work is counted from the generated update code itself (the
exponential-Euler snippet Brian's code generator wrote): the arithmetic
operators of each neuron-step, with the calls of exp / expm1 (``_exprel``) /
pow counted separately (their device implementations are many instructions
each, so the counted flops bound the work from below).  The peak is measured
on the device (libb200_peaks: FMA throughput in float32 and float64).
"""
from __future__ import annotations

import ctypes as C
import re

from . import native

_FUNCS = ("exp", "expm1", "_exprel", "_brian_pow", "pow", "log", "sqrt")


def count_ops(code: str) -> dict:
    """Arithmetic operators and function calls per evaluation of a C snippet:
    binary + - * / (a multiplication by the literal 1.0f, which Brian emits
    for its unit algebra and the compiler removes, is not counted; unary minus
    is a sign change, not a flop), and calls per function name."""
    calls = {f: len(re.findall(r"\b%s\s*\(" % re.escape(f), code)) for f in _FUNCS}
    body = []
    for ln in code.splitlines():
        ln = ln.strip()
        if not ln or ln.startswith("//") or "=" not in ln or re.match(r"^\w+\s*=\s*\w+\s*;$", ln):
            continue
        if re.match(r"^(const\s+)?\w+\s+\w+\s*=\s*_ptr_array_\w+\[_idx\];$", ln):
            continue
        if ln.startswith("_ptr_array_"):
            continue
        body.append(ln.split("=", 1)[1])
    text = " ".join(body).replace("1.0f*", "")
    text = re.sub(r"\d+\.\d*(e[-+]?\d+)?|\d+e[-+]?\d+", "0", text)  # numbers (exponent signs are not operators)
    toks = re.findall(r"[A-Za-z_]\w*|\d+|[-+*/()<>!=,?:;]", text)
    flops = 0
    prev = None
    for t in toks:
        if t in "*/+":
            flops += 1
        elif t == "-":
            if prev is not None and (re.match(r"[A-Za-z_0-9]", prev) or prev == ")"):
                flops += 1  # binary minus
        prev = t
    return {"flops": flops, "calls": {k: v for k, v in calls.items() if v}}


def update_ops(spec: dict, group: int = 0) -> dict:
    """count_ops of a group's state update (vector code, per neuron-step)."""
    return count_ops(spec["groups"][group]["update"]["vector"])


_lib = None


def fma_peak_gflops(fp64: bool, iterations: int | None = None) -> float:
    """Measured FMA throughput of the device in GFLOP/s."""
    global _lib
    if _lib is None:
        _lib = native.load(native.build_peaks())
        _lib.b200p_fma_peak.argtypes = [C.c_int32, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.b200p_last_error.restype = C.c_char_p
    g, ms = C.c_double(), C.c_double()
    it = iterations or (2_000 if fp64 else 100_000)
    r = _lib.b200p_fma_peak(int(bool(fp64)), int(it), C.byref(g), C.byref(ms))
    if r:
        raise RuntimeError("FMA peak measurement failed: " + _lib.b200p_last_error().decode())
    return g.value
