"""Device-side construction of large fixed in-degree networks (libb200_scale).

Used for the 1e6-neuron / 1e9-synapse delay network: every target draws its
sources from a counter-based generator on the GPU and the CSR over
(source, delay slot) is built on the device, then handed to the step engine
with ``b200_set_synapses_csr``.  The construction is restated on the CPU in
``oracle/scale_ref.c`` (test infrastructure) and checked bit for bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .construct import BrianRandom
from .runtime import Model, Network

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = native.load(native.build_scale())
        L.b200s_fixed_indegree_csr.argtypes = [C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                               C.c_double, C.c_double, C.c_double,
                                               C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                               C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                               C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]
        L.b200s_last_error.restype = C.c_char_p
        L.b200s_free.argtypes = [C.c_void_p]
        L.b200s_fill_f32.argtypes = [C.c_void_p, C.c_float, C.c_int64]
        L.b200s_fill_f64.argtypes = [C.c_void_p, C.c_double, C.c_int64]
        L.b200s_to_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        L.b200s_host_draw.argtypes = [C.c_uint32] * 4 + [C.c_uint64, C.c_uint32]
        L.b200s_host_draw.restype = C.c_uint32
        L.b200s_outdegree.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
        _lib = L
    return _lib


class DeviceCSR:
    """A pathway's CSR over (source, delay slot) in device memory."""

    def __init__(self, seed, path_id, n_src, src_off, n_post, K, dmin, dspan, dt):
        L = lib()
        s0, s1 = C.c_int32(), C.c_int32()
        seg, post, pre = C.c_void_p(), C.c_void_p(), C.c_void_p()
        n = C.c_int64()
        r = L.b200s_fixed_indegree_csr(int(seed), int(path_id), int(n_src), int(src_off), int(n_post), int(K),
                                       float(dmin), float(dspan), float(dt), C.byref(s0), C.byref(s1),
                                       C.byref(seg), C.byref(post), C.byref(pre), C.byref(n))
        if r:
            raise RuntimeError("device construction failed: " + L.b200s_last_error().decode())
        self.slot_min, self.slot_max = s0.value, s1.value
        self.seg, self.post, self.pre = seg.value, post.value, pre.value
        self.n_syn = n.value
        self.n_src = n_src
        self.W = self.slot_max - self.slot_min + 1

    def host_arrays(self):
        """(segptr, post, pre) copied to the host (tests, small networks only)."""
        L = lib()
        seg = np.empty(self.n_src * self.W + 1, np.int64)
        post = np.empty(self.n_syn, np.int32)
        pre = np.empty(self.n_syn, np.int32)
        for a, p in ((seg, self.seg), (post, self.post), (pre, self.pre)):
            if a.nbytes and L.b200s_to_host(a.ctypes.data, p, a.nbytes):
                raise RuntimeError(L.b200s_last_error().decode())
        return seg, post, pre

    def outdegree(self):
        out = np.empty(self.n_src, np.int32)
        if lib().b200s_outdegree(self.seg, self.n_src, self.W, out.ctypes.data):
            raise RuntimeError(lib().b200s_last_error().decode())
        return out

    def free(self):
        L = lib()
        for p in (self.seg, self.post, self.pre):
            L.b200s_free(p)
        self.seg = self.post = self.pre = None


def build_delays_scale(spec, N=1_000_000, K=1000, seed=1234, ne_frac=0.8, wscale=1.0 / 50, dmin_ms=0.1,
                       dmax_ms=5.0, threads=256, ctas_per_inst=None, keep_csr=False):
    """The fixed in-degree delay network of ``oracle/brian_configs.py:cuba_delays``
    at full scale: v0 from Brian's stream (as the script), synapses and delays
    from the device generator.  Returns (network, csr list)."""
    from .workloads import DT, delay_constants, _ftype
    c = {x["name"]: x["value"] for x in spec["consts"]}
    Ne = int(N * ne_frac)
    Ke = int(K * ne_frac)
    Ki = K - Ke
    ft = _ftype(spec)
    we, wi, dmin, dspan = delay_constants(wscale, dmin_ms, dmax_ms)
    model = Model.get(spec)
    net = Network(model, [[N]], DT)
    if ctas_per_inst is None:
        ctas_per_inst = 1
    net.configure(threads=threads, ctas_per_inst=ctas_per_inst)
    v0 = BrianRandom(seed).affine_rand(c["Vr"], c["Vt"] - c["Vr"], N).astype(ft)
    net.upload(0, "neurongroup", "v", v0)
    if "i" in model.tables["groups"][0]:
        net.upload(0, "neurongroup", "i", np.arange(N, dtype=np.int32))
    csrs = []
    outdeg = np.zeros(N, np.int64)
    for pw, (lo, hi, k, w) in (("synapses_pre", (0, Ne, Ke, we)), ("synapses_1_pre", (Ne, N, Ki, wi))):
        pid = model.pathway_index[pw]
        d = DeviceCSR(seed, pid, hi - lo, lo, N, k, dmin, dspan, DT)
        net.set_synapses_csr(0, pw, (lo, hi), (0, N), d.slot_min, d.slot_max, d.seg, d.post, d.pre, d.n_syn)
        outdeg[lo:hi] += d.outdegree()
        wp = net.synapse_var_ptr(0, pw, "w")
        fill = lib().b200s_fill_f32 if ft == np.float32 else lib().b200s_fill_f64
        if fill(wp, w, d.n_syn):
            raise RuntimeError(lib().b200s_last_error().decode())
        if keep_csr:
            csrs.append(d)
        else:
            d.free()
    net.outdegree = outdeg  # synapses per source neuron (for counting synaptic events)
    return net, csrs
