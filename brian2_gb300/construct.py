"""Python side of the native construction library (libb200_construct).

:class:`BrianRandom` is a host random stream identical to the one a Brian2
``cpp_standalone`` program draws from after ``seed(s)`` (single thread), and the
``connect_*`` functions reproduce the synapse creation loops of
``brian2/devices/cpp_standalone/templates/synapses_create_generator.cpp`` draw for
draw, so a network built here is the network Brian builds.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class _RngState(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("idx", C.c_int32), ("has_gauss", C.c_int32), ("gauss", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = native.load(native.build_construct())
        P = C.POINTER(_RngState)
        L.b200_rng_seed.argtypes = [P, C.c_uint32]
        L.b200_rng_u32.argtypes = [P]
        L.b200_rng_u32.restype = C.c_uint32
        L.b200_rng_rand.argtypes = [P]
        L.b200_rng_rand.restype = C.c_double
        L.b200_rng_randn.argtypes = [P]
        L.b200_rng_randn.restype = C.c_double
        L.b200_rng_fill_rand.argtypes = [P, _f64p, C.c_int64]
        L.b200_rng_fill_randn.argtypes = [P, _f64p, C.c_int64]
        L.b200_rng_affine_rand.argtypes = [P, C.c_double, C.c_double, _f64p, C.c_int64]
        L.b200_rng_affine_randn.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double, _f64p, C.c_int64]
        L.b200_connect_bernoulli.argtypes = [P, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                             C.c_int32, C.c_int32, _i32p, _i32p, C.c_int64]
        L.b200_connect_bernoulli.restype = C.c_int64
        L.b200_connect_fixed_indegree.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, _i32p, _i32p, C.c_int64]
        L.b200_connect_fixed_indegree.restype = C.c_int64
        L.b200_quantise_delays.argtypes = [_f64p, C.c_int64, C.c_double, _i32p]
        _lib = L
    return _lib


class BrianRandom:
    """mt19937 stream of a single-threaded Brian2 standalone run after seed(s)."""

    def __init__(self, seed: int):
        self.state = _RngState()
        lib().b200_rng_seed(C.byref(self.state), C.c_uint32(int(seed) & 0xFFFFFFFF))

    def u32(self):
        return lib().b200_rng_u32(C.byref(self.state))

    def rand(self, n=None):
        if n is None:
            return lib().b200_rng_rand(C.byref(self.state))
        out = np.empty(int(n), np.float64)
        lib().b200_rng_fill_rand(C.byref(self.state), out.ctypes.data_as(_f64p), out.size)
        return out

    def randn(self, n=None):
        if n is None:
            return lib().b200_rng_randn(C.byref(self.state))
        out = np.empty(int(n), np.float64)
        lib().b200_rng_fill_randn(C.byref(self.state), out.ctypes.data_as(_f64p), out.size)
        return out

    def affine_rand(self, a, b, n):
        """n values of ``a + (b * rand())``."""
        out = np.empty(int(n), np.float64)
        lib().b200_rng_affine_rand(C.byref(self.state), float(a), float(b), out.ctypes.data_as(_f64p), out.size)
        return out

    def affine_randn(self, a, scale, c0, c1, n):
        """n values of ``a + (scale * (c0 + (c1 * randn())))``."""
        out = np.empty(int(n), np.float64)
        lib().b200_rng_affine_randn(C.byref(self.state), float(a), float(scale), float(c0), float(c1),
                                    out.ctypes.data_as(_f64p), out.size)
        return out

    def connect_bernoulli(self, n_pre, n_post, p, i_range=None, no_self=False, cond_uses_j=None):
        """Synapses of ``connect(condition, p=p)`` as (pre, post) int32 arrays.

        The condition is ``i in i_range`` (and ``i != j`` if no_self).  By
        default the condition is taken to depend on j exactly when no_self is
        set, matching how Brian splits outer and inner conditions.
        """
        i_lo, i_hi = i_range if i_range is not None else (0, n_pre)
        if cond_uses_j is None:
            cond_uses_j = bool(no_self)
        cap = max(16, int(n_pre * n_post * p * 1.2 + 10 * np.sqrt(n_pre * n_post * p + 1) + 1024))
        while True:
            st = _RngState()
            C.pointer(st)[0] = self.state
            pre = np.empty(cap, np.int32)
            post = np.empty(cap, np.int32)
            n = lib().b200_connect_bernoulli(C.byref(st), n_pre, n_post, float(p), i_lo, i_hi, int(no_self),
                                             int(cond_uses_j), pre.ctypes.data_as(_i32p),
                                             post.ctypes.data_as(_i32p), cap)
            if n >= 0:
                self.state = st
                return pre[:n].copy(), post[:n].copy()
            cap *= 2

    def connect_fixed_indegree(self, n_pre, n_post, K):
        """Synapses of ``connect(i='k for k in sample(N_pre, size=K)')``."""
        cap = int(n_post) * int(K)
        pre = np.empty(cap, np.int32)
        post = np.empty(cap, np.int32)
        n = lib().b200_connect_fixed_indegree(C.byref(self.state), n_pre, n_post, K, pre.ctypes.data_as(_i32p),
                                              post.ctypes.data_as(_i32p), cap)
        if n < 0:
            raise ValueError("invalid sample size")
        return pre[:n], post[:n]


def quantise_delays(delay_seconds, dt):
    """(int)(delay/dt + 0.5), as ``CSpikeQueue::prepare`` (brian2/synapses/spikequeue.h:85-95)."""
    d = np.ascontiguousarray(delay_seconds, dtype=np.float64)
    out = np.empty(d.size, np.int32)
    lib().b200_quantise_delays(d.ctypes.data_as(_f64p), d.size, float(dt), out.ctypes.data_as(_i32p))
    return out
