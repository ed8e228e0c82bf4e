"""The allocation-free construction entry point (GPU only).

`b200s_fixed_indegree_csr_noalloc` serves callers that may not allocate device
memory while they run (their device memory belongs to another framework's pool
allocator, or they work within a fixed device-memory budget): they pass the
output buffers, and the temporaries come from one fixed 16 MiB device array.
Its output must equal the allocating entry point's, bit for bit, on calls made
one after another (the shared scratch keeps the previous call's contents).
This file is collected last so that a failure here stops a `-x` run only after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from brian2_gb300 import native, workloads as W
from brian2_gb300.scale import DeviceCSR

pytestmark = pytest.mark.gpu


def _lib():
    L = C.CDLL(native.build_scale())
    L.b200s_noalloc_scratch_bytes.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double]
    L.b200s_noalloc_scratch_bytes.restype = C.c_int64
    L.b200s_fixed_indegree_csr_noalloc.argtypes = [
        C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
        C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64]
    L.b200s_last_error.restype = C.c_char_p
    return L


def _noalloc(L, seed, pid, n_src, src_off, n_post, K):
    import torch
    we, wi, dmin, dspan = W.delay_constants()
    s0, s1 = int(dmin / W.DT + 0.5), int((dmin + dspan) / W.DT + 0.5)
    nseg = n_src * (s1 - s0 + 1) + 1
    # the caller owns the outputs (here: tensors from torch's allocator)
    seg = torch.full((nseg,), -1, dtype=torch.int64, device="cuda")
    post = torch.full((n_post * K,), -1, dtype=torch.int32, device="cuda")
    pre = torch.full((n_post * K,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    lo, hi = C.c_int32(), C.c_int32()
    r = L.b200s_fixed_indegree_csr_noalloc(seed, pid, n_src, src_off, n_post, K, dmin, dspan, W.DT,
                                           C.byref(lo), C.byref(hi), seg.data_ptr(), nseg, post.data_ptr(),
                                           pre.data_ptr(), n_post * K)
    assert r == 0, L.b200s_last_error().decode()
    assert (lo.value, hi.value) == (s0, s1)
    return seg.cpu().numpy(), post.cpu().numpy(), pre.cpu().numpy()


def _allocating(seed, pid, n_src, src_off, n_post, K):
    we, wi, dmin, dspan = W.delay_constants()
    d = DeviceCSR(seed, pid, n_src, src_off, n_post, K, dmin, dspan, W.DT)
    out = d.host_arrays()
    d.free()
    return out


def test_noalloc_equals_allocating_entry_point_on_consecutive_calls():
    L = _lib()
    cases = [(5, 0, 1600, 0, 2000, 80), (9, 1, 400, 1600, 900, 20), (5, 0, 1600, 0, 2000, 80), (7, 1, 60, 3, 500, 50)]
    for case in cases:
        assert L.b200s_noalloc_scratch_bytes(case[2], case[4], case[5], 1e-4, 4.9e-3, W.DT) < 16 << 20
        got = _noalloc(L, *case)
        ref = _allocating(*case)
        for a, b, name in zip(got, ref, ("segptr", "post", "pre")):
            np.testing.assert_array_equal(a, b, err_msg=f"{name} differs for {case}")


def test_noalloc_rejects_networks_beyond_its_scratch():
    L = _lib()
    lo, hi = C.c_int32(), C.c_int32()
    # 100,000 targets x 1000 sources needs far more than 16 MiB of temporaries
    assert L.b200s_noalloc_scratch_bytes(800_000, 100_000, 1000, 1e-4, 4.9e-3, W.DT) > 16 << 20
    r = L.b200s_fixed_indegree_csr_noalloc(1, 0, 800_000, 0, 100_000, 1000, 1e-4, 4.9e-3, W.DT,
                                           C.byref(lo), C.byref(hi), None, 0, None, None, 0)
    assert r == 7   # B200S_STATUS_SCRATCH_LIMIT: its own code, apart from a sampling failure (3)
    assert b"too large for the allocation-free path" in L.b200s_last_error()
