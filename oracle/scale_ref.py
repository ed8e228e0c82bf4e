"""THE ORACLE -- test infrastructure only: ctypes wrapper of oracle/scale_ref.c."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "scale_ref.c")
        out = os.path.join(HERE, "_build", "libscale_ref.so")
        if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
            os.makedirs(os.path.dirname(out), exist_ok=True)
            tmp = out + f".tmp{os.getpid()}"
            subprocess.run([shutil.which("gcc") or "gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                            "-fno-fast-math", src, "-o", tmp], check=True)
            os.replace(tmp, out)
        _lib = C.CDLL(out)
    return _lib


def fixed_indegree_csr(seed, path_id, n_src, src_off, n_post, K, dmin, dspan, dt):
    L = lib()
    n = n_post * K
    pre = np.empty(n, np.int32)
    slot = np.empty(n, np.int32)
    r = L.scale_ref_sample(C.c_uint64(seed), C.c_uint32(path_id), C.c_uint32(n_src), C.c_int(K), C.c_int(n_post),
                           C.c_double(dmin), C.c_double(dspan), C.c_double(dt), pre.ctypes.data_as(C.c_void_p),
                           slot.ctypes.data_as(C.c_void_p))
    assert r == 0
    s0, s1 = int(dmin / dt + 0.5), int((dmin + dspan) / dt + 0.5)
    W = s1 - s0 + 1
    seg = np.empty(n_src * W + 1, np.int64)
    post_csr = np.empty(n, np.int32)
    pre_csr = np.empty(n, np.int32)
    L.scale_ref_csr(pre.ctypes.data_as(C.c_void_p), slot.ctypes.data_as(C.c_void_p), C.c_int64(n), C.c_int(K),
                    C.c_int(n_src), C.c_int(s0), C.c_int(W), C.c_int(src_off), seg.ctypes.data_as(C.c_void_p),
                    post_csr.ctypes.data_as(C.c_void_p), pre_csr.ctypes.data_as(C.c_void_p))
    return dict(seg=seg, post=post_csr, pre=pre_csr, slot_min=s0, slot_max=s1, pre_tm=pre, slot_tm=slot)
