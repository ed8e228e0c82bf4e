"""ctypes host for the b200 C ABI (include/b200.h).

:class:`Model` is a compiled network spec (one shared library); :class:`Network`
is a handle on the device: ``n_inst`` independent instances of the model (one
network, or a batched parameter sweep), their state, synapses and monitors.
Every call maps to one ``extern "C"`` entry point; a non-zero status raises
:class:`B200Error` with the library's message, the way Brian's standalone
device raises ``RuntimeError`` for a failed run
(``brian2/devices/cpp_standalone/device.py:1316-1324``).
"""
from __future__ import annotations

import ctypes as C
import numpy as np

from . import native
from .codegen import KIND_NP, spec_tables

_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)

STATUS = {1: "CUDA error", 2: "invalid argument", 3: "capacity", 4: "device wait timed out", 5: "index out of range",
          6: "random stream"}


class B200Error(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"b200 status {status} ({STATUS.get(status, '?')}): {message}")
        self.status = status


def _ptr(a, t=C.c_void_p):
    return a.ctypes.data_as(t)


def _declare(lib):
    h = C.c_void_p
    sig = {
        "b200_create": [C.POINTER(h), C.c_int32, _i32p, C.c_double],
        "b200_destroy": [h],
        "b200_last_error": [h, C.c_char_p, C.c_int64],
        "b200_configure": [h, C.c_int32, _i32p, C.c_int32, C.c_int64, C.c_int32],
        "b200_set_consts": [h, C.c_int32, _f64p, C.c_int32],
        "b200_upload": [h, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64],
        "b200_download": [h, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64],
        "b200_set_synapses": [h, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                              _i32p, _i32p, _i32p, C.c_int32, C.c_int64],
        "b200_set_synapses_csr": [h, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                  C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64],
        "b200_synapse_var_ptr": [h, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)],
        "b200_set_monitor_range": [h, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32],
        "b200_set_statemon": [h, C.c_int32, C.c_int32, _i32p, C.c_int32, _i32p, C.c_int32],
        "b200_run": [h, C.c_int64],
        "b200_get_step": [h, C.c_int32, _i64p],
        "b200_set_step": [h, C.c_int32, C.c_int64],
        "b200_last_run_ms": [h, _f64p],
        "b200_last_kernel_ms": [h, _f64p],
        "b200_spikemon_size": [h, C.c_int32, C.c_int32, _i64p],
        "b200_spikemon_get": [h, C.c_int32, C.c_int32, _i32p, _i32p, _i32p, C.c_int64],
        "b200_spikemon_values": [h, C.c_int32, C.c_int32, C.POINTER(C.c_double), C.c_int64],
        "b200_ratemon_size": [h, C.c_int32, C.c_int32, _i64p],
        "b200_ratemon_get": [h, C.c_int32, C.c_int32, _i32p, C.c_int64],
        "b200_statemon_size": [h, C.c_int32, C.c_int32, _i64p],
        "b200_statemon_get": [h, C.c_int32, C.c_int32, _f64p, C.c_int64],
        "b200_reset_monitors": [h, C.c_int32],
        "b200_model_name": [C.c_char_p, C.c_int64],
        "b200_device_bytes": [h, _i64p],
        "b200_launch_count": [h, _i64p],
        "b200_set_wait_limit": [h, C.c_int64, C.c_int32],
        "b200_set_smem_cache": [h, C.c_int32],
        "b200_set_profiling": [h, C.c_int32],
        "b200_set_clusters": [h, C.c_int32],
        "b200_set_owner": [h, C.c_int32],
        "b200_owner_active": [h, _i32p],
        "b200_set_push": [h, C.c_int32],
        "b200_push_active": [h, _i32p],
        "b200_set_event_capacity": [h, C.c_double],
        "b200_set_generator": [h, C.c_int32, C.c_int32, _i32p, _i32p, C.c_int64, C.c_int32, C.c_int32],
        "b200_set_rng": [h, C.c_int32, C.POINTER(C.c_uint32), C.c_int32],
        "b200_get_rng": [h, C.c_int32, C.POINTER(C.c_uint32), _i32p, _i64p],
        "b200_set_rng_gauss": [h, C.c_int32, C.c_int32, C.c_double],
        "b200_get_rng_gauss": [h, C.c_int32, _i32p, C.POINTER(C.c_double)],
        "b200_get_generator": [h, C.c_int32, C.c_int32, _i32p],
        "b200_launch_plan": [h, _i32p, _i32p, _i32p],
        "b200_profile_phases": [h, _i32p],
        "b200_get_profile": [h, C.c_int32, C.POINTER(C.c_uint64), C.c_int32],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    return lib


class Model:
    """A network spec compiled to its model library."""

    _cache: dict[str, "Model"] = {}

    def __init__(self, spec: dict):
        self.spec = spec
        self.tables = spec_tables(spec)
        self.path = native.build_model(spec)
        self.lib = _declare(native.load(self.path))
        self.group_index = {g["name"]: k for k, g in enumerate(spec["groups"])}
        self.pathway_index = {p["name"]: k for k, p in enumerate(spec.get("pathways", []))}
        self.spkmon_index = {m["name"]: k for k, m in enumerate(spec.get("spike_monitors", []))}
        self.ratemon_index = {m["name"]: k for k, m in enumerate(spec.get("rate_monitors", []))}
        self.statemon_index = {m["name"]: k for k, m in enumerate(spec.get("state_monitors", []))}

    @classmethod
    def get(cls, spec: dict) -> "Model":
        key = native.model_library_path(spec)
        m = cls._cache.get(key)
        if m is None:
            m = cls._cache[key] = Model(spec)
        return m


class Network:
    """Device handle: `n_inst` instances of one model."""

    def __init__(self, model: Model, sizes, dt: float):
        self.model = model
        self.lib = model.lib
        sizes = np.ascontiguousarray(np.asarray(sizes, dtype=np.int32).reshape(-1, len(model.spec["groups"])))
        self.n_inst = sizes.shape[0]
        self.sizes = sizes
        self.dt = float(dt)
        self._h = C.c_void_p()
        self._check(self.lib.b200_create(C.byref(self._h), self.n_inst, _ptr(sizes, _i32p), self.dt))
        self.n_syn = {}

    # -- plumbing -----------------------------------------------------------
    def _check(self, status):
        if status != 0:
            buf = C.create_string_buffer(1024)
            if self._h:
                self.lib.b200_last_error(self._h, buf, 1024)
            raise B200Error(status, buf.value.decode(errors="replace"))

    def close(self):
        if self._h:
            self.lib.b200_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _g(self, group):
        return group if isinstance(group, int) else self.model.group_index[group]

    def _p(self, pw):
        return pw if isinstance(pw, int) else self.model.pathway_index[pw]

    # -- configuration --------------------------------------------------------
    def configure(self, threads=256, ctas_per_inst=1, queue_mode=False, chunk_steps=0, use_graph=False):
        c = np.ascontiguousarray(np.broadcast_to(np.asarray(ctas_per_inst, dtype=np.int32), (self.n_inst,)))
        self._check(self.lib.b200_configure(self._h, int(threads), _ptr(c, _i32p), int(bool(queue_mode)),
                                            int(chunk_steps), int(bool(use_graph))))

    def set_consts(self, inst, values: dict):
        names = self.model.tables["consts"]
        cur = {c["name"]: c["value"] for c in self.model.spec.get("consts", [])}
        cur.update(getattr(self, "_consts", {}).get(inst, {}))
        cur.update(values)
        self.__dict__.setdefault("_consts", {})[inst] = cur
        arr = np.array([float(cur[n]) for n in names], dtype=np.float64)
        self._check(self.lib.b200_set_consts(self._h, int(inst), _ptr(arr, _f64p), len(names)))

    # -- state ----------------------------------------------------------------
    def _var(self, group, var):
        g = self._g(group)
        v = var if isinstance(var, int) else self.model.tables["groups"][g].index(var)
        return g, v, np.dtype(KIND_NP[self.model.tables["group_kinds"][g][v]])

    def upload(self, inst, group, var, values):
        g, v, dt = self._var(group, var)
        a = np.ascontiguousarray(values, dtype=dt)
        self._check(self.lib.b200_upload(self._h, int(inst), 0, g, v, _ptr(a), a.size))

    def download(self, inst, group, var):
        g, v, dt = self._var(group, var)
        a = np.empty(int(self.sizes[inst, g]), dtype=dt)
        self._check(self.lib.b200_download(self._h, int(inst), 0, g, v, _ptr(a), a.size))
        return a

    def set_synapses(self, inst, pathway, pre, post, delay_steps=None, scalar_delay=0,
                     src_range=None, tgt_range=None):
        p = self._p(pathway)
        info = self.model.spec["pathways"][p]
        Ns, Nt = int(self.sizes[inst, info["src"]]), int(self.sizes[inst, info["tgt"]])
        s0, s1 = src_range if src_range is not None else (0, Ns)
        t0, t1 = tgt_range if tgt_range is not None else (0, Nt)
        pre = np.ascontiguousarray(pre, dtype=np.int32)
        post = np.ascontiguousarray(post, dtype=np.int32)
        dptr = None
        if delay_steps is not None:
            d = np.ascontiguousarray(delay_steps, dtype=np.int32)
            dptr = _ptr(d, _i32p)
        self._check(self.lib.b200_set_synapses(self._h, int(inst), p, s0, s1, t0, t1, _ptr(pre, _i32p),
                                               _ptr(post, _i32p), dptr, int(scalar_delay), pre.size))
        self.n_syn[(inst, p)] = pre.size

    def set_synapses_csr(self, inst, pathway, src_range, tgt_range, dmin, dmax, segptr_dev, post_dev,
                         pre_dev, n_syn):
        p = self._p(pathway)
        self._check(self.lib.b200_set_synapses_csr(self._h, int(inst), p, int(src_range[0]), int(src_range[1]),
                                                   int(tgt_range[0]), int(tgt_range[1]), int(dmin), int(dmax),
                                                   C.c_void_p(segptr_dev), C.c_void_p(post_dev),
                                                   C.c_void_p(pre_dev), int(n_syn)))
        self.n_syn[(inst, p)] = int(n_syn)

    def synapse_var_ptr(self, inst, pathway, var):
        p = self._p(pathway)
        v = var if isinstance(var, int) else self.model.tables["pathways"][p].index(var)
        out = C.c_void_p()
        self._check(self.lib.b200_synapse_var_ptr(self._h, int(inst), p, v, C.byref(out)))
        return out.value

    def _svar(self, pathway, var):
        p = self._p(pathway)
        v = var if isinstance(var, int) else self.model.tables["pathways"][p].index(var)
        return p, v, np.dtype(KIND_NP[self.model.tables["pathway_kinds"][p][v]])

    def upload_synapse_var(self, inst, pathway, var, values):
        p, v, dt = self._svar(pathway, var)
        a = np.ascontiguousarray(values, dtype=dt)
        self._check(self.lib.b200_upload(self._h, int(inst), 1, p, v, _ptr(a), a.size))

    def download_synapse_var(self, inst, pathway, var):
        p, v, dt = self._svar(pathway, var)
        a = np.empty(self.n_syn[(inst, p)], dtype=dt)
        self._check(self.lib.b200_download(self._h, int(inst), 1, p, v, _ptr(a), a.size))
        return a

    # -- monitors -------------------------------------------------------------
    def set_generator(self, inst, group, timebins, indices, period_bins=0, last=0):
        """Spikes of a spike generator group: per entry its time bin (sorted)
        and neuron index; the period in bins (0: none) and the cursor."""
        g = self._g(group)
        b = np.ascontiguousarray(timebins, dtype=np.int32)
        i = np.ascontiguousarray(indices, dtype=np.int32)
        if b.shape != i.shape:
            raise ValueError("timebins and indices differ in length")
        self._check(self.lib.b200_set_generator(self._h, int(inst), g, _ptr(b, _i32p), _ptr(i, _i32p), b.size,
                                                int(period_bins), int(last)))

    def set_rng(self, inst, words, position, gauss=None):
        """The random generator of the step loop: the reference's MT19937 state
        (624 words and the position, as the C++ library stores them) and, if
        given, randn()'s kept value as (has, value)."""
        w = np.ascontiguousarray(words, dtype=np.uint32)
        if w.size != 624:
            raise ValueError("624 state words expected")
        self._check(self.lib.b200_set_rng(self._h, int(inst), _ptr(w, C.POINTER(C.c_uint32)), int(position)))
        if gauss is not None and int(gauss[0]):
            self._check(self.lib.b200_set_rng_gauss(self._h, int(inst), 1, float(gauss[1])))

    def rng_gauss(self, inst=0):
        """randn()'s kept value: (has, value)."""
        has, val = C.c_int32(), C.c_double()
        self._check(self.lib.b200_get_rng_gauss(self._h, int(inst), C.byref(has), C.byref(val)))
        return bool(has.value), float(val.value)

    def rng_state(self, inst=0):
        """(words, position, steps generated ahead and not yet consumed)."""
        w = np.zeros(624, np.uint32)
        p, u = C.c_int32(), C.c_int64()
        self._check(self.lib.b200_get_rng(self._h, int(inst), _ptr(w, C.POINTER(C.c_uint32)), C.byref(p), C.byref(u)))
        return w, int(p.value), int(u.value)

    def generator_cursor(self, inst, group):
        """The generator's cursor (the reference's `_lastindex`)."""
        a = C.c_int32(0)
        self._check(self.lib.b200_get_generator(self._h, int(inst), self._g(group), C.byref(a)))
        return int(a.value)

    def set_spikemon_range(self, inst, mon, lo, hi):
        m = mon if isinstance(mon, int) else self.model.spkmon_index[mon]
        self._check(self.lib.b200_set_monitor_range(self._h, int(inst), 0, m, int(lo), int(hi)))

    def set_ratemon_range(self, inst, mon, lo, hi):
        m = mon if isinstance(mon, int) else self.model.ratemon_index[mon]
        self._check(self.lib.b200_set_monitor_range(self._h, int(inst), 1, m, int(lo), int(hi)))

    def set_statemon(self, inst, mon, indices, variables):
        m = mon if isinstance(mon, int) else self.model.statemon_index[mon]
        sm = self.model.spec["state_monitors"][m]
        # a Synapses object's monitor: synapse indices and that pathway's variables
        names = (self.model.tables["pathways"][sm["syn"]] if sm.get("syn", -1) >= 0
                 else self.model.tables["groups"][sm["group"]])
        idx = np.ascontiguousarray(indices, dtype=np.int32)
        vs = np.ascontiguousarray([v if isinstance(v, int) else names.index(v) for v in variables], dtype=np.int32)
        self._check(self.lib.b200_set_statemon(self._h, int(inst), m, _ptr(idx, _i32p), idx.size,
                                               _ptr(vs, _i32p), vs.size))
        self.__dict__.setdefault("_statemon_shape", {})[(inst, m)] = (vs.size, idx.size)

    def spikes(self, inst=0, mon=0, counts=True, out=None):
        """(i, timestep, per-neuron count) recorded by a spike monitor.
        `counts=False` skips the per-neuron counts (None is returned for them);
        `out=(i, ts)` reads into caller-provided int32 arrays (for instance in
        pinned host memory) of at least the recorded length, and returns views
        of them."""
        m = mon if isinstance(mon, int) else self.model.spkmon_index[mon]
        n = C.c_int64()
        self._check(self.lib.b200_spikemon_size(self._h, int(inst), m, C.byref(n)))
        if out is not None:
            i, ts = out[0][:n.value], out[1][:n.value]
            if i.dtype != np.int32 or ts.dtype != np.int32 or i.size < n.value or ts.size < n.value or \
                    not (i.flags.c_contiguous and ts.flags.c_contiguous):
                raise ValueError("spikes(out=...): contiguous int32 arrays of the recorded length needed")
        else:
            i = np.empty(n.value, np.int32)
            ts = np.empty(n.value, np.int32)
        cnt = None
        if counts:
            g = self.model.spec["spike_monitors"][m]["group"]
            cnt = np.empty(int(self.sizes[inst, g]), np.int32)
        self._check(self.lib.b200_spikemon_get(self._h, int(inst), m, _ptr(i, _i32p), _ptr(ts, _i32p),
                                               _ptr(cnt, _i32p) if cnt is not None else None, n.value))
        return i, ts, cnt

    def spike_values(self, inst=0, mon=0):
        """[spikes, n_vars] float64: the values of the monitor's recorded
        variables (``SpikeMonitor(..., variables=...)``) at each spike, in the
        order of spikes()."""
        m = mon if isinstance(mon, int) else self.model.spkmon_index[mon]
        nv = len(self.model.spec["spike_monitors"][m].get("vars", []))
        n = C.c_int64()
        self._check(self.lib.b200_spikemon_size(self._h, int(inst), m, C.byref(n)))
        a = np.empty((n.value, nv), np.float64)
        if nv:
            self._check(self.lib.b200_spikemon_values(self._h, int(inst), m,
                                                      a.ctypes.data_as(C.POINTER(C.c_double)), n.value))
        return a

    def rate_counts(self, inst=0, mon=0):
        m = mon if isinstance(mon, int) else self.model.ratemon_index[mon]
        n = C.c_int64()
        self._check(self.lib.b200_ratemon_size(self._h, int(inst), m, C.byref(n)))
        a = np.empty(n.value, np.int32)
        self._check(self.lib.b200_ratemon_get(self._h, int(inst), m, _ptr(a, _i32p), n.value))
        return a

    def state_trace(self, inst=0, mon=0):
        """[steps, n_vars, n_rec] float64 values recorded at the start of each step."""
        m = mon if isinstance(mon, int) else self.model.statemon_index[mon]
        n_vars, n_rec = self._statemon_shape[(inst, m)]
        n = C.c_int64()
        self._check(self.lib.b200_statemon_size(self._h, int(inst), m, C.byref(n)))
        a = np.empty((n.value, n_vars, n_rec), np.float64)
        self._check(self.lib.b200_statemon_get(self._h, int(inst), m, _ptr(a, _f64p), n.value))
        return a

    def reset_monitors(self, inst=0):
        self._check(self.lib.b200_reset_monitors(self._h, int(inst)))

    # -- running --------------------------------------------------------------
    def run(self, n_steps: int):
        self._check(self.lib.b200_run(self._h, int(n_steps)))

    def step(self, inst=0):
        t = C.c_int64()
        self._check(self.lib.b200_get_step(self._h, int(inst), C.byref(t)))
        return t.value

    def set_step(self, inst, ts):
        self._check(self.lib.b200_set_step(self._h, int(inst), int(ts)))

    def last_run_ms(self):
        v = C.c_double()
        self._check(self.lib.b200_last_run_ms(self._h, C.byref(v)))
        return v.value

    def last_kernel_ms(self):
        v = C.c_double()
        self._check(self.lib.b200_last_kernel_ms(self._h, C.byref(v)))
        return v.value

    def launches(self):
        v = C.c_int64()
        self._check(self.lib.b200_launch_count(self._h, C.byref(v)))
        return v.value

    def set_clusters(self, enable=True):
        self._check(self.lib.b200_set_clusters(self._h, int(bool(enable))))

    def set_owner(self, enable=True):
        """Owner-mode delivery: True (where the model allows it), False, or
        "auto" (the default: on for networks without synaptic delays)."""
        self._check(self.lib.b200_set_owner(self._h, 2 if enable == "auto" else int(bool(enable))))

    def owner_active(self):
        a = C.c_int32()
        self._check(self.lib.b200_owner_active(self._h, C.byref(a)))
        return bool(a.value)

    def set_push(self, enable=True):
        """Push-mode delivery: True (where the model allows it), False, or
        "auto" (the default: on for float32 models with synaptic delays on
        instances of 2+ CTAs)."""
        self._check(self.lib.b200_set_push(self._h, 2 if enable == "auto" else int(bool(enable))))

    def push_active(self):
        a = C.c_int32()
        self._check(self.lib.b200_push_active(self._h, C.byref(a)))
        return bool(a.value)

    def delivery_mode(self):
        """'push', 'owner' or 'classic': the delivery of the current launch plan."""
        return "push" if self.push_active() else ("owner" if self.owner_active() else "classic")

    def set_event_capacity(self, factor):
        self._check(self.lib.b200_set_event_capacity(self._h, float(factor)))

    def launch_plan(self):
        g, c, sb = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self.lib.b200_launch_plan(self._h, C.byref(g), C.byref(c), C.byref(sb)))
        return dict(grid=g.value, cluster=c.value, state_bytes=sb.value)

    def set_profiling(self, enable=True):
        self._check(self.lib.b200_set_profiling(self._h, int(bool(enable))))

    def profile(self, inst=0):
        """{phase: SM cycles summed over the instance's CTAs and steps}."""
        n = C.c_int32()
        self._check(self.lib.b200_profile_phases(self._h, C.byref(n)))
        a = np.zeros(n.value, np.uint64)
        self._check(self.lib.b200_get_profile(self._h, int(inst), a.ctypes.data_as(C.POINTER(C.c_uint64)), n.value))
        from .codegen import profile_slots
        names = profile_slots(self.model.spec, owner=self.owner_active(), push=self.push_active())
        return {k: int(x) for k, x in zip(names, a) if not k.startswith("unused")}

    def set_smem_cache(self, enable=True):
        self._check(self.lib.b200_set_smem_cache(self._h, int(bool(enable))))

    def set_wait_limit(self, limit_ns, fault_rank=-1):
        self._check(self.lib.b200_set_wait_limit(self._h, int(limit_ns), int(fault_rank)))

    def device_bytes(self):
        v = C.c_int64()
        self._check(self.lib.b200_device_bytes(self._h, C.byref(v)))
        return v.value
