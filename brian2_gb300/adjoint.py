"""Adjoint gradients of an exact-linear LIF network (libb200_adjoint).

Workload (the benchmark's "adjoint gradients" configuration): 200 Poisson
inputs (rates uniform in 5-50 Hz, trains pre-generated from a seed) drive 1000
LIF neurons (taum = 20 ms, exponential synaptic current taus = 5 ms, CUBA
threshold/reset: El = -49 mV, Vt = -50 mV, Vr = -60 mV) through a dense weight
matrix W ~ N(0, 0.5 mV); 10 non-spiking readout neurons receive the hidden
spikes through W_out ~ N(0, 0.5 mV); T = 500 ms, dt = 0.1 ms; the loss is the
mean squared error between the readout membrane potentials and sinusoids
(2-20 Hz, amplitude 5 mV around El, from a seed).  Gradients with respect to
W, W_out and taum come from the hand-written adjoint kernel
(csrc/b200_adjoint.cu) behind :class:`LIFAdjoint`, a ``torch.autograd.Function``
with state checkpoints every K = 100 steps.

Device buffers are torch tensors; the kernels run on torch's current stream.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import native

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = native.load(native.build_adjoint())
        for name in ("b200a_forward_f32", "b200a_forward_f64", "b200a_forward_grid_f32", "b200a_forward_grid_f64"):
            getattr(L, name).argtypes = [C.c_void_p] * 11 + [C.c_void_p]
            getattr(L, name).restype = C.c_int
        for name in ("b200a_backward_f32", "b200a_backward_f64"):
            getattr(L, name).argtypes = [C.c_void_p] * 15 + [C.c_void_p]
            getattr(L, name).restype = C.c_int
        L.b200a_last_error.restype = C.c_char_p
        _lib = L
    return _lib


@dataclass
class AdjointConfig:
    n_in: int = 200
    n_h: int = 1000
    n_o: int = 10
    steps: int = 5000
    K: int = 100
    dt: float = 1e-4
    El: float = -49e-3
    Vt: float = -50e-3
    Vr: float = -60e-3
    taus: float = 5e-3
    taum: float = 20e-3
    w_sd: float = 0.5e-3
    seed: int = 42

    def iparams(self):
        return np.array([self.steps, self.K, self.n_in, self.n_h, self.n_o], np.int32)

    def fparams(self, taum):
        return np.array([self.dt, self.El, self.Vt, self.Vr, self.taus, float(taum)], np.float64)


def make_problem(cfg: AdjointConfig):
    """Seeded inputs, weights, initial state and targets (numpy, float64)."""
    rng = np.random.default_rng(cfg.seed)
    rates = rng.uniform(5.0, 50.0, size=cfg.n_in)
    spikes = rng.random((cfg.steps, cfg.n_in)) < rates * cfg.dt           # Poisson trains on the grid
    in_ptr = np.zeros(cfg.steps + 1, np.int32)
    in_ptr[1:] = np.cumsum(spikes.sum(1))
    in_ids = np.nonzero(spikes)[1].astype(np.int32)                       # ascending per step
    W = rng.normal(0.0, cfg.w_sd, size=(cfg.n_in, cfg.n_h))
    W_out = rng.normal(0.0, cfg.w_sd, size=(cfg.n_h, cfg.n_o))
    v0 = cfg.Vr + rng.random(cfg.n_h) * (cfg.Vt - cfg.Vr)
    state0 = np.concatenate([v0, np.zeros(cfg.n_h), np.full(cfg.n_o, cfg.El), np.zeros(cfg.n_o)])
    freqs = rng.uniform(2.0, 20.0, size=cfg.n_o)
    phases = rng.uniform(0, 2 * math.pi, size=cfg.n_o)
    t = (np.arange(cfg.steps) + 1) * cfg.dt
    target = cfg.El + 5e-3 * np.sin(2 * math.pi * freqs[None, :] * t[:, None] + phases[None, :])
    return dict(in_ptr=in_ptr, in_ids=in_ids, W=W, W_out=W_out, state0=state0, target=target, rates=rates)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Ctx:
    """Device copies of the inputs that do not change during training."""

    def __init__(self, cfg, prob, dtype):
        import torch
        self.cfg = cfg
        self.dtype = dtype
        self.in_ptr = torch.as_tensor(prob["in_ptr"], device="cuda")
        self.in_ids = torch.as_tensor(prob["in_ids"] if len(prob["in_ids"]) else np.zeros(1, np.int32), device="cuda")
        self.state0 = torch.as_tensor(prob["state0"], dtype=dtype, device="cuda")
        self.ip = torch.as_tensor(cfg.iparams())   # host, read by the C entry point
        S = 2 * cfg.n_h + 2 * cfg.n_o
        self.nseg = (cfg.steps + cfg.K - 1) // cfg.K
        self.S = S


def _suffix(dtype):
    import torch
    return "f64" if dtype == torch.float64 else "f32"


def forward_trace(ctx: _Ctx, W, W_out, taum, ckpt=None, spike_count=None, io=None, grid=False):
    """Readout trace vo[steps, n_o] (the state after each step).  grid: the
    readout receives hidden spikes at the end of their step (the reference's
    on_pre timing) instead of at the interpolated crossing time."""
    import torch
    cfg = ctx.cfg
    vo = torch.empty((cfg.steps, cfg.n_o), dtype=ctx.dtype, device="cuda")
    fp = cfg.fparams(taum)
    f = getattr(lib(), ("b200a_forward_grid_" if grid else "b200a_forward_") + _suffix(ctx.dtype))
    r = f(ctx.ip.numpy().ctypes.data, fp.ctypes.data, _ptr(W), _ptr(W_out), _ptr(ctx.in_ptr), _ptr(ctx.in_ids),
          _ptr(ctx.state0), _ptr(vo), _ptr(spike_count), _ptr(ckpt), _ptr(io), _stream())
    if r:
        raise RuntimeError("adjoint forward: " + lib().b200a_last_error().decode())
    return vo


def _make_function():
    import torch

    class LIFAdjoint(torch.autograd.Function):
        """vo_trace = LIFAdjoint.apply(W, W_out, taum, ctx): readout membrane
        potentials [steps, n_o]; backward runs the adjoint kernel."""

        @staticmethod
        def forward(fctx, W, W_out, taum, ctx):
            ckpt = torch.empty((ctx.nseg, ctx.S), dtype=ctx.dtype, device="cuda")
            io = torch.empty((ctx.cfg.steps, ctx.cfg.n_o), dtype=ctx.dtype, device="cuda")
            vo = forward_trace(ctx, W.contiguous(), W_out.contiguous(), float(taum), ckpt=ckpt, io=io)
            fctx.save_for_backward(W, W_out, ckpt, vo, io)
            fctx.taum = float(taum)
            fctx.ctx = ctx
            return vo

        @staticmethod
        def backward(fctx, grad_vo):
            W, W_out, ckpt, vo, io = fctx.saved_tensors
            ctx = fctx.ctx
            cfg = ctx.cfg
            dW = torch.zeros_like(W)
            dWo = torch.zeros_like(W_out)
            dt = torch.zeros(1, dtype=ctx.dtype, device="cuda")
            seg = torch.empty((cfg.K, ctx.S), dtype=ctx.dtype, device="cuda")
            fp = cfg.fparams(fctx.taum)
            f = getattr(lib(), "b200a_backward_" + _suffix(ctx.dtype))
            r = f(ctx.ip.numpy().ctypes.data, fp.ctypes.data, _ptr(W.contiguous()), _ptr(W_out.contiguous()),
                  _ptr(ctx.in_ptr), _ptr(ctx.in_ids), _ptr(ckpt), _ptr(grad_vo.contiguous()), _ptr(seg), _ptr(dW),
                  _ptr(dWo), _ptr(dt), _ptr(vo), _ptr(io), _ptr(ctx.state0), _stream())
            if r:
                raise RuntimeError("adjoint backward: " + lib().b200a_last_error().decode())
            return dW, dWo, dt.reshape(()), None

    return LIFAdjoint


_fn = None


def LIFAdjoint():
    global _fn
    if _fn is None:
        _fn = _make_function()
    return _fn


class AdjointProblem:
    """One training problem on the device: loss(W, W_out, taum) with gradients."""

    def __init__(self, cfg: AdjointConfig = None, dtype=None):
        import torch
        self.cfg = cfg or AdjointConfig()
        self.dtype = dtype or torch.float32
        self.prob = make_problem(self.cfg)
        self.ctx = _Ctx(self.cfg, self.prob, self.dtype)
        self.target = torch.as_tensor(self.prob["target"], dtype=self.dtype, device="cuda")

    def params(self, requires_grad=True):
        import torch
        W = torch.as_tensor(self.prob["W"], dtype=self.dtype, device="cuda").requires_grad_(requires_grad)
        Wo = torch.as_tensor(self.prob["W_out"], dtype=self.dtype, device="cuda").requires_grad_(requires_grad)
        taum = torch.tensor(self.cfg.taum, dtype=self.dtype, device="cuda", requires_grad=requires_grad)
        return W, Wo, taum

    def loss(self, W, W_out, taum):
        vo = LIFAdjoint().apply(W, W_out, taum, self.ctx)
        return ((vo - self.target) ** 2).mean()

    def loss_nograd(self, W, W_out, taum):
        import torch
        with torch.no_grad():
            vo = forward_trace(self.ctx, W.detach().contiguous(), W_out.detach().contiguous(), float(taum))
            return float(((vo - self.target) ** 2).mean())
