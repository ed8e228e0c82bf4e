"""THE ORACLE for the adjoint -- test infrastructure only.

The same network as brian2_gb300/csrc/b200_adjoint.cu written as an unrolled
float64 torch program, differentiated by autograd.  The spike rule is the hard
threshold (no surrogate): autograd sees the crossing fraction
phi = (Vt - v)/(vm - v) at spiking neurons and the reset as a `where`, which
is exactly the adjoint's event terms.  Pinned on the CPU by central finite
differences (tests/test_adjoint_ref.py).
"""
import math

import numpy as np
import torch


def forward(W, W_out, taum, prob, cfg, device="cpu"):
    dt, El, Vt, Vr, taus = cfg.dt, cfg.El, cfg.Vt, cfg.Vr, cfg.taus
    dtype = W.dtype
    a_m = torch.exp(-dt / taum)
    a_s = math.exp(-dt / taus)
    c = taus * (a_s - a_m) / (taus - taum)
    s0 = torch.as_tensor(prob["state0"], dtype=dtype, device=device)
    nh, no = cfg.n_h, cfg.n_o
    v, I, vo, Io = s0[:nh], s0[nh:2 * nh], s0[2 * nh:2 * nh + no], s0[2 * nh + no:]
    X = np.zeros((cfg.steps, cfg.n_in))
    for n in range(cfg.steps):
        X[n, prob["in_ids"][prob["in_ptr"][n]:prob["in_ptr"][n + 1]]] = 1.0
    X = torch.as_tensor(X, dtype=dtype, device=device)
    out = []
    for n in range(cfg.steps):
        vm = El + a_m * (v - El) + c * I
        spk = (vm > Vt).detach()
        den = torch.where(spk, vm - v, torch.ones_like(v))
        r = 1 - (Vt - v) / den
        es = torch.exp(-r * dt / taus)
        em = torch.exp(-r * dt / taum)
        f = taus * (es - em) / (taus - taum)
        zero = torch.zeros_like(f)
        sf = torch.where(spk, f, zero)
        se = torch.where(spk, es, zero)
        vo_new = El + a_m * (vo - El) + c * Io + sf @ W_out
        Io_new = a_s * Io + se @ W_out
        v = torch.where(spk, torch.full_like(vm, Vr), vm)
        I = a_s * I + X[n] @ W
        vo, Io = vo_new, Io_new
        out.append(vo)
    return torch.stack(out)


def loss_and_grads(prob, cfg, device="cpu"):
    W = torch.tensor(prob["W"], dtype=torch.float64, device=device, requires_grad=True)
    Wo = torch.tensor(prob["W_out"], dtype=torch.float64, device=device, requires_grad=True)
    taum = torch.tensor(cfg.taum, dtype=torch.float64, device=device, requires_grad=True)
    vo = forward(W, Wo, taum, prob, cfg, device)
    target = torch.as_tensor(prob["target"], dtype=torch.float64, device=device)
    loss = ((vo - target) ** 2).mean()
    loss.backward()
    return loss.item(), W.grad.cpu().numpy(), Wo.grad.cpu().numpy(), float(taum.grad), vo.detach().cpu().numpy()


def loss_at(prob, cfg, W=None, W_out=None, taum=None, device="cpu"):
    with torch.no_grad():
        W = torch.tensor(prob["W"] if W is None else W, dtype=torch.float64, device=device)
        Wo = torch.tensor(prob["W_out"] if W_out is None else W_out, dtype=torch.float64, device=device)
        tm = torch.tensor(cfg.taum if taum is None else taum, dtype=torch.float64, device=device)
        vo = forward(W, Wo, tm, prob, cfg, device)
        target = torch.as_tensor(prob["target"], dtype=torch.float64, device=device)
        return float(((vo - target) ** 2).mean())
