"""The adjoint kernel (GPU only) against the float64 unrolled-autograd
reference and central finite differences."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import adjoint_ref
from brian2_gb300.adjoint import AdjointConfig, AdjointProblem, forward_trace

pytestmark = pytest.mark.gpu


def medium():
    return AdjointConfig(n_in=50, n_h=300, n_o=4, steps=1200, K=100, w_sd=1.5e-3, seed=11)


def test_forward_trace_equals_reference_f64():
    cfg = medium()
    P = AdjointProblem(cfg, dtype=torch.float64)
    W, Wo, tm = P.params(requires_grad=False)
    vo = forward_trace(P.ctx, W, Wo, float(tm)).cpu().numpy()
    ref = adjoint_ref.forward(torch.tensor(P.prob["W"]), torch.tensor(P.prob["W_out"]),
                              torch.tensor(cfg.taum, dtype=torch.float64), P.prob, cfg).numpy()
    np.testing.assert_allclose(vo, ref, rtol=1e-12, atol=1e-15)


def test_adjoint_equals_autograd_reference_f64():
    cfg = medium()
    P = AdjointProblem(cfg, dtype=torch.float64)
    W, Wo, tm = P.params()
    loss = P.loss(W, Wo, tm)
    loss.backward()
    rl, gW, gWo, gT, _ = adjoint_ref.loss_and_grads(P.prob, cfg)
    assert abs(loss.item() - rl) <= 1e-12 * abs(rl)
    for g, r in ((W.grad.cpu().numpy(), gW), (Wo.grad.cpu().numpy(), gWo)):
        assert np.abs(r).max() > 0
        np.testing.assert_allclose(g, r, rtol=1e-8, atol=1e-9 * np.abs(r).max())
    assert abs(float(tm.grad) - gT) <= 1e-8 * abs(gT)


def test_adjoint_matches_central_differences_f64():
    cfg = medium()
    P = AdjointProblem(cfg, dtype=torch.float64)
    W, Wo, tm = P.params()
    P.loss(W, Wo, tm).backward()
    h = 1e-9
    fd = (P.loss_nograd(W, Wo, cfg.taum + h) - P.loss_nograd(W, Wo, cfg.taum - h)) / (2 * h)
    assert abs(fd - float(tm.grad)) <= 1e-5 * abs(float(tm.grad))
    for t, g in ((W, W.grad), (Wo, Wo.grad)):
        flat = torch.argsort(g.abs().flatten(), descending=True)[:3]
        for k in flat.tolist():
            idx = np.unravel_index(k, tuple(g.shape))
            p, m = t.detach().clone(), t.detach().clone()
            p[idx] += 1e-9
            m[idx] -= 1e-9
            args_p = (p, Wo, cfg.taum) if t is W else (W, p, cfg.taum)
            args_m = (m, Wo, cfg.taum) if t is W else (W, m, cfg.taum)
            fd = (P.loss_nograd(*args_p) - P.loss_nograd(*args_m)) / 2e-9
            assert abs(fd - float(g[idx])) <= 1e-4 * abs(float(g[idx])) + 1e-12


def test_float32_gradients_agree_with_float64():
    cfg = medium()
    grads = []
    for dt in (torch.float32, torch.float64):
        P = AdjointProblem(cfg, dtype=dt)
        W, Wo, tm = P.params()
        P.loss(W, Wo, tm).backward()
        grads.append([W.grad.double().cpu().numpy().ravel(), Wo.grad.double().cpu().numpy().ravel(), float(tm.grad)])
    for a, b in zip(grads[0][:2], grads[1][:2]):
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        assert cos > 0.99, cos
    assert abs(grads[0][2] - grads[1][2]) <= 0.05 * abs(grads[1][2])
