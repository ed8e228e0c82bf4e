"""The float64 unrolled-autograd reference of the adjoint network against
central finite differences (CPU; pins the checker before it checks the GPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import adjoint_ref
from brian2_gb300.adjoint import AdjointConfig, make_problem


def small():
    cfg = AdjointConfig(n_in=20, n_h=60, n_o=3, steps=400, K=50, w_sd=2e-3, seed=3)
    return cfg, make_problem(cfg)


def test_reference_gradient_matches_central_differences():
    cfg, prob = small()
    loss, gW, gWo, gT, vo = adjoint_ref.loss_and_grads(prob, cfg)
    assert np.isfinite(loss) and np.abs(gW).max() > 0 and np.abs(gWo).max() > 0
    # taum
    h = 1e-9
    fd = (adjoint_ref.loss_at(prob, cfg, taum=cfg.taum + h) - adjoint_ref.loss_at(prob, cfg, taum=cfg.taum - h)) / (2 * h)
    assert abs(fd - gT) <= 1e-5 * abs(gT) + 1e-12
    # the largest input-weight and readout-weight entries
    for arr, g, key in ((prob["W"], gW, "W"), (prob["W_out"], gWo, "W_out")):
        idx = np.unravel_index(np.argsort(-np.abs(g), axis=None)[:3], g.shape)
        for a, b in zip(*idx):
            eps = 1e-9
            p, m = arr.copy(), arr.copy()
            p[a, b] += eps
            m[a, b] -= eps
            fd = (adjoint_ref.loss_at(prob, cfg, **{key: p}) - adjoint_ref.loss_at(prob, cfg, **{key: m})) / (2 * eps)
            assert abs(fd - g[a, b]) <= 1e-4 * abs(g[a, b]) + 1e-12, (key, a, b, fd, g[a, b])
