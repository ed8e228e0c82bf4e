"""The adjoint benchmark's forward pass pinned to the reference.

The network of the "adjoint gradients" configuration is also written as a
Brian script (oracle/brian_configs.py:adjoint_network): SpikeGeneratorGroup
inputs, the exact-linear LIF hidden layer, the readout driven by on_pre.  The
reference ran it (tests/golden/adjoint_forward_f64: hidden raster, readout
potentials after every step) and set_device('b200') wrote it as a job
(tests/golden/jobs/adjoint_forward).  Checked here: the oracle against the
reference (CPU), the step engine running the plugin's job, and the adjoint
library's forward pass with the readout driven at the step grid, against the
reference (GPU); and what the adjoint's interpolated delivery changes.
"""
import os

import numpy as np
import pytest

from oracle import run_job_on_oracle

HERE = os.path.dirname(os.path.abspath(__file__))
JOB = os.path.join(HERE, "golden", "jobs", "adjoint_forward")
REL = 1e-9  # float64 readout potentials where the arithmetic differs (atomic order, host/device libm)


def fixture():
    z = np.load(os.path.join(HERE, "golden", "adjoint_forward_f64.npz"))
    return {k: z[k] for k in z.files}


def test_oracle_reproduces_reference_forward():
    z = fixture()
    out = run_job_on_oracle(JOB)
    np.testing.assert_array_equal(out["sm0_i"], z["spk_i"])
    np.testing.assert_array_equal(out["sm0_ts"], z["spk_ts"])
    np.testing.assert_array_equal(out["stm0_trace"][:, 0, :], z["vo"])


@pytest.mark.gpu
@pytest.mark.parametrize("ctas", [1, 4])
def test_step_engine_runs_the_plugin_job(ctas):
    """The plugin's job of the script on the GPU: the hidden raster identical
    to the reference's, the readout potentials within 1e-9 (the weights are
    heterogeneous, so the order of a step's float64 additions may differ)."""
    from brian2_gb300.job import run_job
    z = fixture()
    out = run_job(JOB, ctas_per_inst=ctas, write=False)
    np.testing.assert_array_equal(out["sm0_i"], z["spk_i"])
    np.testing.assert_array_equal(out["sm0_ts"], z["spk_ts"])
    vo = out["stm0_trace"][:, 0, :]
    assert np.max(np.abs(vo - z["vo"]) / np.abs(z["vo"])) < REL


@pytest.mark.gpu
def test_adjoint_library_grid_forward_equals_reference():
    """b200a_forward_grid_f64: the hidden spike counts per neuron equal the
    reference raster's and every readout potential agrees within 1e-9 (each
    hidden spike moves the readout by ~0.5 mV, so any raster difference would
    show); the interpolated delivery of the adjoint pass is reported against
    it (loss and potentials)."""
    import torch
    from brian2_gb300.adjoint import AdjointProblem, forward_trace
    z = fixture()
    P = AdjointProblem(dtype=torch.float64)
    W, Wo, tm = P.params(requires_grad=False)
    counts = torch.zeros(P.cfg.n_h, dtype=torch.int32, device="cuda")
    vo = forward_trace(P.ctx, W, Wo, float(tm), spike_count=counts, grid=True).cpu().numpy()
    np.testing.assert_array_equal(counts.cpu().numpy(), np.bincount(z["spk_i"], minlength=P.cfg.n_h))
    rel = np.max(np.abs(vo - z["vo"]) / np.abs(z["vo"]))
    assert rel < REL, rel
    vi = forward_trace(P.ctx, W, Wo, float(tm)).cpu().numpy()
    tgt = P.prob["target"]
    l_grid, l_int = float(((vo - tgt) ** 2).mean()), float(((vi - tgt) ** 2).mean())
    print(f"\nconfig-4 forward: grid delivery vs reference max rel {rel:.2e}; loss grid {l_grid:.6e}, "
          f"interpolated {l_int:.6e} ({(l_int - l_grid) / l_grid:+.3%}); readout max |diff| "
          f"{np.max(np.abs(vi - vo)) * 1e3:.4f} mV")
