"""Spike generator groups on the GPU against the oracle (GPU only): the
spike_generator scenario's network with other spike lists -- no period, a
cursor that starts past the first entries (with and without a period, which
resets it at the first step), no entries at all, every input in the same few
bins -- bit-exact in rasters, state and the final cursor
(templates/spikegenerator.cpp:5-31)."""
import os

import numpy as np
import pytest

from brian2_gb300.job import load_job, run_job, write_job
from oracle import run_job_on_oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _lists(case, n_in, rng):
    if case == "no_period":
        bins = np.sort(rng.integers(0, 1300, 600))
        idx = np.concatenate([rng.permutation(n_in)[: int((bins == b).sum())] for b in np.unique(bins)])
        return bins, idx, 0, 0
    if case in ("cursor", "cursor_wrap"):           # the first 150 entries already emitted
        bins = np.repeat(np.arange(0, 400, 2), 2)
        idx = np.tile([3, 77], 200)
        return bins, idx, (400 if case == "cursor_wrap" else 0), 150
    if case == "empty":
        return np.zeros(0, np.int32), np.zeros(0, np.int32), 0, 0
    if case == "dense":
        bins = np.repeat([5, 6, 7, 300], n_in)
        idx = np.tile(np.arange(n_in), 4)
        return bins, idx, 0, 0
    raise ValueError(case)


@pytest.mark.parametrize("case", ["no_period", "cursor", "cursor_wrap", "empty", "dense"])
@pytest.mark.parametrize("ctas,owner", [(1, "auto"), (4, True), (4, False), (20, "auto")])
def test_generator_matches_oracle(case, ctas, owner, tmp_path):
    spec, init, job = load_job(os.path.join(HERE, "golden", "jobs", "spike_generator"))
    gi = next(k for k, g in enumerate(spec["groups"]) if g.get("generator"))
    n_in = int(init[f"g{gi}_N"])
    bins, idx, period, last = _lists(case, n_in, np.random.default_rng(7))
    order = np.lexsort((idx, bins))                # the reference's order: by time bin, then neuron
    init[f"g{gi}_gen_bins"] = np.asarray(bins, np.int32)[order]
    init[f"g{gi}_gen_index"] = np.asarray(idx, np.int32)[order]
    init[f"g{gi}_gen_period"] = np.int64(period)
    init[f"g{gi}_gen_last"] = np.int64(last)
    write_job(str(tmp_path), spec, init, job["runs"], job["dt"])
    ref = run_job_on_oracle(str(tmp_path))
    out = run_job(str(tmp_path), threads=128, ctas_per_inst=ctas, write=False, owner=owner)
    assert int(out[f"g{gi}_gen_last"]) == int(ref[f"g{gi}_gen_last"])
    for mi in range(len(spec["spike_monitors"])):
        np.testing.assert_array_equal(out[f"sm{mi}_i"], ref[f"sm{mi}_i"])
        np.testing.assert_array_equal(out[f"sm{mi}_ts"], ref[f"sm{mi}_ts"])
    np.testing.assert_array_equal(out["rm0_counts"], ref["rm0_counts"])
    for gk, g in enumerate(spec["groups"]):
        for v in g["vars"]:
            np.testing.assert_array_equal(out[f"g{gk}_{v['name']}"], ref[f"g{gk}_{v['name']}"], err_msg=v["name"])
