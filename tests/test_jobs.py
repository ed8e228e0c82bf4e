"""Jobs written by the set_device('b200') plugin from the reference's own
scripts (tests/golden/make_jobs.py): the network they carry is the
reference's construction, array for array (no GPU)."""
import os

import numpy as np
import pytest

from brian2_gb300.job import load_job

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["cuba_small_f64", "delays_small_f64", "cobahh_small_f64"]
# Brian names the first Synapses object "synapses", the second "synapses_1"
FIXTURE_KEY = {"synapses_pre": "Ce", "synapses_1_pre": "Ci"}


@pytest.mark.parametrize("case", CASES)
def test_job_carries_the_reference_network(case, golden):
    spec, init, job = load_job(os.path.join(HERE, "golden", "jobs", case))
    meta, z = golden(case)
    assert int(init["g0_N"]) == meta["N"]
    np.testing.assert_array_equal(init["g0_v"], z["v0"])
    assert sum(job["runs"]) == meta["n_steps"] and job["dt"] == pytest.approx(1e-4)
    assert len(spec["pathways"]) == 2
    for pi, p in enumerate(spec["pathways"]):
        k = FIXTURE_KEY[p["name"]]
        np.testing.assert_array_equal(init[f"p{pi}_pre"], z[f"{k}_pre"])
        np.testing.assert_array_equal(init[f"p{pi}_post"], z[f"{k}_post"])
        d = z[f"{k}_delay"]
        if d.size > 1:
            np.testing.assert_array_equal(init[f"p{pi}_delay_steps"], (d / 1e-4 + 0.5).astype(np.int32))
        if f"{k}_w" in z:
            np.testing.assert_array_equal(init[f"p{pi}_w"], z[f"{k}_w"])


SCENARIOS = ["lif_refractory", "hetero_delays", "subgroup_monitors", "input_group", "presynaptic_read",
             "spike_generator", "stdp", "gap_junctions", "explicit_methods", "poisson_input", "poisson_drive",
             "noise_inputs", "regular_ops", "host_sets"]


@pytest.mark.parametrize("name", SCENARIOS)
def test_scenario_jobs_describe_their_features(name):
    """The plugin's spec of each scenario carries the feature it exercises."""
    spec, init, job = load_job(os.path.join(HERE, "golden", "jobs", name))
    names = {v["name"] for g in spec["groups"] for v in g["vars"]}
    if name == "lif_refractory":
        assert {"not_refractory", "lastspike"} <= names
    if name == "hetero_delays":
        assert "p0_delay_steps" in init and init["p0_delay_steps"].max() > 0 and "p0_w" in init
    if name == "subgroup_monitors":
        assert tuple(init["sm0_range"]) == (100, 300) and tuple(init["rm0_range"]) == (0, 50)
        assert list(init["stm0_idx"]) == [0, 10, 250, 499]
    if name == "input_group":
        assert len(spec["groups"]) == 2 and {p["src"] for p in spec["pathways"]} == {0, 1}
    if name in ("poisson_input", "poisson_drive", "noise_inputs"):  # the generator state travels
        assert init["rng_words"].dtype == np.uint32 and init["rng_words"].size == 624
        assert 0 <= int(init["rng_position"]) <= 624 and init["rng_gauss"].shape == (2,)
        for si, d in enumerate(spec["draws"]):  # every draw site's calls are its macros
            if d["kind"] in ("rand", "randn"):
                blk = next(b for b in ("update", "threshold") if (spec["groups"][d["group"]].get(b) or {}).get("draw") == si)
                code = spec["groups"][d["group"]][blk]["vector"]
            else:
                code = next(inp for inp in spec["inputs"] if inp["draw"] == si)["code"]["vector"]
            assert code.count(f"_b200_draw_{si}_") == d["calls"] and "_rand(" not in code and "_randn(" not in code
    if name == "poisson_input":  # rand() in two PoissonGroups' thresholds
        assert [d["kind"] for d in spec["draws"]] == ["rand", "rand"]
    if name == "poisson_drive":  # a PoissonGroup, then three inputs by inversion (one reversed)
        assert [d["kind"] for d in spec["draws"]] == ["rand", "binomial", "binomial", "binomial"]
        assert [d["binom"]["reverse"] for d in spec["draws"][1:]] == [False, False, True]
        assert [(d["lo"], d["hi"]) for d in spec["draws"][1:]] == [(0, -1), (50, 250), (300, 400)]
    if name == "noise_inputs":  # randn() in two updates (schedule order: by name), both samplers
        assert [(d["kind"], d["calls"]) for d in spec["draws"]] == [("randn", 1), ("randn", 2), ("binormal", 1),
                                                                    ("binomial", 1)]
        assert int(init["rng_gauss"][0]) == 1  # the initial values left one kept
    if name == "regular_ops":  # run_regularly: slots, clock multiples, a subgroup range
        ops = spec["groups"][0]["ops"]
        assert [(o["when"], o["every"], o["lo"], o["hi"]) for o in ops] == [("start", 10, 0, -1), ("start", 20, 50, 150),
                                                                            ("end", 1, 0, -1)]
        assert "_sub_idx = _b200_abs_idx;" in ops[1]["code"]["vector"] and "__sub_idx[" not in ops[1]["code"]["vector"]
    if name == "host_sets":  # assignments between and after the runs, in the reference's three forms
        assert job["runs"] == [500, 500, 500]
        assert [(a["after"], a["var"], a["indexed"]) for a in job["actions"]] == [
            (0, "I", False), (0, "v", True), (1, "I", True), (2, "I", False)]
        np.testing.assert_array_equal(init["act1_index"], np.arange(10))
        assert init["act2_index"].tolist() == [5] and float(init["act2_values"][0]) == 0.0
    if name == "gap_junctions":  # a summed variable over a Synapses object without on_pre
        (sm,) = spec["summed"]
        pw = spec["pathways"][sm["pathway"]]
        assert pw.get("events") is False and [v["name"] for v in pw["vars"]] == ["w"]
        assert spec["groups"][sm["tgt_group"]]["vars"][sm["tgt_var"]]["name"] == "Igap" and sm["index_post"]
    if name == "stdp":  # on_pre and on_post pathways of one Synapses object share its variables
        pre, post = spec["pathways"]
        assert post.get("alias") == 0 and pre.get("alias", -1) == -1
        assert [v["name"] for v in pre["vars"]] == [v["name"] for v in post["vars"]] == ["Apost", "Apre", "lastupdate", "w"]
        assert (pre["src"], pre["tgt"]) == (post["tgt"], post["src"])
        assert "p1_w" not in init and init["p0_pre"].size == init["p1_pre"].size
        assert int(init["p1_delay_steps"].max()) == 0 and int(init["p0_delay_steps"].max()) > 0
    if name == "spike_generator":
        gi = next(k for k, g in enumerate(spec["groups"]) if g.get("generator"))
        bins = init[f"g{gi}_gen_bins"]
        assert int(init[f"g{gi}_gen_period"]) == 400 and int(init[f"g{gi}_gen_last"]) == 0
        assert bins.size == 400 and np.all(np.diff(bins) >= 0) and bins.max() < 400
        assert [v["name"] for v in spec["groups"][gi]["vars"]] == ["i"]
        assert any(p["src"] == gi for p in spec["pathways"])
    if name == "presynaptic_read":
        assert any("_presynaptic_idx" in (p["on_pre"].get("vector_device") or p["on_pre"]["vector"])
                   for p in spec["pathways"])


def test_progress_report_lines(capsys):
    """run(report='text'/'stderr'): the job runner prints the reference's
    standard report lines (device.py:1843-1887) to the chosen stream."""
    from brian2_gb300.job import _format_time, _report
    assert _format_time(0.2) == "< 1s" and _format_time(61) == "1m 1s" and _format_time(3600) == "1h 0m 0s"
    _report("stdout", 0.0, 0.0, 0.0, 0.5)
    _report("stdout", 2.0, 0.5, 0.0, 0.5)
    _report("stderr", 4.0, 1.0, 0.0, 0.5)
    out, err = capsys.readouterr()
    assert out.splitlines() == ["Starting simulation at t=0 s for duration 0.5 s",
                                "0.25 s (50%) simulated in 2s, estimated 2s remaining."]
    assert err.splitlines() == ["0.5 s (100%) simulated in 4s"]
