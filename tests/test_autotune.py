"""Launch-shape candidates of the autotuner (host logic, no GPU)."""
from brian2_gb300.autotune import candidates


def test_sweep_candidates_are_queue_mode_single_cta():
    c = candidates(8000, 256)
    assert c and all(q and ctas == 1 for _, ctas, q in c)
    assert {t for t, _, _ in c} == {256, 512, 1024}


def test_plain_candidates_cover_clusters_and_one_cta_per_sm():
    c = candidates(4000, 1)
    assert (512, 1, False) in c and (256, 8, False) in c and (256, 152, False) in c
    assert not any(q for _, _, q in c)


def test_tiny_network_gets_no_wide_shapes():
    c = candidates(600, 1)
    assert all(ctas <= 4 for _, ctas, _ in c)
