"""Golden cases: which committed spec and which native builder reproduce each
fixture of tests/golden (generated by tests/golden/make_golden.py)."""
from brian2_gb300 import workloads as W

CASES = {
    # fixture: (spec, builder, steps simulated by the fixture)
    "cuba_small_f64": ("cuba_f64", lambda s: W.build_cuba(s, N=500, seed=7), 5000),
    "cuba_f64": ("cuba_f64", lambda s: W.build_cuba(s, N=4000, seed=1234), 10000),
    "cobahh_small_f64": ("cobahh_f64", lambda s: W.build_cobahh(s, N=400, seed=3), 1000),
    "cobahh_f64": ("cobahh_f64", lambda s: W.build_cobahh(s, N=4000, seed=1234), 1000),
    "cobahh_f32": ("cobahh_f32", lambda s: W.build_cobahh(s, N=4000, seed=1234), 1000),
    "delays_small_f64": ("delays_f64", lambda s: W.build_delays(s, N=2000, K=100, seed=5), 3000),
    "delays_f64": ("delays_f64", lambda s: W.build_delays(s, N=10000, K=1000, seed=1234), 2000),
    # the full simulated second of the benchmark configurations
    "cobahh_1s_f64": ("cobahh_f64", lambda s: W.build_cobahh(s, N=4000, seed=1234), 10000),
    "delays_1s_f64": ("delays_f64", lambda s: W.build_delays(s, N=10000, K=1000, seed=1234), 10000),
}

SYN_KEYS = (("synapses_pre", "Ce"), ("synapses_1_pre", "Ci"))
