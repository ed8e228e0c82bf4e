"""Work counts of the ALU roofline (host logic) and the measured FMA peaks (GPU)."""
import pytest

from brian2_gb300 import roofline, workloads as W


def test_count_ops_of_a_snippet():
    code = ("const double x = _ptr_array_g_x[_idx];\n"
            "const double _x = 1.0f*(a * exp(- x))/(b + (c * _exprel(x - 2.0e-3)));\n"
            "x = _x;\n_ptr_array_g_x[_idx] = x;\n")
    ops = roofline.count_ops(code)
    # a*exp, /, b+, c*, x-  (1.0f* and the unary minus are not counted)
    assert ops["flops"] == 5
    assert ops["calls"] == {"exp": 1, "_exprel": 1}


def test_cobahh_update_counts():
    ops = roofline.update_ops(W.load_spec("cobahh_f64"))
    # the generated exponential-Euler update of the Hodgkin-Huxley benchmark:
    # 11 exp, 8 exprel (expm1), 10 pow calls per neuron-step
    assert ops["calls"] == {"exp": 11, "_exprel": 8, "_brian_pow": 10}
    assert 80 <= ops["flops"] <= 120
    assert roofline.update_ops(W.load_spec("cuba_f64"))["flops"] == 8


@pytest.mark.gpu
def test_fma_peaks_are_measured():
    f32 = roofline.fma_peak_gflops(False)
    f64 = roofline.fma_peak_gflops(True)
    print(f"\nFMA peaks: float32 {f32:.0f} GFLOP/s, float64 {f64:.0f} GFLOP/s")
    assert 5_000 < f32 < 500_000
    assert 100 < f64 < f32
