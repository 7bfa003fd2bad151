"""gb_measure_fma_peaks: the measured FP64 / FP32 FMA-pipe rates used as the CUDA-core kernels'
roofline denominators are positive, in the range a GB300 can reach, and repeatable."""
import pytest

import gbblas

pytestmark = pytest.mark.gpu


def test_fma_peaks_plausible_and_repeatable(cuda):
    a = gbblas.measure_fma_peaks()
    b = gbblas.measure_fma_peaks()
    # GB300: FP64 about 1.2-1.4 TFLOP/s nominal, FP32 about 80 TFLOP/s at the maximum clock
    assert 0.3 < a["fp64_tflops"] < 5.0, a
    assert 20.0 < a["fp32_tflops"] < 200.0, a
    assert abs(a["fp64_tflops"] - b["fp64_tflops"]) < 0.2 * a["fp64_tflops"]
    assert abs(a["fp32_tflops"] - b["fp32_tflops"]) < 0.2 * a["fp32_tflops"]
