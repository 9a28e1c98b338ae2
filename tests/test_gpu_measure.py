"""The library's measurement entry points on the GPU: the FP32 rate of a
plain FMA-chain kernel and the FMA / MUFU tanh rates per SM clock, which the
benchmark reports beside its roofline figures."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_fp32_peak_and_pipe_rates_are_plausible():
    import torch
    import tiralib_gb300 as tv
    L = tv.lib()
    tf, mhz = ctypes.c_double(0.0), ctypes.c_double(0.0)
    assert L.tvgb_fp32_peak(ctypes.byref(tf), ctypes.byref(mhz), None) == 0
    props = torch.cuda.get_device_properties(0)
    nominal = props.multi_processor_count * 128 * 2 * mhz.value * 1e6 / 1e12
    assert 200.0 < mhz.value < 4000.0
    assert 0.3 * nominal < tf.value <= 1.05 * nominal
    rates = (ctypes.c_double * 4)()
    assert L.tvgb_pipe_rates(rates, None) == 0
    fma, tanh32, tanh16, clk = list(rates)
    assert 32.0 < fma <= 130.0            # FP32 FMAs per SM clock (128 lanes)
    assert 2.0 < tanh32 <= 40.0 and 2.0 < tanh16 <= 80.0
    assert abs(clk - mhz.value) < 0.2 * mhz.value
    assert L.tvgb_fp32_peak(None, None, None) == 1       # a NULL result is refused
