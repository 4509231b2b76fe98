"""Device helpers checked against CUDA's own results: the integer-pipe FP32<->FP64
conversions of the mixed form against the hardware casts (bit for bit), and the FP64 peak
probe that serves as the roofline denominator."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_integer_pipe_conversions_match_hardware_casts(gpu, cns):
    lib = cns.load()
    for seed in (1, 2, 3):
        bad = ctypes.c_ulonglong(99)
        cns._lib.check(lib.cns_selftest_conversions(1 << 24, seed, ctypes.byref(bad)))
        assert bad.value == 0


def test_fp64_peak_probe_is_plausible(gpu, cns):
    lib = cns.load()
    tf = ctypes.c_double()
    cns._lib.check(lib.cns_measure_fp64_peak(ctypes.byref(tf)))
    assert 0.3 < tf.value < 100.0
