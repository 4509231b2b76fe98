"""The exact stencil sums as the device computes them (cns_selftest_exact_sums) against the
rational model of tests/test_exact_sum.py: the same bits, and the FP64 fallback reported for
exactly the same tap sets."""
import ctypes

import numpy as np
import pytest

from test_exact_sum import W1, W2, model, tap_sets

pytestmark = pytest.mark.gpu


def test_device_exact_sums_match_the_rational_model(gpu, cns):
    from cns_nospec_gb300 import _lib as L
    sets = tap_sets(16000, seed=12)
    taps = np.ascontiguousarray(np.array(sets, dtype=np.uint64).view(np.float64))
    n = len(sets)
    sums = np.zeros(2 * n)
    ok = np.zeros(2 * n, dtype=np.int32)
    L.check(gpu.cns_selftest_exact_sums(L.dptr(taps), n, L.dptr(sums),
                                        ok.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    bits = sums.view(np.uint64)
    fallbacks = 0
    for q, s in enumerate(sets):
        for col, (w, sgn) in enumerate(((W1, -1), (W2, 1))):
            want = model(s, w, sgn)
            if want is None:
                assert ok[2 * q + col] == 0, (s, w)
                fallbacks += 1
            else:
                assert ok[2 * q + col] == 1 and int(bits[2 * q + col]) == want, (s, w, hex(int(bits[2 * q + col])), hex(want))
    assert 0 < fallbacks < n
