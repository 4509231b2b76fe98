"""Failure detection without a GPU fault: the bounded waits inside the kernels give up and
report instead of hanging (an mbarrier nothing arrives on), and the context stays usable."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports(gpu, cns):
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    status = ctypes.c_int(-1)
    L.check(gpu.cns_selftest_bounded_wait(ctypes.byref(status)))
    assert status.value == L.CNS_HEALTH_TIMEOUT
    # the device still works: a short advance afterwards matches a fresh one bit for bit
    n = 12
    U0 = I.initial_state(n, perturb=1e-3, seed=3)
    a, b = U0.copy(), U0.copy()
    cns.advance_host(a, 2, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    cns.advance_host(b, 2, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    assert np.array_equal(a, b) and np.isfinite(a).all()
