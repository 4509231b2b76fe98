"""cns_diffterm_noalloc: diffterm for callers that cannot allocate device memory while they run
(their device memory belongs to another allocator or a fixed budget, or they cannot afford
cudaMalloc's synchronisation).  It takes caller-owned device buffers and keeps its
temporaries in one fixed device array.  Checked through the C ABI on two calls in a row (the
second call finds the first call's data in the shared array): the first against the golden D
the reference's own diffterm produced (tests/golden/ops_6x9x11.npz), the second against the
oracle's diffterm on another box, with the normwise tolerance of the other FP64 parity tests.
Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from conftest import FP64_TOL, golden, normwise
from cns_nospec_gb300 import initdata as I

pytestmark = pytest.mark.gpu


def _noalloc(lib, L, torch, Q, dx, eta, alam):
    n = [Q.shape[a] - 8 for a in range(3)]
    lo, hi = [4, 4, 4], [x + 3 for x in n]
    q_dev = torch.from_numpy(np.ascontiguousarray(Q)).cuda()
    d_dev = torch.full(tuple(n) + (5,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.cns_diffterm_noalloc(L.iarr(lo), L.iarr(hi), 4, L.darr(dx), ctypes.c_void_p(q_dev.data_ptr()),
                                  ctypes.c_void_p(d_dev.data_ptr()), float(eta), float(alam), None)
    L.check(rc)
    torch.cuda.synchronize()
    return d_dev.cpu().numpy()


def test_diffterm_noalloc_matches_reference_twice(gpu, cns, oracle):
    torch = pytest.importorskip("torch")
    from cns_nospec_gb300 import _lib as L
    lib = cns.load()
    g = golden("ops_6x9x11.npz")
    first = (g["Q"], tuple(g["dx"]), float(g["eta"]), float(g["alam"]), g["D"])
    n2 = (12, 10, 8)
    Q2, _ = oracle.ctoprim(I.initial_state(n2, perturb=1e-3, seed=31), I.box_dx(n2))
    eta2, alam2 = I.ETA * 1.1, I.ALAM * 0.9
    second = (Q2, I.box_dx(n2), eta2, alam2, oracle.diffterm(Q2, I.box_dx(n2), eta2, alam2))
    for Q, dx, eta, alam, want in (first, second):
        got = _noalloc(lib, L, torch, Q, dx, eta, alam)
        assert np.all(np.isfinite(got))
        assert normwise(got, want, interior_only=False).max() <= FP64_TOL


def test_diffterm_noalloc_rejects_boxes_above_its_limit(gpu, cns):
    from cns_nospec_gb300 import _lib as L
    lib = cns.load()
    # 33^3 interior -> 41^3 = 68,921 ghost-inclusive points > 64,000; rejected before any GPU work
    rc = lib.cns_diffterm_noalloc(L.iarr([4, 4, 4]), L.iarr([36, 36, 36]), 4, L.darr([0.1] * 3),
                                  ctypes.c_void_p(16), ctypes.c_void_p(16), 1e-4, 100.0, None)
    assert rc == L.CNS_ERR_CAPACITY
    assert b"64000" in lib.cns_last_error()
