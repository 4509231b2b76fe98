"""Host arrays moved in place by the GPU over the CPU-GPU link against the staged path (a copy
through a device buffer): bit-identical results from cns_new_advance, cns_advance_host (FP64
and mixed; 0, 1 and 3 steps; a non-cubic box) and Box upload/download, ghost cells included.
In place: page-locked memory, and pageable memory on a device that reads host memory through
the host's page tables (NVLink-C2C); staged: pageable memory with that turned off
(cns_set_pageable_in_place(0)).  The input's ghost cells are filled with garbage: only the
interior may be read."""
import contextlib
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned_copy(a):
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    out = t.numpy()
    out[...] = a
    return out, t  # the tensor owns the page-locked memory


def garbage_ghosts(U, seed):
    rng = np.random.default_rng(seed)
    G = U.copy()
    inner = np.zeros(U.shape[:3], dtype=bool)
    inner[4:-4, 4:-4, 4:-4] = True
    G[~inner] = rng.uniform(-1e3, 1e3, size=(int((~inner).sum()), U.shape[3]))
    return G


def in_place(lib, a, nbytes=None):
    flag = ctypes.c_int(-1)
    nb = a.nbytes if nbytes is None else nbytes
    assert lib.cns_host_in_place(ctypes.c_void_p(a.ctypes.data), ctypes.c_longlong(nb), ctypes.byref(flag)) == 0
    return flag.value


@contextlib.contextmanager
def staged_pageable(lib):
    """Pageable host arrays take the staged path inside the block."""
    assert lib.cns_set_pageable_in_place(0) == 0
    try:
        yield
    finally:
        lib.cns_set_pageable_in_place(1)


def pageable_in_place_supported(lib):
    return in_place(lib, np.zeros((8, 8, 8, 5))) == 1


def test_in_place_query(gpu, cns):
    a = np.zeros((8, 8, 8, 5))
    p, _keep = pinned_copy(a)
    assert in_place(gpu, p) == 1
    with staged_pageable(gpu):
        assert in_place(gpu, a) == 0
        assert in_place(gpu, p) == 1  # page-locked memory is unaffected
    # a range running past the end of the page-locked allocation is refused
    assert in_place(gpu, p, nbytes=1 << 40) == 0


def test_new_advance_pinned_equals_pageable(gpu, cns):
    from cns_nospec_gb300 import initdata as I
    n = 24
    U0 = garbage_ghosts(I.initial_state(n, perturb=1e-3, seed=5), 1)
    h = cns.read_configurations(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    Ua = U0.copy()
    Ub, _keep = pinned_copy(U0)
    assert in_place(gpu, Ub) == 1
    for _ in range(2):
        with staged_pageable(gpu):
            dta = cns.new_advance(Ua, None, None, None, None, h)
        dtb = cns.new_advance(Ub, None, None, None, None, h)
        assert dta == dtb
        assert np.array_equal(Ua.view(np.uint64), Ub.view(np.uint64))


@pytest.mark.parametrize("precision,n", [(0, (20, 12, 36)), (1, (20, 12, 36)), (0, (4, 5, 6))])
@pytest.mark.parametrize("nsteps", [0, 1, 3])
def test_advance_host_pinned_equals_pageable(gpu, cns, precision, n, nsteps):
    # (4, 5, 6): every interior cell is within 4 of both faces, so each has images on both sides
    from cns_nospec_gb300 import initdata as I
    U0 = garbage_ghosts(I.initial_state(n, perturb=1e-3, seed=7), 2)
    Ua = U0.copy()
    Ub, _keep = pinned_copy(U0)
    with staged_pageable(gpu):
        dta = cns.advance_host(Ua, nsteps, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision)
    dtb = cns.advance_host(Ub, nsteps, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision)
    assert np.array_equal(dta, dtb)
    assert np.array_equal(Ua.view(np.uint64), Ub.view(np.uint64))
    if nsteps == 0:  # the interior is unchanged and the ghosts are its periodic images
        assert np.array_equal(Ub, I.fill_periodic(U0.copy()))


@pytest.mark.parametrize("precision", [0, 1])
def test_box_upload_download_pinned_equals_pageable(gpu, cns, precision):
    from cns_nospec_gb300 import initdata as I
    n = (16, 28, 20)
    U0 = garbage_ghosts(I.initial_state(n, perturb=1e-3, seed=9), 3)
    outs = []
    for pin in (False, True):
        src, keep = pinned_copy(U0) if pin else (U0.copy(), None)
        box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=precision)
        dst, keep2 = pinned_copy(np.full(U0.shape, np.nan)) if pin else (np.full(U0.shape, np.nan), None)
        with contextlib.ExitStack() as stack:
            if not pin:
                stack.enter_context(staged_pageable(gpu))
            box.upload(src)
            box.advance(3)
            box.download(dst)
            box.sync()
        outs.append(dst.copy())
        box.close()
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))


@pytest.mark.parametrize("precision", [0, 1])
def test_named_entry_points_equal_advance_host(gpu, cns, precision):
    """cns_advance_f64 / cns_advance_mixed are cns_advance_host with the precision fixed."""
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    n = (12, 16, 20)
    U0 = I.initial_state(n, perturb=1e-3, seed=11)
    a, b = U0.copy(), U0.copy()
    cns.advance_host(a, 2, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision)
    fn = gpu.cns_advance_f64 if precision == 0 else gpu.cns_advance_mixed
    dts = np.zeros(2)
    L.check(fn(L.dptr(b), L.iarr(list(n)), L.darr(I.box_dx(n)), I.CFL, I.ETA, I.ALAM, 2, L.dptr(dts)))
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_offset_inside_larger_pinned_allocation(gpu, cns):
    """U as the second of two arrays carved from one page-locked allocation: in place, and the
    first array (outside U's range) is left untouched."""
    from cns_nospec_gb300 import initdata as I
    n = (12, 16, 20)
    U0 = garbage_ghosts(I.initial_state(n, perturb=1e-3, seed=13), 4)
    t = torch.empty((2,) + U0.shape, dtype=torch.float64, pin_memory=True)
    both = t.numpy()
    both[0] = 7.0
    both[1] = U0
    Ub = both[1]
    assert Ub.flags.c_contiguous and in_place(gpu, Ub) == 1
    Ua = U0.copy()
    with staged_pageable(gpu):
        dta = cns.advance_host(Ua, 2, I.box_dx(n), I.CFL, I.ETA, I.ALAM, 0)
    dtb = cns.advance_host(Ub, 2, I.box_dx(n), I.CFL, I.ETA, I.ALAM, 0)
    assert np.array_equal(dta, dtb)
    assert np.array_equal(Ua.view(np.uint64), Ub.view(np.uint64))
    assert np.all(both[0] == 7.0)


@pytest.mark.parametrize("precision", [0, 1])
def test_pageable_in_place_equals_staged(gpu, cns, precision):
    """Pageable (malloc'd) arrays used in place by a device that reads host memory through the
    host's page tables: the same bits as the staged path, through cns_new_advance (FP64),
    cns_advance_host and Box upload/download."""
    from cns_nospec_gb300 import initdata as I
    if not pageable_in_place_supported(gpu):
        pytest.skip("this device does not address pageable host memory")
    n = (20, 12, 36)
    U0 = garbage_ghosts(I.initial_state(n, perturb=1e-3, seed=17), 5)
    Ua, Ub = U0.copy(), U0.copy()
    with staged_pageable(gpu):
        dta = cns.advance_host(Ua, 3, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision)
    dtb = cns.advance_host(Ub, 3, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision)
    assert np.array_equal(dta, dtb)
    assert np.array_equal(Ua.view(np.uint64), Ub.view(np.uint64))
    if precision == 0:
        m = 24
        V0 = garbage_ghosts(I.initial_state(m, perturb=1e-3, seed=19), 6)
        h = cns.read_configurations(m, I.box_dx(m), I.CFL, I.ETA, I.ALAM)
        Va, Vb = V0.copy(), V0.copy()
        for _ in range(2):
            with staged_pageable(gpu):
                da = cns.new_advance(Va, None, None, None, None, h)
            db = cns.new_advance(Vb, None, None, None, None, h)
            assert da == db
            assert np.array_equal(Va.view(np.uint64), Vb.view(np.uint64))
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=precision)
    box.upload(U0)
    box.advance(2)
    outs = []
    for staged in (True, False):
        dst = np.full(U0.shape, np.nan)
        with contextlib.ExitStack() as stack:
            if staged:
                stack.enter_context(staged_pageable(gpu))
            box.download(dst)
            box.sync()
        outs.append(dst)
    box.close()
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))
