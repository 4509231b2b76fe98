"""Host API: the reference's call surface over the GB300 library.

Functions keep the reference's names and argument meaning (cpu/header.h:98-156,
cpu/helper_functions.h:171-176):

    ctoprim(lo, hi, u, q, dx, ng, courno=None) -> courno
    hypterm(lo, hi, ng, dx, cons, q, flux)
    diffterm(lo, hi, ng, dx, q, difflux, eta, alam)
    fill_boundary(U, dim, dim_ng)
    new_advance(U, Unew, Q, D, F, h_const) -> dt
    read_configurations(...) -> h_const         (cpu/helper_functions.cpp:38-83, from arguments)

Arrays are numpy float64 in the reference host layout ([i][j][k][l], C order).  Outputs are
written in place, as in the reference.  Every call runs on the GPU through the C ABI; errors
raise CnsError instead of exiting.  ``Box`` and ``Batch`` keep state resident on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .initdata import NC, NG

CnsError = L.CnsError


def _f64(a, name):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError(f"{name} must be a C-contiguous float64 numpy array")
    return a


def ctoprim(lo, hi, u, q, dx, ng, courno=None):
    """cpu/ctoprim.cpp:11-105.  Writes q; returns max(courno, Courant max) when courno is given."""
    lib = L.load()
    _f64(u, "u"), _f64(q, "q")
    c = C.c_double(courno) if courno is not None else None
    L.check(lib.cns_ctoprim(L.iarr(lo), L.iarr(hi), L.dptr(u), L.dptr(q), L.darr(dx), int(ng),
                            C.byref(c) if c is not None else None))
    return c.value if c is not None else None


def hypterm(lo, hi, ng, dx, cons, q, flux):
    """cpu/hypterm.cpp:11-209.  Writes flux (interior-indexed)."""
    lib = L.load()
    _f64(cons, "cons"), _f64(q, "q"), _f64(flux, "flux")
    L.check(lib.cns_hypterm(L.iarr(lo), L.iarr(hi), int(ng), L.darr(dx), L.dptr(cons), L.dptr(q), L.dptr(flux)))


def diffterm(lo, hi, ng, dx, q, difflux, eta, alam):
    """cpu/diffterm.cpp:22-320.  Writes difflux (interior-indexed)."""
    lib = L.load()
    _f64(q, "q"), _f64(difflux, "difflux")
    L.check(lib.cns_diffterm(L.iarr(lo), L.iarr(hi), int(ng), L.darr(dx), L.dptr(q), L.dptr(difflux),
                             float(eta), float(alam)))


def fill_boundary(U, dim, dim_ng):
    """cpu/helper_functions.cpp:226-262, in place."""
    lib = L.load()
    _f64(U, "U")
    L.check(lib.cns_fill_boundary(L.dptr(U), L.iarr(dim), L.iarr(dim_ng)))


def read_configurations(n, dx, cfl, eta, alam, nsteps=0, ng=NG, nc=NC) -> L.GlobalConst:
    """The reference fills h_const from ../testcases/general_input
    (cpu/helper_functions.cpp:38-83); this builds the same struct from arguments."""
    if isinstance(n, int):
        n = (n, n, n)
    h = L.GlobalConst()
    h.ng, h.nc, h.ncells, h.nsteps = ng, nc, int(n[0]), int(nsteps)
    for a in range(3):
        h.lo[a], h.hi[a] = 0, int(n[a]) - 1
        h.dim[a], h.dim_g[a] = int(n[a]), int(n[a]) + 2 * ng
        h.dx[a], h.dxinv[a] = float(dx[a]), 1.0 / float(dx[a])
    h.comp_offset_g = h.dim_g[0] * h.dim_g[1] * h.dim_g[2]
    h.comp_offset = h.dim[0] * h.dim[1] * h.dim[2]
    h.plane_offset_g = h.dim_g[1] * h.dim_g[2]
    h.plane_offset = h.dim[1] * h.dim[2]
    h.cfl, h.eta, h.alam = float(cfl), float(eta), float(alam)
    h.ALP, h.BET, h.GAM, h.DEL = 0.8, -0.2, 4.0 / 105.0, -1.0 / 280.0
    h.OneThird, h.TwoThirds, h.FourThirds = 1.0 / 3.0, 2.0 / 3.0, 4.0 / 3.0
    h.OneQuarter, h.ThreeQuarters = 0.25, 0.75
    h.CENTER, h.OFF1, h.OFF2, h.OFF3, h.OFF4 = -205.0 / 72.0, 8.0 / 5.0, -0.2, 8.0 / 315.0, -1.0 / 560.0
    return h


def new_advance(U, Unew, Q, D, F, h_const) -> float:
    """cpu/advance.cpp:13-154: one RK3 step of U in place; returns dt.  Unew/Q/D/F are
    accepted for signature compatibility (may be None) and are not written."""
    lib = L.load()
    _f64(U, "U")
    dt = C.c_double(0.0)
    L.check(lib.cns_new_advance(C.byref(h_const), L.dptr(U), None, None, None, None, C.byref(dt)))
    return dt.value


def advance_host(U, nsteps, dx, cfl, eta, alam, precision=L.CNS_FP64):
    """nsteps RK3 steps of the host array U in place (one copy in, one out); returns dt per step."""
    lib = L.load()
    _f64(U, "U")
    n = [U.shape[a] - 2 * NG for a in range(3)]
    dts = np.zeros(max(int(nsteps), 1), dtype=np.float64)
    L.check(lib.cns_advance_host(L.dptr(U), L.iarr(n), L.darr(dx), float(cfl), float(eta), float(alam),
                                 int(nsteps), int(precision), L.dptr(dts)))
    return dts[:nsteps]


class Box:
    """One periodic box with its state resident in HBM."""

    def __init__(self, n, dx, cfl, eta, alam, precision=L.CNS_FP64):
        if isinstance(n, int):
            n = (n, n, n)
        self.lib = L.load()
        self.n = tuple(int(x) for x in n)
        self.desc = L.BoxDesc()
        for a in range(3):
            self.desc.n[a] = self.n[a]
            self.desc.dx[a] = float(dx[a])
        self.desc.cfl, self.desc.eta, self.desc.alam = float(cfl), float(eta), float(alam)
        self.desc.precision = int(precision)
        self.precision = int(precision)
        self.h = C.c_void_p()
        L.check(self.lib.cns_box_create(C.byref(self.desc), C.byref(self.h)))

    @staticmethod
    def bytes_for(n, precision=L.CNS_FP64) -> int:
        if isinstance(n, int):
            n = (n, n, n)
        d = L.BoxDesc()
        for a in range(3):
            d.n[a] = int(n[a])
            d.dx[a] = 1.0 / int(n[a])
        d.cfl, d.eta, d.alam, d.precision = 0.5, 1.0, 1.0, int(precision)
        return int(L.load().cns_box_bytes(C.byref(d)))

    def shape(self):
        return tuple(x + 2 * NG for x in self.n) + (NC,)

    def upload(self, U):
        _f64(U, "U")
        if U.shape != self.shape():
            raise ValueError(f"U has shape {U.shape}, expected {self.shape()}")
        L.check(self.lib.cns_box_upload(self.h, L.dptr(U)))

    def init_field(self, amp=(1.0, 1.0, 1.0), perturb=0.0, seed=1):
        """Generate the CNS_NoSpec initial field on the device (no host array)."""
        a = (C.c_double * 3)(*[float(x) for x in amp])
        L.check(self.lib.cns_box_init_field(self.h, a, float(perturb), C.c_ulonglong(int(seed))))

    def save(self, path):
        L.check(self.lib.cns_box_save(self.h, str(path).encode()))

    def load(self, path):
        L.check(self.lib.cns_box_load(self.h, str(path).encode()))

    def download(self, out=None):
        out = np.empty(self.shape(), dtype=np.float64) if out is None else _f64(out, "out")
        L.check(self.lib.cns_box_download(self.h, L.dptr(out)))
        return out

    def set_stream(self, stream_handle):
        L.check(self.lib.cns_box_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    def advance(self, nsteps):
        L.check(self.lib.cns_box_advance(self.h, int(nsteps)))

    def advance_ms(self, nsteps) -> float:
        """nsteps graph-replayed RK3 steps; waits for them and returns their device time (ms,
        CUDA events on the box's stream)."""
        ms = C.c_double()
        L.check(self.lib.cns_box_advance_ms(self.h, int(nsteps), C.byref(ms)))
        return ms.value

    def advance_timed(self, nsteps):
        ms = (C.c_double * L.KERN_COUNT)()
        launches = (C.c_int * L.KERN_COUNT)()
        total = C.c_double()
        L.check(self.lib.cns_box_advance_timed(self.h, int(nsteps), ms, launches, C.byref(total)))
        return list(ms), list(launches), total.value

    def sync(self):
        hb = C.c_int(0)
        L.check(self.lib.cns_box_sync(self.h, C.byref(hb)))

    def health(self) -> int:
        hb = C.c_int(0)
        self.lib.cns_box_sync(self.h, C.byref(hb))
        return hb.value

    def last_dt(self):
        dt, n = C.c_double(), C.c_int()
        L.check(self.lib.cns_box_last_dt(self.h, C.byref(dt), C.byref(n)))
        return dt.value, n.value

    def tile(self):
        t = (C.c_int * 3)()
        L.check(self.lib.cns_box_get_tile(self.h, t))
        return tuple(t)

    def set_tile(self, tlog):
        L.check(self.lib.cns_box_set_tile(self.h, (C.c_int * 3)(*tlog)))

    def autotune(self, trial_steps=2):
        """Pick the fastest tile shape (and, for mixed boxes, assembly kernel) by timing trial
        steps (state restored afterwards).  Returns (tile log2 shape, kernel, ms per step)."""
        t = (C.c_int * 3)()
        k = C.c_int()
        ms = C.c_double()
        L.check(self.lib.cns_box_autotune(self.h, int(trial_steps), t, C.byref(k), C.byref(ms)))
        return tuple(t), k.value, ms.value

    def kernel(self) -> int:
        k = C.c_int()
        L.check(self.lib.cns_box_get_kernel(self.h, C.byref(k)))
        return k.value

    def set_kernel(self, kernel: int):
        L.check(self.lib.cns_box_set_kernel(self.h, int(kernel)))

    def launches_per_step(self) -> int:
        return int(self.lib.cns_box_launches_per_step(self.h))

    def close(self):
        if self.h:
            self.lib.cns_box_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Boxes advanced together: one launch per kernel and RK stage for all members."""

    def __init__(self):
        self.lib = L.load()
        self.h = C.c_void_p()
        L.check(self.lib.cns_batch_create(C.byref(self.h)))
        self.members = []

    def add(self, box: Box):
        L.check(self.lib.cns_batch_add(self.h, box.h))
        self.members.append(box)

    def remove(self, box: Box):
        L.check(self.lib.cns_batch_remove(self.h, box.h))
        self.members.remove(box)

    def set_stream(self, stream_handle):
        L.check(self.lib.cns_batch_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    def advance(self, nsteps=1):
        L.check(self.lib.cns_batch_advance(self.h, int(nsteps)))

    def advance_ms(self, nsteps) -> float:
        """nsteps graph-replayed steps of every member; waits and returns their device time (ms)."""
        ms = C.c_double()
        L.check(self.lib.cns_batch_advance_ms(self.h, int(nsteps), C.byref(ms)))
        return ms.value

    def sync(self):
        L.check(self.lib.cns_batch_sync(self.h))

    def autotune(self, trial_steps=2):
        """Time each tile-shape policy on the members (states restored) and keep the fastest;
        returns (policy, ms per step): policy 0 = per-box least padding, 1+s = candidate s."""
        pol = C.c_int()
        ms = C.c_double()
        L.check(self.lib.cns_batch_autotune(self.h, int(trial_steps), C.byref(pol), C.byref(ms)))
        return pol.value, ms.value

    def close(self):
        if self.h:
            for b in list(self.members):
                self.lib.cns_batch_remove(self.h, b.h)
            self.members = []
            self.lib.cns_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
