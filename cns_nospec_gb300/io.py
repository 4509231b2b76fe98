"""The reference's file formats and snapshots, over the library's native readers and writers.

    read_general_input(path) -> GlobalConst       cpu/helper_functions.cpp:38-83
    write_general_input(path, h)
    read_3d(path, dims, ncomp) -> array           cpu/helper_functions.cpp:166-175 (multistep_input)
    write_3d(path, a)
    print_4d(path, a, header=True)                cpu/helper_functions.cpp:85-98 + cpu/main.cpp:36-40
    read_4d(path, dims, ncomp, header=True) -> array

Arrays are float64 (d0, d1, d2, ncomp) in the reference host layout.  Snapshots of device
boxes are Box.save / Box.load.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L


def _p(path) -> bytes:
    return str(path).encode()


def read_general_input(path) -> L.GlobalConst:
    h = L.GlobalConst()
    L.check(L.load().cns_read_general_input(_p(path), L.C.byref(h)))
    return h


def write_general_input(path, h: L.GlobalConst) -> None:
    L.check(L.load().cns_write_general_input(_p(path), L.C.byref(h)))


def read_3d(path, dims, ncomp: int) -> np.ndarray:
    a = np.zeros(tuple(int(x) for x in dims) + (int(ncomp),), dtype=np.float64)
    L.check(L.load().cns_read_3d(_p(path), L.dptr(a), L.iarr(dims), int(ncomp)))
    return a


def write_3d(path, a: np.ndarray) -> None:
    a = np.ascontiguousarray(a, dtype=np.float64)
    L.check(L.load().cns_write_3d(_p(path), L.dptr(a), L.iarr(a.shape[:3]), int(a.shape[3])))


def print_4d(path, a: np.ndarray, header: bool = True) -> None:
    a = np.ascontiguousarray(a, dtype=np.float64)
    L.check(L.load().cns_print_4d(_p(path), L.dptr(a), L.iarr(a.shape[:3]), int(a.shape[3]), int(bool(header))))


def read_4d(path, dims, ncomp: int, header: bool = True) -> np.ndarray:
    a = np.zeros(tuple(int(x) for x in dims) + (int(ncomp),), dtype=np.float64)
    L.check(L.load().cns_read_4d(_p(path), L.dptr(a), L.iarr(dims), int(ncomp), int(bool(header))))
    return a
