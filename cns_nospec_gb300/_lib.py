"""ctypes binding of libcns_gb300.so (the C ABI in include/cns_gb300.h).

The library is the product path: there is no CPU fallback.  Loading fails loudly when the
shared library has not been built (``cns_nospec_gb300.build.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_VP = C.c_void_p

CNS_OK, CNS_ERR_INVALID, CNS_ERR_NOMEM, CNS_ERR_NONFINITE, CNS_ERR_CUDA, CNS_ERR_CAPACITY, CNS_ERR_NODEVICE = range(7)
CNS_FP64, CNS_MIXED = 0, 1
CNS_HEALTH_NONPOS_RHO, CNS_HEALTH_NONFINITE, CNS_HEALTH_NONPOS_EINT, CNS_HEALTH_TIMEOUT = 1, 2, 4, 8
CNS_ASSEMBLE_DIRECT, CNS_ASSEMBLE_TMA, CNS_ASSEMBLE_TMA_WS, CNS_ASSEMBLE_TMA_FX, CNS_ASSEMBLE_FX = 0, 1, 2, 3, 4
KERN_DERIV, KERN_ASSEMBLE, KERN_STEPEND, KERN_PRIM, KERN_COUNT = range(5)
KERNEL_NAMES = ("k_deriv", "k_assemble", "k_stepend", "k_prim")


class CnsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cns error {code}: {msg}")
        self.code = code


class BoxDesc(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("dx", C.c_double * 3), ("cfl", C.c_double), ("eta", C.c_double),
                ("alam", C.c_double), ("precision", C.c_int)]


class GlobalConst(C.Structure):
    """Field-for-field image of the reference's global_const_t (cpu/header.h:47-86)."""
    _fields_ = [("ng", C.c_int), ("nc", C.c_int), ("ncells", C.c_int), ("lo", C.c_int * 3), ("hi", C.c_int * 3),
                ("dim", C.c_int * 3), ("dim_g", C.c_int * 3), ("comp_offset_g", C.c_int), ("comp_offset", C.c_int),
                ("plane_offset_g", C.c_int), ("plane_offset", C.c_int), ("nsteps", C.c_int), ("dt", C.c_double),
                ("dx", C.c_double * 3), ("dxinv", C.c_double * 3), ("cfl", C.c_double), ("eta", C.c_double),
                ("alam", C.c_double), ("temp", C.c_void_p * 27), ("ALP", C.c_double), ("BET", C.c_double),
                ("GAM", C.c_double), ("DEL", C.c_double), ("OneThird", C.c_double), ("TwoThirds", C.c_double),
                ("FourThirds", C.c_double), ("OneQuarter", C.c_double), ("ThreeQuarters", C.c_double),
                ("CENTER", C.c_double), ("OFF1", C.c_double), ("OFF2", C.c_double), ("OFF3", C.c_double),
                ("OFF4", C.c_double)]


# name -> (restype, argtypes); every symbol include/cns_gb300.h declares
SIGNATURES = {
    "cns_last_error": (C.c_char_p, []),
    "cns_version": (C.c_int, []),
    "cns_set_device": (C.c_int, [C.c_int]),
    "cns_device_synchronize": (C.c_int, []),
    "cns_measure_fp64_peak": (C.c_int, [_D]),
    "cns_selftest_bounded_wait": (C.c_int, [_I]),
    "cns_selftest_exact_sums": (C.c_int, [_D, C.c_int, _D, _I]),
    "cns_ctoprim": (C.c_int, [_I, _I, _D, _D, _D, C.c_int, _D]),
    "cns_hypterm": (C.c_int, [_I, _I, C.c_int, _D, _D, _D, _D]),
    "cns_diffterm": (C.c_int, [_I, _I, C.c_int, _D, _D, _D, C.c_double, C.c_double]),
    "cns_diffterm_noalloc": (C.c_int, [_I, _I, C.c_int, _D, _VP, _VP, C.c_double, C.c_double, _VP]),
    "cns_fill_boundary": (C.c_int, [_D, _I, _I]),
    "cns_new_advance": (C.c_int, [C.POINTER(GlobalConst), _D, _D, _D, _D, _D, _D]),
    "cns_host_in_place": (C.c_int, [_VP, C.c_longlong, _I]),
    "cns_set_pageable_in_place": (C.c_int, [C.c_int]),
    "cns_advance_host": (C.c_int, [_D, _I, _D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _D]),
    "cns_advance_f64": (C.c_int, [_D, _I, _D, C.c_double, C.c_double, C.c_double, C.c_int, _D]),
    "cns_advance_mixed": (C.c_int, [_D, _I, _D, C.c_double, C.c_double, C.c_double, C.c_int, _D]),
    "cns_box_bytes": (C.c_longlong, [C.POINTER(BoxDesc)]),
    "cns_box_create": (C.c_int, [C.POINTER(BoxDesc), C.POINTER(_VP)]),
    "cns_box_destroy": (C.c_int, [_VP]),
    "cns_box_set_stream": (C.c_int, [_VP, _VP]),
    "cns_box_upload": (C.c_int, [_VP, _D]),
    "cns_box_download": (C.c_int, [_VP, _D]),
    "cns_box_upload_device": (C.c_int, [_VP, _VP]),
    "cns_box_download_device": (C.c_int, [_VP, _VP]),
    "cns_box_advance": (C.c_int, [_VP, C.c_int]),
    "cns_box_advance_timed": (C.c_int, [_VP, C.c_int, _D, _I, _D]),
    "cns_box_advance_ms": (C.c_int, [_VP, C.c_int, _D]),
    "cns_box_sync": (C.c_int, [_VP, _I]),
    "cns_box_last_dt": (C.c_int, [_VP, _D, _I]),
    "cns_box_launches_per_step": (C.c_int, [_VP]),
    "cns_box_init_field": (C.c_int, [_VP, _D, C.c_double, C.c_ulonglong]),
    "cns_box_save": (C.c_int, [_VP, C.c_char_p]),
    "cns_box_load": (C.c_int, [_VP, C.c_char_p]),
    "cns_read_general_input": (C.c_int, [C.c_char_p, C.POINTER(GlobalConst)]),
    "cns_write_general_input": (C.c_int, [C.c_char_p, C.POINTER(GlobalConst)]),
    "cns_read_3d": (C.c_int, [C.c_char_p, _D, _I, C.c_int]),
    "cns_write_3d": (C.c_int, [C.c_char_p, _D, _I, C.c_int]),
    "cns_print_4d": (C.c_int, [C.c_char_p, _D, _I, C.c_int, C.c_int]),
    "cns_read_4d": (C.c_int, [C.c_char_p, _D, _I, C.c_int, C.c_int]),
    "cns_batch_create": (C.c_int, [C.POINTER(_VP)]),
    "cns_batch_destroy": (C.c_int, [_VP]),
    "cns_batch_set_stream": (C.c_int, [_VP, _VP]),
    "cns_batch_add": (C.c_int, [_VP, _VP]),
    "cns_batch_remove": (C.c_int, [_VP, _VP]),
    "cns_batch_size": (C.c_int, [_VP]),
    "cns_batch_advance": (C.c_int, [_VP, C.c_int]),
    "cns_batch_sync": (C.c_int, [_VP]),
    "cns_batch_advance_ms": (C.c_int, [_VP, C.c_int, _D]),
    "cns_box_get_tile": (C.c_int, [_VP, _I]),
    "cns_box_set_tile": (C.c_int, [_VP, _I]),
    "cns_box_autotune": (C.c_int, [_VP, C.c_int, _I, _I, _D]),
    "cns_box_get_kernel": (C.c_int, [_VP, _I]),
    "cns_box_set_kernel": (C.c_int, [_VP, C.c_int]),
    "cns_batch_autotune": (C.c_int, [_VP, C.c_int, _I, _D]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the CUDA library (no fallback: raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise OSError(f"{path} is not built; run cns_nospec_gb300.build.build() (nvcc, sm_103a)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != CNS_OK:
        msg = load().cns_last_error()
        raise CnsError(rc, msg.decode() if msg else "")


def dptr(a):
    return a.ctypes.data_as(_D)


def iarr(v):
    return (C.c_int * 3)(*[int(x) for x in v])


def darr(v):
    return (C.c_double * 3)(*[float(x) for x in v])
