"""ctypes front end to the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two libraries stand behind the same Python calls:

* ``port`` -- oracle/libcns_oracle.so, the C restatement in cns_oracle.c (built anywhere);
* ``ref``  -- oracle/_ref/libcnsref.so, the reference's own cpu/ sources compiled unmodified
  (only where the reference tree is present; see oracle/Makefile).

Only tests, the smoke check and the benchmark's CPU-baseline leg import this module.
Arrays use the reference host layout: ghost-inclusive (n0+8, n1+8, n2+8, ncomp) float64,
C order (cpu/helper_functions.cpp:100-122).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libcns_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcnsref.so")
# Where the reference tree lies (its cpu/ sources are compiled unmodified by the Makefile's
# `ref` target); CNS_REFERENCE_DIR overrides it.  Absent on machines without the tree.
REF_ROOT = os.environ.get("CNS_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "cpu")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_libs: dict = {}


def build(ref: bool = True, quiet: bool = True) -> None:
    """Compile the port (always) and the reference objects (when the reference tree exists)."""
    out = subprocess.DEVNULL if quiet else None
    r = subprocess.run(["make", "-C", HERE, "all"], stdout=out, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        # retry without OpenMP (a host compiler without libgomp)
        r = subprocess.run(["make", "-C", HERE, "all", "OMP=0", "-B"], stdout=out, stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
    if ref and os.path.isdir(REF_SRC):
        r = subprocess.run(["make", "-C", HERE, "ref", "REFDIR=" + REF_SRC], stdout=out,
                           stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stderr)


def have_ref() -> bool:
    return os.path.exists(REF_SO)


def _lib(which: str):
    if which in _libs:
        return _libs[which]
    path = PORT_SO if which == "port" else REF_SO
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is not built (run oracle.build())")
    lib = C.CDLL(path)
    pre = "oracle_" if which == "port" else "ref_"
    if which == "port":
        lib.oracle_num_threads.argtypes = [C.c_int]
        lib.oracle_num_threads.restype = C.c_int
        lib.oracle_fill_boundary.argtypes = [_D, _I, _I]
        lib.oracle_advance.argtypes = [_D, _I, _D, C.c_double, C.c_double, C.c_double, C.c_int, _D]
    else:
        lib.ref_fill_boundary.argtypes = [_D, _I]
        lib.ref_new_advance.argtypes = [_D, C.c_int, _D, C.c_double, C.c_double, C.c_double, C.c_int, _D]
    getattr(lib, pre + "ctoprim").argtypes = [_I, _I, _D, _D, _D, C.c_int, _D]
    getattr(lib, pre + "hypterm").argtypes = [_I, _I, C.c_int, _D, _D, _D, _D]
    getattr(lib, pre + "diffterm").argtypes = [_I, _I, C.c_int, _D, _D, _D, C.c_double, C.c_double]
    _libs[which] = lib
    return lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def _ip(v):
    return (C.c_int * 3)(*[int(x) for x in v])


def _dv(v):
    return (C.c_double * 3)(*[float(x) for x in v])


def set_threads(n: int) -> int:
    return _lib("port").oracle_num_threads(int(n))


def interior_dims(U: np.ndarray, ng: int = 4):
    return tuple(int(U.shape[a]) - 2 * ng for a in range(3))


def lo_hi(dims, ng: int = 4):
    """Ghost-offset interior bounds, as new_advance sets them (cpu/advance.cpp:33-34)."""
    return [ng] * 3, [d - 1 + ng for d in dims]


def fill_boundary(U: np.ndarray, which: str = "port") -> np.ndarray:
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    dims = interior_dims(U)
    if which == "port":
        _lib("port").oracle_fill_boundary(_dp(U), _ip(dims), _ip([d + 8 for d in dims]))
    else:
        _lib("ref").ref_fill_boundary(_dp(U), _ip(dims))
    return U


def ctoprim(U: np.ndarray, dx, with_courno: bool = True, courno_in: float = 1.0e-50, which: str = "port"):
    U = np.ascontiguousarray(U, dtype=np.float64)
    dims = interior_dims(U)
    lo, hi = lo_hi(dims)
    Q = np.zeros(U.shape[:3] + (6,), dtype=np.float64)
    c = C.c_double(courno_in)
    fn = getattr(_lib(which), ("oracle_" if which == "port" else "ref_") + "ctoprim")
    fn(_ip(lo), _ip(hi), _dp(U), _dp(Q), _dv(dx), 4, C.byref(c) if with_courno else None)
    return Q, (c.value if with_courno else None)


def hypterm(U: np.ndarray, Q: np.ndarray, dx, which: str = "port") -> np.ndarray:
    U = np.ascontiguousarray(U, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    dims = interior_dims(U)
    lo, hi = lo_hi(dims)
    F = np.zeros(tuple(dims) + (5,), dtype=np.float64)
    fn = getattr(_lib(which), ("oracle_" if which == "port" else "ref_") + "hypterm")
    fn(_ip(lo), _ip(hi), 4, _dv(dx), _dp(U), _dp(Q), _dp(F))
    return F


def diffterm(Q: np.ndarray, dx, eta: float, alam: float, which: str = "port") -> np.ndarray:
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    dims = interior_dims(Q)
    lo, hi = lo_hi(dims)
    D = np.zeros(tuple(dims) + (5,), dtype=np.float64)
    fn = getattr(_lib(which), ("oracle_" if which == "port" else "ref_") + "diffterm")
    fn(_ip(lo), _ip(hi), 4, _dv(dx), _dp(Q), _dp(D), float(eta), float(alam))
    return D


def advance(U: np.ndarray, nsteps: int, dx, cfl: float, eta: float, alam: float, which: str = "port"):
    """nsteps RK3 steps; returns (U_after, dt per step).  'ref' needs a cubic box."""
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    dims = interior_dims(U)
    dts = np.zeros(max(int(nsteps), 1), dtype=np.float64)
    if which == "port":
        _lib("port").oracle_advance(_dp(U), _ip(dims), _dv(dx), float(cfl), float(eta), float(alam), int(nsteps),
                                    _dp(dts))
    else:
        if not (dims[0] == dims[1] == dims[2]):
            raise ValueError("the reference new_advance handles cubic boxes only (cpu/advance.cpp:34)")
        _lib("ref").ref_new_advance(_dp(U), int(dims[0]), _dv(dx), float(cfl), float(eta), float(alam),
                                    int(nsteps), _dp(dts))
    return U, dts[:nsteps]


# ---- the reference's own file I/O (oracle/_ref only) ---------------------------------------
def ref_print_4d(path, A: np.ndarray) -> None:
    lib = _lib("ref")
    A = np.ascontiguousarray(A, dtype=np.float64)
    lib.ref_print_4D.argtypes = [C.c_char_p, _D, _I, C.c_int]
    if lib.ref_print_4D(str(path).encode(), _dp(A), _ip(A.shape[:3]), int(A.shape[3])) != 0:
        raise OSError(path)


def ref_read_3d(path, dims, ncomp: int) -> np.ndarray:
    lib = _lib("ref")
    A = np.zeros(tuple(dims) + (ncomp,), dtype=np.float64)
    lib.ref_read_3D.argtypes = [C.c_char_p, _D, _I, C.c_int]
    if lib.ref_read_3D(str(path).encode(), _dp(A), _ip(dims), int(ncomp)) != 0:
        raise OSError(path)
    return A


def ref_read_configurations(workdir, out_struct) -> None:
    """Run the reference's read_configurations, which opens ../testcases/general_input
    relative to the working directory, from `workdir`; fills the ctypes struct `out_struct`."""
    lib = _lib("ref")
    lib.ref_read_configurations.argtypes = [C.c_void_p, C.c_int]
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        rc = lib.ref_read_configurations(C.addressof(out_struct), C.sizeof(out_struct))
    finally:
        os.chdir(cwd)
    if rc != 0:
        raise RuntimeError("struct size mismatch")
