"""The C ABI boundary without a GPU: the library builds for sm_103a, loads, exports every
function include/*.h declares, and the ctypes signatures cover exactly those."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(cns_[a-z0-9_]+)\s*\(", src))
    return names


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_library_exports_every_declared_symbol(cns):
    from cns_nospec_gb300 import _lib
    decl = declared_functions()
    assert len(decl) >= 25
    syms = exported(_lib.lib_path())
    missing = decl - syms
    assert not missing, f"declared but not exported: {sorted(missing)}"
    # the ctypes layer binds exactly the declared surface
    assert set(_lib.SIGNATURES) == decl


def test_library_loads_and_binds(cns):
    lib = cns.load()
    for name in cns._lib.SIGNATURES:
        assert hasattr(lib, name)
    assert lib.cns_version() >= 100


def test_invalid_arguments_are_rejected_before_any_device_work(cns):
    from cns_nospec_gb300 import _lib as L
    lib = cns.load()
    d = L.BoxDesc()
    d.n[0], d.n[1], d.n[2] = 3, 16, 16  # below the 4-cell minimum
    for a in range(3):
        d.dx[a] = 0.1
    d.cfl, d.eta, d.alam, d.precision = 0.5, 1e-4, 100.0, 0
    h = ctypes.c_void_p()
    assert lib.cns_box_create(ctypes.byref(d), ctypes.byref(h)) == L.CNS_ERR_INVALID
    assert b"interior cells" in lib.cns_last_error()
    assert lib.cns_box_bytes(ctypes.byref(d)) == -1
    d.n[0] = 16
    d.precision = 7
    assert lib.cns_box_create(ctypes.byref(d), ctypes.byref(h)) == L.CNS_ERR_INVALID
    lo = L.iarr([4, 4, 4])
    hi = L.iarr([11, 11, 11])
    assert lib.cns_ctoprim(lo, hi, None, None, L.darr([1, 1, 1]), 4, None) == L.CNS_ERR_INVALID
    assert lib.cns_ctoprim(lo, hi, None, None, L.darr([1, 1, 1]), 2, None) == L.CNS_ERR_INVALID
    assert lib.cns_box_advance(None, 1) == L.CNS_ERR_INVALID
    taps, sums, ok = (ctypes.c_double * 8)(*([1.0] * 8)), (ctypes.c_double * 2)(), (ctypes.c_int * 2)()
    assert lib.cns_selftest_exact_sums(None, 1, sums, ok) == L.CNS_ERR_INVALID
    assert lib.cns_selftest_exact_sums(taps, -1, sums, ok) == L.CNS_ERR_INVALID
    assert lib.cns_selftest_exact_sums(taps, 1 << 25, sums, ok) == L.CNS_ERR_INVALID
    assert lib.cns_selftest_exact_sums(taps, 0, sums, ok) == 0  # nothing to do, no device work


def test_box_bytes_accounts_for_state_and_stencil_sets(cns):
    from cns_nospec_gb300 import Box
    b64 = Box.bytes_for(64, 0)
    b32 = Box.bytes_for(64, 1)
    g = 72
    pk = (g + 7) // 8 * 8
    fs = g * g * pk
    assert b64 >= fs * 8 * (5 + 5 + 16 * 2 + 4)
    assert b32 < b64 and b32 >= fs * (8 * 10 + 4 * 36)


def test_global_const_layout_matches_reference_struct():
    """cns_global_const_t must be layout-compatible with global_const_t (cpu/header.h:47-86)."""
    from cns_nospec_gb300 import _lib as L
    # ints: 3 + 4*3 + 4 + 1 = 20 ints (80 B) then doubles (aligned): dt, dx[3], dxinv[3], cfl, eta, alam
    assert L.GlobalConst.dt.offset == 80
    assert L.GlobalConst.temp.offset == 80 + 8 * 10
    assert ctypes.sizeof(L.GlobalConst) == 80 + 8 * 10 + 8 * 27 + 8 * 14


def test_global_const_layout_against_reference_header(tmp_path):
    from oracle import oracle as O
    hdr = os.path.join(O.REF_SRC, "header.h")
    if not os.path.exists(hdr):
        pytest.skip("reference tree not present")
    src = tmp_path / "probe.cpp"
    src.write_text(
        '#include "header.h"\n#include "%s"\n#include <cstddef>\n#include <cstdio>\n'
        'int main(){printf("%%zu %%zu %%zu %%zu\\n", sizeof(global_const_t), sizeof(cns_global_const_t),'
        ' offsetof(global_const_t, OFF4), offsetof(cns_global_const_t, OFF4));}\n' % os.path.join(ROOT, "include",
                                                                                                 "cns_gb300.h"))
    exe = tmp_path / "probe"
    subprocess.run(["g++", "-I" + O.REF_SRC, str(src), "-o", str(exe)], check=True)
    a, b, c, d = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert a == b and c == d
