"""The C++ drop-in (cns_nospec_gb300/dropin/advance_gb300.cpp): the reference's own signatures
(double**** trees, h_const, double& dt) over the C ABI.

CPU: it compiles against the reference's real header and links with the reference's own
cpu/main.cpp and cpu/helper_functions.cpp in place of advance/ctoprim/hypterm/diffterm.cpp.
GPU: a driver written like cpu/main.cpp runs it and matches the reference's golden outputs."""
import os
import subprocess

import numpy as np
import pytest

from conftest import FP64_TOL, ROOT, golden, normwise

DROPIN = os.path.join(ROOT, "cns_nospec_gb300", "dropin", "advance_gb300.cpp")
LIBDIR = os.path.join(ROOT, "cns_nospec_gb300")
from oracle.oracle import REF_SRC as REF  # noqa: E402


def _build_driver(tmp, header_dir):
    exe = os.path.join(tmp, "driver")
    cmd = ["g++", "-O2", "-std=c++17", "-I" + header_dir, "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "driver.cpp"), DROPIN, "-L" + LIBDIR, "-lcns_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_dropin_links_with_reference_main(cns, tmp_path):
    if not os.path.isdir(REF):
        pytest.skip("reference tree not present")
    exe = tmp_path / "cpu_gb300"
    cmd = ["g++", "-O2", "-w", "-I" + REF, "-I" + os.path.join(ROOT, "include"), os.path.join(REF, "main.cpp"),
           os.path.join(REF, "helper_functions.cpp"), DROPIN, "-L" + LIBDIR, "-lcns_gb300", "-Wl,-rpath," + LIBDIR,
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()


def test_dropin_driver_builds_with_standin_header(cns, tmp_path):
    assert os.path.exists(_build_driver(str(tmp_path), os.path.join(ROOT, "tests", "dropin")))


@pytest.mark.gpu
def test_dropin_advance_matches_golden(gpu, tmp_path):
    exe = _build_driver(str(tmp_path), os.path.join(ROOT, "tests", "dropin"))
    g = golden("advance_8.npz")
    U0 = g["U0"]
    src, dst = tmp_path / "in.bin", tmp_path / "out.bin"
    U0.tofile(src)
    r = subprocess.run([exe, "advance", "8", str(int(g["nsteps"])), str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("dt, courno") == int(g["nsteps"])
    out = np.fromfile(dst, dtype=np.float64)
    U = out[:-1].reshape(U0.shape)
    assert normwise(U, g["U"]).max() <= FP64_TOL
    assert abs(out[-1] - g["dts"][-1]) <= 1e-13 * g["dts"][-1]


@pytest.mark.gpu
def test_dropin_operators_match_golden(gpu, tmp_path):
    exe = _build_driver(str(tmp_path), os.path.join(ROOT, "tests", "dropin"))
    g = golden("ops_6x9x11.npz")
    src, dst = tmp_path / "U.bin", tmp_path / "o.bin"
    g["U"].tofile(src)
    r = subprocess.run([exe, "ops", "6", "9", "11", str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(dst, dtype=np.float64)
    nq, ni = g["Q"].size, g["F"].size
    Q = out[:nq].reshape(g["Q"].shape)
    courno = out[nq]
    F = out[nq + 1:nq + 1 + ni].reshape(g["F"].shape)
    D = out[nq + 1 + ni:].reshape(g["D"].shape)
    assert np.abs(Q - g["Q"]).max() <= 1e-14 * np.abs(g["Q"]).max()
    assert abs(courno - float(g["courno"])) <= 1e-14 * float(g["courno"])
    assert normwise(F, g["F"], interior_only=False).max() <= FP64_TOL
    assert normwise(D, g["D"], interior_only=False).max() <= FP64_TOL
