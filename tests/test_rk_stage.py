"""The RK3 stage kept between stages as U1 / 4 (cns_nospec_gb300/csrc/cns_exact.cuh's quarter()),
on the CPU: the header compiled for the host.  quarter(x) is x / 4 exactly for every finite x of
magnitude at least 2^-1020, keeps infinities and NaNs, and gives a zero of x's sign below that;
and the second stage's fma(dt / 4, L, U1 / 4) has the bits of the reference's
0.25 * (U1 + dt L) formed as 0.25 * fma(dt, L, U1) (cpu/advance.cpp:110-119)."""
import os
import subprocess

import numpy as np
import pytest

from cns_nospec_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("rk") / "rk_stage_host")
    cmd = [B.nvcc(), "-x", "cu", "-std=c++17", "-O2", "--expt-relaxed-constexpr",
           "-I" + os.path.join(ROOT, "cns_nospec_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
           "-o", exe, os.path.join(ROOT, "tests", "rk_stage_host.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    return exe


def run(driver, x, dt, r):
    inp = "".join("%016x %016x %016x\n" % t for t in zip(x.view(np.uint64), dt.view(np.uint64), r.view(np.uint64)))
    out = subprocess.run([driver], input=inp, capture_output=True, text=True, check=True).stdout.split()
    q = np.array([int(v, 16) for v in out[0::2]], dtype=np.uint64).view(np.float64)
    same = np.array([int(v) for v in out[1::2]], dtype=bool)
    return q, same


def test_quarter_is_exact_and_keeps_specials(driver):
    rng = np.random.default_rng(11)
    n = 20000
    e = rng.integers(-1074, 1024, n)
    x = rng.uniform(1.0, 2.0, n) * np.ldexp(1.0, e) * rng.choice([-1.0, 1.0], n)
    edge = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, np.ldexp(1.0, -1022),
                     np.ldexp(1.0, -1021), np.ldexp(1.0, -1020), -np.ldexp(1.5, -1020), np.ldexp(1.999, -1021),
                     np.finfo(np.float64).max, -np.finfo(np.float64).max])
    x = np.concatenate([x, edge])
    q, _ = run(driver, x, np.ones_like(x), np.zeros_like(x))
    big = np.isfinite(x) & (np.abs(x) >= np.ldexp(1.0, -1020))
    assert np.array_equal(q[big].view(np.uint64), (x[big] / 4.0).view(np.uint64))
    tiny = np.isfinite(x) & ~big
    assert np.all(q[tiny] == 0.0) and np.array_equal(np.signbit(q[tiny]), np.signbit(x[tiny]))
    assert np.array_equal(q[np.isinf(x)], x[np.isinf(x)]) and np.all(np.isnan(q[np.isnan(x)]))


def test_second_stage_combine_keeps_the_bits(driver):
    rng = np.random.default_rng(12)
    n = 20000
    dt = rng.uniform(1e-9, 1e-6, n)
    r = (rng.uniform(-1.0, 1.0, n) * np.ldexp(1.0, rng.integers(-10, 40, n))).astype(np.float32).astype(np.float64)
    x = rng.uniform(-1.0, 1.0, n) * np.ldexp(1.0, rng.integers(-20, 35, n))
    x[: n // 4] = -dt[: n // 4] * r[: n // 4] * (1.0 + rng.uniform(-1e-9, 1e-9, n // 4))  # cancelling sums
    _, same = run(driver, x, dt, r)
    assert same.all(), int((~same).sum())
