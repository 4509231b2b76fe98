"""The exact stencil sums of the plain form (cns_nospec_gb300/csrc/cns_exact.cuh), on the CPU:
the header's arithmetic, compiled for the host, against an independent model in exact
rational arithmetic.  The model places each tap's significand 9 bits below the ulp of the
largest tap (truncating what lies below, as the header does), sums with the integer weights
and rounds once to nearest even; the header must give the same bits, and must report the
FP64 fallback exactly for non-finite taps and sums outside the normal range.  A second test
bounds the result against the untruncated sum sum_m w_m f[m] itself: it is within half an ulp
of the result plus sum|w| * 2^(emax - 1084) (emax the largest tap's biased exponent field), a
few ulp of the largest tap, also where the largest taps cancel."""
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from cns_nospec_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
W1 = (672, -168, 32, -3)
W2 = (8064, -1008, 128, -9)


def model(taps, w, sgn):
    """taps: eight IEEE bit patterns f[+1..+4], f[-1..-4]; None where the header falls back."""
    emax = max([1] + [(u >> 52) & 0x7FF for u in taps])
    if emax == 0x7FF:
        return None
    S = 0
    for u, wm in zip(taps, list(w) + [sgn * x for x in w]):
        e = (u >> 52) & 0x7FF
        m = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
        t = (m << 9) >> min(emax - max(e, 1), 63)
        S += (-wm if u >> 63 else wm) * t
    if S == 0:
        return 0
    e2 = emax - 1075 - 9
    be = abs(S).bit_length() - 1 + e2 + 1023
    if be < 1 or be > 2045:
        return None
    x = float(Fraction(S) * Fraction(2) ** e2)  # correctly rounded, ties to even
    return int(np.float64(x).view(np.uint64))


def tap_sets(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        kind = q % 9
        x = np.arange(-4, 5)
        A = 2.0 ** rng.uniform(-100, 100) * rng.choice([-1.0, 1.0])
        if kind == 0:    # smooth, sign changes
            v = A * np.sin(rng.uniform(0, 6.3) + rng.uniform(0.001, 0.3) * x)
        elif kind == 1:  # smooth with an offset
            v = A * (rng.uniform(1, 4) + np.sin(rng.uniform(0, 6.3) + rng.uniform(0.001, 0.3) * x))
        elif kind == 2:  # small exact values: ties in the rounding
            v = np.ldexp(rng.integers(-8, 8, 9).astype(np.float64), int(rng.integers(-20, 20)))
        elif kind == 3:  # taps spread over many binades (truncation below the guard bits)
            v = rng.choice([-1.0, 1.0], 9) * 2.0 ** rng.uniform(-40, 0, 9) * abs(A)
        elif kind == 4:  # zeros among the taps
            v = A * np.sin(0.1 * x + rng.uniform(0, 6.3))
            v[rng.integers(0, 9, 3)] = 0.0
        elif kind == 5:  # subnormal range
            v = rng.uniform(-0.5, 0.5, 9) * 2.0 ** rng.uniform(-1070, -1040)
        elif kind == 6:  # near the top of the range
            v = rng.uniform(-0.5, 0.5, 9) * 2.0 ** rng.uniform(1000, 1023)
        elif kind == 7:  # a non-finite tap
            v = A * np.sin(0.1 * x)
            v[int(rng.integers(0, 9))] = [np.inf, -np.inf, np.nan][q % 3]
        else:            # f[+1] = f[-1] dominate (locally even data) and cancel in a first
            # derivative; the other taps lie 10-30 binades below them
            v = A * 2.0 ** -rng.uniform(10, 30) * rng.uniform(-1, 1, 9)
            v[3] = v[5] = A
        bits = v.astype(np.float64).view(np.uint64)
        # f[+1..+4], f[-1..-4] around the centre index 4
        out.append([int(bits[4 + m]) for m in range(1, 5)] + [int(bits[4 - m]) for m in range(1, 5)])
    return out


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("xs") / "exact_sum_host")
    cmd = [B.nvcc(), "-x", "cu", "-std=c++17", "-O2", "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "cns_nospec_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           "-o", exe, os.path.join(ROOT, "tests", "exact_sum_host.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_exact_sums_match_the_rational_model(driver):
    sets = tap_sets(16000, seed=11)
    inp = "\n".join(" ".join("%016x" % u for u in s) for s in sets) + "\n"
    r = subprocess.run([driver], input=inp, capture_output=True, text=True, check=True)
    lines = r.stdout.split("\n")[:len(sets)]
    assert len(lines) == len(sets)
    fallbacks = 0
    for s, line in zip(sets, lines):
        ok1, b1, ok2, b2 = line.split()
        for ok, b, (w, sgn) in ((ok1, b1, (W1, -1)), (ok2, b2, (W2, 1))):
            want = model(s, w, sgn)
            if want is None:
                assert ok == "0", (s, w)
                fallbacks += 1
            else:
                assert ok == "1" and int(b, 16) == want, (s, w, b, hex(want))
    # the fallback is exercised (non-finite taps, subnormal and top-of-range sums) but rare
    assert 0 < fallbacks < len(sets)


def test_exact_sums_error_bound_against_the_untruncated_sum(driver):
    """|result - sum_m w_m f[m]| <= ulp(result)/2 + sum|w| 2^(emax-1084): the truncation below the
    guard bits costs less than one unit of 2^(emax-1084) per tap, the final rounding half an ulp."""
    import math
    sets = tap_sets(9000, seed=12)
    inp = "\n".join(" ".join("%016x" % u for u in s) for s in sets) + "\n"
    r = subprocess.run([driver], input=inp, capture_output=True, text=True, check=True)
    lines = r.stdout.split("\n")[:len(sets)]
    checked = cancelling = 0
    for q, (s, line) in enumerate(zip(sets, lines)):
        ok1, b1, ok2, b2 = line.split()
        vals = [float(np.uint64(u).view(np.float64)) for u in s]
        if not all(math.isfinite(v) for v in vals):
            continue  # the FP64 chain (checked by the test above)
        taps = [Fraction(v) for v in vals]
        emax = max([1] + [(u >> 52) & 0x7FF for u in s])
        for ok, b, (w, sgn) in ((ok1, b1, (W1, -1)), (ok2, b2, (W2, 1))):
            if ok != "1":
                continue
            ws = list(w) + [sgn * x for x in w]
            exact = sum(wm * t for wm, t in zip(ws, taps))
            got = float(np.uint64(int(b, 16)).view(np.float64))
            bound = Fraction(math.ulp(got)) / 2 + sum(abs(x) for x in ws) * Fraction(2) ** (emax - 1084)
            assert abs(Fraction(got) - exact) <= bound, (s, w, got, float(exact))
            checked += 1
            cancelling += q % 9 == 8 and sgn == -1
    assert checked > 12000 and cancelling > 900
