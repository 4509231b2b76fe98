"""The plain form's fixed-point stencil copies (cns_nospec_gb300/csrc/cns_exact.cuh), on the CPU:
the header's arithmetic, compiled for the host, against an independent model in exact rational
arithmetic.  The model truncates each value toward zero onto the grid 2^E, flags values that do
not fit (|v| >= 2^(E + 62) by the exponent test, or not finite), splits each word into its two
31-bit chunks, sums with the integer weights exactly and rounds once to nearest even; the header
must give the same words and bits.  A second test bounds each sum against the exact
sum_m w_m v_m: within half an ulp of the result plus sum|w| * 2^E."""
import math
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from cns_nospec_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
W1 = (672, -168, 32, -3)
W2 = (8064, -1008, 128, -9)


def model_word(u, E):
    """(word, bad) for the FP64 bit pattern u at exponent E."""
    e = (u >> 52) & 0x7FF
    m = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
    sh = max(e, 1) - 1075 - E
    if e == 0x7FF or sh > 9:
        return None, True
    X = m << sh if sh >= 0 else m >> min(-sh, 63)
    if u >> 63:
        X = -X
    lo, hi = X & 0x7FFFFFFF, X >> 31
    return ((hi & 0xFFFFFFFF) << 32) | lo, False


def model_sum(words, w, sgn, E, weights_given=False):
    """The rounded sum of the words (None outside FP64's normal range): eight words with the
    weights w at +m and sgn * w at -m, or with weights_given, any words with the weights w."""
    S = 0
    for word, wm in zip(words, list(w) if weights_given else list(w) + [sgn * x for x in w]):
        lo, hi = word & 0xFFFFFFFF, word >> 32
        hi = hi - (1 << 32) if hi >= 1 << 31 else hi
        S += wm * (hi * (1 << 31) + lo)
    if S == 0:
        return 0
    be = abs(S).bit_length() - 1 + E + 1023
    if be < 1 or be > 2045:
        return None
    return int(np.float64(float(Fraction(S) * Fraction(2) ** E)).view(np.uint64))


def cases(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        kind = q % 6
        x = np.arange(-4, 5)
        M = 2.0 ** rng.uniform(-60, 60)
        if kind == 0:    # smooth around zero: the field's magnitude sets E
            v = M * np.sin(rng.uniform(0, 6.3) + rng.uniform(0.001, 0.3) * x)
        elif kind == 1:  # a large background with small variations (pressure-like)
            v = M * (1.0 + 1e-4 * np.sin(rng.uniform(0, 6.3) + 0.1 * x))
        elif kind == 2:  # values far below the field's magnitude (truncated on the grid)
            v = M * 2.0 ** -rng.uniform(20, 70, 9) * rng.choice([-1.0, 1.0], 9)
        elif kind == 3:  # exact small integers: ties in the rounding
            v = np.ldexp(rng.integers(-8, 8, 9).astype(np.float64), int(rng.integers(-20, 20)))
            M = 8.0 * 2.0 ** 20
        elif kind == 4:  # values that outgrew the exponent (flagged)
            v = M * np.sin(0.1 * x + rng.uniform(0, 6.3))
            v[int(rng.integers(0, 9))] = M * 2.0 ** rng.uniform(2.5, 6)
        else:            # a non-finite value (flagged)
            v = M * np.sin(0.1 * x)
            v[int(rng.integers(0, 9))] = [np.inf, -np.inf, np.nan][q % 3]
        emax = (int(np.float64(abs(M)).view(np.uint64)) >> 52) & 0x7FF
        E = max(emax, 1) - 1082
        bits = v.astype(np.float64).view(np.uint64)
        out.append((E, [int(bits[4 + m]) for m in range(1, 5)] + [int(bits[4 - m]) for m in range(1, 5)]))
    return out


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("fx") / "fixed_point_host")
    cmd = [B.nvcc(), "-x", "cu", "-std=c++17", "-O2", "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "cns_nospec_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           "-o", exe, os.path.join(ROOT, "tests", "fixed_point_host.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(driver, cs):
    inp = "\n".join(f"{E} " + " ".join("%016x" % u for u in taps) for E, taps in cs) + "\n"
    r = subprocess.run([driver], input=inp, capture_output=True, text=True, check=True)
    return r.stdout.split("\n")[:len(cs)]


def test_fixed_point_words_and_sums_match_the_model(driver):
    cs = cases(12000, seed=21)
    lines = run(driver, cs)
    assert len(lines) == len(cs)
    flagged = 0
    for (E, taps), line in zip(cs, lines):
        f = line.split()
        words, bad = [int(x, 16) for x in f[:8]], f[8] == "1"
        model = [model_word(u, E) for u in taps]
        assert bad == any(b for _, b in model), (E, taps)
        if bad:
            flagged += 1
            continue
        assert words == [w for w, _ in model], (E, taps)
        for ok, b, (w, sgn) in ((f[9], f[10], (W1, -1)), (f[11], f[12], (W2, 1))):
            want = model_sum(words, w, sgn, E)
            if want is None:
                assert ok == "0"
            else:
                assert ok == "1" and int(b, 16) == want, (E, taps, w)
    assert 0 < flagged < len(cs) // 2


def test_merged_second_difference_sums_match_the_model(driver):
    """fx_d2acc2 / fx_d2acc3 (the Laplacians of cubic cells): one exact sum over the taps of two or
    three stencils, rounded once; here the words as given, mirrored and rotated."""
    cs = cases(6000, seed=23)
    lines = run(driver, cs)
    checked = 0
    for (E, taps), line in zip(cs, lines):
        f = line.split()
        if f[8] == "1":
            continue
        words = [int(x, 16) for x in f[:8]]
        plus, minus = words[:4], words[4:]
        mirrored = minus + plus
        rotated = plus[1:] + plus[:1] + minus[1:] + minus[:1]
        ws = list(W2) + list(W2)
        for ok, b, sets in ((f[13], f[14], (words, mirrored)), (f[15], f[16], (words, mirrored, rotated))):
            want = model_sum([w for st in sets for w in st], ws * len(sets), 1, E, weights_given=True)
            if want is None:
                assert ok == "0"
            else:
                assert ok == "1" and int(b, 16) == want, (E, taps, len(sets))
                checked += 1
    assert checked > 3000


def test_fixed_point_sums_are_within_the_stated_bound(driver):
    """|result - sum_m w_m v_m| <= ulp(result) / 2 + sum|w| 2^E for every value that fits."""
    cs = cases(6000, seed=22)
    lines = run(driver, cs)
    checked = 0
    for (E, taps), line in zip(cs, lines):
        f = line.split()
        if f[8] == "1":
            continue
        vals = [Fraction(float(np.uint64(u).view(np.float64))) for u in taps]
        for ok, b, (w, sgn) in ((f[9], f[10], (W1, -1)), (f[11], f[12], (W2, 1))):
            if ok != "1":
                continue
            ws = list(w) + [sgn * x for x in w]
            exact = sum(wm * v for wm, v in zip(ws, vals))
            got = float(np.uint64(int(b, 16)).view(np.float64))
            bound = Fraction(math.ulp(got)) / 2 + sum(abs(x) for x in ws) * Fraction(2) ** E
            assert abs(Fraction(got) - exact) <= bound, (E, taps, w)
            checked += 1
    assert checked > 6000
