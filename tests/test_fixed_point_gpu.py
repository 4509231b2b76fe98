"""The plain form on fixed-point copies of its fields: the TMA assembly (CNS_ASSEMBLE_TMA_FX,
every Laplacian and flux-divergence stencil on 62-bit fixed-point copies staged by TMA) and the
direct kernels (CNS_ASSEMBLE_FX, the stencils of u, v, w and e that the FP64 form sums exactly
reading the copies).  Against the oracle within the FP64 parity bar (cubic, non-cubic and
smaller-than-a-tile boxes), within 1e-13 of the direct kernel; a snapshot resumes and an
autotuned box continues bit for bit; batched boxes equal their runs alone; switching between
the kernels between steps stays within the bar."""
import os

import numpy as np
import pytest

from conftest import FP64_TOL, normwise
from cns_nospec_gb300 import initdata as I

pytestmark = pytest.mark.gpu


def run(cns, n, U0, steps, kernel):
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b.set_kernel(kernel)
    assert b.kernel() == kernel
    b.upload(U0)
    b.advance(steps)
    b.sync()
    out = b.download(), b.last_dt()
    b.close()
    return out


FX_KERNELS = ["CNS_ASSEMBLE_TMA_FX", "CNS_ASSEMBLE_FX"]


@pytest.mark.parametrize("kernel", FX_KERNELS)
@pytest.mark.parametrize("n,steps", [(32, 10), ((40, 36, 48), 6), ((19, 23, 37), 3), ((6, 7, 5), 3)])
def test_fixed_point_assembly_matches_the_oracle(gpu, cns, oracle, n, steps, kernel):
    U0 = I.initial_state(n, perturb=1e-3, seed=41)
    ref, rdt = oracle.advance(U0, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    fx, (dt, done) = run(cns, n, U0, steps, getattr(cns, kernel))
    assert done == steps and abs(dt - rdt[-1]) <= 1e-12 * rdt[-1]
    assert normwise(fx, ref).max() <= FP64_TOL
    direct, _ = run(cns, n, U0, steps, cns.CNS_ASSEMBLE_DIRECT)
    assert normwise(fx, direct).max() <= 1e-13


@pytest.mark.parametrize("kernel", FX_KERNELS)
def test_fixed_point_assembly_resumes_and_autotunes_bit_for_bit(gpu, cns, tmp_path, kernel):
    n = (40, 36, 48)
    U0 = I.initial_state(n, perturb=1e-3, seed=42)
    kernel = getattr(cns, kernel)
    boxes = []
    for _ in range(3):
        b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
        b.set_kernel(kernel)
        b.upload(U0)
        boxes.append(b)
    a, b, c = boxes
    a.advance(6)
    b.advance(3)
    b.save(tmp_path / "s.bin")
    c.load(tmp_path / "s.bin")
    c.advance(3)
    t, k, ms = b.autotune(trial_steps=1)
    assert k == kernel  # the tuner keeps the arithmetic
    b.advance(3)
    want = a.download()
    assert np.array_equal(want.view(np.uint64), c.download().view(np.uint64))
    assert np.array_equal(want.view(np.uint64), b.download().view(np.uint64))
    for x in boxes:
        x.close()


def test_fixed_point_boxes_batched_equal_alone(gpu, cns):
    specs = [((40, 24, 72), cns.CNS_FP64, cns.CNS_ASSEMBLE_TMA_FX), ((20, 36, 33), cns.CNS_FP64, cns.CNS_ASSEMBLE_FX),
             ((24, 24, 24), cns.CNS_FP64, cns.CNS_ASSEMBLE_DIRECT), ((33, 17, 40), cns.CNS_MIXED, cns.CNS_ASSEMBLE_TMA_WS),
             ((17, 40, 23), cns.CNS_FP64, cns.CNS_ASSEMBLE_FX)]

    def boxes():
        out = []
        for q, (n, prec, k) in enumerate(specs):
            b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
            b.set_kernel(k)
            b.upload(I.initial_state(n, perturb=1e-3, seed=50 + q))
            out.append(b)
        return out

    mix = boxes()
    bt = cns.Batch()
    for b in mix:
        bt.add(b)
    bt.advance(4)
    bt.sync()
    for m, a in zip(mix, boxes()):
        a.advance(4)
        assert np.array_equal(m.download().view(np.uint64), a.download().view(np.uint64))
        a.close()
    bt.close()


def test_switching_between_the_fixed_point_kernels_between_steps(gpu, cns, oracle):
    n = (40, 36, 48)
    U0 = I.initial_state(n, perturb=1e-3, seed=43)
    seq = (cns.CNS_ASSEMBLE_DIRECT, cns.CNS_ASSEMBLE_TMA_FX, cns.CNS_ASSEMBLE_FX, cns.CNS_ASSEMBLE_TMA_FX,
           cns.CNS_ASSEMBLE_DIRECT, cns.CNS_ASSEMBLE_FX)
    ref, _ = oracle.advance(U0, 3 * len(seq), I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b.upload(U0)
    for k in seq:
        b.set_kernel(k)
        b.advance(3)
    b.sync()
    assert normwise(b.download(), ref).max() <= FP64_TOL
    b.close()
    m = cns.Box(16, I.box_dx(16), I.CFL, I.ETA, I.ALAM, precision=cns.CNS_MIXED)
    for k in (cns.CNS_ASSEMBLE_TMA_FX, cns.CNS_ASSEMBLE_FX):
        with pytest.raises(cns.CnsError):
            m.set_kernel(k)
    m.close()


@pytest.mark.parametrize("amp", [(1.0, 0.0, 0.0), (1e-6, 1.0, 1e-3), (0.0, 0.0, 0.0)])
def test_fixed_point_copies_of_fields_that_start_at_zero_or_differ_in_scale(gpu, cns, oracle, amp):
    """Velocity components that start at zero (their exponents then come from nothing, and the
    first values written do not fit: the kernels fall back to the FP64 fields until the maxima
    catch up) or differ by six orders of magnitude (one exponent per field): the default kernels
    stay within the FP64 bar of the oracle and within 1e-13 of the FP64-tap kernels."""
    n, steps = (24, 20, 28), 6
    U0 = I.initial_state(n, amp=amp, perturb=1e-3, seed=44)
    ref, _ = oracle.advance(U0, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    fx, _ = run(cns, n, U0, steps, cns.CNS_ASSEMBLE_FX)
    assert normwise(fx, ref).max() <= FP64_TOL
    direct, _ = run(cns, n, U0, steps, cns.CNS_ASSEMBLE_DIRECT)
    assert normwise(fx, direct).max() <= 1e-13


def test_snapshot_taken_right_after_an_upload_resumes_bit_for_bit(gpu, cns, tmp_path):
    """A snapshot of a freshly uploaded box carries that its first step reads the FP64 fields in
    the derivative pass (as the upload fused with that pass does); resumed, it continues as the
    box it was taken from, bit for bit."""
    n = 32
    U0 = I.initial_state(n, perturb=1e-3, seed=45)
    a = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    a.upload(U0)
    a.save(tmp_path / "fresh.bin")
    a.advance(3)
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b.load(tmp_path / "fresh.bin")
    b.advance(3)
    assert np.array_equal(a.download().view(np.uint64), b.download().view(np.uint64))
    a.close()
    b.close()
