"""The plain form's fixed-point TMA assembly (CNS_ASSEMBLE_TMA_FX): FP64 boxes whose Laplacian
and flux-divergence stencils read 62-bit fixed-point copies of their fields, staged by TMA.
Against the oracle within the FP64 parity bar (cubic, non-cubic and smaller-than-a-tile boxes),
within 1e-13 of the direct kernel; a snapshot resumes and an autotuned box continues bit for bit;
batched boxes equal their runs alone; switching onto it between steps stays within the bar."""
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


@pytest.mark.parametrize("n,steps", [(32, 10), ((40, 36, 48), 6), ((19, 23, 37), 3), ((6, 7, 5), 3)])
def test_fixed_point_assembly_matches_the_oracle(gpu, cns, oracle, n, steps):
    U0 = I.initial_state(n, perturb=1e-3, seed=41)
    ref, rdt = oracle.advance(U0, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    fx, (dt, done) = run(cns, n, U0, steps, cns.CNS_ASSEMBLE_TMA_FX)
    assert done == steps and abs(dt - rdt[-1]) <= 1e-12 * rdt[-1]
    assert normwise(fx, ref).max() <= FP64_TOL
    direct, _ = run(cns, n, U0, steps, cns.CNS_ASSEMBLE_DIRECT)
    assert normwise(fx, direct).max() <= 1e-13


def test_fixed_point_assembly_resumes_and_autotunes_bit_for_bit(gpu, cns, tmp_path):
    n = (40, 36, 48)
    U0 = I.initial_state(n, perturb=1e-3, seed=42)
    boxes = []
    for _ in range(3):
        b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
        b.set_kernel(cns.CNS_ASSEMBLE_TMA_FX)
        b.upload(U0)
        boxes.append(b)
    a, b, c = boxes
    a.advance(6)
    b.advance(3)
    b.save(tmp_path / "s.bin")
    c.load(tmp_path / "s.bin")
    c.advance(3)
    t, k, ms = b.autotune(trial_steps=1)
    assert k == cns.CNS_ASSEMBLE_TMA_FX  # the tuner keeps the arithmetic
    b.advance(3)
    want = a.download()
    assert np.array_equal(want.view(np.uint64), c.download().view(np.uint64))
    assert np.array_equal(want.view(np.uint64), b.download().view(np.uint64))
    for x in boxes:
        x.close()


def test_fixed_point_boxes_batched_equal_alone(gpu, cns):
    specs = [((40, 24, 72), cns.CNS_FP64, cns.CNS_ASSEMBLE_TMA_FX), ((20, 36, 33), cns.CNS_FP64, cns.CNS_ASSEMBLE_TMA_FX),
             ((24, 24, 24), cns.CNS_FP64, cns.CNS_ASSEMBLE_DIRECT), ((33, 17, 40), cns.CNS_MIXED, cns.CNS_ASSEMBLE_TMA_WS)]

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


def test_switching_onto_the_fixed_point_assembly_between_steps(gpu, cns, oracle):
    n = (40, 36, 48)
    U0 = I.initial_state(n, perturb=1e-3, seed=43)
    ref, _ = oracle.advance(U0, 9, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b.upload(U0)
    for k in (cns.CNS_ASSEMBLE_DIRECT, cns.CNS_ASSEMBLE_TMA_FX, cns.CNS_ASSEMBLE_DIRECT):
        b.set_kernel(k)
        b.advance(3)
    b.sync()
    assert normwise(b.download(), ref).max() <= FP64_TOL
    b.close()
    m = cns.Box(16, I.box_dx(16), I.CFL, I.ETA, I.ALAM, precision=cns.CNS_MIXED)
    with pytest.raises(cns.CnsError):
        m.set_kernel(cns.CNS_ASSEMBLE_TMA_FX)
    m.close()
