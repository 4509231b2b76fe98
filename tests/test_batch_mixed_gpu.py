"""Batched advance (many boxes per launch, graph-replayed) and the mixed-precision form."""
import numpy as np
import pytest

from conftest import FP64_TOL, MIXED_TOL, normwise
from cns_nospec_gb300 import initdata as I

pytestmark = pytest.mark.gpu


def _boxes(cns, specs):
    out = []
    for n, prec, amp, eta_f, seed in specs:
        dx = I.box_dx(n)
        U0 = I.initial_state(n, amp=amp, perturb=1e-3, seed=seed)
        b = cns.Box(n, dx, I.CFL, I.ETA * eta_f, I.ALAM * eta_f, precision=prec)
        b.upload(U0)
        out.append((b, U0, n, prec, eta_f))
    return out


SPECS = [((16, 24, 20), 0, (1.0, 0.9, 1.1), 1.0, 1), ((33, 17, 40), 1, (0.8, 1.2, 1.0), 0.9, 2),
         ((20, 20, 20), 0, (1.1, 1.1, 0.85), 1.15, 3), ((48, 16, 17), 1, (1.0, 1.0, 1.0), 1.05, 4),
         ((9, 40, 12), 0, (0.95, 1.05, 1.2), 0.8, 5)]


def test_batch_equals_alone_bitwise(gpu, cns):
    """Every box's result in the mix is bit-identical to the same box advanced alone."""
    mix = _boxes(cns, SPECS)
    batch = cns.Batch()
    for b, *_ in mix:
        batch.add(b)
    batch.advance(5)
    batch.sync()
    alone = _boxes(cns, SPECS)
    for (bm, U0, n, prec, _), (ba, *_rest) in zip(mix, alone):
        ba.advance(5)
        A = ba.download()
        M = bm.download()
        assert np.array_equal(A, M), n
    batch.close()


def test_continuous_batching_join_and_leave(gpu, cns):
    """Boxes that join or leave between steps still match their solo runs bit for bit."""
    mix = _boxes(cns, SPECS[:3])
    batch = cns.Batch()
    batch.add(mix[0][0])
    batch.add(mix[1][0])
    batch.advance(2)            # boxes 0, 1: 2 steps
    batch.add(mix[2][0])        # box 2 joins
    batch.advance(3)            # boxes 0, 1: 5 steps; box 2: 3
    batch.remove(mix[0][0])     # box 0 leaves at 5 steps
    batch.advance(1)            # box 1: 6; box 2: 4
    batch.sync()
    expect = [5, 6, 4]
    alone = _boxes(cns, SPECS[:3])
    for (bm, *_), (ba, *_r), k in zip(mix, alone, expect):
        ba.advance(k)
        assert np.array_equal(ba.download(), bm.download())
        assert bm.last_dt()[1] == k
    batch.close()


def test_batch_fp64_members_match_oracle(gpu, cns, oracle):
    mix = _boxes(cns, [s for s in SPECS if s[1] == 0])
    batch = cns.Batch()
    for b, *_ in mix:
        batch.add(b)
    batch.advance(3)
    batch.sync()
    for b, U0, n, prec, f in mix:
        ref, _ = oracle.advance(U0, 3, I.box_dx(n), I.CFL, I.ETA * f, I.ALAM * f)
        assert normwise(b.download(), ref).max() <= FP64_TOL
    batch.close()


def test_mixed_32cube_10_steps_vs_oracle(gpu, cns, oracle):
    n = 32
    U0 = I.initial_state(n)
    ref, rdt = oracle.advance(U0, 10, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    U = U0.copy()
    dts = cns.advance_host(U, 10, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=cns.CNS_MIXED)
    err = normwise(U, ref)
    assert err.max() <= MIXED_TOL, err
    assert np.allclose(dts, rdt, rtol=1e-6)


def test_mixed_128cube_100_steps_vs_fp64(gpu, cns):
    """Mixed form against the (oracle-validated) FP64 form: 128^3, 100 steps, <= 1e-6."""
    n = 128
    U0 = I.initial_state(n, perturb=1e-3, seed=1)
    out = {}
    for prec in (cns.CNS_FP64, cns.CNS_MIXED):
        b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
        b.upload(U0)
        b.advance(100)
        b.sync()
        out[prec] = b.download()
        b.close()
    err = normwise(out[cns.CNS_MIXED], out[cns.CNS_FP64])
    assert err.max() <= MIXED_TOL, err


def test_every_tile_shape_gives_identical_bits(gpu, cns):
    n = (19, 23, 37)
    U0 = I.initial_state(n, perturb=1e-3, seed=13)
    ref = None
    # (-1, 0, 0): linear tiles of 256 consecutive cells (here they cross k rows and j planes)
    shapes = [(1, 2, 5), (0, 3, 5), (0, 2, 6), (2, 2, 4), (2, 3, 3), (3, 2, 3), (1, 4, 3), (-1, 0, 0)]
    for prec in (0, 1):
        ref = None
        for t in shapes:
            b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
            b.set_kernel(cns.CNS_ASSEMBLE_DIRECT)  # the direct kernels are the ones that use the shape
            b.set_tile(t)
            assert b.tile() == t
            b.upload(U0)
            b.advance(3)
            out = b.download()
            b.close()
            if ref is None:
                ref = out
            assert np.array_equal(out, ref), (prec, t)
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    for bad in [(1, 2, 2), (4, 4, 0), (0, 0, 9), (3, 3, 2), (-1, 1, 0), (-2, 0, 0)]:
        with pytest.raises(cns.CnsError):
            b.set_tile(bad)


def test_autotune_keeps_results_and_state(gpu, cns):
    """Autotuning runs trial steps, then restores every member: results equal the untuned run."""
    mix = _boxes(cns, SPECS)
    batch = cns.Batch()
    for b, *_ in mix:
        batch.add(b)
    batch.advance(2)
    pol, ms = batch.autotune(trial_steps=1)
    assert 0 <= pol < 14 * 3 and ms > 0  # 1 + 13 shapes, times the assembly kernels
    batch.advance(3)
    batch.sync()
    alone = _boxes(cns, SPECS)
    for (bm, *_), (ba, *_r) in zip(mix, alone):
        ba.advance(5)
        assert np.array_equal(ba.download(), bm.download())
        assert bm.last_dt()[1] == 5
    batch.close()
    box = cns.Box(24, I.box_dx(24), I.CFL, I.ETA, I.ALAM)
    box.upload(I.initial_state(24, perturb=1e-3, seed=3))
    t, k, ms = box.autotune(trial_steps=1)
    assert (sum(t) == 8 or t == (-1, 0, 0)) and k == cns.CNS_ASSEMBLE_FX and ms > 0  # FP64 keeps its kernel
    box.advance(2)
    other = cns.Box(24, I.box_dx(24), I.CFL, I.ETA, I.ALAM)
    other.upload(I.initial_state(24, perturb=1e-3, seed=3))
    other.advance(2)
    assert np.array_equal(box.download(), other.download())


KERNELS = ("CNS_ASSEMBLE_DIRECT", "CNS_ASSEMBLE_TMA", "CNS_ASSEMBLE_TMA_WS")


# (128, 128, 128) and (96, 80, 128): 1024 and 480 TMA tiles, several per block, so the
# warp-specialised kernel reuses both stash slots and flips every barrier's parity.  (6, 7, 5):
# smaller than one tile, every TMA box reaches past the tensor on every axis (zero fill).
@pytest.mark.parametrize("n", [(19, 23, 37), (8, 8, 32), (33, 17, 40), (64, 64, 64), (96, 80, 128), (128, 128, 128),
                               (6, 7, 5)])
def test_tma_assemblies_equal_direct_bitwise(gpu, cns, n):
    """The TMA-staged assemblies and the direct one do the same arithmetic in the same order."""
    U0 = I.initial_state(n, perturb=1e-3, seed=17)
    out = []
    for name in KERNELS:
        kern = getattr(cns, name)
        b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=cns.CNS_MIXED)
        b.set_kernel(kern)
        assert b.kernel() == kern
        b.upload(U0)
        b.advance(4)
        b.sync()
        out.append(b.download())
        b.close()
    for name, o in zip(KERNELS[1:], out[1:]):
        assert np.array_equal(out[0], o), name


def test_courant_near_ties_equal_direct_bitwise(gpu, cns):
    """A nearly uniform state (velocity amplitudes 1e-6, perturbation 1e-9): every cell's
    Courant number ties with the maximum to within the FP32 estimate's error, so the TMA
    kernels' exact-maximum search has to evaluate (almost) every cell in FP64; dt and the state
    must still equal the direct kernel's bit for bit."""
    n = (40, 36, 64)
    U0 = I.initial_state(n, amp=(1e-6, 1e-6, 1e-6), perturb=1e-9, seed=23)
    out = []
    for name in KERNELS:
        b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=cns.CNS_MIXED)
        b.set_kernel(getattr(cns, name))
        b.upload(U0)
        b.advance(3)
        b.sync()
        out.append((b.download(), b.last_dt()))
        b.close()
    for name, (u, dt) in zip(KERNELS[1:], out[1:]):
        assert dt == out[0][1], name
        assert np.array_equal(u, out[0][0]), name


def test_batched_boxes_on_every_assembly_kernel_match(gpu, cns):
    """Mixed boxes batched on each assembly kernel (one kernel per batch, and all three in one
    batch) give the same bits as on the direct kernel."""
    sizes = [(40, 24, 72), (64, 64, 64), (20, 36, 33)]
    U0 = [I.initial_state(n, perturb=1e-3, seed=30 + q) for q, n in enumerate(sizes)]

    def run(kernels):
        bt = cns.Batch()
        boxes = []
        for n, u, k in zip(sizes, U0, kernels):
            b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=cns.CNS_MIXED)
            b.set_kernel(getattr(cns, k))
            b.upload(u)
            bt.add(b)
            boxes.append(b)
        bt.advance(3)
        bt.sync()
        res = [b.download() for b in boxes]
        bt.close()
        for b in boxes:
            b.close()
        return res

    ref = run([KERNELS[0]] * 3)
    for ks in ([KERNELS[1]] * 3, [KERNELS[2]] * 3, list(KERNELS)):
        for a, r in zip(run(ks), ref):
            assert np.array_equal(a, r), ks


@pytest.mark.parametrize("n,ties", [((20, 12, 36), False), ((37, 19, 70), False), ((8, 8, 32), False),
                                     ((40, 36, 64), True)])
def test_fp64_tma_assembly_equals_direct(gpu, cns, n, ties):
    """FP64 boxes: the TMA-staged assembly (FP64 tensor maps, one block per SM) gives the direct
    assembly's bits, dt included (with ties: a nearly uniform state, where every cell is a
    Courant candidate); it is an option (slower on GB300), never the default, and the
    warp-specialised assembly stays mixed-only."""
    kw = dict(amp=(1e-6, 1e-6, 1e-6), perturb=1e-9, seed=23) if ties else dict(perturb=1e-3, seed=3)
    outs = []
    for kern in (cns.CNS_ASSEMBLE_DIRECT, cns.CNS_ASSEMBLE_TMA):
        b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
        try:
            assert b.kernel() == cns.CNS_ASSEMBLE_FX  # a new FP64 box's kernel
            b.set_kernel(kern)
            b.upload(I.initial_state(n, **kw))
            b.advance(4)
            outs.append((b.download(), b.last_dt()))
            b.sync()
            with pytest.raises(cns.CnsError):
                b.set_kernel(cns.CNS_ASSEMBLE_TMA_WS)
        finally:
            b.close()
    assert outs[0][1] == outs[1][1]
    assert np.array_equal(outs[0][0].view(np.uint64), outs[1][0].view(np.uint64))
