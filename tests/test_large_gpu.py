"""The largest boxes.  Thin boxes at the per-axis maximum (4096 cells) against the oracle run
live; and a 512^3 box, whose stencil sets hold more than 2^31 elements, against a 256^3 box:
a periodic box holding two periods of a field along each axis, with the same cell size,
advances exactly as one period does, so the 512^3 result is the 256^3 result tiled 2 x 2 x 2,
bit for bit (dt included), in both forms and through both the resident and the host-array
paths."""
import numpy as np
import pytest

from conftest import FP64_TOL, normwise
from cns_nospec_gb300 import initdata as I

pytestmark = pytest.mark.gpu


def bits(a):
    return a.view(np.uint64)


@pytest.mark.parametrize("n", [(4, 4, 4096), (4096, 5, 4), (6, 4096, 4)])
def test_axis_maximum_matches_oracle(gpu, cns, oracle, n):
    U0 = I.initial_state(n, perturb=1e-3, seed=7)
    dx = I.box_dx(n)
    ref, rdt = oracle.advance(U0, 2, dx, I.CFL, I.ETA, I.ALAM)
    U = U0.copy()
    dts = cns.advance_host(U, 2, dx, I.CFL, I.ETA, I.ALAM)
    err = normwise(U, ref)
    assert err.max() <= FP64_TOL, (n, err)
    assert np.allclose(dts, rdt, rtol=1e-13, atol=0)


def two_periods(U):
    """The ghost-inclusive state of the box that holds the interior of U twice along each axis."""
    n = U.shape[0] - 8
    big = np.empty((2 * n + 8,) * 3 + (5,))
    big[4:-4, 4:-4, 4:-4] = np.tile(U[4:-4, 4:-4, 4:-4], (2, 2, 2, 1))
    I.fill_periodic(big)
    return big


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_512cube_is_256cube_tiled(gpu, cns, precision):
    n, steps = 256, 2
    dx = I.box_dx(n)  # both boxes: cells of 1/256
    U0 = I.initial_state(n, perturb=1e-3, seed=3)
    small = cns.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=precision)
    small.upload(U0)
    small.advance(steps)
    small.sync()
    A = small.download()
    dt_a = small.last_dt()
    small.close()

    big_in = two_periods(U0)
    del U0
    big = cns.Box(2 * n, dx, I.CFL, I.ETA, I.ALAM, precision=precision)
    big.upload(big_in)
    big.advance(steps)
    big.sync()
    B = big.download()
    assert big.last_dt() == dt_a
    big.close()
    expect = np.tile(A[4:-4, 4:-4, 4:-4], (2, 2, 2, 1))
    assert np.array_equal(bits(expect), bits(B[4:-4, 4:-4, 4:-4]))
    del B

    if precision == 0:
        # the host-array path (page-locked: the fused upload and derivative kernel, stage 3
        # writing straight into the array) gives the same bits
        torch = pytest.importorskip("torch")
        t = torch.empty(big_in.shape, dtype=torch.float64, pin_memory=True)
        H = t.numpy()
        H[...] = big_in
        dts = cns.advance_host(H, steps, dx, I.CFL, I.ETA, I.ALAM)
        assert dts[-1] == dt_a[0]
        assert np.array_equal(bits(expect), bits(H[4:-4, 4:-4, 4:-4]))
        # release the 512^3 box the host path keeps for its next call
        cns.advance_host(I.initial_state(8), 0, I.box_dx(8), I.CFL, I.ETA, I.ALAM)
