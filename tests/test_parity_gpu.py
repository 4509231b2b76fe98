"""Parity of the GPU library (called through the C ABI) with the reference's cpu/ path.

Small cases compare against the committed golden fixtures (made by the reference itself) and
against the oracle run live on identical inputs, up to 128^3 x 100 steps and 256^3 x 3 steps;
full-size cases also check properties that do not need the oracle (bitwise periodic
shift-equivariance, mass conservation).  Tolerance:
normwise relative error per conserved variable <= 1e-12 (FP64_TOL)."""
import numpy as np
import pytest

from conftest import FP64_TOL, MIXED_TOL, golden, normwise
from cns_nospec_gb300 import initdata as I

pytestmark = pytest.mark.gpu


def _lohi(U):
    n = [U.shape[a] - 8 for a in range(3)]
    return [4, 4, 4], [x + 3 for x in n], n


def test_ctoprim_matches_golden(gpu, cns):
    g = golden("ops_6x9x11.npz")
    U = g["U"].copy()
    lo, hi, _ = _lohi(U)
    Q = np.zeros(U.shape[:3] + (6,))
    c = cns.ctoprim(lo, hi, U, Q, tuple(g["dx"]), 4, courno=1.0e-50)
    # q over every cell, ghosts included (cpu/ctoprim.cpp:26-43): pointwise relative
    rel = np.abs(Q - g["Q"]) / np.maximum(np.abs(g["Q"]), 1e-300)
    assert rel.max() < 1e-14
    assert abs(c - float(g["courno"])) <= 1e-14 * float(g["courno"])
    # without courno the q output is the same
    Q2 = np.zeros_like(Q)
    assert cns.ctoprim(lo, hi, U, Q2, tuple(g["dx"]), 4) is None
    assert np.array_equal(Q, Q2)


def test_hypterm_matches_golden(gpu, cns):
    g = golden("ops_6x9x11.npz")
    lo, hi, n = _lohi(g["U"])
    F = np.zeros(tuple(n) + (5,))
    cns.hypterm(lo, hi, 4, tuple(g["dx"]), g["U"], g["Q"], F)
    err = normwise(F, g["F"], interior_only=False)
    assert err.max() <= FP64_TOL, err


def test_diffterm_matches_golden(gpu, cns):
    g = golden("ops_6x9x11.npz")
    lo, hi, n = _lohi(g["U"])
    D = np.full(tuple(n) + (5,), 7.0)
    cns.diffterm(lo, hi, 4, tuple(g["dx"]), g["Q"], D, float(g["eta"]), float(g["alam"]))
    assert np.all(D[..., 0] == 0.0)
    err = normwise(D, g["D"], interior_only=False)
    assert err.max() <= FP64_TOL, err


def test_fill_boundary_matches_golden_bitwise(gpu, cns):
    g = golden("fill_7x5x6.npz")
    U = g["U_in"].copy()
    cns.fill_boundary(U, [7, 5, 6], [15, 13, 14])
    assert np.array_equal(U, g["U_out"])


@pytest.mark.parametrize("name", ["advance_8.npz", "advance_12.npz"])
def test_advance_matches_golden(gpu, cns, name):
    g = golden(name)
    U = g["U0"].copy()
    n = U.shape[0] - 8
    dts = cns.advance_host(U, int(g["nsteps"]), I.box_dx(n), float(g["cfl"]), float(g["eta"]), float(g["alam"]))
    err = normwise(U, g["U"])
    assert err.max() <= FP64_TOL, err
    assert np.allclose(dts, g["dts"], rtol=1e-13, atol=0)
    # ghost cells: the reference leaves the fill made at the start of the last step
    assert normwise(U, g["U"], interior_only=False).max() <= FP64_TOL


def test_new_advance_dropin_one_step(gpu, cns, oracle):
    """new_advance with the reference's h_const: interior within 1e-12, ghosts bit-identical."""
    n = 10
    U0 = I.initial_state(n, perturb=1e-3, seed=21)
    ref, rdt = oracle.advance(U0, 1, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    h = cns.read_configurations(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, nsteps=1)
    U = U0.copy()
    dt = cns.new_advance(U, None, None, None, None, h)
    assert abs(dt - rdt[0]) <= 1e-13 * rdt[0]
    assert normwise(U, ref).max() <= FP64_TOL
    inner = np.zeros(U.shape[:3], bool)
    inner[4:-4, 4:-4, 4:-4] = True
    assert np.array_equal(U[~inner], ref[~inner])


def test_advance_config0_32cube_10_steps(gpu, cns, oracle):
    """32^3, 10 RK3 steps, the reference's initial field: <= 1e-12 normwise per variable."""
    n = 32
    U0 = I.initial_state(n)
    ref, rdt = oracle.advance(U0, 10, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    U = U0.copy()
    dts = cns.advance_host(U, 10, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    err = normwise(U, ref)
    assert err.max() <= FP64_TOL, err
    assert np.allclose(dts, rdt, rtol=1e-13, atol=0)


@pytest.mark.parametrize("n", [(20, 24, 16), (17, 9, 33), (4, 6, 5)])
def test_advance_noncubic_matches_oracle(gpu, cns, oracle, n):
    U0 = I.initial_state(n, perturb=1e-3, seed=5)
    dx = I.box_dx(n)
    ref, rdt = oracle.advance(U0, 3, dx, I.CFL, I.ETA, I.ALAM)
    U = U0.copy()
    dts = cns.advance_host(U, 3, dx, I.CFL, I.ETA, I.ALAM)
    err = normwise(U, ref)
    assert err.max() <= FP64_TOL, (n, err)
    assert np.allclose(dts, rdt, rtol=1e-13, atol=0)


@pytest.mark.parametrize("tile", [(3, 1, 4), (1, 3, 4), (2, 2, 4)])
def test_banded_tile_walk_matches_oracle(gpu, cns, oracle, tile):
    """A box long enough in k for its tiles to be walked in several bands of j rows, the last one
    partial (200 rows in bands of 16 or 32), in both forms, against the oracle; the band sizes
    follow the tile shape."""
    n = (12, 200, 264)
    U0 = I.initial_state(n, perturb=1e-3, seed=6)
    dx = I.box_dx(n)
    ref, _ = oracle.advance(U0, 2, dx, I.CFL, I.ETA, I.ALAM)
    for prec, tol in ((cns.CNS_FP64, FP64_TOL), (cns.CNS_MIXED, MIXED_TOL)):
        box = cns.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=prec)
        try:
            box.set_tile(tile)
            box.upload(U0)
            box.advance(2)
            box.sync()
            err = normwise(box.download(), ref)
        finally:
            box.close()
        assert err.max() <= tol, (prec, tile, err)


def test_advance_perturbed_128cube_100_steps(gpu, cns, oracle):
    """128^3, perturbed field, 100 RK3 steps against the oracle run live."""
    n = 128
    U0 = I.initial_state(n, perturb=1e-3, seed=1)
    ref, rdt = oracle.advance(U0, 100, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box.upload(U0)
    box.advance(100)
    box.sync()
    U = box.download()
    err = normwise(U, ref)
    assert err.max() <= FP64_TOL, err
    dt, steps = box.last_dt()
    assert steps == 100 and abs(dt - rdt[-1]) <= 1e-12 * rdt[-1]


def test_advance_256cube_3_steps(gpu, cns, oracle):
    """256^3 (the mixed-form comparison size), 3 RK3 steps against the oracle run live: the FP64
    form within FP64_TOL, the mixed form within MIXED_TOL."""
    n = 256
    U0 = I.initial_state(n, perturb=1e-3, seed=1)
    ref, rdt = oracle.advance(U0, 3, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    for prec, tol in ((cns.CNS_FP64, FP64_TOL), (cns.CNS_MIXED, MIXED_TOL)):
        box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
        try:
            box.upload(U0)
            box.advance(3)
            box.sync()
            U = box.download()
        finally:
            box.close()
        err = normwise(U, ref)
        assert err.max() <= tol, (prec, err)


def test_resident_box_equals_host_path_bitwise(gpu, cns):
    n = (24, 20, 28)
    U0 = I.initial_state(n, perturb=1e-3, seed=8)
    dx = I.box_dx(n)
    A = U0.copy()
    cns.advance_host(A, 4, dx, I.CFL, I.ETA, I.ALAM)
    box = cns.Box(n, dx, I.CFL, I.ETA, I.ALAM)
    box.upload(U0)
    box.advance(2)
    box.advance(2)
    B = box.download()
    assert np.array_equal(A[4:-4, 4:-4, 4:-4], B[4:-4, 4:-4, 4:-4])
    # a resident download carries the periodic images of the current state
    C = B.copy()
    I.fill_periodic(C)
    assert np.array_equal(B, C)


def test_timed_path_equals_graph_path(gpu, cns):
    n = 24
    U0 = I.initial_state(n, perturb=1e-3, seed=9)
    a = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    a.upload(U0)
    b.upload(U0)
    a.advance(3)
    ms, launches, total = b.advance_timed(3)
    assert launches == [3 * 3, 3 * 3, 3, 0]
    assert total > 0 and all(x >= 0 for x in ms)
    assert np.array_equal(a.download(), b.download())


def test_full_size_256_shift_equivariance_and_mass(gpu, cns):
    """At 256^3 (no oracle): advancing a periodically shifted state gives the shifted result
    bit for bit, and total mass is conserved to rounding."""
    n = 256
    U0 = I.initial_state(n, perturb=1e-3, seed=1)
    inner = U0[4:-4, 4:-4, 4:-4]
    shifted = np.ascontiguousarray(np.roll(inner, (37, -11, 5), axis=(0, 1, 2)))
    U1 = np.zeros_like(U0)
    U1[4:-4, 4:-4, 4:-4] = shifted
    I.fill_periodic(U1)
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box.upload(U0)
    box.advance(3)
    A = box.download()
    box.upload(U1)
    box.advance(3)
    B = box.download()
    assert np.array_equal(np.roll(A[4:-4, 4:-4, 4:-4], (37, -11, 5), axis=(0, 1, 2)), B[4:-4, 4:-4, 4:-4])
    m0 = inner[..., 0].sum()
    m1 = A[4:-4, 4:-4, 4:-4, 0].sum()
    assert abs(m1 - m0) <= 1e-12 * abs(m0)


def test_bad_state_raises_status_not_fault(gpu, cns):
    n = 16
    U0 = I.initial_state(n)
    U0[9, 9, 9, 0] = -1e-3  # negative density at one cell
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box.upload(U0)
    box.advance(1)
    with pytest.raises(cns.CnsError) as ei:
        box.sync()
    assert ei.value.code == 3
    assert box.health() & 1
    # the context stays usable: a clean state advances normally afterwards
    box.upload(I.initial_state(n))
    box.advance(1)
    box.sync()


@pytest.mark.parametrize("n,steps,perturb", [(32, 10, 0.0), (64, 40, 1e-3)])
def test_pointwise_relative_error_against_the_oracle(gpu, cns, oracle, n, steps, perturb):
    """Cell by cell: |GPU - oracle| / |oracle| <= 1e-12 for every cell of rho and rho E (which keep
    away from zero) and for every cell of the momenta whose magnitude is at least a tenth of its
    field's maximum; down to a thousandth of the maximum, near the momenta's zero crossings,
    <= 1e-11 (measured: 6.7e-14 and 4.1e-12 at 128^3 x 100 steps)."""
    U0 = I.initial_state(n, perturb=perturb, seed=1)
    ref, _ = oracle.advance(U0, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box.upload(U0)
    box.advance(steps)
    box.sync()
    a = box.download()[4:-4, 4:-4, 4:-4].reshape(-1, 5)
    box.close()
    r = ref[4:-4, 4:-4, 4:-4].reshape(-1, 5)
    for l in range(5):
        mag = np.abs(r[:, l])
        for thr, tol in ((0.1, 1e-12), (1e-3, 1e-11)):
            m = mag >= (0.0 if l in (0, 4) else thr) * mag.max()
            rel = (np.abs(a[m, l] - r[m, l]) / mag[m]).max()
            assert rel <= (1e-12 if l in (0, 4) else tol), (l, thr, rel)
