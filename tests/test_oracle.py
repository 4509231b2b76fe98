"""The oracle itself: the C restatement (oracle/cns_oracle.c) against the reference's own
cpu/ code -- bit for bit, through the committed golden fixtures (made by the reference) and,
where the reference tree is present, live against oracle/_ref."""
import numpy as np
import pytest

from conftest import golden
from cns_nospec_gb300 import initdata as I


def test_port_matches_golden_advance(oracle):
    for name in ("advance_8.npz", "advance_12.npz"):
        g = golden(name)
        n = g["U0"].shape[0] - 8
        U, dts = oracle.advance(g["U0"], int(g["nsteps"]), I.box_dx(n), float(g["cfl"]), float(g["eta"]),
                                float(g["alam"]))
        assert np.array_equal(U, g["U"]), name
        assert np.array_equal(dts, g["dts"]), name


def test_port_matches_golden_operators(oracle):
    g = golden("ops_6x9x11.npz")
    dx = tuple(g["dx"])
    Q, courno = oracle.ctoprim(g["U"], dx, True, 1.0e-50)
    assert np.array_equal(Q, g["Q"])
    assert courno == float(g["courno"])
    assert np.array_equal(oracle.hypterm(g["U"], g["Q"], dx), g["F"])
    assert np.array_equal(oracle.diffterm(g["Q"], dx, float(g["eta"]), float(g["alam"])), g["D"])


def test_port_matches_golden_fill_boundary(oracle):
    g = golden("fill_7x5x6.npz")
    assert np.array_equal(oracle.fill_boundary(g["U_in"]), g["U_out"])


def test_fill_boundary_is_periodic_image(oracle):
    g = golden("fill_7x5x6.npz")
    U = g["U_in"].copy()
    I.fill_periodic(U)
    assert np.array_equal(U, g["U_out"])


def test_port_thread_count_does_not_change_bits(oracle):
    U0 = I.initial_state((10, 12, 9), perturb=1e-3, seed=4)
    dx = I.box_dx((10, 12, 9))
    oracle.set_threads(1)
    a, da = oracle.advance(U0, 2, dx, I.CFL, I.ETA, I.ALAM)
    oracle.set_threads(4)
    b, db = oracle.advance(U0, 2, dx, I.CFL, I.ETA, I.ALAM)
    assert np.array_equal(a, b) and np.array_equal(da, db)


@pytest.mark.parametrize("n,steps", [(16, 2), (24, 1)])
def test_port_matches_reference_live(oracle, n, steps):
    if not oracle.have_ref():
        pytest.skip("reference tree not present; parity pinned by the golden fixtures")
    U0 = I.initial_state(n, perturb=1e-3, seed=2)
    a, da = oracle.advance(U0, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM, which="port")
    b, db = oracle.advance(U0, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM, which="ref")
    assert np.array_equal(a, b) and np.array_equal(da, db)


def test_port_operators_match_reference_live_noncubic(oracle):
    if not oracle.have_ref():
        pytest.skip("reference tree not present")
    n = (5, 13, 8)
    rng = np.random.default_rng(3)
    U = I.initial_state(n, perturb=1e-3, seed=9) * (1 + 1e-4 * rng.standard_normal((13, 21, 16, 5)))
    dx = (0.07, 0.03, 0.05)
    Qa, ca = oracle.ctoprim(U, dx, True, 1e-50, which="port")
    Qb, cb = oracle.ctoprim(U, dx, True, 1e-50, which="ref")
    assert np.array_equal(Qa, Qb) and ca == cb
    assert np.array_equal(oracle.hypterm(U, Qa, dx, "port"), oracle.hypterm(U, Qa, dx, "ref"))
    assert np.array_equal(oracle.diffterm(Qa, dx, 2e-4, 120.0, "port"), oracle.diffterm(Qa, dx, 2e-4, 120.0, "ref"))


def test_ctoprim_without_courno_leaves_q_identical(oracle):
    g = golden("ops_6x9x11.npz")
    dx = tuple(g["dx"])
    Q1, _ = oracle.ctoprim(g["U"], dx, True)
    Q2, c2 = oracle.ctoprim(g["U"], dx, False)
    assert c2 is None and np.array_equal(Q1, Q2)


def test_initial_state_matches_spec():
    n = 16
    U = I.initial_state(n)
    x = 2 * np.pi * (np.arange(n) + 0.5) / n
    i, j, k = 3, 5, 7
    X, Y, Z = x[i], x[j], x[k]
    rho = 1e-3 + 1e-5 * np.sin(X) * np.cos(2 * Y) * np.cos(3 * Z)
    u = 1.1e4 * np.sin(X) * np.sin(2 * Y) * np.sin(3 * Z)
    c = U[i + 4, j + 4, k + 4]
    assert abs(c[0] - rho) < 1e-18
    assert abs(c[1] / c[0] - u) < 1e-9
    # ghosts are periodic images
    assert np.array_equal(U[0, 4:-4, 4:-4], U[n, 4:-4, 4:-4])
    assert np.array_equal(U[-1, 4:-4, 4:-4], U[7, 4:-4, 4:-4])


def test_perturbation_is_seeded_and_bounded():
    a = I.initial_state(8, perturb=1e-3, seed=1)
    b = I.initial_state(8, perturb=1e-3, seed=1)
    c = I.initial_state(8, perturb=1e-3, seed=2)
    base = I.initial_state(8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    r = a[..., 0] / base[..., 0] - 1
    assert np.abs(r).max() <= 1e-3 + 1e-15 and np.abs(r).max() > 5e-4
