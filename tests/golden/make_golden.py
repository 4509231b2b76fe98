"""Generate the golden fixtures in this folder from the reference's own cpu/ code.

The reference ships no fixtures (its harnesses open ../testcases/*, which is absent), so the
goldens are produced by running the reference's unmodified cpu/ sources, compiled by
oracle/Makefile into oracle/_ref/libcnsref.so, on seeded inputs.  Run from the repository
root where the reference tree is available:

    python tests/golden/make_golden.py

Fixtures (numpy .npz, float64):
  advance_8.npz     8^3 box, perturbed field (seed 1), 3 new_advance steps: U0, U3, dts
  advance_12.npz    12^3 box, velocity amplitudes (0.9, 1.1, 1.2), eta x1.1, alam x0.9,
                    perturbed (seed 7), 2 steps: U0, U2, dts, eta, alam
  ops_6x9x11.npz    non-cubic 6x9x11 box with non-periodic ghost data: U, Q = ctoprim(U),
                    courno, F = hypterm(U, Q), D = diffterm(Q)
  fill_7x5x6.npz    fill_boundary on a 7x5x6 box whose ghosts hold noise: U_in, U_out
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cns_nospec_gb300 import initdata as I  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    O.build(ref=True)
    if not O.have_ref():
        raise SystemExit("the reference library is not built (needs the reference tree)")

    U0 = I.initial_state(8, perturb=1e-3, seed=1)
    U3, dts = O.advance(U0, 3, I.box_dx(8), I.CFL, I.ETA, I.ALAM, which="ref")
    np.savez_compressed(os.path.join(HERE, "advance_8.npz"), U0=U0, U=U3, dts=dts, nsteps=3,
                        cfl=I.CFL, eta=I.ETA, alam=I.ALAM)

    eta, alam = I.ETA * 1.1, I.ALAM * 0.9
    U0 = I.initial_state(12, amp=(0.9, 1.1, 1.2), perturb=1e-3, seed=7)
    U2, dts = O.advance(U0, 2, I.box_dx(12), I.CFL, eta, alam, which="ref")
    np.savez_compressed(os.path.join(HERE, "advance_12.npz"), U0=U0, U=U2, dts=dts, nsteps=2,
                        cfl=I.CFL, eta=eta, alam=alam)

    n = (6, 9, 11)
    rng = np.random.default_rng(11)
    U = I.initial_state(n, perturb=1e-3, seed=3)
    U = U * (1.0 + 1e-3 * rng.standard_normal(U.shape))  # ghost data that is not a periodic image
    dx = I.box_dx(n)
    Q, courno = O.ctoprim(U, dx, True, 1.0e-50, which="ref")
    F = O.hypterm(U, Q, dx, which="ref")
    D = O.diffterm(Q, dx, I.ETA, I.ALAM, which="ref")
    np.savez_compressed(os.path.join(HERE, "ops_6x9x11.npz"), U=U, Q=Q, courno=courno, F=F, D=D,
                        dx=np.array(dx), eta=I.ETA, alam=I.ALAM)

    n = (7, 5, 6)
    U = I.initial_state(n, perturb=1e-3, seed=5)
    U[:4] = rng.standard_normal(U[:4].shape)
    U[:, -4:] = rng.standard_normal(U[:, -4:].shape)
    U[:, :, :4] = rng.standard_normal(U[:, :, :4].shape)
    Uo = O.fill_boundary(U, which="ref")
    np.savez_compressed(os.path.join(HERE, "fill_7x5x6.npz"), U_in=U, U_out=Uo)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
