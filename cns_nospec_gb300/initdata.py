"""Synthetic initial states for periodic CNS boxes.

The field is the CNS_NoSpec test problem (the reference's Fortran initialiser,
fortran90/init_data.f90:61-81), evaluated cell-centred on the unit cube:
X = 2*pi*(i+1/2)/n0, Y = 2*pi*(j+1/2)/n1, Z = 2*pi*(k+1/2)/n2, dx = 1/n per axis, and

    u   = 1.1e4 * sin(X)  * sin(2Y) * sin(3Z)
    v   = 1.0e4 * sin(2X) * sin(4Y) * sin(Z)
    w   = 1.2e4 * sin(3X) * cos(2Y) * sin(2Z)
    rho = 1e-3 + 1e-5 * sin(X) * cos(2Y) * cos(3Z)
    e   = 2.5e9 + 1e-3 * sin(X) * cos(2Y) * sin(2Z)

with U = (rho, rho u, rho v, rho w, rho (e + |u|^2/2)).

Arrays use the reference's host layout (allocate_4D, cpu/helper_functions.cpp:100-122):
shape (n0+2*ng, n1+2*ng, n2+2*ng, 5), C order, component fastest.  Ghost cells hold the
periodic images of the interior (what fill_boundary, cpu/helper_functions.cpp:226-262,
produces).

Optional seeded perturbations: ``perturb`` multiplies rho, u, v, w by (1 + U(-perturb,
perturb)) drawn from a counter-based SplitMix64 stream (one draw per (cell, field), counter
= ((i*n1 + j)*n2 + k)*4 + field, field order rho, u, v, w), so any box size gives the same
draws on every machine.  ``amp`` scales the three velocity amplitudes.
"""
from __future__ import annotations

import math

import numpy as np

NG = 4
NC = 5

GAMMA = 1.4
CV = 8.3333333333e6
ETA = 1.8e-4
ALAM = 1.5e2
CFL = 0.5

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(counter: np.ndarray, seed: int) -> np.ndarray:
    """SplitMix64 finaliser of (seed * golden + counter); returns uint64 per element."""
    with np.errstate(over="ignore"):
        z = counter.astype(np.uint64) + np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * np.uint64(0x9E3779B97F4A7C15)
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(counter: np.ndarray, seed: int) -> np.ndarray:
    """Uniform doubles in [0, 1) from the top 53 bits of splitmix64."""
    return (splitmix64(counter, seed) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def fill_periodic(U: np.ndarray, ng: int = NG) -> np.ndarray:
    """Write the periodic images of the interior into every ghost cell (in place)."""
    n = [U.shape[a] - 2 * ng for a in range(3)]
    for a in range(3):
        idx = [slice(None)] * 4
        src = [slice(None)] * 4
        idx[a] = slice(0, ng)
        src[a] = slice(n[a], n[a] + ng)
        U[tuple(idx)] = U[tuple(src)]
        idx[a] = slice(n[a] + ng, n[a] + 2 * ng)
        src[a] = slice(ng, 2 * ng)
        U[tuple(idx)] = U[tuple(src)]
    return U


def initial_state(n, amp=(1.0, 1.0, 1.0), perturb: float = 0.0, seed: int = 1, ng: int = NG) -> np.ndarray:
    """Ghost-inclusive conserved state of shape (n0+2ng, n1+2ng, n2+2ng, 5), float64."""
    if isinstance(n, int):
        n = (n, n, n)
    n0, n1, n2 = (int(x) for x in n)
    twopi = 2.0 * math.pi
    X = twopi * (np.arange(n0) + 0.5) / n0
    Y = twopi * (np.arange(n1) + 0.5) / n1
    Z = twopi * (np.arange(n2) + 0.5) / n2
    sx, s2x, s3x = np.sin(X), np.sin(2 * X), np.sin(3 * X)
    s2y, s4y, c2y = np.sin(2 * Y), np.sin(4 * Y), np.cos(2 * Y)
    sz, s2z, s3z, c3z = np.sin(Z), np.sin(2 * Z), np.sin(3 * Z), np.cos(3 * Z)
    u = (1.1e4 * amp[0]) * (sx[:, None, None] * s2y[None, :, None] * s3z[None, None, :])
    v = (1.0e4 * amp[1]) * (s2x[:, None, None] * s4y[None, :, None] * sz[None, None, :])
    w = (1.2e4 * amp[2]) * (s3x[:, None, None] * c2y[None, :, None] * s2z[None, None, :])
    rho = 1.0e-3 + 1.0e-5 * (sx[:, None, None] * c2y[None, :, None] * c3z[None, None, :])
    e = 2.5e9 + 1.0e-3 * (sx[:, None, None] * c2y[None, :, None] * s2z[None, None, :])
    if perturb:
        cells = np.arange(n0 * n1 * n2, dtype=np.uint64).reshape(n0, n1, n2) * np.uint64(4)
        fac = [1.0 + perturb * (2.0 * uniform(cells + np.uint64(f), seed) - 1.0) for f in range(4)]
        rho = rho * fac[0]
        u = u * fac[1]
        v = v * fac[2]
        w = w * fac[3]
    U = np.empty((n0 + 2 * ng, n1 + 2 * ng, n2 + 2 * ng, NC), dtype=np.float64)
    inner = U[ng:ng + n0, ng:ng + n1, ng:ng + n2]
    inner[..., 0] = rho
    inner[..., 1] = rho * u
    inner[..., 2] = rho * v
    inner[..., 3] = rho * w
    inner[..., 4] = rho * (e + (u * u + v * v + w * w) / 2.0)
    return fill_periodic(U, ng)


def box_dx(n):
    """Cell sizes of an n0 x n1 x n2 box on the unit cube."""
    if isinstance(n, int):
        n = (n, n, n)
    return tuple(1.0 / float(x) for x in n)


def interior(U: np.ndarray, ng: int = NG) -> np.ndarray:
    return U[ng:-ng, ng:-ng, ng:-ng]


def normwise_error(a: np.ndarray, ref: np.ndarray, ng: int = NG):
    """Per-variable max|a-ref| / max|ref| over interior cells, and the RMS analogue."""
    ai, ri = interior(a, ng), interior(ref, ng)
    d = np.abs(ai - ri).reshape(-1, ai.shape[-1])
    r = np.abs(ri).reshape(-1, ri.shape[-1])
    mx = d.max(axis=0) / r.max(axis=0)
    rms = np.sqrt((d ** 2).mean(axis=0)) / np.sqrt((r ** 2).mean(axis=0))
    return mx, rms
