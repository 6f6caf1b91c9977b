"""Seeded, layout-independent initial conditions.

The reference starts from u = 1, v = w = 0 everywhere
(inc/run/RUN_CPU_PC_METHOD.hpp:77-87).  The workloads add a uniform random
perturbation in [-amp, amp] on every interior face of u, v and w.  Each value
is a pure function of (seed, component, global interior index), drawn with
splitmix64, so any decomposition or memory layout reproduces the same field.
"""
from __future__ import annotations

import numpy as np

DEFAULT_SEED = 20261203
_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser over uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, comp: int, index: np.ndarray) -> np.ndarray:
    key = np.uint64(seed) ^ (np.uint64(comp) << np.uint64(56)) ^ index.astype(np.uint64)
    return (splitmix64(key) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def perturbation(nxc: int, nyc: int, nzc: int, comp: int, amp: float = 1e-3,
                 seed: int = DEFAULT_SEED) -> np.ndarray:
    """(nxc, nyc, nzc) block of uniform values in [-amp, amp]."""
    idx = np.arange(nxc * nyc * nzc, dtype=np.uint64)
    return (amp * (2.0 * uniform01(seed, comp, idx) - 1.0)).reshape(nxc, nyc, nzc)


def initial_velocity(nxc: int, nyc: int, nzc: int, amp: float = 1e-3, seed: int = DEFAULT_SEED,
                     u_inf: float = 1.0, spanwise: float = 0.0):
    """Ghosted (u, v, w) arrays in the reference layout (k fastest).

    u = u_inf + perturbation, v = w = perturbation on interior faces; ghost
    values are the uniform start (the first boundary update overwrites them).
    spanwise > 0 adds spanwise * sin(2 pi k / nzc) to v (z-periodic seed).
    """
    nx, ny, nz = nxc + 4, nyc + 4, nzc + 4
    out = []
    for comp, base in enumerate((u_inf, 0.0, 0.0)):
        a = np.full((nx, ny, nz), base)
        if amp:
            a[2:-2, 2:-2, 2:-2] += perturbation(nxc, nyc, nzc, comp, amp, seed)
        if comp == 1 and spanwise:
            k = np.arange(nzc)
            a[2:-2, 2:-2, 2:-2] += spanwise * np.sin(2.0 * np.pi * k / nzc)[None, None, :]
        out.append(np.ascontiguousarray(a.ravel()))
    return tuple(out)


def seeded_field(n: int, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """Flat array of n seeded uniform values in [lo, hi) (test inputs)."""
    u = uniform01(seed, 0, np.arange(n, dtype=np.uint64))
    return lo + (hi - lo) * u
