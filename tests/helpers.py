"""Helpers shared by the test modules: seeded inputs and tolerances."""
from __future__ import annotations

import numpy as np

from cfd_nssolver_forhpc_gb300.initial import seeded_field

# Per-kernel tolerance of the FP64 CUDA kernels against the FP64 oracle.  The
# kernels replace divisions by multiplications with tabulated reciprocals and
# use fused multiply-adds, so they differ from the reference by rounding only.
KERNEL_RTOL = 1e-13


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| (0 when both vanish)."""
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    return d / scale if scale > 0 else d


SEEDS = dict(u0=11, v0=12, w0=13, u1=14, v1=15, w1=16, p=17, f=18, x=19, bc=20, sor_p=21)


def kernel_inputs(ng: int, n: int) -> dict:
    """Seeded inputs of the single-kernel fixtures (velocities O(1)); the
    same inputs tests/golden/make_golden.py fed to the reference."""
    s = SEEDS
    return dict(
        u0=1.0 + 0.3 * seeded_field(ng, s["u0"]), v0=0.3 * seeded_field(ng, s["v0"]),
        w0=0.3 * seeded_field(ng, s["w0"]), u1=seeded_field(ng, s["u1"]),
        v1=seeded_field(ng, s["v1"]), w1=seeded_field(ng, s["w1"]), p=seeded_field(ng, s["p"]),
        f=seeded_field(3 * n, s["f"]), x=seeded_field(n, s["x"]),
        bc=[seeded_field(ng, s["bc"] + q) for q in range(4)],
        sor_p=0.01 * seeded_field(ng, s["sor_p"]))


def seeded(n: int, seed: int, lo=-1.0, hi=1.0) -> np.ndarray:
    return seeded_field(n, seed, lo, hi)
