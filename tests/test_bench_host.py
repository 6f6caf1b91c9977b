"""Host logic of bench.py (CPU): the per-field comparison of the mixed and
FP64 legs.  The pressure of the all-Neumann problem is defined up to a
constant, so it is compared over the interior cells with its mean removed;
the ghost cells (two layers) are left out, since the edge and corner ghosts
follow no boundary condition and keep values independent of the solution's
constant."""
from __future__ import annotations

import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import bench  # noqa: E402


def _fields(w, rng, p_offset=0.0, stale_ghosts=0.0):
    gc = 2
    shape = (w.nxc + 2 * gc, w.nyc + 2 * gc, w.nzc + 2 * gc)
    u = rng.standard_normal(shape).ravel()
    p = rng.standard_normal(shape)
    p[gc:-gc, gc:-gc, gc:-gc] += p_offset
    p[:gc, :gc, :] = stale_ghosts  # edge ghosts no boundary condition writes
    return {"U0": u, "P": p.ravel()}


def test_pressure_compared_over_the_interior_without_its_constant():
    w = SimpleNamespace(nxc=6, nyc=5, nzc=4)
    a = _fields(w, np.random.default_rng(1), p_offset=0.0, stale_ghosts=7.0)
    b = _fields(w, np.random.default_rng(1), p_offset=3.25, stale_ghosts=-2.0)
    e = bench.field_errors(a, b, w)
    assert e["P"]["max_rel"] < 1e-14 and e["P"]["l2_rel"] < 1e-14
    assert e["U0"]["max_rel"] == 0.0


def test_field_errors_see_an_interior_difference():
    w = SimpleNamespace(nxc=6, nyc=5, nzc=4)
    a = _fields(w, np.random.default_rng(2))
    b = {k: v.copy() for k, v in a.items()}
    p = b["P"].reshape(w.nxc + 4, w.nyc + 4, w.nzc + 4)
    p[4, 3, 3] += 0.5
    e = bench.field_errors(a, b, w)
    assert e["P"]["max_rel"] > 0.05
