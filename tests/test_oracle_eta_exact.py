"""Exact-area option of the cylinder's volume fraction (an extension: the
reference sub-samples cut cells nsub x nsub).  The oracle's area routine is
checked against closed forms and numerical quadrature, the plane of fractions
against the disc area, and the reference's sub-sampling against it."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from oracle.oracle import Grid


@pytest.fixture(scope="module")
def area(oracle):
    f = oracle.lib.og_disc_rect_area
    f.restype = C.c_double
    f.argtypes = [C.c_double] * 5
    return f


def test_area_closed_forms(area):
    r = 0.7
    assert area(-1, 1, -1, 1, r) == pytest.approx(math.pi * r * r, rel=1e-14)
    assert area(0, 1, 0, 1, r) == pytest.approx(math.pi * r * r / 4, rel=1e-14)
    assert area(-1, 0, -1, 1, r) == pytest.approx(math.pi * r * r / 2, rel=1e-14)
    assert area(0.8, 1.0, -1, 1, r) == 0.0
    assert area(-0.1, 0.1, -0.1, 0.1, r) == pytest.approx(0.04, rel=1e-14)  # inside


def test_area_matches_quadrature(area):
    from scipy.integrate import quad
    rng = np.random.default_rng(9)
    r = 0.5
    for _ in range(40):
        x0, y0 = rng.uniform(-0.7, 0.5, 2)
        x1, y1 = x0 + rng.uniform(0.01, 0.4), y0 + rng.uniform(0.01, 0.4)

        def chord(t):
            s = math.sqrt(max(r * r - t * t, 0.0))
            return max(0.0, min(y1, s) - max(y0, -s))
        a, b = max(x0, -r), min(x1, r)
        want = quad(chord, a, b, epsabs=1e-14, epsrel=1e-13, limit=200)[0] if a < b else 0.0
        assert area(x0, x1, y0, y1, r) == pytest.approx(want, rel=1e-10, abs=1e-14)


@pytest.mark.parametrize("name", ["g1", "c1"])
def test_exact_plane_sums_to_the_disc_area(oracle, name):
    w = WORKLOADS[name]
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y, w.radius, nsub=0)
    plane = eta.reshape(g.nx, g.ny, g.nz)[2:-2, 2:-2, 0]
    dx, dy = g.m["Dx"][2:-2], g.m["Dy"][2:-2]
    total = (plane * np.outer(dx, dy)).sum()
    assert total == pytest.approx(math.pi * w.radius ** 2, rel=1e-12)
    assert plane.min() >= 0.0 and plane.max() <= 1.0


def test_subsampling_converges_to_exact(oracle):
    w = WORKLOADS["c1"]
    g = Grid.of(w, oracle)
    ex = oracle.eta_cylinder_z(g, w.cx, w.center_y, w.radius, nsub=0)
    errs = []
    for nsub in (10, 40, 160):
        sub = oracle.eta_cylinder_z(g, w.cx, w.center_y, w.radius, nsub=nsub)
        errs.append(np.abs(sub - ex).max())
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 2.0 / 160
