"""The exact-area cylinder fraction on the GPU (cfd_eta_cylinder_z with nsub =
0) against the oracle's, which the CPU tests pin to closed forms, quadrature
and the disc area."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["g1", "c1"])
def test_exact_eta_matches_oracle(oracle, name):
    w = WORKLOADS[name]
    g = Grid.of(w, oracle)
    want = oracle.eta_cylinder_z(g, w.cx, w.center_y, w.radius, nsub=0)
    with Simulation(w) as S:
        S.grid_uniform()
        S.DFIB_CylinderZ(w.cx, w.center_y, w.radius, 0)
        got = S.download("ETA")
    assert np.abs(got - want).max() < 1e-13
    with Simulation(w, precision=capi.PREC_MIXED) as S:
        S.grid_uniform()
        S.DFIB_CylinderZ(w.cx, w.center_y, w.radius, 0)
        got32 = S.download("ETA")
    assert np.abs(got32 - want).max() < 1e-7
