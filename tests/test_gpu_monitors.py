"""Monitors on the GPU against the oracle (itself pinned bitwise to the
reference's get_Cfl, timestepper and CheckSteadyStatebyMaxVal_omp): the CFL
number, the running velocity extremes and the next time step of two
successive calls, and the steady-state difference, all bitwise."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import seeded_field
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["g1", "g2"])
def test_cfl_timestepper_and_steady_state_match_oracle(oracle, name):
    w = WORKLOADS[name]
    g = Grid.of(w, oracle)
    with Simulation(w) as S:
        S.grid_uniform()
        S.start()
        umax = umin = None
        cmax = 0.0
        for seed in (1, 2):
            f = [seeded_field(g.ng, 10 * seed + q, lo, hi) for q, (lo, hi) in
                 enumerate([(0.2, 1.6 * seed), (-0.5, 0.5), (-0.3 * seed, 0.3)])]
            for q, nm in enumerate(("U0", "V0", "W0")):
                S.upload(nm, f[q])
            got = S.get_Cfl(capi.T0)
            c, umax, umin, cmax = oracle.cfl(g, w.dt, *f, umax=umax, umin=umin, cfl_max=cmax)
            assert got["cfl"] == c
            assert got["cfl_max"] == cmax
            assert got["u_max"] == list(umax) and got["u_min"] == list(umin)
            assert got["dt_next"] == oracle.timestepper(w.re, umax, umin)
        f3 = [seeded_field(g.ng, 70 + q, -1.0, 1.0) for q in range(3)]
        for q, nm in enumerate(("U3", "V3", "W3")):
            S.upload(nm, f3[q])
        f0 = [S.download(nm) for nm in ("U0", "V0", "W0")]
        want = oracle.steady_max(g, *f0, *f3)
        assert S.CheckSteadyStatebyMaxVal(capi.T0, capi.T3) == tuple(want)
