"""Smagorinsky LES option on the GPU (TERBULENCE_SMAGORINSKY in the
reference): the eddy viscosity and the convection-diffusion with nu + nu_t
against the oracle, whose LES functions are pinned bitwise to the reference
compiled with the model on (test_oracle_vs_reference.py).  The GPU evaluates
delta = (Dx Dy Dz)^(1/3) with CUDA's pow, so agreement is to a few ulp."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity, seeded_field
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _fields(g, seed):
    return [seeded_field(g.ng, seed + q, lo, hi) for q, (lo, hi) in enumerate([(0.5, 1.5), (-0.4, 0.4), (-0.4, 0.4)])]


@pytest.mark.parametrize("name", ["g1", "g2"])
def test_eddy_viscosity_and_les_convdiff_match_oracle(oracle, name):
    w = WORKLOADS[name]
    g = Grid.of(w, oracle)
    f = _fields(g, 31)
    vis_o = oracle.smagorinsky(g, *f)
    out_o = [g.zeros() for _ in range(3)]
    oracle.convdiff_les(g, w.dt, 1.0 / w.re, vis_o, *f, *out_o)
    with Simulation(w, les=True) as S:
        S.grid_uniform()
        for nm, a in zip(("U0", "V0", "W0"), f):
            S.upload(nm, a)
        S.SmagorinskyModel(capi.T0)
        vis = S.download("VIS")
        np.testing.assert_allclose(vis, vis_o, rtol=1e-14, atol=0)
        for nm in ("U1", "V1", "W1"):
            S.upload(nm, np.zeros(g.ng))
        S.ConvectionDifussion(capi.T0, capi.T1)
        for nm, b in zip(("U1", "V1", "W1"), out_o):
            assert rel_err(S.download(nm), b) < 1e-13, nm


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_les_steps_run_and_change_the_flow(prec):
    w = WORKLOADS["c1"]
    out = {}
    for les in (False, True):
        with Simulation(w, tol=1e-8, precision=prec, les=les) as S:
            S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
            hist = [S.step() for _ in range(4)]
            out[les] = (np.array([h["cd"] for h in hist]), S.download("U0"))
            if les:
                vis = S.download("VIS")
                assert np.all(np.isfinite(vis)) and vis.max() > 0
    assert np.all(np.isfinite(out[True][0]))
    assert not np.array_equal(out[True][1], out[False][1])
    # a small eddy viscosity on this grid: the drag moves, but little
    np.testing.assert_allclose(out[True][0], out[False][0], rtol=5e-2)
