"""The warm start of the defect-correction solves (GPU).

The reference starts every Poisson solve from the previous solve's solution
(the previous pass's).  The mixed and FP64-defect-correction contexts start
pass k from its own solutions of the last two steps, extrapolated linearly
in time (CFDGPU_WARM=prev keeps the reference's start).  Both converge every
solve to the tolerance, so the steps agree to it.  Past the impulsive
start's transient (its first steps change the pressure too fast for the
extrapolation) the extrapolated start needs fewer defect-correction sweeps:
measured at 512x256x32 from step 20 on, 8 sweeps a step against 12."""
from __future__ import annotations

import os

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu


def _run(w, warm, steps, **kw):
    old = os.environ.get("CFDGPU_WARM")
    os.environ["CFDGPU_WARM"] = warm
    try:
        with Simulation(w, tol=1e-10, **kw) as S:
            S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
            hist = [S.step() for _ in range(steps)]
            return hist, {k: S.download(k) for k in ("U0", "V0", "W0")}
    finally:
        if old is None:
            os.environ.pop("CFDGPU_WARM", None)
        else:
            os.environ["CFDGPU_WARM"] = old


@pytest.mark.parametrize("precision,periodic", [(capi.PREC_MIXED, False), (capi.PREC_FP64_DC, False),
                                                (capi.PREC_MIXED, True)])
def test_extrapolated_warm_start_agrees_and_saves_sweeps(precision, periodic):
    w = WORKLOADS["c1"]
    h1, f1 = _run(w, "extrapolate", 30, precision=precision, periodic_z=periodic)
    h0, f0 = _run(w, "prev", 30, precision=precision, periodic_z=periodic)
    # two solves to relative residual 1e-10 leave the pressure accurate to
    # about the condition number times that, which reaches the drag at 1e-7
    # (measured 2.3e-7 over 30 steps); the mixed-vs-FP64 drag criterion
    np.testing.assert_allclose([h["cd"] for h in h1], [h["cd"] for h in h0], rtol=1e-6)
    for h in h1[1:]:
        assert all(r < 1e-10 for r in h["relres"]), h["relres"]
    for k in f1:
        d = np.abs(f1[k] - f0[k]).max() / np.abs(f0[k]).max()
        assert d < 1e-6, (k, d)
    # past the transient
    assert sum(sum(h["outer"]) for h in h1[15:]) < sum(sum(h["outer"]) for h in h0[15:])
