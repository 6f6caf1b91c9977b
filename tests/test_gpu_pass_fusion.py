"""The fused predictor-corrector step against the reference's call sequence
(GPU).

cfd_step evaluates the convection-diffusion of T0 once per step (every pass
of RUN_CPU_PC_METHOD.hpp:287-627 starts from the same T0), forms T1 = C +
source and the Poisson right-hand side in one pass kernel, and fuses the
source accumulation and the drag/lift sums into the projection.  The call
sequence through the individual entry points (ConvectionDifussion,
add_source, createBMatrix, pSolver, Pressure_transform_X_result,
update_UandF, accumulate_source, copy, BC_staggered_main/copy,
Delay_IO_CD_CL) is the reference's loop one function at a time.  In FP64
both do the same arithmetic in the same order, so they agree to the last
bits; the mixed path's right-hand side runs in float-float from the FP32
velocities, against FP64 arithmetic in the call sequence.
"""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _call_sequence(S, steps):
    """The reference's main loop through the individual entry points (the
    reference's index convention for the source coupling)."""
    cds = []
    for s in range(steps):
        S.clear_source()
        for p in range(4):
            S.ConvectionDifussion(S.T0, S.T1)
            S.add_source(S.T1)
            if s > 0:
                S.createBMatrix(S.T1)
                S.pSolver()
                S.Pressure_transform_X_result()
            S.update_UandF(S.T1, S.T3)
            if p < 3:
                S.accumulate_source()
        S.copy_velocity(S.T3, S.T0)
        S.BC_staggered_main(S.T0)
        S.BC_staggered_copy(S.T0, S.T1)
        cds.append(S.Delay_IO_CD_CL()[0])
    return cds


@pytest.mark.parametrize("name,precision", [("g1", capi.PREC_FP64), ("c1", capi.PREC_FP64),
                                            ("c1", capi.PREC_MIXED)])
def test_fused_step_matches_call_sequence(name, precision):
    w = WORKLOADS[name]
    steps = 3
    st = initial_velocity(w.nxc, w.nyc, w.nzc)
    with Simulation(w, tol=1e-10, precision=precision) as A, Simulation(w, tol=1e-10, precision=precision) as B:
        A.setup_cylinder(*st)
        B.setup_cylinder(*st)
        hist = [A.step() for _ in range(steps)]
        cds = _call_sequence(B, steps)
        fields = {k: (A.download(k), B.download(k)) for k in ("U0", "V0", "W0", "P", "F", "SRC")}
    rtol = 1e-13 if precision == capi.PREC_FP64 else 1e-6
    np.testing.assert_allclose([h["cd"] for h in hist], cds, rtol=rtol)
    for k, (a, b) in fields.items():
        assert rel_err(a, b) <= rtol, (k, rel_err(a, b))
