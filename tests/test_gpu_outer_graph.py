"""The mixed defect correction as one CUDA graph (GPU).

With the multigrid-CG inner solve, a Poisson solve of the mixed and
FP64-defect-correction paths runs as one graph: the first residual, then a
WHILE node over the sweeps whose body nests the inner solve's own WHILE node
(api.cu, solve_mixed_graph).  CFDGPU_OUTER_LOOP=host gives the host loop
(two waits a sweep).  Both issue the same kernels in the same order, so the
steps agree bit for bit, with the same iteration and sweep counts."""
from __future__ import annotations

import os

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu


def _run(w, host, steps=3, **kw):
    old = os.environ.get("CFDGPU_OUTER_LOOP")
    if host:
        os.environ["CFDGPU_OUTER_LOOP"] = "host"
    else:
        os.environ.pop("CFDGPU_OUTER_LOOP", None)
    try:
        with Simulation(w, tol=1e-10, **kw) as S:
            S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
            hist = [S.step() for _ in range(steps)]
            return hist, {k: S.download(k) for k in ("U0", "V0", "W0", "P")}
    finally:
        if old is None:
            os.environ.pop("CFDGPU_OUTER_LOOP", None)
        else:
            os.environ["CFDGPU_OUTER_LOOP"] = old


@pytest.mark.parametrize("precision,periodic", [(capi.PREC_MIXED, False), (capi.PREC_FP64_DC, False),
                                                (capi.PREC_MIXED, True)])
def test_defect_correction_graph_matches_host_loop(precision, periodic):
    w = WORKLOADS["c1"]
    h1, f1 = _run(w, False, precision=precision, periodic_z=periodic)
    h0, f0 = _run(w, True, precision=precision, periodic_z=periodic)
    for key in ("cd", "iters", "outer", "relres"):
        assert [h[key] for h in h1] == [h[key] for h in h0], key
    assert all(r < 1e-10 for h in h1[1:] for r in h["relres"])
    for k in f1:
        np.testing.assert_array_equal(f1[k], f0[k], err_msg=k)
