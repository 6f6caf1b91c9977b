"""The discrete adjoint at the 256x128x16 workload's specification (GPU;
long: runs only with CFDGPU_LONG_TESTS=1, a few minutes).

J = mean Cd over steps 250..500 of a 500-step run from the seeded start,
Re 100, dt 2e-3; parameters: the 128-value inflow profile (u on the x-min
face, one value per y cell) and the whole eta field; checkpoints every 50
steps with recompute.

* The FP64 gradient against FP64 central finite differences along 8 seeded
  directions: 4 in the inflow profile, 4 in eta restricted to the cells the
  cylinder touches (eta > 0).  FP64 here is CFD_PREC_FP64_DC (FP64 fields,
  the Poisson equation by FP64 defect correction to 1e-13).  J is piecewise
  smooth: QUICK's upwind selection switches where a face velocity changes
  sign, and the adjoint is the derivative with the base run's switches, so
  central differences agree only to the extent that they cross no switch;
  and a solve to relative residual 1e-13 leaves the solution accurate to
  about the condition number times that, a noise in J near 1e-8 relative.
  Measured (eps from 1e-6 to 1e-3): inflow 2e-5 to 8e-4, eta near the
  cylinder 1e-4 to 4e-4 at eps 1e-3 and up to 0.6 at eps 1e-6 (noise over
  eps), eta perturbed everywhere up to 0.2 at eps 1e-3 (the far field's
  near-zero v and w switch).  The test uses eps 1e-3 and asserts 1e-3 along
  the inflow directions (measured 2e-4 to 4e-4) and 2e-2 along the eta ones
  (measured 1e-4 to 1.5e-2, the largest where the directional derivative is
  smallest); the 1e-5 agreement holds on the small grid, where the
  differences cross no switch (tests/test_gpu_adjoint.py).
* The gradient with the FP32 forward and FP64-refined solves against the FP64
  gradient (measured 5e-7).
* The adjoint/forward time ratio at this specification, for both forwards
  (measured 2.27 FP64, 2.31 mixed; target at most 3).
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.adjoint import MeanDrag
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("CFDGPU_LONG_TESTS") != "1",
                                 reason="long run: set CFDGPU_LONG_TESTS=1")]

FIRST, LAST, INTERVAL = 250, 500, 50
EPS = 1e-3
DIRECTIONS = 8
GRAD_RTOL = 1e-3


def _model(precision, tol):
    return MeanDrag(WORKLOADS["c4"], FIRST, LAST, INTERVAL, precision=precision, tol=tol, maxit=50000)


def test_c4_gradient_against_fd_along_8_directions():
    w = WORKLOADS["c4"]
    out = {}
    m = _model(capi.PREC_FP64_DC, 1e-13)
    try:
        eta0 = m.default_eta().numpy()
        prof0 = np.full(w.nyc, float(w.bc_dir[0][0]))
        J0 = m.objective(prof0, eta0)
        g_in, g_eta = m.gradient()
        out["fp64"] = {"J": J0, "forward_s": m.last_run["forward_seconds"],
                       "adjoint_s": m.last_run["adjoint_seconds"],
                       "ratio": m.last_run["adjoint_seconds"] / m.last_run["forward_seconds"]}
        rng = np.random.default_rng(20261204)
        band = (eta0 > 0).astype(np.float64)
        errs = []
        for d in range(DIRECTIONS):
            inflow = d < DIRECTIONS // 2
            dp = rng.standard_normal(w.nyc) if inflow else np.zeros(w.nyc)
            de = np.zeros_like(eta0) if inflow else rng.standard_normal(eta0.size) * band
            jp = m.objective(prof0 + EPS * dp, eta0 + EPS * de)
            jm = m.objective(prof0 - EPS * dp, eta0 - EPS * de)
            fd = (jp - jm) / (2 * EPS)
            ad = float(np.dot(g_in, dp) + np.dot(g_eta, de))
            errs.append({"kind": "inflow" if inflow else "eta", "fd": fd, "adjoint": ad,
                         "rel": abs(ad - fd) / abs(fd)})
        out["directions"] = errs
    finally:
        m.close()
    mm = _model(capi.PREC_MIXED, w.tol)
    try:
        mm.objective(prof0, eta0)
        mg_in, mg_eta = mm.gradient()
        out["mixed"] = {"J": mm.last_run["J"], "forward_s": mm.last_run["forward_seconds"],
                        "adjoint_s": mm.last_run["adjoint_seconds"],
                        "ratio": mm.last_run["adjoint_seconds"] / mm.last_run["forward_seconds"],
                        "grad_rel_vs_fp64": float(np.linalg.norm(np.concatenate([mg_in - g_in, mg_eta - g_eta]))
                                                  / np.linalg.norm(np.concatenate([g_in, g_eta])))}
    finally:
        mm.close()
    print("\nC4ADJOINT " + json.dumps(out))
    assert max(e["rel"] for e in out["directions"] if e["kind"] == "inflow") < GRAD_RTOL
    assert max(e["rel"] for e in out["directions"] if e["kind"] == "eta") < 20 * GRAD_RTOL
    assert out["mixed"]["grad_rel_vs_fp64"] < 1e-3
    assert out["mixed"]["ratio"] < 3.0
