"""Strouhal number of the 128x64x8 cylinder wake on the GPU (long: it runs
only with CFDGPU_LONG_TESTS=1; about ten minutes of GPU time and two of CPU).

The reference computes no Strouhal number, it logs Cd and Cl only
(RUN_CPU_PC_METHOD.hpp:414-435), so the shedding frequency is estimated from
the lift history (cfd_nssolver_forhpc_gb300/strouhal.py, tested on synthetic
signals in tests/test_strouhal.py).  The run: the mixed-precision step for
60 time units from the seeded start, which develops the shedding; then, from
that one state, 30 more time units in mixed precision and in FP64.  Checks:

* the two continuations shed at the same Strouhal number (1e-4) with the
  same mean drag (1e-5); measured on GB300: St 0.16131 for both (relative
  difference 1e-6), mean drag 1.45319 (2e-6), from a spin-up shedding at
  0.157 (FFT 0.165);
* the FP64 continuation follows the oracle (the C restatement of the
  reference's step) from the same state: drag and lift (relative to the
  drag) within 1e-6 over the first 100 steps, the workload's solver
  tolerance being 1e-8 (measured 3.0e-7 and 7.1e-8: the two BiCGSTAB
  implementations sum in different orders and stop at different iterates
  inside the tolerance).  The oracle needs about half a second per step
  here, so it covers 0.2 time units, not a period.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from cfd_nssolver_forhpc_gb300.strouhal import strouhal
from oracle.oracle import Grid

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("CFDGPU_LONG_TESTS") != "1",
                                 reason="long run: set CFDGPU_LONG_TESTS=1")]

SPINUP, CONTINUE, ORACLE_STEPS = 60.0, 30.0, 100


def _run(S, steps):
    t, cd, cl = [], [], []
    for _ in range(steps):
        h = S.step()
        t.append(h["time"])
        cd.append(h["cd"])
        cl.append(h["cl"])
    return np.array(t), np.array(cd), np.array(cl)


def test_strouhal_mixed_vs_fp64_and_fp64_vs_oracle(oracle):
    w = WORKLOADS["c1"]
    with Simulation(w, precision=capi.PREC_MIXED) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        t, cd, cl = _run(S, int(round(SPINUP / w.dt)))
        state = S.state()
    spin = strouhal(t, cl, settle=0.5)
    res, hist = {"spinup": spin}, {}
    steps = int(round(CONTINUE / w.dt))
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        with Simulation(w, precision=prec, maxit=50000) as S:
            S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
            S.restore(state)
            hist[name] = _run(S, steps)
        res[name] = strouhal(hist[name][0], hist[name][2], settle=0.0)
        res[name]["cd_mean"] = float(hist[name][1].mean())
    # the oracle from the same state
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    O = oracle.sim(g, method=0, solver=0, compat=True, dt=w.dt, nu=1.0 / w.re, tol=w.tol, bc_dir=w.bc_dir,
                   bc_num=w.bc_num, eta=eta)
    O.init()
    for f, k in (("u0", "U0"), ("v0", "V0"), ("w0", "W0"), ("u1", "U1"), ("v1", "V1"), ("w1", "W1"),
                 ("u3", "U3"), ("v3", "V3"), ("w3", "W3"), ("p", "P"), ("x", "X"), ("eta", "ETA")):
        O.field(f)[:] = state[k]
    O.loop = state["clock"][0]
    ocd, ocl = np.array([O.step()[:2] for _ in range(ORACLE_STEPS)]).T
    gcd, gcl = hist["fp64"][1][:ORACLE_STEPS], hist["fp64"][2][:ORACLE_STEPS]
    res["oracle"] = {"steps": ORACLE_STEPS, "cd_max_rel": float(np.max(np.abs(gcd / ocd - 1.0))),
                     "cl_max_diff_rel_to_cd": float(np.max(np.abs(gcl - ocl) / np.abs(ocd))),
                     "cl_amplitude_in_window": float(np.ptp(ocl))}
    print("\nSTROUHAL " + json.dumps(res))
    m, f = res["mixed"], res["fp64"]
    assert spin["st"] is not None and m["st"] is not None and f["st"] is not None
    assert abs(m["st"] / f["st"] - 1.0) < 1e-4
    assert abs(m["cd_mean"] / f["cd_mean"] - 1.0) < 1e-5
    assert res["oracle"]["cd_max_rel"] < 1e-6
    assert res["oracle"]["cl_max_diff_rel_to_cd"] < 1e-6
