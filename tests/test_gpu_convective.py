"""Convective outflow at the x-max face (an extension of the reference's BC
table) on the GPU against the oracle's FP64 restatement, which the CPU tests
pin to a numpy statement of the formulas and to mass conservation."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

UC = 1.0


def _oracle_run(oracle, w, steps):
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=0, solver=0, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-10, omega=w.omega,
                   bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta, conv_uc=UC)
    S.init()
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    S.field("u0")[:] = u0
    S.field("v0")[:] = v0
    S.field("w0")[:] = w0
    S.start()
    return g, S, [S.step() for _ in range(steps)]


def _flux_balance(w, U):
    g = Grid.of(w)
    U = U.reshape(g.nx, g.ny, g.nz)
    js, ks = slice(2, g.ny - 2), slice(2, g.nz - 2)
    area = np.outer(g.m["Dy"][js], g.m["Dz"][ks])
    q_in = (U[1, js, ks] * area).sum()
    return abs((U[g.nx - 3, js, ks] * area).sum() - q_in) / abs(q_in)


@pytest.mark.parametrize("name", ["g1", "c1"])
def test_convective_outflow_steps_match_oracle(oracle, name):
    w = WORKLOADS[name]
    g, O, ohist = _oracle_run(oracle, w, 4)
    with Simulation(w, tol=1e-10, conv_outflow_uc=UC) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        hist = [S.step() for _ in range(4)]
        np.testing.assert_allclose([h["cd"] for h in hist], [h[0] for h in ohist], rtol=1e-7)
        for k, f in (("U0", "u0"), ("V0", "v0"), ("W0", "w0")):
            assert rel_err(S.download(k), O.field(f)) < 1e-7, k
        U = S.download("U0")
        # the outflow face and its ghosts carry the convective values
        np.testing.assert_allclose(U.reshape(g.nx, g.ny, g.nz)[g.nx - 3], O.field("u0").reshape(g.nx, g.ny, g.nz)[g.nx - 3],
                                   rtol=1e-7, atol=1e-12)
        assert _flux_balance(w, U) < 1e-12


def test_convective_outflow_mixed_precision_conserves_mass():
    w = WORKLOADS["c1"]
    with Simulation(w, tol=1e-10, precision=capi.PREC_MIXED, conv_outflow_uc=UC) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        for _ in range(3):
            h = S.step()
        assert all(r < 1e-10 for r in h["relres"])
        assert _flux_balance(w, S.download("U0")) < 1e-6  # FP32 face values


def test_adjoint_rejects_convective_outflow():
    w = WORKLOADS["g1"]
    with Simulation(w, tol=1e-10, conv_outflow_uc=UC) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        with pytest.raises(capi.CfdError):
            S.adj_enable(1)
