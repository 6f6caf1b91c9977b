"""Convective outflow at the x-max face (an extension: the reference's velocity
BC is only its Dirichlet/Neumann table).  The oracle's restatement is checked
here on the CPU against an independent numpy statement of the same formulas,
for mass conservation across the domain's open faces, and for leaving the
reference path untouched when it is off."""
from __future__ import annotations

import numpy as np

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from oracle.oracle import Grid


def _numpy_convective(g, dt, uc, u0, v0, w0, u3, v3, w3):
    """The convective update written out with numpy (first-order upwind from
    the old field, then the outflow flux scaled to the inflow flux)."""
    sh = (g.nx, g.ny, g.nz)
    U0, V0, W0 = (a.reshape(sh) for a in (u0, v0, w0))
    U3, V3, W3 = (a.reshape(sh).copy() for a in (u3, v3, w3))
    nx = g.nx
    Dx, Dxs, Dy, Dz = g.m["Dx"], g.m["Dxs"], g.m["Dy"], g.m["Dz"]
    js, ks = slice(2, g.ny - 2), slice(2, g.nz - 2)
    C = uc * dt / Dx[nx - 3]
    Ct = uc * dt / Dxs[nx - 3]
    ub = U0[nx - 3, js, ks] - C * (U0[nx - 3, js, ks] - U0[nx - 4, js, ks])
    vg = V0[nx - 2, js, ks] - Ct * (V0[nx - 2, js, ks] - V0[nx - 3, js, ks])
    wg = W0[nx - 2, js, ks] - Ct * (W0[nx - 2, js, ks] - W0[nx - 3, js, ks])
    area = np.outer(Dy[js], Dz[ks])
    scale = (U0[1, js, ks] * area).sum() / (ub * area).sum()
    for i in (nx - 3, nx - 2, nx - 1):
        U3[i, js, ks] = ub * scale
    for i in (nx - 2, nx - 1):
        V3[i, js, ks] = vg
        W3[i, js, ks] = wg
    return U3.ravel(), V3.ravel(), W3.ravel()


def test_convective_update_matches_numpy_statement(oracle):
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle)
    rng = np.random.default_rng(4)
    u0, v0, w0 = (1.0 + 0.1 * rng.standard_normal(g.ng) for _ in range(3))
    u3, v3, w3 = (rng.standard_normal(g.ng) for _ in range(3))
    want = _numpy_convective(g, w.dt, 1.3, u0, v0, w0, u3, v3, w3)
    oracle.bc_convective(g, w.dt, 1.3, u0, v0, w0, u3, v3, w3)
    for got, ref in zip((u3, v3, w3), want):
        np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15)


def _sim(oracle, w, conv_uc, steps):
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=0, solver=0, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-10, omega=w.omega,
                   bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta, conv_uc=conv_uc)
    S.init()
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    S.field("u0")[:] = u0
    S.field("v0")[:] = v0
    S.field("w0")[:] = w0
    S.start()
    hist = [S.step() for _ in range(steps)]
    return g, S, hist


def test_convective_outflow_conserves_mass_and_differs_from_zero_gradient(oracle):
    w = WORKLOADS["g1"]
    g, S, _ = _sim(oracle, w, 1.0, 4)
    U = S.field("u0").reshape(g.nx, g.ny, g.nz)
    js, ks = slice(2, g.ny - 2), slice(2, g.nz - 2)
    area = np.outer(g.m["Dy"][js], g.m["Dz"][ks])
    q_in = (U[1, js, ks] * area).sum()
    q_out = (U[g.nx - 3, js, ks] * area).sum()
    assert abs(q_out - q_in) <= 1e-12 * abs(q_in)
    np.testing.assert_array_equal(U[g.nx - 2, js, ks], U[g.nx - 3, js, ks])
    g0, S0, _ = _sim(oracle, w, 0.0, 4)
    U0 = S0.field("u0").reshape(g.nx, g.ny, g.nz)
    assert np.abs(U[g.nx - 3, js, ks] - U0[g.nx - 3, js, ks]).max() > 1e-8


def test_convective_off_leaves_the_reference_path_unchanged(oracle):
    """conv_uc = 0 is the reference's table BC, bit for bit."""
    w = WORKLOADS["g1"]
    _, S, h = _sim(oracle, w, 0.0, 3)
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    R = oracle.sim(g, method=0, solver=0, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-10, omega=w.omega,
                   bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    R.init()
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    R.field("u0")[:] = u0
    R.field("v0")[:] = v0
    R.field("w0")[:] = w0
    R.start()
    hr = [R.step() for _ in range(3)]
    assert [x[0] for x in h] == [x[0] for x in hr]
    np.testing.assert_array_equal(S.field("u0"), R.field("u0"))
