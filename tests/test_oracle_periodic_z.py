"""Periodic z in the oracle (an extension: the reference's z faces are the
Dirichlet/Neumann table and its pressure operator is Neumann-only).  With no
reference to compare against, the restatement is checked through properties
that only a periodic discretisation has: the solution commutes with a cyclic
shift in z, and a doubled domain initialised with two copies stays two exact
copies.  The GPU path will be checked against this oracle."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from oracle.oracle import Grid


def _z_varying_state(w, nzc):
    """Seeded interior perturbation plus a z-varying w so the z coupling matters."""
    u0, v0, w0 = (a.copy() for a in initial_velocity(w.nxc, w.nyc, nzc))
    shape = (w.nxc + 4, w.nyc + 4, nzc + 4)
    kz = np.arange(nzc)
    W = w0.reshape(shape)
    W[2:-2, 2:-2, 2:-2] += 0.05 * np.sin(2 * np.pi * kz / nzc)[None, None, :]
    return u0, v0, w0


def _run(oracle, w, nzc, lz, state, steps, solver=0):
    # aligned source coupling: the reference's compact-index coupling does not
    # commute with a shift in z
    g = Grid(w.nxc, w.nyc, nzc, w.lx, w.ly, lz, oracle=oracle, periodic_z=True)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=0, solver=solver, aligned_src=True, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-12,
                   omega=w.omega, bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    S.init()
    for f, a in zip(("u0", "v0", "w0"), state):
        S.field(f)[:] = a
    S.start()
    hist = [S.step() for _ in range(steps)]
    return g, S, hist


def _interior(g, a):
    return a.reshape(g.nx, g.ny, g.nz)[2:-2, 2:-2, 2:-2]


@pytest.mark.parametrize("solver", [0, 1])
def test_periodic_solution_commutes_with_a_z_shift(oracle, solver):
    w = WORKLOADS["g1"]
    nzc, shift = w.nzc, 2
    base = _z_varying_state(w, nzc)
    rolled = []
    for a in base:
        b = a.copy()
        A = b.reshape(w.nxc + 4, w.nyc + 4, nzc + 4)
        A[2:-2, 2:-2, 2:-2] = np.roll(a.reshape(A.shape)[2:-2, 2:-2, 2:-2], shift, axis=2)
        rolled.append(b)
    g, S, h = _run(oracle, w, nzc, w.lz, base, 3, solver)
    _, R, hr = _run(oracle, w, nzc, w.lz, rolled, 3, solver)
    np.testing.assert_allclose([x[0] for x in hr], [x[0] for x in h], rtol=1e-9)
    for f in ("u0", "v0", "w0", "p"):
        a = np.roll(_interior(g, S.field(f)), shift, axis=2)
        b = _interior(g, R.field(f))
        scale = np.abs(a).max() + 1e-30
        if f == "p":  # pressure is defined up to a constant
            a, b = a - a.mean(), b - b.mean()
        assert np.abs(a - b).max() <= 1e-8 * scale, f


def test_doubled_periodic_domain_stays_two_copies(oracle):
    w = WORKLOADS["g1"]
    nzc = w.nzc
    base = _z_varying_state(w, nzc)
    tiled = []
    for a in base:
        A = a.reshape(w.nxc + 4, w.nyc + 4, nzc + 4)
        T = np.zeros((w.nxc + 4, w.nyc + 4, 2 * nzc + 4))
        T[:, :, 2:-2] = np.concatenate([A[:, :, 2:-2], A[:, :, 2:-2]], axis=2)
        tiled.append(T.ravel())
    g1, S1, h1 = _run(oracle, w, nzc, w.lz, base, 3)
    g2, S2, h2 = _run(oracle, w, 2 * nzc, 2 * w.lz, tiled, 3)
    np.testing.assert_allclose([x[0] for x in h2], [x[0] for x in h1], rtol=1e-9)
    for f in ("u0", "v0", "w0"):
        one = _interior(g1, S1.field(f))
        two = _interior(g2, S2.field(f))
        scale = np.abs(one).max()
        assert np.abs(two[:, :, :nzc] - one).max() <= 1e-8 * scale, f
        assert np.abs(two[:, :, nzc:] - one).max() <= 1e-8 * scale, f


def test_periodic_differs_from_neumann_and_keeps_ghosts_periodic(oracle):
    w = WORKLOADS["g1"]
    state = _z_varying_state(w, w.nzc)
    g, S, _ = _run(oracle, w, w.nzc, w.lz, state, 2)
    W = S.field("w0").reshape(g.nx, g.ny, g.nz)
    np.testing.assert_array_equal(W[:, :, 1], W[:, :, g.nz - 3])
    np.testing.assert_array_equal(W[:, :, g.nz - 2], W[:, :, 2])
    gn = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(gn, w.cx, w.center_y)
    N = oracle.sim(gn, method=0, solver=0, aligned_src=True, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-12,
                   omega=w.omega, bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    N.init()
    for f, a in zip(("u0", "v0", "w0"), state):
        N.field(f)[:] = a
    N.start()
    for _ in range(2):
        N.step()
    assert np.abs(_interior(g, S.field("w0")) - _interior(gn, N.field("w0"))).max() > 1e-6


def test_sor_is_refused_with_periodic_z(oracle):
    w = WORKLOADS["g1"]
    with pytest.raises(ValueError):
        _run(oracle, w, w.nzc, w.lz, _z_varying_state(w, w.nzc), 1, solver=3)
