"""Periodic z on the GPU (an extension: the reference's z faces are the
Dirichlet/Neumann table of Boundary_Condition.hpp:4-31 and its pressure
operator is Neumann-only) against the oracle's periodic restatement, which
tests/test_oracle_periodic_z.py pins by the properties only a periodic
discretisation has.

* Whole steps, SPE and ELL BiCGSTAB, both source-index conventions: Cd and
  fields against the oracle at solver tolerance 1e-10, as for the
  non-periodic steps; the z ghost planes are exact copies of the interior
  planes one period away.
* The boundary update alone: bitwise against og_bc_main on a periodic grid.
* Mixed precision (FP32 multigrid-CG, wrapped smoother and coarse operators)
  against the FP64 periodic run.
* A cyclic shift in z of the initial state shifts the solution.
"""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid
from tests.helpers import kernel_inputs, rel_err

pytestmark = pytest.mark.gpu


def _state(w):
    """Seeded perturbation plus a z-varying w, so the z coupling matters."""
    u0, v0, w0 = (a.copy() for a in initial_velocity(w.nxc, w.nyc, w.nzc))
    W = w0.reshape(w.nxc + 4, w.nyc + 4, w.nzc + 4)
    W[2:-2, 2:-2, 2:-2] += 0.05 * np.sin(2 * np.pi * np.arange(w.nzc) / w.nzc)[None, None, :]
    return u0, v0, w0


def _oracle_run(oracle, w, steps, state, solver=0, aligned=False, tol=1e-10):
    g = Grid.of(w, oracle, periodic_z=True)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=0, solver=solver, aligned_src=aligned, compat=True, dt=w.dt, nu=1.0 / w.re, tol=tol,
                   omega=w.omega, bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    S.init()
    for f, a in zip(("u0", "v0", "w0"), state):
        S.field(f)[:] = a
    S.start()
    return g, S, [S.step() for _ in range(steps)]


def _gpu_run(w, steps, state, **kw):
    S = Simulation(w, periodic_z=True, **kw)
    S.setup_cylinder(*state)
    return S, [S.step() for _ in range(steps)]


@pytest.mark.parametrize("name,steps", [("g1", 5), ("c1", 3)])
@pytest.mark.parametrize("solver", [capi.SOLVER_BICG_SPE, capi.SOLVER_BICG_ELL])
@pytest.mark.parametrize("aligned", [False, True])
def test_periodic_steps_match_oracle(oracle, name, steps, solver, aligned):
    w = WORKLOADS[name]
    st = _state(w)
    g, O, ohist = _oracle_run(oracle, w, steps, st, solver=solver, aligned=aligned)
    S, hist = _gpu_run(w, steps, st, solver=solver, aligned_source=aligned, tol=1e-10)
    try:
        np.testing.assert_allclose([h["cd"] for h in hist], [h[0] for h in ohist], rtol=1e-7)
        for k, f in (("U0", "u0"), ("V0", "v0"), ("W0", "w0")):
            assert rel_err(S.download(k), O.field(f)) < 1e-7, k
        assert rel_err(S.download("P"), O.field("p")) < 1e-6
        W = S.download("W0").reshape(g.nx, g.ny, g.nz)
        np.testing.assert_array_equal(W[:, :, 1], W[:, :, g.nz - 3])
        np.testing.assert_array_equal(W[:, :, g.nz - 2], W[:, :, 2])
        P = S.download("P").reshape(g.nx, g.ny, g.nz)
        np.testing.assert_array_equal(P[:, :, 0], P[:, :, g.nzc])
    finally:
        S.close()


def test_periodic_bc_main_bitwise(oracle):
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle, periodic_z=True)
    ins = kernel_inputs(g.ng, g.n)
    u, v, ww, p = (a.copy() for a in ins["bc"])
    with Simulation(w, periodic_z=True) as S:
        S.grid_uniform()
        for k, a in (("U0", u), ("V0", v), ("W0", ww), ("P", p)):
            S.upload(k, a)
        S.BC_staggered_main(S.T0)
        got = {k: S.download(k) for k in ("U0", "V0", "W0", "P")}
    oracle.bc_main(g, w.bc_dir, w.bc_num, u, v, ww, p)
    for k, a in (("U0", u), ("V0", v), ("W0", ww), ("P", p)):
        np.testing.assert_array_equal(got[k], a, err_msg=k)


def test_periodic_mixed_close_to_fp64():
    w = WORKLOADS["c1"]
    st = _state(w)
    S64, h64 = _gpu_run(w, 6, st, tol=1e-10)
    S32, h32 = _gpu_run(w, 6, st, tol=1e-10, precision=capi.PREC_MIXED)
    try:
        np.testing.assert_allclose([h["cd"] for h in h32], [h["cd"] for h in h64], rtol=1e-6)
        assert all(r < 1e-10 for h in h32[1:] + h64[1:] for r in h["relres"])
        assert rel_err(S32.download("U0"), S64.download("U0")) < 1e-5
        assert rel_err(S32.download("W0"), S64.download("W0")) < 1e-4
    finally:
        S64.close()
        S32.close()


def test_periodic_run_commutes_with_a_z_shift():
    """Aligned source coupling (the reference's compact-index coupling does
    not commute with a shift); FP64, tolerance 1e-12."""
    w = WORKLOADS["g1"]
    shift = 2
    base = _state(w)
    shape = (w.nxc + 4, w.nyc + 4, w.nzc + 4)
    rolled = []
    for a in base:
        b = a.copy().reshape(shape)
        b[2:-2, 2:-2, 2:-2] = np.roll(a.reshape(shape)[2:-2, 2:-2, 2:-2], shift, axis=2)
        rolled.append(b.ravel())
    S, h = _gpu_run(w, 3, base, aligned_source=True, tol=1e-12)
    R, hr = _gpu_run(w, 3, rolled, aligned_source=True, tol=1e-12)
    try:
        np.testing.assert_allclose([x["cd"] for x in hr], [x["cd"] for x in h], rtol=1e-9)
        for k in ("U0", "V0", "W0"):
            a = np.roll(S.download(k).reshape(shape)[2:-2, 2:-2, 2:-2], shift, axis=2)
            b = R.download(k).reshape(shape)[2:-2, 2:-2, 2:-2]
            assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max(), k
    finally:
        S.close()
        R.close()


def test_sor_and_adjoint_refuse_periodic_z():
    w = WORKLOADS["g1"]
    with pytest.raises(capi.CfdError) as e:
        Simulation(w, periodic_z=True, solver=capi.SOLVER_SOR_RB)
    assert e.value.status == -1
    import ctypes as C
    with Simulation(w, periodic_z=True) as S:
        S.grid_uniform()
        assert capi.lib().cfd_adj_enable(S.handle, 4) == -1
        assert "periodic" in capi.lib().cfd_last_error().decode()
        del C
