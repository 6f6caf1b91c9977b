"""Failure paths of the GPU solvers (none faults, traps or hangs the GPU).

* A non-finite Poisson residual returns CFD_ERR_NAN from the mixed-precision
  defect correction (cfd_bicgstab and cfd_step).
* bicgstabRe2's NaN/Inf reset at the iteration cap (bicgstabRe2.hpp:143-163):
  non-finite entries of x take the previous initial guess px1, and when more
  than 10 % were reset x becomes the guess before that, px2.  The oracle runs
  the same sequence and is the checker.
* Every device-side wait is bounded.  cfd_set_test_limits lowers the bounds so
  they run out on purpose: the trip cap of the CUDA-graph WHILE loop of a
  solve, and the try-wait count of the TMA pipeline of the FP32 CG stencil.
  Both return CFD_ERR_TIMEOUT, and the context stays usable.
"""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.capi import lib
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid
from tests.helpers import kernel_inputs

pytestmark = pytest.mark.gpu

ERR_NOCONV, ERR_NAN, ERR_TIMEOUT = -4, -5, -6


def _rhs(oracle, g):
    x_true = kernel_inputs(g.ng, g.n)["x"]
    co, _, jp = oracle.spe_setup(g)
    b = np.zeros(g.n)
    oracle.spe_spmv(g, co, jp, x_true, b)
    return b


def _solve_status(S):
    import ctypes as C
    it, res = C.c_int(), C.c_double()
    return lib().cfd_bicgstab(S.handle, C.byref(it), C.byref(res)), it.value, res.value


def test_mixed_nan_rhs_returns_err_nan(oracle):
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle)
    b = _rhs(oracle, g)
    b[g.n // 3] = np.nan
    with Simulation(w, precision=capi.PREC_MIXED, tol=1e-10) as S:
        S.grid_uniform()
        S.upload("B", b)
        S.upload("X", np.zeros(g.n))
        st, _, res = _solve_status(S)
        assert st == ERR_NAN
        assert not np.isfinite(res)
        # the context stays usable: a finite system solves
        b[g.n // 3] = 0.0
        S.upload("B", _rhs(oracle, g))
        S.upload("X", np.zeros(g.n))
        st, _, res = _solve_status(S)
        assert st == 0 and res < 1e-10


def test_mixed_step_with_nan_velocity_returns_err_nan():
    w = WORKLOADS["c1"]
    with Simulation(w, precision=capi.PREC_MIXED, tol=1e-10) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        S.step()  # the first step solves no Poisson equation
        u = S.download("U0")
        ny, nz = w.nyc + 4, w.nzc + 4
        u[(w.nxc // 2 + 2) * ny * nz + (w.nyc // 2 + 2) * nz + w.nzc // 2 + 2] = np.nan  # an interior face
        S.upload("U0", u)
        with pytest.raises(capi.CfdError) as e:
            S.step()
        assert e.value.status == ERR_NAN


def test_fp64_nan_at_cap_resets_x_like_the_reference(oracle):
    """Solve 1 (finite, capped) from x0; solve 2 with a NaN in b: every entry
    of x turns non-finite, all are reset (to px1 = x1), more than 10 % were
    reset, so x = px2 = x0, bit for bit."""
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle)
    b = _rhs(oracle, g)
    x0 = 0.1 * kernel_inputs(g.ng, g.n)["p"][: g.n]
    bn = b.copy()
    bn[g.n // 2] = np.nan
    maxit = 4
    co, _, jp = oracle.spe_setup(g)
    ref = oracle.bicg(g, 1e-14, spe=(co, jp), maxit=maxit)
    xr = x0.copy()
    _, _, capped1 = ref.solve(b, xr)
    x1_ref = xr.copy()
    _, _, capped2 = ref.solve(bn, xr)
    assert capped1 and capped2
    with Simulation(w, tol=1e-14, maxit=maxit) as S:
        S.grid_uniform()
        S.upload("X", x0)
        S.upload("B", b)
        st, it, _ = _solve_status(S)
        assert st == ERR_NOCONV and it == maxit
        x1 = S.download("X")
        assert np.all(np.isfinite(x1))
        np.testing.assert_allclose(x1, x1_ref, rtol=1e-9, atol=1e-12)
        S.upload("B", bn)
        st, it, res = _solve_status(S)
        assert st == ERR_NOCONV and it == maxit and not np.isfinite(res)
        x2 = S.download("X")
    assert np.array_equal(xr, x0)       # the oracle: x = px2
    assert np.array_equal(x2, x0)       # the GPU: the same, bitwise


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_solve_loop_trip_cap_returns_timeout(oracle, precision):
    """A trip cap of one body run: the FP64 BiCGSTAB (16 iterations per body)
    and the mixed path's Jacobi-PCG inner solve (8 pairs per body) both need
    many more at tolerance 1e-10 on c1."""
    w = WORKLOADS["c1"]
    g = Grid.of(w, oracle)
    b = _rhs(oracle, g)
    with Simulation(w, precision=precision, tol=1e-10, inner_solver=capi.INNER_CG) as S:
        S.grid_uniform()
        check_limits(S, 1, -1)
        S.upload("B", b)
        S.upload("X", np.zeros(g.n))
        st, _, _ = _solve_status(S)
        assert st == ERR_TIMEOUT
        assert "did not report completion" in lib().cfd_last_error().decode()
        check_limits(S, 0, -1)
        S.upload("X", np.zeros(g.n))
        st, _, res = _solve_status(S)
        assert st == 0 and res < 1e-10


def test_tma_pipeline_wait_limit_returns_timeout(oracle):
    """c1 has nz = 8, a multiple of 4, so the inner CG stencil is the TMA-fed
    kernel.  With a try-wait limit of 0 every block gives up at its first
    plane, waits out the copies it issued and skips its work; the solve
    reports the timeout.  With the default limit the same context solves."""
    w = WORKLOADS["c1"]
    g = Grid.of(w, oracle)
    b = _rhs(oracle, g)
    with Simulation(w, precision=capi.PREC_MIXED, tol=1e-10) as S:
        S.grid_uniform()
        S.upload("B", b)
        S.upload("X", np.zeros(g.n))
        st, _, res_ok = _solve_status(S)
        assert st == 0
        check_limits(S, 0, 0)
        S.upload("X", np.zeros(g.n))
        st, _, _ = _solve_status(S)
        assert st == ERR_TIMEOUT
        assert "bounded wait" in lib().cfd_last_error().decode()
        check_limits(S, 0, -1)
        S.upload("X", np.zeros(g.n))
        st, _, res = _solve_status(S)
        assert st == 0 and res < 1e-10


def check_limits(S, cap, wait):
    assert lib().cfd_set_test_limits(S.handle, cap, wait) == 0
