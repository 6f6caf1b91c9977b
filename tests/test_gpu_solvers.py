"""Poisson solvers on the GPU against the oracle.

BiCGSTAB: the GPU and the oracle run the same algorithm (bicgstabRe2) on
the same system with different summation orders, so the iteration count
agrees to a few iterations and both solutions satisfy the tolerance; the
solutions themselves agree to tol x (condition number), checked after
removing the constant null-space component of the Neumann operator.
SOR: the GPU and the oracle run the same red-black sweeps; the iterates
agree to rounding, and both agree with the reference's lexicographic SOR at
the converged fixed point."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid
from tests.helpers import kernel_inputs, rel_err

pytestmark = pytest.mark.gpu


def _centered(a):
    return a - a.mean()


def _consistent_rhs(oracle, g, solver):
    x_true = kernel_inputs(g.ng, g.n)["x"]
    b = np.zeros(g.n)
    if solver == capi.SOLVER_BICG_SPE:
        co, _, jp = oracle.spe_setup(g)
        oracle.spe_spmv(g, co, jp, x_true, b)
        op = dict(spe=(co, jp))
    else:
        cols, vals, _ = oracle.ell_assemble(g)
        oracle.ell_spmv(g.n, cols, vals, x_true, b)
        op = dict(ell=(cols, vals))
    return b, op


def _residual(oracle, g, op, x, b):
    r = np.zeros(g.n)
    if "spe" in op:
        co, jp = op["spe"]
        oracle.spe_spmv(g, co, jp, x, r)
    else:
        cols, vals = op["ell"]
        oracle.ell_spmv(g.n, cols, vals, x, r)
    return np.linalg.norm(b - r) / np.linalg.norm(b)


@pytest.mark.parametrize("name", ["g1", "c1"])
@pytest.mark.parametrize("solver", [capi.SOLVER_BICG_SPE, capi.SOLVER_BICG_ELL])
def test_bicgstab_matches_oracle(oracle, name, solver):
    w = WORKLOADS[name]
    g = Grid.of(w, oracle)
    b, op = _consistent_rhs(oracle, g, solver)
    tol = 1e-10
    ref = oracle.bicg(g, tol, **op)
    x_ref = np.zeros(g.n)
    it_ref, res_ref, _ = ref.solve(b, x_ref)
    with Simulation(w, solver=solver, tol=tol) as S:
        S.grid_uniform()
        S.upload("B", b)
        S.upload("X", np.zeros(g.n))
        it, res = S.pSolver()
        x = S.download("X")
    assert res < tol
    assert _residual(oracle, g, op, x, b) < 2 * tol
    assert abs(it - it_ref) <= max(3, 0.1 * it_ref)
    assert rel_err(_centered(x), _centered(x_ref)) < 1e-6


def test_bicgstab_warm_start_and_counters(oracle):
    """Solves warm-start from the previous solution (Mx.X_result is never
    reset, RUN_CPU_PC_METHOD.hpp:130,354): a second solve of the same system
    takes zero iterations beyond the first check."""
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle)
    b, _ = _consistent_rhs(oracle, g, capi.SOLVER_BICG_SPE)
    with Simulation(w, tol=1e-10) as S:
        S.grid_uniform()
        S.upload("B", b)
        it1, _ = S.pSolver()
        it2, res2 = S.pSolver()
    assert it1 > 10
    assert it2 <= 1 and res2 < 1e-10


def test_bicgstab_iteration_cap_reports_noconv(oracle):
    """The cap path (bicgstabRe2.hpp:143-163) returns CFD_ERR_NOCONV with a
    finite x (no NaN/Inf were present, so nothing is reset)."""
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle)
    b, _ = _consistent_rhs(oracle, g, capi.SOLVER_BICG_SPE)
    with Simulation(w, tol=1e-14, maxit=3) as S:
        S.grid_uniform()
        S.upload("B", b)
        with pytest.raises(capi.CfdError) as e:
            S.pSolver()
        assert e.value.status == -4
        it, res = S.pSolver(allow_noconv=True)
        assert it == 3 and res > 1e-14
        assert np.all(np.isfinite(S.download("X")))


def test_zero_rhs_returns_immediately():
    w = WORKLOADS["g0"]
    with Simulation(w, tol=1e-10) as S:
        S.grid_uniform()
        S.upload("B", np.zeros(w.n_cells))
        it, res = S.pSolver()
        assert it == 0 and res == 0.0


@pytest.mark.parametrize("solver,inner", [(capi.SOLVER_BICG_SPE, capi.INNER_CG),
                                          (capi.SOLVER_BICG_SPE, capi.INNER_MG),
                                          (capi.SOLVER_BICG_SPE, capi.INNER_BICGSTAB),
                                          (capi.SOLVER_BICG_ELL, capi.INNER_BICGSTAB)])
def test_mixed_precision_defect_correction(oracle, solver, inner):
    """FP32 inner solves (CG on the symmetric finite-volume form, or
    restarted BiCGSTAB) + FP64 defect correction reach the FP64 tolerance on
    the FP64 residual."""
    w = WORKLOADS["c1"]
    g = Grid.of(w, oracle)
    b, op = _consistent_rhs(oracle, g, solver)
    tol = 1e-10
    with Simulation(w, solver=solver, tol=tol, precision=capi.PREC_MIXED, inner_solver=inner) as S:
        S.grid_uniform()
        S.upload("B", b)
        it, res = S.pSolver()
        x = S.download("X")
    assert res < tol
    assert _residual(oracle, g, op, x, b) < 2 * tol
    assert it > 0


def _sor_workload(name):
    if name == "g2_odd":  # nz odd: one colour has one cell fewer in every row
        return WORKLOADS["g2"].with_(nzc=7, lz=0.875)
    return WORKLOADS[name]


@pytest.mark.parametrize("name,loop", [("g1", "device"), ("c1", "device"), ("c1", "host"), ("g2_odd", "device"),
                                       ("g2_odd", "host")])
def test_sor_redblack_matches_oracle_bitwise(monkeypatch, oracle, name, loop):
    """The sweeps form every value with the reference's operations in its
    order, one rounding each, and the cells of one colour do not read each
    other, so p, the sweep count and the last max change are those of the
    oracle's sequential red-black loop, bit for bit (device WHILE loop or
    host-polled batches; an odd nz leaves the last slot of every other row
    unused)."""
    monkeypatch.setenv("CFDGPU_SOLVE_LOOP", loop)
    w = _sor_workload(name)
    g = Grid.of(w, oracle)
    I = kernel_inputs(g.ng, g.n)
    u1, v1, w1 = (0.01 * I[k] for k in ("u1", "v1", "w1"))
    p0 = I["sor_p"]
    cf = oracle.sor_coef(g)
    oracle.sor_rhs(g, w.dt, u1, v1, w1, cf)
    p_ref = p0.copy()
    it_ref, err_ref = oracle.sor(g, 1.7, 1e-9, 400, cf, p_ref, redblack=True)
    with Simulation(w, solver=capi.SOLVER_SOR_RB, tol=1e-9, omega=1.7, sor_maxit=400,
                    check_every=7) as S:
        S.grid_uniform()
        S.upload("P", p0)
        for k, a in (("U1", u1), ("V1", v1), ("W1", w1)):
            S.upload(k, a)
        it, err = S.SorPipeLine(S.T1)
        p = S.download("P")
        # a second solve from the converged p stops after one sweep
        it2, err2 = S.SorPipeLine(S.T1)
    assert it == it_ref and err == err_ref
    np.testing.assert_array_equal(p, p_ref)  # ghost pressures untouched (SorPipeLine.seq.hpp:74-104)
    assert it2 == 0 and err2 <= 1e-9


def test_sor_sweep_cap(oracle):
    """p_sor_iter_max sweeps, then the solve stops above tolerance and
    reports iters = cap - 1 with the last max change, as the reference."""
    w = WORKLOADS["g1"]
    g = Grid.of(w, oracle)
    I = kernel_inputs(g.ng, g.n)
    u1, v1, w1 = (0.01 * I[k] for k in ("u1", "v1", "w1"))
    cf = oracle.sor_coef(g)
    oracle.sor_rhs(g, w.dt, u1, v1, w1, cf)
    p_ref = I["sor_p"].copy()
    it_ref, err_ref = oracle.sor(g, 1.7, 1e-14, 37, cf, p_ref, redblack=True)
    with Simulation(w, solver=capi.SOLVER_SOR_RB, tol=1e-14, omega=1.7, sor_maxit=37, check_every=5) as S:
        S.grid_uniform()
        S.upload("P", I["sor_p"])
        for k, a in (("U1", u1), ("V1", v1), ("W1", w1)):
            S.upload(k, a)
        it, err = S.SorPipeLine(S.T1)
        p = S.download("P")
    assert it == it_ref == 36 and err == err_ref and err > 1e-14
    np.testing.assert_array_equal(p, p_ref)


@pytest.mark.parametrize("name", ["g1", "c1", "g2_odd"])
def test_sor_fp32_sweeps_reach_the_fp64_fixed_point(oracle, name):
    """Mixed-precision contexts sweep in FP32 on the correction between FP64
    sweeps, whose max change is the reference's stop test.  At a tight
    tolerance both runs reach the same fixed point, and the FP32 sweeps take
    about as many sweeps as FP64 ones (the count includes them; the stop test
    runs once per loop body of 4 x check_every FP32 sweeps).  The velocities
    are FP32 values, so both contexts hold the same right-hand side."""
    w = _sor_workload(name)
    g = Grid.of(w, oracle)
    I = kernel_inputs(g.ng, g.n)
    u1, v1, w1 = ((0.01 * I[k]).astype(np.float32).astype(np.float64) for k in ("u1", "v1", "w1"))
    out = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        with Simulation(w, solver=capi.SOLVER_SOR_RB, precision=prec, tol=1e-12, omega=1.7, sor_maxit=20000,
                        check_every=4) as S:
            S.grid_uniform()
            S.upload("P", I["sor_p"])
            for k, a in (("U1", u1), ("V1", v1), ("W1", w1)):
                S.upload(k, a)
            it, err = S.SorPipeLine(S.T1)
            out[prec] = (it, err, S.download("P"))
    (it64, err64, p64), (it32, err32, p32) = out[capi.PREC_FP64], out[capi.PREC_MIXED]
    assert err64 <= 1e-12 and err32 <= 1e-12
    assert it64 < 20000 and it32 < 20000
    assert abs(it32 - it64) <= 17 + 0.1 * it64, (it32, it64)
    assert rel_err(g.interior(p32), g.interior(p64)) < 1e-9


@pytest.mark.parametrize("dims", [(64, 48, 32), (24, 40, 64), (32, 20, 8), (16, 24, 12)])
def test_cg_stencil_tma_matches_plain_kernel(monkeypatch, dims):
    """The TMA-fed CG stencil (z and p planes streamed into shared memory,
    halos zero-filled by the TMA) and the plain 2.5D kernel compute the same
    operator: the mixed-precision solve agrees to the FP64 tolerance and takes
    nearly the same number of inner iterations.  Covers k tiles of 32 (one and
    two per column), 16 and 8 cells."""
    nx, ny, nz = dims
    w = WORKLOADS["c1"].with_(nxc=nx, nyc=ny, nzc=nz, lx=nx * 0.25, ly=ny * 0.25, lz=nz * 0.25, cx=nx * 0.1)
    rng = np.random.default_rng(11)
    out = []
    for flag in ("0", "1"):
        monkeypatch.setenv("CFDGPU_NO_TMA", flag)
        with Simulation(w, tol=1e-10, precision=capi.PREC_MIXED, inner_solver=capi.INNER_CG, inner_tol=1e-2) as S:
            S.grid_uniform()
            jp = S.download("JP")
            r = rng.standard_normal(w.n_cells) if flag == "0" else out[0][2]
            b = r - jp * np.mean(r / jp)
            S.upload("B", b)
            it, res = S.pSolver()
            out.append((it, res, r, S.download("X")))
    (it_t, res_t, _, x_t), (it_p, res_p, _, x_p) = out
    assert res_t < 1e-10 and res_p < 1e-10
    assert abs(it_t - it_p) <= 0.05 * it_p + 4
    d_t, d_p = x_t - x_t.mean(), x_p - x_p.mean()
    assert np.linalg.norm(d_t - d_p) <= 1e-8 * np.linalg.norm(d_p)


@pytest.mark.parametrize("dims", [(64, 48, 32), (32, 20, 8), (30, 18, 6)])
def test_multigrid_inner_solve_reaches_tolerance_in_few_iterations(dims):
    """Multigrid-preconditioned FP32 CG inside the FP64 defect correction:
    the FP64 tolerance is reached, with far fewer inner iterations than
    Jacobi-PCG (the 30x18x6 grid does not coarsen to a small level, so it
    falls back to Jacobi-PCG and must still converge)."""
    nx, ny, nz = dims
    w = WORKLOADS["c1"].with_(nxc=nx, nyc=ny, nzc=nz, lx=nx * 0.25, ly=ny * 0.25, lz=nz * 0.25, cx=nx * 0.1)
    rng = np.random.default_rng(5)
    its = {}
    for inner in (capi.INNER_CG, capi.INNER_MG):
        with Simulation(w, tol=1e-10, precision=capi.PREC_MIXED, inner_solver=inner) as S:
            S.grid_uniform()
            jp = S.download("JP")
            r = rng.standard_normal(w.n_cells) if inner == capi.INNER_CG else r
            S.upload("B", r - jp * np.mean(r / jp))
            it, res = S.pSolver()
            assert res < 1e-10
            its[inner] = it
    if dims != (30, 18, 6):
        assert its[capi.INNER_MG] * 5 < its[capi.INNER_CG], its


@pytest.mark.parametrize("dims", [(64, 48, 32), (70, 40, 32), (96, 56, 16)])
def test_fused_sweeps_match_colour_launches_bitwise(monkeypatch, dims):
    """The fused red-black sweep (both colours in one plane-marching pass,
    ping-pong buffers) computes every cell with the same operations in the
    same order as the two colour launches, so the multigrid-CG solve is
    bitwise identical either way.  Covers partial j tiles (ny not a multiple
    of the tile), chunks that do not divide nx, and 8 and 4 quads per k line."""
    nx, ny, nz = dims
    w = WORKLOADS["c1"].with_(nxc=nx, nyc=ny, nzc=nz, lx=nx * 0.25, ly=ny * 0.25, lz=nz * 0.25, cx=nx * 0.1)
    rng = np.random.default_rng(21)
    r = rng.standard_normal(w.n_cells)
    out = []
    for flag in ("0", "1"):
        monkeypatch.setenv("CFDGPU_MG_FUSED", flag)
        with Simulation(w, tol=1e-10, precision=capi.PREC_MIXED, inner_solver=capi.INNER_MG) as S:
            S.grid_uniform()
            jp = S.download("JP")
            S.upload("B", r - jp * np.mean(r / jp))
            it, res = S.pSolver()
            assert res < 1e-10
            out.append((it, S.download("X")))
    assert out[0][0] == out[1][0]
    np.testing.assert_array_equal(out[0][1], out[1][1])
