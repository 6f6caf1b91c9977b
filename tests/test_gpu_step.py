"""Whole time steps on the GPU against the oracle and the reference's golden
runs: predictor-corrector and plain drivers, SPE / ELL BiCGSTAB and
red-black SOR, both source-index conventions, FP64 and mixed precision.

Tolerances: Cd agrees with the oracle to 1e-7 relative and fields to 1e-7
relative after several steps at solver tolerance 1e-10 (the two sides sum
dot products in different orders, so their Krylov iterates differ at the
tolerance level); mixed precision is compared with the FP64 GPU run."""
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


def oracle_run(oracle, w, steps, *, method=0, solver=0, aligned=False, tol=1e-10):
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=method, solver=solver, aligned_src=aligned, compat=True, dt=w.dt,
                   nu=1.0 / w.re, tol=tol, omega=w.omega, bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    S.init()
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    S.field("u0")[:] = u0
    S.field("v0")[:] = v0
    S.field("w0")[:] = w0
    S.start()
    hist = [S.step() for _ in range(steps)]
    return S, hist


def gpu_run(w, steps, **kw):
    S = Simulation(w, **kw)
    S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
    hist = [S.step() for _ in range(steps)]
    return S, hist


@pytest.mark.parametrize("name,steps", [("g1", 6), ("c1", 4)])
@pytest.mark.parametrize("solver", [capi.SOLVER_BICG_SPE, capi.SOLVER_BICG_ELL])
def test_pc_steps_match_oracle(oracle, name, steps, solver):
    w = WORKLOADS[name]
    O, ohist = oracle_run(oracle, w, steps, solver=solver)
    S, hist = gpu_run(w, steps, solver=solver, tol=1e-10)
    cd = np.array([h["cd"] for h in hist])
    ocd = np.array([h[0] for h in ohist])
    np.testing.assert_allclose(cd, ocd, rtol=1e-7)
    assert hist[0]["iters"] == [0, 0, 0, 0]
    for k, f in (("U0", "u0"), ("V0", "v0"), ("W0", "w0")):
        assert rel_err(S.download(k), O.field(f)) < 1e-7, k
    assert rel_err(S.download("P"), O.field("p")) < 1e-6
    # near tol 1e-10 the two summation orders stagnate differently, so single
    # solves may differ by half; the totals agree to 15%
    its = [h["iters"] for h in hist[1:]]
    oits = [oh[2] for oh in ohist[1:]]
    for h, oh in zip(its, oits):
        assert all(abs(a - b) <= max(5, 0.5 * b) for a, b in zip(h, oh)), (its, oits)
    tot, otot = sum(map(sum, its)), sum(map(sum, oits))
    assert abs(tot - otot) <= 0.15 * otot, (its, oits)
    S.close()


def test_pc_steps_match_reference_golden(golden):
    """20 steps of the 128x64x8 cylinder against the reference's own run."""
    w = WORKLOADS["c1"]
    G = golden("c1_run")
    S, hist = gpu_run(w, 20, tol=1e-8)
    cd = np.array([h["cd"] for h in hist])
    cl = np.array([h["cl"] for h in hist])
    np.testing.assert_allclose(cd, G["spe_cd"], rtol=1e-6)
    np.testing.assert_allclose(cl, G["spe_cl"], rtol=1e-3, atol=1e-4)
    u = S.download("U0")
    ref = G["spe_u_summary"]
    np.testing.assert_allclose([u.sum(), np.abs(u).sum(), np.abs(u).max()], ref[:3], rtol=1e-7)
    S.close()


def test_golden_g0_fields(golden):
    G = golden("g0_run")
    w = WORKLOADS["g0"]
    S, hist = gpu_run(w, 5, tol=1e-10)
    for k, f in (("U0", "spe_u"), ("V0", "spe_v"), ("W0", "spe_w")):
        assert rel_err(S.download(k), G[f]) < 1e-8, k
    np.testing.assert_allclose([h["cd"] for h in hist], G["spe_cd"], rtol=1e-8)
    S.close()


@pytest.mark.parametrize("aligned", [False, True])
def test_plain_and_aligned_variants(oracle, aligned):
    w = WORKLOADS["g1"]
    for method in (capi.METHOD_PC, capi.METHOD_PLAIN):
        O, ohist = oracle_run(oracle, w, 4, method=method, aligned=aligned)
        S, hist = gpu_run(w, 4, method=method, aligned_source=aligned, tol=1e-10)
        np.testing.assert_allclose([h["cd"] for h in hist], [h[0] for h in ohist], rtol=1e-7)
        assert rel_err(S.download("U0"), O.field("u0")) < 1e-7
        S.close()


def test_sor_steps_match_oracle(oracle):
    w = WORKLOADS["g1"]
    O, ohist = oracle_run(oracle, w, 4, solver=3, tol=1e-9)
    S, hist = gpu_run(w, 4, solver=capi.SOLVER_SOR_RB, tol=1e-9, omega=w.omega)
    np.testing.assert_allclose([h["cd"] for h in hist], [h[0] for h in ohist], rtol=1e-8)
    for h, oh in zip(hist, ohist):
        assert all(abs(a - b) <= 1 for a, b in zip(h["iters"], oh[2]))
    assert rel_err(S.download("P"), O.field("p")) < 1e-8
    S.close()


def test_mixed_sor_steps_close_to_fp64_sor():
    """FP32 fields with the red-black SOR of the mixed path (FP32 sweeps on the
    correction between FP64 sweeps); a mixed SOR context holds no FP32 Krylov
    tables, so the metric set-up must convert only what exists.  Both runs
    converge every solve (the iteration cap is out of reach)."""
    w = WORKLOADS["c1"]
    S64, h64 = gpu_run(w, 4, solver=capi.SOLVER_SOR_RB, tol=1e-9, omega=w.omega, sor_maxit=30000)
    S32, h32 = gpu_run(w, 4, solver=capi.SOLVER_SOR_RB, tol=1e-9, omega=w.omega, sor_maxit=30000,
                       precision=capi.PREC_MIXED)
    try:
        np.testing.assert_allclose([h["cd"] for h in h32], [h["cd"] for h in h64], rtol=1e-5)
        assert rel_err(S32.download("U0"), S64.download("U0")) < 1e-5
        assert all(h["iters"][0] > 0 for h in h32[1:])
        assert all(max(h["iters"]) < 30000 for h in h32 + h64)
    finally:
        S64.close()
        S32.close()


def test_steps_are_bitwise_reproducible():
    w = WORKLOADS["g1"]
    a, ha = gpu_run(w, 4, tol=1e-10)
    b, hb = gpu_run(w, 4, tol=1e-10)
    assert [h["cd"] for h in ha] == [h["cd"] for h in hb]
    np.testing.assert_array_equal(a.download("P"), b.download("P"))
    a.close()
    b.close()


@pytest.mark.parametrize("inner", [capi.INNER_CG, capi.INNER_MG])
def test_mixed_precision_step_close_to_fp64(inner):
    w = WORKLOADS["c1"]
    S64, h64 = gpu_run(w, 4, tol=1e-10)
    S32, h32 = gpu_run(w, 4, tol=1e-10, precision=capi.PREC_MIXED, inner_solver=inner)
    cd64 = np.array([h["cd"] for h in h64])
    cd32 = np.array([h["cd"] for h in h32])
    np.testing.assert_allclose(cd32, cd64, rtol=1e-4)
    assert rel_err(S32.download("U0"), S64.download("U0")) < 1e-5
    assert all(r < 1e-10 for h in h32[1:] for r in h["relres"])
    S64.close()
    S32.close()


def test_divergence_of_projected_field():
    """After a converged solve the projected field T2 = u* - dt grad p has, in
    every cell, the uniform divergence -dt * (removed RHS mean): the
    zero-gradient outflow lets mass leave and the compatibility projection
    assigns that loss evenly.  The deviation from it is at solver level."""
    w = WORKLOADS["g1"]
    with Simulation(w, tol=1e-12) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        S.step()
        S.ConvectionDifussion(S.T0, S.T1)
        mean = S.createBMatrix(S.T1)
        S.pSolver()
        S.Pressure_transform_X_result()
        div, dev = S.div_projected(S.T1)
    assert abs(div - abs(w.dt * mean)) <= 1e-8 * max(1.0, div)
    assert dev < 1e-8 * max(1.0, div)


def test_pc_steps_on_sml_grid_match_oracle(oracle):
    """The reference's default stretched SML grid (fine cells around the
    cylinder in x and y): GPU steps against the oracle on the same metrics
    (the SML generator is pinned bitwise to the reference on the CPU)."""
    from cfd_nssolver_forhpc_gb300.simulation import sml_metrics
    w = WORKLOADS["s1"]
    m = sml_metrics(w)
    g = Grid(w.nxc, w.nyc, w.nzc, w.lx, w.ly, w.lz, oracle=oracle, metrics=m)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    O = oracle.sim(g, method=0, solver=0, aligned_src=False, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-10,
                   omega=w.omega, bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    O.init()
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    for f, a in (("u0", u0), ("v0", v0), ("w0", w0)):
        O.field(f)[:] = a
    O.start()
    ohist = [O.step() for _ in range(3)]
    with Simulation(w, tol=1e-10) as S:
        S.grid_sml()
        S.init_uniform(1.0, 0.0, 0.0)
        S.DFIB_CylinderZ(w.cx, w.center_y, w.radius, w.nsub)
        np.testing.assert_array_equal(S.download("ETA"), eta)
        for nm, a in (("U0", u0), ("V0", v0), ("W0", w0)):
            S.upload(nm, a)
        S.start()
        hist = [S.step() for _ in range(3)]
        np.testing.assert_allclose([h["cd"] for h in hist], [h[0] for h in ohist], rtol=1e-7)
        for k, f in (("U0", "u0"), ("V0", "v0"), ("W0", "w0")):
            assert rel_err(S.download(k), O.field(f)) < 1e-7, k
