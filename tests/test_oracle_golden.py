"""The C oracle against the golden fixtures produced by the reference itself
(tests/golden/make_golden.py).  Elementwise kernels must match bit for bit
(both sides evaluate the same expressions in the same order without fused
multiply-adds); reductions and solvers match to their summation-order /
tolerance limits."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from oracle.oracle import Grid
from tests.helpers import kernel_inputs, rel_err


@pytest.fixture(scope="module")
def g0(oracle):
    return Grid.of(WORKLOADS["g0"], oracle)


@pytest.fixture(scope="module")
def G(golden):
    return golden("g0_kernels")


def test_grid_metrics_bitwise(g0, G):
    for k, v in g0.m.items():
        np.testing.assert_array_equal(v, G[f"grid_{k}"], err_msg=k)


def test_eta_cylinder_bitwise(oracle, g0, G):
    w = WORKLOADS["g0"]
    eta = oracle.eta_cylinder_z(g0, w.cx, w.center_y, w.radius, w.nsub)
    np.testing.assert_array_equal(eta, G["eta"])
    assert 0.0 < eta.max() <= 1.0 and eta.min() == 0.0


def test_convdiff_bitwise(oracle, g0, G):
    w = WORKLOADS["g0"]
    I = kernel_inputs(g0.ng, g0.n)
    u1, v1, w1 = I["u1"].copy(), I["v1"].copy(), I["w1"].copy()
    oracle.convdiff(g0, w.dt, 1.0 / w.re, I["u0"], I["v0"], I["w0"], u1, v1, w1)
    np.testing.assert_array_equal(u1, G["cd_u1"])
    np.testing.assert_array_equal(v1, G["cd_v1"])
    np.testing.assert_array_equal(w1, G["cd_w1"])


def test_operators_bitwise(oracle, g0, G):
    w = WORKLOADS["g0"]
    I = kernel_inputs(g0.ng, g0.n)
    co, val, jp = oracle.spe_setup(g0)
    cols, vals, jpe = oracle.ell_assemble(g0)
    np.testing.assert_array_equal(jp, G["jp_spe"])
    np.testing.assert_array_equal(jpe, G["jp_ell"])
    for jj, key in ((jp, "rhs_spe"), (jpe, "rhs_ell")):
        b = np.zeros(g0.n)
        oracle.rhs(g0, w.dt, jj, I["u1"], I["v1"], I["w1"], b)
        np.testing.assert_array_equal(b, G[key])
    r = np.zeros(g0.n)
    oracle.spe_spmv(g0, co, jp, I["x"], r)
    np.testing.assert_array_equal(r, G["spmv_spe"])
    oracle.ell_spmv(g0.n, cols, vals, I["x"], r)
    np.testing.assert_array_equal(r, G["spmv_ell"])
    # ELL layout: padding slots point at the last row with value 0
    pad = vals.reshape(-1, 7) == 0.0
    assert np.all(cols.reshape(-1, 7)[pad] == g0.n - 1)


@pytest.mark.parametrize("kind", ["spe", "ell"])
def test_bicgstab_solution(oracle, g0, G, kind):
    co, val, jp = oracle.spe_setup(g0)
    cols, vals, _ = oracle.ell_assemble(g0)
    solver = oracle.bicg(g0, 1e-10, spe=(co, jp)) if kind == "spe" else \
        oracle.bicg(g0, 1e-10, ell=(cols, vals))
    b = G[f"bicg_{kind}_b"].copy()
    x = np.zeros(g0.n)
    it, res, capped = solver.solve(b, x)
    ref_it, ref_res = G[f"bicg_{kind}_it"]
    assert not capped and res < 1e-10
    assert abs(it - ref_it) <= max(3, 0.1 * ref_it)
    assert rel_err(x, G[f"bicg_{kind}_x"]) < 1e-8


def test_sor_sequential_bitwise(oracle, g0, G):
    w = WORKLOADS["g0"]
    I = kernel_inputs(g0.ng, g0.n)
    cf = oracle.sor_coef(g0)
    oracle.sor_rhs(g0, w.dt, I["u1"], I["v1"], I["w1"], cf)
    p = I["sor_p"].copy()
    it, err = oracle.sor(g0, 1.7, 1e-10, 5000, cf, p)
    np.testing.assert_array_equal(p, G["sor_p"])
    assert (it, err) == tuple(G["sor_it"])


def test_sor_redblack_same_fixed_point(oracle, g0, G):
    """Red-black and lexicographic SOR converge to the same fixed point."""
    w = WORKLOADS["g0"]
    I = kernel_inputs(g0.ng, g0.n)
    cf = oracle.sor_coef(g0)
    oracle.sor_rhs(g0, w.dt, I["u1"], I["v1"], I["w1"], cf)
    p = I["sor_p"].copy()
    it, err = oracle.sor(g0, 1.7, 1e-12, 20000, cf, p, redblack=True)
    assert err <= 1e-12
    assert rel_err(g0.interior(p), g0.interior(G["sor_p"])) < 1e-7


def test_update_uf_bitwise(oracle, g0, G):
    w = WORKLOADS["g0"]
    I = kernel_inputs(g0.ng, g0.n)
    eta = G["eta"]
    u3, v3, w3, f = np.zeros(g0.ng), np.zeros(g0.ng), np.zeros(g0.ng), I["f"].copy()
    oracle.update_uf(g0, w.dt, I["p"], eta, I["u1"], I["v1"], I["w1"], u3, v3, w3, f)
    np.testing.assert_array_equal(u3, G["uf_u3"])
    np.testing.assert_array_equal(v3, G["uf_v3"])
    np.testing.assert_array_equal(w3, G["uf_w3"])
    np.testing.assert_array_equal(f, G["uf_f"])


def test_cdcl(oracle, g0, G):
    I = kernel_inputs(g0.ng, g0.n)
    cd, cl = oracle.cdcl(g0, I["f"])
    np.testing.assert_allclose([cd, cl], G["cdcl"], rtol=1e-13)


def test_boundary_conditions_bitwise(oracle, g0, G):
    w = WORKLOADS["g0"]
    I = kernel_inputs(g0.ng, g0.n)
    a = [x.copy() for x in I["bc"]]
    oracle.bc_main(g0, w.bc_dir, w.bc_num, *a)
    for x, k in zip(a, ("bc_u", "bc_v", "bc_w", "bc_p")):
        np.testing.assert_array_equal(x, G[k])
    b = [x.copy() for x in I["bc"][1:]]
    oracle.bc_copy(g0, *I["bc"][:3], *b)
    for x, k in zip(b, ("bccopy_u", "bccopy_v", "bccopy_w")):
        np.testing.assert_array_equal(x, G[k])


def _run(oracle, name, steps, tol, solver):
    w = WORKLOADS[name]
    g = Grid.of(w, oracle)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=0, solver=solver, compat=True, dt=w.dt, nu=1.0 / w.re, tol=tol,
                   bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    S.init()
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    S.field("u0")[:] = u0
    S.field("v0")[:] = v0
    S.field("w0")[:] = w0
    S.start()
    res = [S.step() for _ in range(steps)]
    return S, np.array([r[0] for r in res]), np.array([r[1] for r in res]), np.array([r[2] for r in res])


@pytest.mark.parametrize("solver,tag", [(0, "spe"), (1, "ell")])
def test_pc_run_g0_fields(oracle, golden, solver, tag):
    G = golden("g0_run")
    S, cd, cl, it = _run(oracle, "g0", 5, 1e-10, solver)
    np.testing.assert_allclose(cd, G[f"{tag}_cd"], rtol=1e-8)
    np.testing.assert_allclose(cl, G[f"{tag}_cl"], rtol=1e-6, atol=1e-7)
    for k, f in (("u", "u0"), ("v", "v0"), ("w", "w0")):
        assert rel_err(S.field(f), G[f"{tag}_{k}"]) < 1e-9
    assert rel_err(S.field("p"), G[f"{tag}_p"]) < 1e-7
    assert np.all(np.abs(it - G[f"{tag}_iters"]) <= np.maximum(3, 0.1 * G[f"{tag}_iters"]))


@pytest.mark.parametrize("solver,tag", [(0, "spe"), (1, "ell")])
def test_pc_run_g1_history(oracle, golden, solver, tag):
    G = golden("g1_run")
    _, cd, cl, _ = _run(oracle, "g1", 10, 1e-10, solver)
    np.testing.assert_allclose(cd, G[f"{tag}_cd"], rtol=1e-8)
    np.testing.assert_allclose(cl, G[f"{tag}_cl"], rtol=1e-6, atol=1e-7)


def test_pc_run_c1_history(oracle, golden):
    """First 8 steps of the 128x64x8 cylinder at tol 1e-8 (Cd/Cl within the
    tolerance-limited 1e-6 relative of two independent solves)."""
    G = golden("c1_run")
    _, cd, cl, it = _run(oracle, "c1", 8, 1e-8, 0)
    np.testing.assert_allclose(cd, G["spe_cd"][:8], rtol=1e-6)
    np.testing.assert_allclose(cl, G["spe_cl"][:8], rtol=1e-4, atol=1e-5)
    assert cd[0] == pytest.approx(785.4022426870018, rel=1e-12)
