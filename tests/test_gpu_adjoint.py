"""Discrete adjoint (GPU): every adjoint kernel against the linearisation of
its forward kernel, the adjoint of a whole time step, and the gradient of the
time-averaged drag against FP64 central finite differences.

Dot-product tests: for a forward map F with linearisation J at x and random
directions d (inputs) and l (outputs),

    <l, (F(x + eps d) - F(x - eps d)) / (2 eps)> = <J^T l, d>.

The central difference is exact for the affine and bilinear kernels and for
the piecewise-quadratic convection-diffusion (no upwind switch flips at eps
1e-6), so the two sides agree to rounding.  Steps and runs include the
iterative Poisson solves; they are solved to 1e-13.  QUICK's upwind switch
makes the step non-smooth where a face velocity crosses zero (inside the
body), so finite differences of eta converge only for small eps: the runs use
eps = 1e-6 (measured agreement ~1e-7), the single step eps = 1e-5.  Inflow and
eta directions are checked separately: their derivatives are of similar size
and opposite sign, and a combined direction would cancel.
"""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu

T0, T1, T3 = capi.T0, capi.T1, capi.T3
VEL = {0: ("U0", "V0", "W0"), 1: ("U1", "V1", "W1"), 3: ("U3", "V3", "W3")}

# rounding-level agreement of the dot-product tests (single kernels)
DOT_RTOL = 1e-9
# steps with solves at 1e-13 and eps = 1e-5, relative to the sum of the
# magnitudes of the per-input terms
STEP_RTOL = 1e-5
# objective gradient vs central differences (eps = 1e-6)
GRAD_RTOL = 1e-5


def rng(seed):
    return np.random.default_rng(seed)


def dot3(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


def make(w, **kw):
    S = Simulation(w, **kw)
    S.grid_uniform()
    S.adj_enable(1)
    return S


@pytest.fixture
def w():
    return WORKLOADS["g1"]


def test_convection_diffusion_adjoint(w):
    ng = w.n_ghosted
    r = rng(1)
    base = [1.0 + 0.3 * r.standard_normal(ng), 0.3 * r.standard_normal(ng), 0.3 * r.standard_normal(ng)]
    d = [r.standard_normal(ng) for _ in range(3)]
    lam = [r.standard_normal(ng) for _ in range(3)]
    eps = 1e-6
    with make(w) as S:
        def fwd(sign):
            for q, name in enumerate(VEL[0]):
                S.upload(name, base[q] + sign * eps * d[q])
            for name in VEL[1]:
                S.upload(name, np.zeros(ng))
            S.ConvectionDifussion(T0, T1)
            return [S.download(n) for n in VEL[1]]
        p, m = fwd(1.0), fwd(-1.0)
        lhs = dot3(lam, [(a - b) / (2 * eps) for a, b in zip(p, m)])
        for q, name in enumerate(VEL[0]):
            S.upload(name, base[q])
        S.adj_zero()
        for q, name in enumerate(("CDU", "CDV", "CDW")):
            S.adj_upload(name, lam[q])
        S.adj_ConvectionDifussion(T0)
        rhs = dot3([S.adj_download(n) for n in VEL[0]], d)
    assert rhs == pytest.approx(lhs, rel=1e-7)


def test_update_uf_adjoint_with_drag_lift(w):
    ng, n = w.n_ghosted, w.n_cells
    r = rng(2)
    t1 = [1.0 + 0.3 * r.standard_normal(ng), 0.3 * r.standard_normal(ng), 0.3 * r.standard_normal(ng)]
    p0 = r.standard_normal(ng)
    eta = r.uniform(0.0, 1.0, ng)
    dt1 = [r.standard_normal(ng) for _ in range(3)]
    dp = r.standard_normal(ng)
    de = r.standard_normal(ng)
    l3 = [r.standard_normal(ng) for _ in range(3)]
    lf = r.standard_normal(3 * n)
    wcd, wcl = 0.7, -0.3
    eps = 1e-6
    with make(w) as S:
        def fwd(sign):
            for q, name in enumerate(VEL[1]):
                S.upload(name, t1[q] + sign * eps * dt1[q])
            for name in VEL[3]:
                S.upload(name, np.zeros(ng))
            S.upload("P", p0 + sign * eps * dp)
            S.upload("ETA", eta + sign * eps * de)
            S.upload("F", np.zeros(3 * n))
            S.update_UandF(T1, T3)
            cd, cl = S.Delay_IO_CD_CL()
            return [S.download(nm) for nm in VEL[3]], S.download("F"), cd, cl
        a, b = fwd(1.0), fwd(-1.0)
        lhs = (dot3(l3, [(x - y) / (2 * eps) for x, y in zip(a[0], b[0])])
               + float(np.dot(lf, (a[1] - b[1]) / (2 * eps)))
               + wcd * (a[2] - b[2]) / (2 * eps) + wcl * (a[3] - b[3]) / (2 * eps))
        for q, name in enumerate(VEL[1]):
            S.upload(name, t1[q])
        S.upload("P", p0)
        S.upload("ETA", eta)
        S.adj_zero()
        for q, name in enumerate(VEL[3]):
            S.adj_upload(name, l3[q])
        S.adj_upload("F", lf)
        S.adj_update_UandF(T1, wcd, wcl)
        nx, ny, nz = w.nxc + 4, w.nyc + 4, w.nzc + 4
        dp_int = dp.reshape(nx, ny, nz)[2:-2, 2:-2, 2:-2].ravel()
        rhs = (dot3([S.adj_download(nm) for nm in VEL[1]], dt1) + float(np.dot(S.adj_download("X"), dp_int))
               + float(np.dot(S.adj_download("ETA"), de)))
    assert rhs == pytest.approx(lhs, rel=DOT_RTOL)


@pytest.mark.parametrize("compat", [True, False])
def test_create_b_adjoint(w, compat):
    ng, n = w.n_ghosted, w.n_cells
    r = rng(3)
    t1 = [r.standard_normal(ng) for _ in range(3)]
    d = [r.standard_normal(ng) for _ in range(3)]
    lam = r.standard_normal(n)
    with make(w, compat_rhs=compat) as S:
        def fwd(sign):
            for q, name in enumerate(VEL[1]):
                S.upload(name, t1[q] + sign * d[q])
            S.createBMatrix(T1)
            return S.download("B")
        lhs = float(np.dot(lam, (fwd(1.0) - fwd(-1.0)) / 2.0))
        S.adj_zero()
        S.adj_upload("B", lam)
        S.adj_createBMatrix()
        rhs = dot3([S.adj_download(nm) for nm in VEL[1]], d)
    assert rhs == pytest.approx(lhs, rel=DOT_RTOL)


def test_pressure_solve_adjoint(w):
    """<lx', A^+ db> = <A^-T lx, db> for a compatible db (uniform grid: equal
    cell volumes) and lx' = lx without its mean (the constant is free)."""
    n = w.n_cells
    r = rng(4)
    lx = r.standard_normal(n)
    with make(w, tol=1e-12, maxit=20000) as S:
        jp = S.download("JP")
        rb = r.standard_normal(n)
        db = rb - jp * np.mean(rb / jp)
        S.upload("B", db)
        S.upload("X", np.zeros(n))
        S.pSolver()
        x = S.download("X")
        lhs = float(np.dot(lx - lx.mean(), x))
        S.adj_zero()
        S.adj_upload("X", lx)
        S.adj_pSolver()
        rhs = float(np.dot(S.adj_download("B"), db))
    assert rhs == pytest.approx(lhs, rel=1e-8)


def test_bc_main_adjoint_with_inflow_profile(w):
    ng = w.n_ghosted
    r = rng(5)
    base = [r.standard_normal(ng) for _ in range(3)]
    d = [r.standard_normal(ng) for _ in range(3)]
    prof = 1.0 + 0.1 * r.standard_normal(w.nyc)
    dprof = r.standard_normal(w.nyc)
    lam = [r.standard_normal(ng) for _ in range(3)]
    with make(w) as S:
        def fwd(sign):
            for q, name in enumerate(VEL[0]):
                S.upload(name, base[q] + sign * d[q])
            S.set_inflow_profile(prof + sign * dprof)
            S.BC_staggered_main(T0)
            return [S.download(nm) for nm in VEL[0]]
        lhs = dot3(lam, [(a - b) / 2.0 for a, b in zip(fwd(1.0), fwd(-1.0))])
        S.set_inflow_profile(prof)
        S.adj_zero()
        for q, name in enumerate(VEL[0]):
            S.adj_upload(name, lam[q])
        S.adj_BC_staggered_main()
        rhs = dot3([S.adj_download(nm) for nm in VEL[0]], d) + float(np.dot(S.adj_download("INFLOW"), dprof))
    assert rhs == pytest.approx(lhs, rel=DOT_RTOL)


def test_bc_copy_adjoint(w):
    ng = w.n_ghosted
    r = rng(6)
    b0 = [r.standard_normal(ng) for _ in range(3)]
    b1 = [r.standard_normal(ng) for _ in range(3)]
    d0 = [r.standard_normal(ng) for _ in range(3)]
    d1 = [r.standard_normal(ng) for _ in range(3)]
    l0 = [r.standard_normal(ng) for _ in range(3)]
    l1 = [r.standard_normal(ng) for _ in range(3)]
    with make(w) as S:
        def fwd(sign):
            for q in range(3):
                S.upload(VEL[0][q], b0[q] + sign * d0[q])
                S.upload(VEL[1][q], b1[q] + sign * d1[q])
            S.BC_staggered_copy(T0, T1)
            return [S.download(nm) for nm in VEL[0]], [S.download(nm) for nm in VEL[1]]
        a, b = fwd(1.0), fwd(-1.0)
        lhs = dot3(l0, [(x - y) / 2.0 for x, y in zip(a[0], b[0])]) + dot3(l1, [(x - y) / 2.0 for x, y in zip(a[1], b[1])])
        S.adj_zero()
        for q in range(3):
            S.adj_upload(VEL[0][q], l0[q])
            S.adj_upload(VEL[1][q], l1[q])
        S.adj_BC_staggered_copy()
        rhs = dot3([S.adj_download(nm) for nm in VEL[0]], d0) + dot3([S.adj_download(nm) for nm in VEL[1]], d1)
    assert rhs == pytest.approx(lhs, rel=DOT_RTOL)


@pytest.mark.parametrize("aligned", [False, True])
def test_add_source_adjoint(w, aligned):
    ng, n = w.n_ghosted, w.n_cells
    r = rng(7)
    b1 = [r.standard_normal(ng) for _ in range(3)]
    src = r.standard_normal(3 * n)
    d1 = [r.standard_normal(ng) for _ in range(3)]
    ds = r.standard_normal(3 * n)
    l1 = [r.standard_normal(ng) for _ in range(3)]
    with make(w, aligned_source=aligned) as S:
        def fwd(sign):
            for q in range(3):
                S.upload(VEL[1][q], b1[q] + sign * d1[q])
            S.upload("SRC", src + sign * ds)
            S.add_source(T1)
            return [S.download(nm) for nm in VEL[1]]
        lhs = dot3(l1, [(x - y) / 2.0 for x, y in zip(fwd(1.0), fwd(-1.0))])
        S.adj_zero()
        for q in range(3):
            S.adj_upload(VEL[1][q], l1[q])
        S.adj_add_source()
        rhs = dot3([S.adj_download(nm) for nm in VEL[1]], d1) + float(np.dot(S.adj_download("SRC"), ds))
    assert rhs == pytest.approx(lhs, rel=DOT_RTOL)


def _cylinder(w, **kw):
    S = Simulation(w, **kw)
    S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
    return S


@pytest.mark.parametrize("aligned", [False, True])
def test_step_adjoint_against_central_differences(w, aligned):
    """One predictor-corrector step (4 passes, 4 Poisson solves) at a state
    after three steps: <l, dStep[d]> by central differences against the
    reversed step, for T0, eta and inflow directions one at a time."""
    ng = w.n_ghosted
    r = rng(8)
    prof = 1.0 + 0.05 * r.standard_normal(w.nyc)
    with _cylinder(w, tol=1e-13, maxit=40000, aligned_source=aligned) as S:
        S.set_inflow_profile(prof)
        for _ in range(3):
            S.step()
        S.adj_enable(1)
        S.checkpoint_alloc(1)
        S.checkpoint_save(0)
        base = [S.download(nm) for nm in VEL[0]]
        eta = S.download("ETA")
        d0 = [1e-2 * r.standard_normal(ng) for _ in range(3)]
        de = 1e-2 * r.standard_normal(ng)
        dprof = 1e-2 * r.standard_normal(w.nyc)
        l0 = [r.standard_normal(ng) for _ in range(3)]
        l1 = [r.standard_normal(ng) for _ in range(3)]
        wcd, wcl = 1.3, 0.4
        eps = 1e-5

        def fwd(a0, ae, ap):
            S.checkpoint_load(0)
            for q, nm in enumerate(VEL[0]):
                S.upload(nm, base[q] + a0 * d0[q])
            S.upload("ETA", eta + ae * de)
            S.set_inflow_profile(prof + ap * dprof)
            h = S.step()
            return ([S.download(nm) for nm in VEL[0]], [S.download(nm) for nm in VEL[1]], h["cd"], h["cl"])

        def dJ(a, b):
            return (dot3(l0, [(x - y) / (2 * eps) for x, y in zip(a[0], b[0])])
                    + dot3(l1, [(x - y) / (2 * eps) for x, y in zip(a[1], b[1])])
                    + wcd * (a[2] - b[2]) / (2 * eps) + wcl * (a[3] - b[3]) / (2 * eps))
        fd = [dJ(fwd(eps, 0, 0), fwd(-eps, 0, 0)), dJ(fwd(0, eps, 0), fwd(0, -eps, 0)),
              dJ(fwd(0, 0, eps), fwd(0, 0, -eps))]
        S.checkpoint_load(0)
        S.upload("ETA", eta)
        S.set_inflow_profile(prof)
        S.step_record(0)
        S.adj_zero()
        for q in range(3):
            S.adj_upload(VEL[0][q], l0[q])
            S.adj_upload(VEL[1][q], l1[q])
        S.adj_step(0, wcd, wcl)
        ad = [dot3([S.adj_download(nm) for nm in VEL[0]], d0), float(np.dot(S.adj_download("ETA"), de)),
              float(np.dot(S.adj_download("INFLOW"), dprof))]
    scale = sum(abs(x) for x in ad)
    for a, f in zip(ad, fd):
        assert abs(a - f) <= STEP_RTOL * scale, (ad, fd)


def _objective_model(w, first, last, interval, **kw):
    from cfd_nssolver_forhpc_gb300.adjoint import MeanDrag
    return MeanDrag(w, first, last, interval, tol=1e-13, maxit=40000, **kw)


def test_mean_drag_gradient_against_central_differences(w):
    """J = mean Cd over steps 4..8 of an 8-step run, in 3-step checkpoint
    segments; the gradient w.r.t. the inflow profile and eta along seeded
    random directions vs FP64 central differences (eps = 1e-6)."""
    m = _objective_model(w, 4, 8, 3)
    try:
        eta0 = m.default_eta().numpy()
        prof0 = np.full(w.nyc, 1.0)
        m.objective(prof0, eta0)
        g_in, g_eta = m.gradient()
        assert np.all(np.isfinite(g_in)) and np.all(np.isfinite(g_eta))
        r = rng(9)
        eps = 1e-6
        for _ in range(2):
            dp = r.standard_normal(w.nyc)
            de = r.standard_normal(eta0.size)
            fd_in = (m.objective(prof0 + eps * dp, eta0) - m.objective(prof0 - eps * dp, eta0)) / (2 * eps)
            fd_eta = (m.objective(prof0, eta0 + eps * de) - m.objective(prof0, eta0 - eps * de)) / (2 * eps)
            assert float(np.dot(g_in, dp)) == pytest.approx(fd_in, rel=GRAD_RTOL)
            assert float(np.dot(g_eta, de)) == pytest.approx(fd_eta, rel=GRAD_RTOL)
    finally:
        m.close()


def test_gradient_does_not_depend_on_checkpoint_interval(w):
    grads = []
    for interval in (1, 8):
        m = _objective_model(w, 4, 8, interval)
        try:
            eta0 = m.default_eta().numpy()
            m.objective(np.full(w.nyc, 1.0), eta0)
            grads.append(m.gradient())
        finally:
            m.close()
    for a, b in zip(grads[0], grads[1]):
        assert np.allclose(a, b, rtol=1e-10, atol=1e-12 * np.abs(a).max())


def test_autograd_harness_matches_direct_gradient(w):
    import torch
    m = _objective_model(w, 2, 5, 5)
    try:
        eta = m.default_eta().requires_grad_()
        inflow = m.default_inflow().requires_grad_()
        J = m(inflow, eta)
        J.backward()
        m.objective(inflow.detach().numpy(), eta.detach().numpy())
        g_in, g_eta = m.gradient()
        assert torch.allclose(inflow.grad, torch.from_numpy(g_in), rtol=1e-10, atol=0)
        assert torch.allclose(eta.grad, torch.from_numpy(g_eta), rtol=1e-10, atol=1e-300)
    finally:
        m.close()


def test_mixed_precision_forward_gradient_close_to_fp64(w):
    """FP32 forward / FP64-refined Poisson solves: gradient close to the FP64
    gradient (the linearisation point differs by FP32 rounding)."""
    out = []
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        m = _objective_model(w, 2, 6, 3, precision=prec)
        try:
            eta0 = m.default_eta().numpy()
            m.objective(np.full(w.nyc, 1.0), eta0)
            out.append(m.gradient())
        finally:
            m.close()
    for a, b in zip(out[0], out[1]):
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(a)
