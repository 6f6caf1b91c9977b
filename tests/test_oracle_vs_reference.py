"""The oracle against the reference's own code, live (CPU).

oracle/build_ref.py compiles oracle/ref_harness.cpp against a patched copy of
the reference headers; these tests feed both sides fresh seeded inputs on
grids other than the golden ones and require bitwise equality for every
elementwise kernel.  Skipped where the reference sources are unavailable."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity, seeded_field
from oracle.oracle import Grid


def _harness(name):
    from oracle import build_ref
    from oracle.oracle import RefHarness
    try:
        build_ref.build(name)
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference sources unavailable: {e}")
    return RefHarness(name, build=False)


@pytest.fixture(scope="module", params=["g1", "g2"])
def pair(request, oracle):
    # one OpenMP thread: BC_staggered_main races between its face loops
    # when multi-threaded (Boundary_Condition.hpp:72-142)
    w = WORKLOADS[request.param]
    R = _harness(w.name)
    R.set_threads(1)
    R.setup(w.dt, w.re, 1e-10, True)
    return w, R, Grid.of(w, oracle)


def inputs(g, seed):
    f = lambda n, k, lo=-1.0, hi=1.0: seeded_field(n, seed * 100 + k, lo, hi)  # noqa: E731
    return dict(u0=f(g.ng, 1, 0.5, 1.5), v0=f(g.ng, 2, -.4, .4), w0=f(g.ng, 3, -.4, .4),
                u1=f(g.ng, 4), v1=f(g.ng, 5), w1=f(g.ng, 6), p=f(g.ng, 7), f=f(3 * g.n, 8),
                x=f(g.n, 9))


@pytest.mark.parametrize("seed", [3, 4])
def test_elementwise_kernels_bitwise(pair, oracle, seed):
    w, R, g = pair
    I = inputs(g, seed)
    for k, v in R.grid_metrics().items():
        np.testing.assert_array_equal(v, g.m[k], err_msg=k)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    np.testing.assert_array_equal(eta, R.eta())
    a = [I["u1"].copy(), I["v1"].copy(), I["w1"].copy()]
    b = [x.copy() for x in a]
    R.convdiff(I["u0"], I["v0"], I["w0"], *a)
    oracle.convdiff(g, w.dt, 1.0 / w.re, I["u0"], I["v0"], I["w0"], *b)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    co, _, jp = oracle.spe_setup(g)
    cols, vals, jpe = oracle.ell_assemble(g)
    rs, re_ = R.jp()
    np.testing.assert_array_equal(rs, jp)
    np.testing.assert_array_equal(re_, jpe)
    bo = np.zeros(g.n)
    oracle.rhs(g, w.dt, jp, I["u1"], I["v1"], I["w1"], bo)
    np.testing.assert_array_equal(R.rhs(0, I["u1"], I["v1"], I["w1"]), bo)
    r = np.zeros(g.n)
    oracle.spe_spmv(g, co, jp, I["x"], r)
    np.testing.assert_array_equal(R.spe_spmv(I["x"]), r)
    oracle.ell_spmv(g.n, cols, vals, I["x"], r)
    np.testing.assert_array_equal(R.ell_spmv(I["x"]), r)
    R.set_eta(eta)
    ua = [np.zeros(g.ng) for _ in range(3)] + [I["f"].copy()]
    ub = [x.copy() for x in ua]
    R.update_uf(I["p"], I["u1"], I["v1"], I["w1"], *ua)
    oracle.update_uf(g, w.dt, I["p"], eta, I["u1"], I["v1"], I["w1"], *ub)
    for x, y in zip(ua, ub):
        np.testing.assert_array_equal(x, y)
    c = [I["u0"].copy(), I["v0"].copy(), I["w0"].copy(), I["p"].copy()]
    d = [x.copy() for x in c]
    R.bc_main(*c)
    oracle.bc_main(g, w.bc_dir, w.bc_num, *d)
    for x, y in zip(c, d):
        np.testing.assert_array_equal(x, y)


def test_pc_run_matches_reference(pair, oracle):
    """Five predictor-corrector steps, BiCGSTAB SPE at tol 1e-10 with the
    compatibility projection applied on both sides."""
    w, R, g = pair
    R.setup(w.dt, w.re, 1e-10, True)
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    R.pc_start(u0, v0, w0)
    cd_r, cl_r, it_r, _ = R.pc_run(5, 0, 0, True)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S = oracle.sim(g, method=0, solver=0, compat=True, dt=w.dt, nu=1.0 / w.re, tol=1e-10,
                   bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
    S.init()
    S.field("u0")[:] = u0
    S.field("v0")[:] = v0
    S.field("w0")[:] = w0
    S.start()
    res = [S.step() for _ in range(5)]
    np.testing.assert_allclose([r[0] for r in res], cd_r, rtol=1e-8)
    st = R.state()
    assert np.max(np.abs(st["u"] - S.field("u0"))) < 1e-9


@pytest.mark.parametrize("seed", [3, 4])
def test_monitors_bitwise(pair, oracle, seed):
    """get_Cfl, timestepper and CheckSteadyStatebyMaxVal_omp of the oracle
    equal the reference's on seeded fields (signed velocities, so the
    signed-sum and signed-difference conventions are exercised)."""
    w, R, g = pair
    I = inputs(g, seed)
    c_r, umax_r, umin_r = R.cfl(I["u0"], I["v0"], I["w0"])
    c_o, umax_o, umin_o, cm = oracle.cfl(g, R_dt(R, w), I["u0"], I["v0"], I["w0"])
    assert c_o == c_r and cm == c_r
    np.testing.assert_array_equal(umax_o, umax_r)
    np.testing.assert_array_equal(umin_o, umin_r)
    assert oracle.timestepper(w.re, umax_o, umin_o) == R.timestepper(umax_r, umin_r)
    u3 = I["u0"] + seeded_field(g.ng, 900 + seed, -0.2, 0.2)
    np.testing.assert_array_equal(oracle.steady_max(g, I["u0"], I["v0"], I["w0"], u3, I["v0"], I["w0"] * 0.5),
                                  R.steady_max(I["u0"], I["v0"], I["w0"], u3, I["v0"], I["w0"] * 0.5))


def R_dt(R, w):
    """the dt the harness was set up with (the pair fixture uses w.dt)"""
    return w.dt


def test_smagorinsky_les_bitwise(oracle):
    """The LES option: the reference compiled with TERBULENCE_SMAGORINSKY (its
    one misspelt `auto` corrected in the scratch copy).  The oracle's eddy
    viscosity and its convection-diffusion with nu + nu_t equal the
    reference's bitwise."""
    from oracle import build_ref
    from oracle.oracle import RefHarness
    w = WORKLOADS["g1"]
    try:
        build_ref.build(w.name, les=True)
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference sources unavailable: {e}")
    R = RefHarness(w.name + "_les", build=False)
    R.set_threads(1)
    R.setup(w.dt, w.re, 1e-8, True)
    g = Grid.of(w, oracle)
    I = inputs(g, 7)
    vis_r = R.smagorinsky(I["u0"], I["v0"], I["w0"])
    vis_o = oracle.smagorinsky(g, I["u0"], I["v0"], I["w0"])
    assert vis_o.max() > 0
    np.testing.assert_array_equal(vis_o, vis_r)
    out_r = [g.zeros() for _ in range(3)]
    out_o = [g.zeros() for _ in range(3)]
    R.convdiff(I["u0"], I["v0"], I["w0"], *out_r)
    oracle.convdiff_les(g, w.dt, 1.0 / w.re, vis_o, I["u0"], I["v0"], I["w0"], *out_o)
    for a, b in zip(out_o, out_r):
        np.testing.assert_array_equal(a, b)
