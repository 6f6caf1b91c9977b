"""Per-kernel parity of the CUDA library (through the C ABI) with the FP64
oracle and with the reference's golden outputs.

Tolerances: kernels whose reference code is a chain of sums and products
without division (boundary conditions, source coupling, projection copy,
eta, jp, ELL assembly) are bitwise equal.  Kernels in which the reference
divides by a cell width multiply by a tabulated reciprocal on the GPU and
use fused multiply-adds: max |gpu - oracle| / max |oracle| <= 1e-13."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.simulation import Simulation
from oracle.oracle import Grid
from tests.helpers import KERNEL_RTOL, kernel_inputs, rel_err

pytestmark = pytest.mark.gpu

CASES = ["g0", "g2", "c1"]


@pytest.fixture(scope="module", params=CASES)
def case(request, oracle):
    w = WORKLOADS[request.param]
    g = Grid.of(w, oracle)
    sims = {}

    def sim(solver=capi.SOLVER_BICG_SPE):
        if solver not in sims:
            s = Simulation(w, solver=solver, tol=1e-10)
            s.grid_uniform()
            sims[solver] = s
        return sims[solver]
    yield w, g, sim
    for s in sims.values():
        s.close()


def test_eta_bitwise(case, oracle):
    w, g, sim = case
    S = sim()
    S.DFIB_CylinderZ(w.cx, w.center_y, w.radius, w.nsub)
    eta = S.download("ETA")
    np.testing.assert_array_equal(eta, oracle.eta_cylinder_z(g, w.cx, w.center_y, w.radius, w.nsub))


def test_convdiff(case, oracle, golden):
    w, g, sim = case
    S = sim()
    I = kernel_inputs(g.ng, g.n)
    for k in ("U0", "V0", "W0", "U1", "V1", "W1"):
        S.upload(k, I[k.lower()])
    S.ConvectionDifussion(S.T0, S.T1)
    u1, v1, w1 = I["u1"].copy(), I["v1"].copy(), I["w1"].copy()
    oracle.convdiff(g, w.dt, 1.0 / w.re, I["u0"], I["v0"], I["w0"], u1, v1, w1)
    for k, ref in (("U1", u1), ("V1", v1), ("W1", w1)):
        assert rel_err(S.download(k), ref) <= KERNEL_RTOL, k
    if w.name == "g0":
        G = golden("g0_kernels")
        assert rel_err(S.download("U1"), G["cd_u1"]) <= KERNEL_RTOL


@pytest.mark.parametrize("solver", [capi.SOLVER_BICG_SPE, capi.SOLVER_BICG_ELL])
def test_jp_rhs_and_operator(case, oracle, solver):
    w, g, sim = case
    S = sim(solver)
    I = kernel_inputs(g.ng, g.n)
    if solver == capi.SOLVER_BICG_SPE:
        co, _, jp = oracle.spe_setup(g)
    else:
        cols, vals, jp = oracle.ell_assemble(g)
    np.testing.assert_array_equal(S.download("JP"), jp)
    for k in ("U1", "V1", "W1"):
        S.upload(k, I[k.lower()])
    S.createBMatrix(S.T1)
    b = np.zeros(g.n)
    oracle.rhs(g, w.dt, jp, I["u1"], I["v1"], I["w1"], b, compat=True)
    assert rel_err(S.download("B"), b) <= KERNEL_RTOL
    S.upload("X", I["x"])
    S.multiply()
    r = np.zeros(g.n)
    if solver == capi.SOLVER_BICG_SPE:
        oracle.spe_spmv(g, co, jp, I["x"], r)
    else:
        oracle.ell_spmv(g.n, cols, vals, I["x"], r)
    assert rel_err(S.download("B"), r) <= KERNEL_RTOL


def test_update_uf_and_transform(case, oracle):
    w, g, sim = case
    S = sim()
    I = kernel_inputs(g.ng, g.n)
    eta = oracle.eta_cylinder_z(g, w.cx, w.center_y)
    S.upload("ETA", eta)
    S.upload("P", I["p"])
    for k in ("U1", "V1", "W1"):
        S.upload(k, I[k.lower()])
    zeros = np.zeros(g.ng)
    for k in ("U3", "V3", "W3"):
        S.upload(k, zeros)
    S.upload("F", I["f"])
    S.update_UandF(S.T1, S.T3)
    u3, v3, w3, f = zeros.copy(), zeros.copy(), zeros.copy(), I["f"].copy()
    oracle.update_uf(g, w.dt, I["p"], eta, I["u1"], I["v1"], I["w1"], u3, v3, w3, f)
    for k, ref in (("U3", u3), ("V3", v3), ("W3", w3), ("F", f)):
        assert rel_err(S.download(k), ref) <= KERNEL_RTOL, k
    # Pressure_transform_X_result is a pure copy
    S.upload("X", I["x"])
    S.upload("P", I["p"])
    S.Pressure_transform_X_result()
    p = I["p"].copy()
    oracle.pressure_transform(g, I["x"], p)
    np.testing.assert_array_equal(S.download("P"), p)


def test_cdcl(case, oracle):
    w, g, sim = case
    S = sim()
    I = kernel_inputs(g.ng, g.n)
    S.upload("F", I["f"])
    cd, cl = S.Delay_IO_CD_CL()
    rcd, rcl = oracle.cdcl(g, I["f"])
    assert cd == pytest.approx(rcd, rel=1e-12, abs=1e-12)
    assert cl == pytest.approx(rcl, rel=1e-12, abs=1e-12)


def test_boundary_conditions_bitwise(case, oracle, golden):
    w, g, sim = case
    S = sim()
    I = kernel_inputs(g.ng, g.n)
    a = [x.copy() for x in I["bc"]]
    for k, x in zip(("U0", "V0", "W0", "P"), a):
        S.upload(k, x)
    S.BC_staggered_main(S.T0)
    oracle.bc_main(g, w.bc_dir, w.bc_num, *a)
    for k, x in zip(("U0", "V0", "W0", "P"), a):
        np.testing.assert_array_equal(S.download(k), x, err_msg=k)
    old = I["bc"][:3]
    cur = [x.copy() for x in I["bc"][1:]]
    for k, x in zip(("U0", "V0", "W0"), old):
        S.upload(k, x)
    for k, x in zip(("U1", "V1", "W1"), cur):
        S.upload(k, x)
    S.BC_staggered_copy(S.T0, S.T1)
    oracle.bc_copy(g, *old, *cur)
    for k, x in zip(("U1", "V1", "W1"), cur):
        np.testing.assert_array_equal(S.download(k), x, err_msg=k)
    if w.name == "g0":
        G = golden("g0_kernels")
        np.testing.assert_array_equal(a[0], G["bc_u"])


@pytest.mark.parametrize("aligned", [False, True])
def test_source_coupling_bitwise(case, oracle, aligned):
    w, g, _ = case
    with Simulation(w, aligned_source=aligned) as S:
        S.grid_uniform()
        I = kernel_inputs(g.ng, g.n)
        for k in ("U1", "V1", "W1"):
            S.upload(k, I[k.lower()])
        S.upload("SRC", I["f"])
        S.add_source(S.T1)
        u1, v1, w1 = I["u1"].copy(), I["v1"].copy(), I["w1"].copy()
        oracle.src_add(g, aligned, u1, v1, w1, I["f"])
        for k, ref in (("U1", u1), ("V1", v1), ("W1", w1)):
            np.testing.assert_array_equal(S.download(k), ref, err_msg=k)
        src = I["f"].copy()
        S.upload("F", I["x"].repeat(3))
        S.upload("SRC", src)
        S.accumulate_source()
        oracle.src_accumulate(g, w.dt, src, I["x"].repeat(3))
        assert rel_err(S.download("SRC"), src) <= 1e-15


def test_argument_errors_on_device():
    w = WORKLOADS["g0"]
    with Simulation(w) as S:
        with pytest.raises(capi.CfdError, match="metrics"):
            S.ConvectionDifussion()
        S.grid_uniform()
        with pytest.raises(capi.CfdError, match="slot"):
            S.ConvectionDifussion(0, 2)
        with pytest.raises(capi.CfdError, match="element count"):
            S.upload("U0", np.zeros(5))
        with pytest.raises(capi.CfdError, match="SOR"):
            S.SorPipeLine()
