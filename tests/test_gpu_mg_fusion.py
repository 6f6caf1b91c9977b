"""Alternative forms of V-cycle kernels against the plain ones (GPU).

* Fused sweep ends (CFDGPU_MG_FUSE_ENDS=1, off by default): on float4 levels
  the first pre-smoothing sweep (both colours from x = 0) and the
  prolongation with the first post-smoothing colour each run as one kernel.
* Float4-row transfers (default; CFDGPU_MG_TRANSFER4=0 gives the scalar
  kernels): the restriction reads the children's rows as float4 quads, the
  prolongation adds to one quad per thread.
* The coarse levels in one thread-block cluster (CFDGPU_MG_CLUSTER=1, off by
  default: measured slower), against the single-block kernel of the small
  levels (CFDGPU_MG_FD=0): a different summation in the coarsest solve, so
  the runs agree to the solver tolerance rather than bit for bit.
* The separable solve of the coarsest level (default) against the small
  levels with the dense coarsest solve (CFDGPU_MG_FD=0): a different
  preconditioner, so the steps agree to the solver tolerance, and the exact
  coarse solve needs no more iterations.
* Two-row colour launches (default on levels of at least 2^21 cells;
  CFDGPU_MG_ROWS2=0 turns them off): a thread updates one quad in each of two
  neighbouring j rows.  c1's levels are below the size, so the test runs a
  512x256x32 grid for one step.
* The two-row colour pass marching along x (CFDGPU_MG_MARCH=ci planes a
  thread; off by default): on 512x256x32, with a chunk that divides the 512
  planes and one that does not.
* Tiled smoothing phases (default on the grid-wide levels below the finest
  of at most 2^17 cells; CFDGPU_MG_TILE_SPLIT=1 adds those up to 2^20 cells
  one sweep a launch; CFDGPU_MG_TILE=0 gives the colour launches,
  CFDGPU_MG_TILE_FROM=l tiles every level from l on, l = 0 the finest
  level's pre-smoothing too): one launch per phase over tiles with a
  recomputed halo.  The 512x256x32 grid runs with both of its levels below
  the finest tiled, the 128x64x8 grid (none below the finest) with the
  finest level's pre-smoothing tiled.

Both keep the arithmetic of the plain launches term for term, so steps agree
bit for bit, with the multigrid-preconditioned inner solve of the mixed path
and with the FP64 defect-correction variant, on grids whose levels are all
float4 rows and on one (periodic z) whose z axis stops coarsening early."""
from __future__ import annotations

import os

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu


def _run_env(w, env, steps=3, sml=False, **kw):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        with Simulation(w, tol=1e-10, **kw) as S:
            if sml:  # the reference's stretched grid instead of the uniform one
                S.grid_sml()
                S.init_uniform(1.0, 0.0, 0.0)
                S.DFIB_CylinderZ(w.cx, w.center_y, w.radius, w.nsub)
                for nm, a in zip(("U0", "V0", "W0"), initial_velocity(w.nxc, w.nyc, w.nzc)):
                    S.upload(nm, a)
                S.start()
            else:
                S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
            hist = [S.step() for _ in range(steps)]
            return hist, {k: S.download(k) for k in ("U0", "V0", "W0", "P")}
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _run(w, fuse, var="CFDGPU_MG_FUSE_ENDS", steps=3, **kw):
    return _run_env(w, {var: "1" if fuse else "0"}, steps, **kw)


@pytest.mark.parametrize("precision,periodic", [(capi.PREC_MIXED, False), (capi.PREC_FP64_DC, False),
                                                (capi.PREC_MIXED, True)])
def test_fused_sweep_ends_bitwise(precision, periodic):
    w = WORKLOADS["c1"]
    h1, f1 = _run(w, True, precision=precision, periodic_z=periodic)
    h0, f0 = _run(w, False, precision=precision, periodic_z=periodic)
    assert [h["cd"] for h in h1] == [h["cd"] for h in h0]
    assert [h["iters"] for h in h1] == [h["iters"] for h in h0]
    for k in f1:
        np.testing.assert_array_equal(f1[k], f0[k], err_msg=k)


@pytest.mark.parametrize("precision,periodic", [(capi.PREC_MIXED, False), (capi.PREC_FP64_DC, False),
                                                (capi.PREC_MIXED, True)])
def test_float4_transfers_bitwise(precision, periodic):
    w = WORKLOADS["c1"]
    h1, f1 = _run(w, True, "CFDGPU_MG_TRANSFER4", precision=precision, periodic_z=periodic)
    h0, f0 = _run(w, False, "CFDGPU_MG_TRANSFER4", precision=precision, periodic_z=periodic)
    assert [h["cd"] for h in h1] == [h["cd"] for h in h0]
    assert [h["iters"] for h in h1] == [h["iters"] for h in h0]
    for k in f1:
        np.testing.assert_array_equal(f1[k], f0[k], err_msg=k)


@pytest.mark.parametrize("precision,periodic", [(capi.PREC_MIXED, False), (capi.PREC_MIXED, True)])
def test_two_row_smoother_bitwise(precision, periodic):
    w = WORKLOADS["c2"]
    h1, f1 = _run(w, True, "CFDGPU_MG_ROWS2", precision=precision, periodic_z=periodic, steps=2)
    h0, f0 = _run(w, False, "CFDGPU_MG_ROWS2", precision=precision, periodic_z=periodic, steps=2)
    assert [h["cd"] for h in h1] == [h["cd"] for h in h0]
    assert [h["iters"] for h in h1] == [h["iters"] for h in h0]
    for k in f1:
        np.testing.assert_array_equal(f1[k], f0[k], err_msg=k)


@pytest.mark.parametrize("name,precision,periodic", [("c1", capi.PREC_MIXED, False), ("c1", capi.PREC_FP64_DC, False),
                                                     ("c1", capi.PREC_MIXED, True)])
def test_cluster_coarse_levels_match_single_block(name, precision, periodic):
    w = WORKLOADS[name]
    h1, f1 = _run(w, True, "CFDGPU_MG_CLUSTER", precision=precision, periodic_z=periodic)
    h0, f0 = _run_env(w, {"CFDGPU_MG_CLUSTER": "0", "CFDGPU_MG_FD": "0"}, precision=precision, periodic_z=periodic)
    np.testing.assert_allclose([h["cd"] for h in h1], [h["cd"] for h in h0], rtol=1e-8)
    for a, b in zip(h1, h0):
        assert all(abs(x - y) <= 2 for x, y in zip(a["iters"], b["iters"])), (a["iters"], b["iters"])
        assert all(r < 1e-10 for r in a["relres"][1:] if r > 0)
    for k in ("U0", "V0", "W0"):
        d = np.abs(f1[k] - f0[k]).max() / np.abs(f0[k]).max()
        assert d < 1e-6, (k, d)


@pytest.mark.parametrize("name,precision,periodic,tile_from",
                         [("c2", capi.PREC_MIXED, False, "1"), ("c2", capi.PREC_MIXED, True, "1"),
                          ("c2", capi.PREC_MIXED, False, None), ("c2", capi.PREC_MIXED, True, None),
                          ("c2", capi.PREC_MIXED, False, "split"), ("c2", capi.PREC_MIXED, True, "split"),
                          ("c1", capi.PREC_MIXED, False, "0"), ("c1", capi.PREC_FP64_DC, True, "0")])
def test_tiled_phases_bitwise(name, precision, periodic, tile_from):
    """tile_from None: the default (the levels of at most 2^17 cells);
    "split": also the 524 288-cell level of 512x256x32, one sweep a launch."""
    w = WORKLOADS[name]
    steps = 2 if name == "c2" else 3
    env = ({"CFDGPU_MG_TILE": "1"} if tile_from is None else {"CFDGPU_MG_TILE_SPLIT": "1"} if tile_from == "split"
           else {"CFDGPU_MG_TILE_FROM": tile_from})
    h1, f1 = _run_env(w, env, steps, precision=precision, periodic_z=periodic)
    h0, f0 = _run_env(w, {"CFDGPU_MG_TILE": "0"}, steps, precision=precision, periodic_z=periodic)
    assert [h["cd"] for h in h1] == [h["cd"] for h in h0]
    assert [h["iters"] for h in h1] == [h["iters"] for h in h0]
    for k in f1:
        np.testing.assert_array_equal(f1[k], f0[k], err_msg=k)


@pytest.mark.parametrize("name,precision,periodic", [("c1", capi.PREC_MIXED, False), ("c1", capi.PREC_FP64_DC, False),
                                                     ("c1", capi.PREC_MIXED, True), ("s1", capi.PREC_MIXED, False)])
def test_separable_coarse_solve_matches_small_levels(name, precision, periodic):
    w = WORKLOADS[name]
    kw = dict(precision=precision, periodic_z=periodic, sml=name == "s1")
    h1, f1 = _run_env(w, {"CFDGPU_MG_FD": "1"}, **kw)
    h0, f0 = _run_env(w, {"CFDGPU_MG_FD": "0"}, **kw)
    np.testing.assert_allclose([h["cd"] for h in h1], [h["cd"] for h in h0], rtol=1e-8)
    for a, b in zip(h1, h0):
        assert all(r < 1e-10 for r in a["relres"][1:] if r > 0)
        assert sum(a["iters"]) <= sum(b["iters"]) + 2, (a["iters"], b["iters"])
    for k in ("U0", "V0", "W0"):
        d = np.abs(f1[k] - f0[k]).max() / np.abs(f0[k]).max()
        assert d < 1e-6, (k, d)


@pytest.mark.parametrize("march,periodic", [("4", False), ("3", False), ("4", True)])
def test_marching_colour_pass_bitwise(march, periodic):
    w = WORKLOADS["c2"]
    h1, f1 = _run_env(w, {"CFDGPU_MG_MARCH": march}, 2, precision=capi.PREC_MIXED, periodic_z=periodic)
    h0, f0 = _run_env(w, {"CFDGPU_MG_MARCH": "0"}, 2, precision=capi.PREC_MIXED, periodic_z=periodic)
    assert [h["cd"] for h in h1] == [h["cd"] for h in h0]
    assert [h["iters"] for h in h1] == [h["iters"] for h in h0]
    for k in f1:
        np.testing.assert_array_equal(f1[k], f0[k], err_msg=k)
