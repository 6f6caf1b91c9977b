"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run in a checkout that has the reference sources (the harness is compiled
from a patched scratch copy by oracle/build_ref.py):

    python tests/golden/make_golden.py

Every input is regenerated from a seed by
cfd_nssolver_forhpc_gb300.initial.seeded_field, so only the seeds and the
reference's outputs are stored.

* g0_kernels.npz  -- one call of each hot-path function on a 10x8x6 grid
* g0_run.npz      -- 5 predictor-corrector steps (BiCGSTAB SPE, tol 1e-10)
* g1_run.npz      -- 10 predictor-corrector steps on 16x12x6, SPE and ELL
Everything runs with one OpenMP thread (see the note on BC_staggered_main).

* c1_run.npz      -- 20 predictor-corrector steps on the 128x64x8 cylinder
                     (tol 1e-8), drag/lift history and field summaries
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

# BC_staggered_main runs its six face loops as `omp for nowait`
# (Boundary_Condition.hpp:72-142) although faces 2..5 read interior faces that
# faces 1 and 3 write, so multi-threaded runs race.  The fixtures record the
# single-thread (sequential) semantics.
os.environ["OMP_NUM_THREADS"] = "1"

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS  # noqa: E402
from cfd_nssolver_forhpc_gb300.initial import initial_velocity  # noqa: E402
from oracle.oracle import RefHarness  # noqa: E402
from tests.helpers import SEEDS, kernel_inputs  # noqa: E402

def summary(a: np.ndarray) -> np.ndarray:
    return np.array([a.sum(), np.abs(a).sum(), np.abs(a).max(), (a * a).sum()])


def make_g0() -> None:
    w = WORKLOADS["g0"]
    R = RefHarness("g0")
    R.set_threads(1)
    R.setup(w.dt, w.re, 1e-10, True)
    ng, n = R.ng, R.n
    I = kernel_inputs(ng, n)
    out = {"seeds": np.array(list(SEEDS.values()))}
    out.update({f"grid_{k}": v for k, v in R.grid_metrics().items()})
    out["eta"] = R.eta()
    jps, jpe = R.jp()
    out["jp_spe"], out["jp_ell"] = jps, jpe
    u1, v1, w1 = I["u1"].copy(), I["v1"].copy(), I["w1"].copy()
    R.convdiff(I["u0"], I["v0"], I["w0"], u1, v1, w1)
    out["cd_u1"], out["cd_v1"], out["cd_w1"] = u1, v1, w1
    out["rhs_spe"] = R.rhs(0, I["u1"], I["v1"], I["w1"])
    out["rhs_ell"] = R.rhs(1, I["u1"], I["v1"], I["w1"])
    out["spmv_spe"] = R.spe_spmv(I["x"])
    out["spmv_ell"] = R.ell_spmv(I["x"])
    # a consistent system: b = A x_true, solved from x = 0
    for kind, name in ((0, "spe"), (1, "ell")):
        b = R.spe_spmv(I["x"]) if kind == 0 else R.ell_spmv(I["x"])
        x = np.zeros(n)
        it, res = R.bicg(kind, b, x)
        out[f"bicg_{name}_b"], out[f"bicg_{name}_x"] = b, x
        out[f"bicg_{name}_it"] = np.array([it, res])
    pr = I["sor_p"].copy()
    it, err = R.sor_seq(I["u1"], I["v1"], I["w1"], pr, 1.7, 1e-10, 5000)
    out["sor_p"], out["sor_it"] = pr, np.array([it, err])
    u3 = np.zeros(ng); v3 = np.zeros(ng); w3 = np.zeros(ng); f = I["f"].copy()
    R.update_uf(I["p"], I["u1"], I["v1"], I["w1"], u3, v3, w3, f)
    out["uf_u3"], out["uf_v3"], out["uf_w3"], out["uf_f"] = u3, v3, w3, f
    out["cdcl"] = np.array(R.cdcl(I["f"]))
    a = [x.copy() for x in I["bc"]]
    R.bc_main(*a)
    out["bc_u"], out["bc_v"], out["bc_w"], out["bc_p"] = a
    b = [x.copy() for x in I["bc"][1:]]
    R.bc_copy(*I["bc"][:3], *b)
    out["bccopy_u"], out["bccopy_v"], out["bccopy_w"] = b
    np.savez_compressed(HERE / "g0_kernels.npz", **out)


def run_pc(name: str, steps: int, tol: float, solvers=(0,), with_fields=True) -> dict:
    w = WORKLOADS[name]
    out = {}
    for solver in solvers:
        R = RefHarness(name)
        R.set_threads(1)
        R.setup(w.dt, w.re, tol, True)
        u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
        R.pc_start(u0, v0, w0)
        cd, cl, it, _ = R.pc_run(steps, 0, solver, True)
        st = R.state()
        tag = {0: "spe", 1: "ell", 2: "sor"}[solver]
        out[f"{tag}_cd"], out[f"{tag}_cl"], out[f"{tag}_iters"] = cd, cl, it
        for k in ("u", "v", "w", "p"):
            if with_fields:
                out[f"{tag}_{k}"] = st[k]
            out[f"{tag}_{k}_summary"] = summary(st[k])
    out["tol"] = np.array([tol])
    return out


def main() -> None:
    make_g0()
    np.savez_compressed(HERE / "g0_run.npz", **run_pc("g0", 5, 1e-10, solvers=(0, 1)))
    np.savez_compressed(HERE / "g1_run.npz", **run_pc("g1", 10, 1e-10, solvers=(0, 1), with_fields=False))
    np.savez_compressed(HERE / "c1_run.npz", **run_pc("c1", 20, 1e-8, solvers=(0,), with_fields=False))
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
