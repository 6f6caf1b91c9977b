"""Time each hot kernel of a workload on the GPU (CUDA events on the
library's stream) and print one JSON line.

    python -m cfd_nssolver_forhpc_gb300.profile_kernels --workload p1 --reps 3

The context is set up as for a run (grid, cylinder, seeded initial field, one
step), the Poisson right-hand side of the first predictor pass is formed, and
then `cfd_time_kernels` launches every hot kernel `reps` times back to back.
The program is short and its launches are few, which makes it the target of
the ncu captures summarised under profiles/.

    python -m cfd_nssolver_forhpc_gb300.profile_kernels --workload c2 --precision mixed \
        --tol 1e-10 --profile-step 3

instead runs 3 untimed steps and then one step between cudaProfilerStart and
cudaProfilerStop, the window of `ncu --profile-from-start off` (the launch
list of one whole step).  ncu cannot profile the kernels of graphs with
conditional nodes, so such a capture sets CFDGPU_SOLVE_LOOP=host: the same
kernels, with the solve loops polled from the host.
"""
from __future__ import annotations

import argparse
import json

from . import capi
from .configs import WORKLOADS
from .initial import initial_velocity
from .simulation import Simulation


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="p1")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--solver", default="spe", choices=["spe", "ell", "sor"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--tol", type=float, default=None, help="Poisson tolerance (default: the workload's)")
    ap.add_argument("--profile-step", type=int, default=None, metavar="K",
                    help="run K steps, then one step inside the profiler window")
    a = ap.parse_args(argv)
    w = WORKLOADS[a.workload]
    solver = {"spe": capi.SOLVER_BICG_SPE, "ell": capi.SOLVER_BICG_ELL, "sor": capi.SOLVER_SOR_RB}[a.solver]
    prec = capi.PREC_MIXED if a.precision == "mixed" else capi.PREC_FP64
    tol = a.tol if a.tol is not None else w.tol
    if a.profile_step is not None:
        import torch  # the profiler window API of the CUDA runtime
        with Simulation(w, solver=solver, precision=prec, tol=tol) as S:
            S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
            for _ in range(a.profile_step):
                S.step()
            S.sync()
            torch.cuda.cudart().cudaProfilerStart()
            info = S.step()
            S.sync()
            torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"workload": a.workload, "cells": w.n_cells, "solver": a.solver, "precision": a.precision,
                          "tol": tol, "warm_steps": a.profile_step, "step": info}))
        return
    with Simulation(w, solver=solver, precision=prec, tol=tol) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        S.step()
        S.ConvectionDifussion(S.T0, S.T1)
        if solver != capi.SOLVER_SOR_RB:
            S.createBMatrix(S.T1)
        ms = S.time_kernels(a.reps)
    print(json.dumps({"workload": a.workload, "cells": w.n_cells, "solver": a.solver,
                      "precision": a.precision, "reps": a.reps, "ms_per_launch": ms}))


if __name__ == "__main__":
    main()
