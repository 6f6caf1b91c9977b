"""Gradient of the time-averaged drag through the discrete adjoint, as a
torch.autograd.Function.

    model = MeanDrag(WORKLOADS["c4"].with_(...), first=250, last=500, interval=50)
    inflow = torch.ones(model.ny, dtype=torch.float64, requires_grad=True)
    eta = model.default_eta().requires_grad_()
    J = model(inflow, eta)          # forward run with checkpoints (cfd_adj_forward)
    J.backward()                    # reverse sweep (cfd_adj_reverse)
    inflow.grad, eta.grad

The parameters are the inflow profile (u on the x-min face, one value per
interior y cell; the workload's bc_dir[0][0] is the unperturbed value) and the
volume-fraction field eta in the reference's ghosted layout.  Every call
restarts the simulation from the same seeded initial velocity, so J is a
deterministic function of the parameters.  The tensors live on the host: the
state and the adjoint stay on the device inside the library context, and only
the parameters and their gradients cross the boundary.
"""
from __future__ import annotations

import numpy as np

from . import capi
from .configs import Workload
from .initial import initial_velocity
from .simulation import Simulation


class MeanDrag:
    """J(inflow, eta) = mean Cd over steps first..last of a cylinder run."""

    def __init__(self, w: Workload, first: int, last: int, interval: int, *, precision: int = capi.PREC_FP64,
                 tol: float | None = None, seed_velocity=None, **sim_kw):
        self.w = w
        self.first, self.last, self.interval = first, last, interval
        self.sim = Simulation(w, precision=precision, tol=tol, **sim_kw)
        self.sim.grid_uniform()
        self.sim.adj_enable(interval)
        self.ny = w.nyc
        self.u0 = initial_velocity(w.nxc, w.nyc, w.nzc) if seed_velocity is None else seed_velocity
        self.last_run: dict | None = None

    def close(self):
        self.sim.close()

    def default_eta(self):
        """The cylinder's eta of the workload (DFIB_CylinderZ) as a tensor."""
        import torch
        self.sim.init_uniform(1.0, 0.0, 0.0)
        self.sim.DFIB_CylinderZ(self.w.cx, self.w.center_y, self.w.radius, self.w.nsub)
        return torch.from_numpy(self.sim.download("ETA").copy())

    def default_inflow(self):
        import torch
        return torch.full((self.ny,), float(self.w.bc_dir[0][0]), dtype=torch.float64)

    def restart(self, inflow: np.ndarray, eta: np.ndarray):
        """Initial state of the run for the given parameters (cfd_start)."""
        s = self.sim
        s.init_uniform(1.0, 0.0, 0.0)
        s.upload("ETA", eta)
        for name, a in zip(("U0", "V0", "W0"), self.u0):
            s.upload(name, a)
        s.set_inflow_profile(inflow)
        s.start()

    def objective(self, inflow: np.ndarray, eta: np.ndarray) -> float:
        """J only (one forward run with checkpoints)."""
        self.restart(inflow, eta)
        self.last_run = self.sim.adj_forward(self.first, self.last, self.interval, allow_noconv=True)
        return self.last_run["J"]

    def gradient(self) -> tuple[np.ndarray, np.ndarray]:
        """Reverse sweep of the last objective(): (dJ/dinflow, dJ/deta)."""
        rev = self.sim.adj_reverse(allow_noconv=True)
        if self.last_run is not None:
            self.last_run.update({k: rev[k] for k in ("adjoint_seconds", "adjoint_iters")})
        return self.sim.adj_download("INFLOW"), self.sim.adj_download("ETA")

    def __call__(self, inflow, eta):
        return _MeanDragFn.apply(inflow, eta, self)


def _torch_fn():
    import torch

    class MeanDragFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, inflow, eta, model: MeanDrag):
            J = model.objective(inflow.detach().cpu().numpy().astype(np.float64),
                                eta.detach().cpu().numpy().astype(np.float64))
            ctx.model = model
            ctx.devices = (inflow.device, eta.device)
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            g_in, g_eta = ctx.model.gradient()
            gj = gJ.detach().cpu().double()
            return (torch.from_numpy(g_in).mul(gj).to(ctx.devices[0]),
                    torch.from_numpy(g_eta).mul(gj).to(ctx.devices[1]), None)

    return MeanDragFn


class _Lazy:
    _fn = None

    def apply(self, *args):
        if _Lazy._fn is None:
            _Lazy._fn = _torch_fn()
        return _Lazy._fn.apply(*args)


_MeanDragFn = _Lazy()
