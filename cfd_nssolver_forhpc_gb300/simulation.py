"""Host-side mirror of the reference's call surface over the C ABI.

`Simulation` owns one device context (`cfd_ctx`).  Its methods carry the
names of the reference functions they replace and take the same slot
arguments (T0 / T1 / T3 are the reference's velocity objects, p, eta, f,
source_termF and Mx live in the context):

    ConvectionDifussion(T0, T1)       convection_and_difussion.hpp:168
    add_source(T1)                    RUN_CPU_PC_METHOD.hpp:309-316
    accumulate_source()               RUN_CPU_PC_METHOD.hpp:393-401
    createBMatrix(T1)                 b_matrix.hpp:51
    pSolver()                         bicgstabRe2.hpp:46 (operator())
    Pressure_transform_X_result()     Transform.hpp:8
    SorPipeLine(T1)                   SorPipeLine.seq.hpp:4 (red-black)
    update_UandF(T1, T3)              updateUandF.hpp:95
    Delay_IO_CD_CL()                  virtualForceIntergrator.hpp:108
    BC_staggered_main(T0)             Boundary_Condition.hpp:37
    BC_staggered_copy(T0, T1)         updateBC.hpp:6
    DFIB_CylinderZ(cx, cy, r, nsub)   setEta.hpp:136
    step()                            one iteration of the driver's main loop

Fields move in the reference's own layouts (ghosted k-fastest, compact
icelCal), as float64 numpy arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import FIELD, check, dptr, lib
from .configs import Workload


def make_config(w: Workload, *, method: int = capi.METHOD_PC, solver: int = capi.SOLVER_BICG_SPE,
                precision: int = capi.PREC_FP64, tol: float | None = None, maxit: int = 5000,
                omega: float | None = None, sor_maxit: int = 5000, aligned_source: bool = False,
                compat_rhs: bool = True, check_every: int = 16, inner_tol: float = 1e-3,
                max_outer: int = 30, inner_solver: int = capi.INNER_MG, les: bool = False,
                conv_outflow_uc: float = 0.0, periodic_z: bool = False) -> capi.CfdConfig:
    cfg = capi.CfdConfig()
    check(lib().cfd_config_default(C.byref(cfg), w.nxc, w.nyc, w.nzc))
    cfg.lx, cfg.ly, cfg.lz = w.lx, w.ly, w.lz
    cfg.re, cfg.dt = w.re, w.dt
    cfg.method, cfg.solver, cfg.precision = method, solver, precision
    cfg.p_criteria = w.tol if tol is None else tol
    cfg.p_iter_max = maxit
    cfg.p_sor_omega = w.omega if omega is None else omega
    cfg.p_sor_iter_max = sor_maxit
    cfg.aligned_source = int(aligned_source)
    cfg.compat_rhs = int(compat_rhs)
    for b in range(6):
        for c in range(3):
            cfg.bc_dir[b][c] = w.bc_dir[b][c]
            cfg.bc_num[b][c] = w.bc_num[b][c]
    cfg.check_every = check_every
    cfg.inner_tol = inner_tol
    cfg.max_outer = max_outer
    cfg.inner_solver = inner_solver
    cfg.les_smagorinsky = int(les)
    cfg.conv_outflow_uc = conv_outflow_uc
    cfg.periodic_z = int(periodic_z)
    return cfg


class Simulation:
    T0, T1, T3 = capi.T0, capi.T1, capi.T3

    def __init__(self, w: Workload, **cfg_kw):
        self.w = w
        self.cfg = make_config(w, **cfg_kw)
        self._h = C.c_void_p()
        check(lib().cfd_create(C.byref(self.cfg), C.byref(self._h)))
        self.ng = w.n_ghosted
        self.n = w.n_cells

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if self._h:
            lib().cfd_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- grid and state ---------------------------------------------------
    def grid_uniform(self):
        check(lib().cfd_grid_uniform(self._h))

    def grid_sml(self, cfg=None):
        """The reference's stretched SML grid (structureGrid.hpp:326-405);
        cfg = capi.CfdSmlConfig or None for the reference's settings."""
        cfg = sml_default() if cfg is None else cfg
        check(lib().cfd_grid_sml(self._h, C.byref(cfg)))

    def set_metrics(self, m: dict):
        arrs = [np.ascontiguousarray(m[k], dtype=np.float64) for k in
                ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs")]
        check(lib().cfd_set_metrics(self._h, *[dptr(a) for a in arrs]))

    def count(self, field: str) -> int:
        return int(lib().cfd_field_count(self._h, FIELD[field]))

    def upload(self, field: str, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        check(lib().cfd_upload(self._h, FIELD[field], dptr(a), a.size))

    def download(self, field: str, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.count(field))
        check(lib().cfd_download(self._h, FIELD[field], dptr(out), out.size))
        return out

    def init_uniform(self, ui=1.0, vi=0.0, wi=0.0):
        check(lib().cfd_init_uniform(self._h, ui, vi, wi))

    def start(self):
        check(lib().cfd_start(self._h))

    def setup_cylinder(self, u0=None, v0=None, w0=None, eta=True):
        """Uniform grid, eta of the workload's cylinder, initial state and the
        first boundary update (RUN_CPU_PC_METHOD.hpp:75-119, 257-266)."""
        self.grid_uniform()
        self.init_uniform(1.0, 0.0, 0.0)
        if eta:
            self.DFIB_CylinderZ(self.w.cx, self.w.center_y, self.w.radius, self.w.nsub)
        for name, a in (("U0", u0), ("V0", v0), ("W0", w0)):
            if a is not None:
                self.upload(name, a)
        self.start()

    # -- the reference's operators ----------------------------------------
    def ConvectionDifussion(self, src=T0, dst=T1):
        check(lib().cfd_convection_diffusion(self._h, src, dst))

    def add_source(self, slot=T1):
        check(lib().cfd_add_source(self._h, slot))

    def accumulate_source(self):
        check(lib().cfd_accumulate_source(self._h))

    def clear_source(self):
        check(lib().cfd_clear_source(self._h))

    def createBMatrix(self, slot=T1) -> float:
        mean = C.c_double()
        check(lib().cfd_create_b(self._h, slot, C.byref(mean)))
        return mean.value

    def pSolver(self, allow_noconv=False):
        """bicgstabRe2::operator()(Mx.matB, Mx.X_result) -> (iters, relres)."""
        it, res = C.c_int(), C.c_double()
        check(lib().cfd_bicgstab(self._h, C.byref(it), C.byref(res)),
              allow=(-4,) if allow_noconv else ())
        return it.value, res.value

    def multiply(self):
        """Mx.B = A Mx.X with the configured operator."""
        check(lib().cfd_apply_operator(self._h))

    def Pressure_transform_X_result(self):
        check(lib().cfd_pressure_transform(self._h))

    def SorPipeLine(self, slot=T1):
        it, err = C.c_int(), C.c_double()
        check(lib().cfd_sor(self._h, slot, C.byref(it), C.byref(err)))
        return it.value, err.value

    def update_UandF(self, src=T1, dst=T3):
        check(lib().cfd_update_uf(self._h, src, dst))

    def Delay_IO_CD_CL(self):
        cd, cl = C.c_double(), C.c_double()
        check(lib().cfd_cdcl(self._h, C.byref(cd), C.byref(cl)))
        return cd.value, cl.value

    def BC_staggered_main(self, slot=T0):
        check(lib().cfd_bc_main(self._h, slot))

    def BC_staggered_copy(self, src=T0, dst=T1):
        check(lib().cfd_bc_copy(self._h, src, dst))

    def copy_velocity(self, src=T3, dst=T0):
        check(lib().cfd_copy_velocity(self._h, src, dst))

    def DFIB_CylinderZ(self, cx, cy, radius=0.5, nsub=100):
        """nsub >= 1: the reference's sub-sampling; nsub = 0: exact cut-cell areas."""
        check(lib().cfd_eta_cylinder_z(self._h, cx, cy, radius, nsub))

    def div_inf(self, slot=T0) -> float:
        out = C.c_double()
        check(lib().cfd_div_inf(self._h, slot, C.byref(out)))
        return out.value

    def div_projected(self, slot=T1) -> tuple[float, float]:
        """(max |div T2|, max |div T2 + dt * removed mean|) of T2 = u* - dt grad p."""
        a, b = C.c_double(), C.c_double()
        check(lib().cfd_div_projected(self._h, slot, C.byref(a), C.byref(b)))
        return a.value, b.value

    STATE_FIELDS = ("U0", "V0", "W0", "U1", "V1", "W1", "U3", "V3", "W3", "P", "X", "ETA")

    def set_clock(self, loop: int, time: float):
        """simuClass::loop / ::time (a restart from fields set by upload)."""
        check(lib().cfd_set_clock(self._h, int(loop), float(time)))

    def clock(self) -> tuple[int, float]:
        loop, t = C.c_longlong(), C.c_double()
        check(lib().cfd_get_clock(self._h, C.byref(loop), C.byref(t)))
        return loop.value, t.value

    def state(self) -> dict:
        """The fields a restart needs (FP64 host arrays) and the clock."""
        out = {k: self.download(k) for k in self.STATE_FIELDS}
        out["clock"] = self.clock()
        return out

    def restore(self, st: dict):
        """Continue from state() of any context of the same grid and either
        precision (FP32 fields widen exactly; FP64 fields round to FP32)."""
        for k in self.STATE_FIELDS:
            self.upload(k, st[k])
        self.set_clock(*st["clock"])

    def sync_periodic_z(self, slot):
        """Periodic z: ghost planes of velocity slot `slot` (or p for -1)."""
        check(lib().cfd_sync_periodic_z(self._h, slot))

    def divergence_check(self, on: bool = True):
        """Measure the projected divergence inside every later step."""
        check(lib().cfd_set_step_divergence_check(self._h, int(on)))

    def step_divergence(self) -> dict:
        """Last step's (max |div T2|, max |div T2 + dt m|, max |div u*|)."""
        out = (C.c_double * 3)()
        check(lib().cfd_step_divergence(self._h, out))
        return {"div_T2_inf": out[0], "dev_inf": out[1], "div_ustar_inf": out[2]}

    def step(self, allow_noconv=False) -> dict:
        info = capi.CfdStepInfo()
        check(lib().cfd_step(self._h, C.byref(info)), allow=(-4,) if allow_noconv else ())
        return {"loop": info.loop, "time": info.time, "iters": list(info.iters),
                "relres": list(info.relres), "outer": list(info.outer), "cd": info.cd, "cl": info.cl}

    def stream(self) -> int:
        """cudaStream_t of the context (an integer handle)."""
        out = C.c_void_p()
        check(lib().cfd_stream(self._h, C.byref(out)))
        return out.value or 0

    def launch_count(self) -> int:
        n = C.c_longlong()
        check(lib().cfd_launch_count(self._h, C.byref(n)))
        return n.value

    def time_kernels(self, reps: int = 20) -> dict:
        """Mean ms per launch of each hot kernel (CUDA events on the context
        stream); kernels the context does not use are omitted."""
        ms = (C.c_double * len(capi.KERNELS))()
        check(lib().cfd_time_kernels(self._h, reps, ms, len(capi.KERNELS)))
        return {k: v for k, v in zip(capi.KERNELS, ms) if v >= 0}

    def sync(self):
        check(lib().cfd_sync(self._h))

    # -- monitors -----------------------------------------------------------
    def get_Cfl(self, slot=T0) -> dict:
        """analyses/cfl.hpp:3 + simuClass::timestepper: cfl of `slot`, running
        cfl_max / U_max / U_min since start(), and the next dt."""
        info = capi.CfdCflInfo()
        check(lib().cfd_cfl(self._h, slot, C.byref(info)))
        return {"cfl": info.cfl, "cfl_max": info.cfl_max, "u_max": list(info.u_max), "u_min": list(info.u_min),
                "dt_next": info.dt_next}

    def SmagorinskyModel(self, slot=T0):
        """source/smagorinskyModel.hpp:31: eddy viscosity of `slot` into VIS."""
        check(lib().cfd_smagorinsky(self._h, slot))

    def CheckSteadyStatebyMaxVal(self, new=T0, old=T3) -> tuple:
        """analyses/CheckSteadystate.hpp:166: max(0, max(new - old)) per component."""
        out = np.zeros(3)
        check(lib().cfd_steady_max(self._h, new, old, dptr(out)))
        return tuple(out)

    # -- files: Plot3D (the reference's format) and the FP64 state ---------
    def OutputPlot3D_Xfile(self, path):
        """Cell-centre grid file (io/Plot3D/xfileWrite.hpp:6)."""
        check(lib().cfd_write_plot3d_x(self._h, str(path).encode()))

    def OutputPLOT3D_Qfile(self, path, slot=T3):
        """p, cell-centred u, v, w and eta of `slot` (io/Plot3D/qfile.hpp:7)."""
        check(lib().cfd_write_plot3d_q(self._h, slot, str(path).encode()))

    def save_state(self, path):
        """Bitwise restart file (T0, T1, eta, p, x, solver scalars, counters)."""
        check(lib().cfd_save_state(self._h, str(path).encode()))

    def load_state(self, path):
        check(lib().cfd_load_state(self._h, str(path).encode()))

    # -- inflow profile and the discrete adjoint --------------------------
    def set_inflow_profile(self, u_in):
        """Per-j inflow u on the x-min face (None restores bc_dir[0][0])."""
        if u_in is None:
            check(lib().cfd_set_inflow_profile(self._h, None, 0))
            return
        a = np.ascontiguousarray(u_in, dtype=np.float64)
        check(lib().cfd_set_inflow_profile(self._h, dptr(a), a.size))

    def adj_enable(self, tape_len: int = 1):
        check(lib().cfd_adj_enable(self._h, tape_len))

    def adj_zero(self):
        check(lib().cfd_adj_zero(self._h))

    def adj_count(self, field: str) -> int:
        return int(lib().cfd_adj_field_count(self._h, capi.ADJ_FIELD[field]))

    def adj_upload(self, field: str, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        check(lib().cfd_adj_upload(self._h, capi.ADJ_FIELD[field], dptr(a), a.size))

    def adj_download(self, field: str) -> np.ndarray:
        out = np.empty(self.adj_count(field))
        check(lib().cfd_adj_download(self._h, capi.ADJ_FIELD[field], dptr(out), out.size))
        return out

    def adj_ConvectionDifussion(self, src=T0):
        check(lib().cfd_adj_convection_diffusion(self._h, src))

    def adj_update_UandF(self, src=T1, wcd=0.0, wcl=0.0):
        check(lib().cfd_adj_update_uf(self._h, src, wcd, wcl))

    def adj_createBMatrix(self):
        check(lib().cfd_adj_create_b(self._h))

    def adj_pSolver(self, allow_noconv=False):
        it, res = C.c_int(), C.c_double()
        check(lib().cfd_adj_pressure_solve(self._h, C.byref(it), C.byref(res)),
              allow=(-4,) if allow_noconv else ())
        return it.value, res.value

    def adj_add_source(self):
        check(lib().cfd_adj_add_source(self._h))

    def adj_BC_staggered_main(self):
        check(lib().cfd_adj_bc_main(self._h))

    def adj_BC_staggered_copy(self):
        check(lib().cfd_adj_bc_copy(self._h))

    def step_record(self, pos: int = 0, allow_noconv=False) -> dict:
        info = capi.CfdStepInfo()
        check(lib().cfd_step_record(self._h, pos, C.byref(info)), allow=(-4,) if allow_noconv else ())
        return {"loop": info.loop, "iters": list(info.iters), "cd": info.cd, "cl": info.cl}

    def adj_step(self, pos: int = 0, wcd: float = 0.0, wcl: float = 0.0, allow_noconv=False) -> dict:
        info = capi.CfdAdjStepInfo()
        check(lib().cfd_adj_step(self._h, pos, wcd, wcl, C.byref(info)), allow=(-4,) if allow_noconv else ())
        return {"iters": list(info.iters), "relres": list(info.relres)}

    def adj_finish(self):
        check(lib().cfd_adj_finish(self._h))

    def checkpoint_alloc(self, count: int):
        check(lib().cfd_checkpoint_alloc(self._h, count))

    def checkpoint_save(self, slot: int):
        check(lib().cfd_checkpoint_save(self._h, slot))

    def checkpoint_load(self, slot: int):
        check(lib().cfd_checkpoint_load(self._h, slot))

    @staticmethod
    def _run_dict(res) -> dict:
        return {"J": res.J, "forward_seconds": res.forward_seconds, "adjoint_seconds": res.adjoint_seconds,
                "forward_iters": res.forward_iters, "adjoint_iters": res.adjoint_iters,
                "checkpoints": res.checkpoints}

    def adj_forward(self, first: int, last: int, interval: int, allow_noconv=False) -> dict:
        cfg = capi.CfdAdjRunConfig(first, last, interval)
        res = capi.CfdAdjRunResult()
        check(lib().cfd_adj_forward(self._h, C.byref(cfg), C.byref(res)), allow=(-4,) if allow_noconv else ())
        return self._run_dict(res)

    def adj_reverse(self, allow_noconv=False) -> dict:
        res = capi.CfdAdjRunResult()
        check(lib().cfd_adj_reverse(self._h, C.byref(res)), allow=(-4,) if allow_noconv else ())
        return self._run_dict(res)

    def adj_mean_drag(self, first: int, last: int, interval: int, allow_noconv=False) -> dict:
        """J = mean Cd over steps first..last and its gradient (ADJ_ETA,
        ADJ_INFLOW) by checkpointed reverse time stepping."""
        cfg = capi.CfdAdjRunConfig(first, last, interval)
        res = capi.CfdAdjRunResult()
        check(lib().cfd_adj_mean_drag(self._h, C.byref(cfg), C.byref(res)), allow=(-4,) if allow_noconv else ())
        return self._run_dict(res)


def plot3d_q_host(path, w: Workload, re: float, time: float, p, u, v, w_, eta):
    """Plot3D q file from ghosted FP64 host arrays (the same bytes as
    Simulation.OutputPLOT3D_Qfile)."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (p, u, v, w_, eta)]
    check(lib().cfd_plot3d_q_host(str(path).encode(), w.nxc, w.nyc, w.nzc, re, time, *[dptr(a) for a in arrs]))


def QfileRead(path, w: Workload):
    """io/Plot3D/qfileRead.hpp:6: ((mach, alpha, Re, time), p, u, v, w, eta)
    as ghosted FP64 arrays with the staggered faces rebuilt from the centres."""
    cond = np.zeros(4)
    out = [np.empty(w.n_ghosted) for _ in range(5)]
    check(lib().cfd_read_plot3d_q(str(path).encode(), w.nxc, w.nyc, w.nzc, dptr(cond), *[dptr(a) for a in out]))
    return (tuple(cond), *out)


def sml_default() -> capi.CfdSmlConfig:
    cfg = capi.CfdSmlConfig()
    check(lib().cfd_sml_default(C.byref(cfg)))
    return cfg


def sml_metrics(w: Workload, cfg=None) -> dict:
    """Host-side SML metrics of workload w: X, Y, Z (n+1 nodes) and the
    ghosted widths Dx..Dzs, as cfd_set_metrics takes them."""
    cfg = sml_default() if cfg is None else cfg
    n = (w.nxc + 4, w.nyc + 4, w.nzc + 4)
    out = {k: np.zeros(n[a] + 1) for a, k in enumerate(("X", "Y", "Z"))}
    for pre in ("D", "Ds"):
        for a, ax in enumerate("xyz"):
            out[pre[0] + ax + pre[1:]] = np.zeros(n[a])
    names = ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs")
    check(lib().cfd_sml_metrics(w.nxc, w.nyc, w.nzc, w.lx, w.ly, w.lz, C.byref(cfg),
                                *[dptr(out[k]) for k in names]))
    return out
