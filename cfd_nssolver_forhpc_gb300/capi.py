"""ctypes binding of libcfdgpu.so (include/cfdgpu.h).

The library is the only compute path: importing this module when the
extension has not been built raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libcfdgpu.so"

CFD_OK = 0
STATUS = {0: "CFD_OK", -1: "CFD_ERR_ARG", -2: "CFD_ERR_CUDA", -3: "CFD_ERR_NOMEM",
          -4: "CFD_ERR_NOCONV", -5: "CFD_ERR_NAN", -6: "CFD_ERR_TIMEOUT", -7: "CFD_ERR_STATE"}

SOLVER_BICG_SPE, SOLVER_BICG_ELL, SOLVER_SOR_RB = 0, 1, 3
METHOD_PC, METHOD_PLAIN = 0, 1
PREC_FP64, PREC_MIXED, PREC_FP64_DC = 0, 1, 2
INNER_CG, INNER_BICGSTAB, INNER_MG = 0, 1, 2
T0, T1, T3 = 0, 1, 3
KERNELS = ["bicg_ap", "bicg_s", "bicg_as", "bicg_xr", "bicg_p", "convdiff", "update_uf", "rhs",
           "sor_sweep", "cg_pq", "cg_upd", "residual64", "mg_smooth", "mg_restrict", "mg_prolong", "mg_coarse",
           "mg_vcycle", "mg_upd", "mg_rho", "mg_sweep", "pass", "update_pass",
           "sor32_sweep"]
FIELDS = ["U0", "V0", "W0", "U1", "V1", "W1", "U3", "V3", "W3", "P", "ETA", "F", "SRC", "X", "B", "JP", "VIS"]
FIELD = {name: i for i, name in enumerate(FIELDS)}
ADJ_FIELDS = ["U0", "V0", "W0", "U1", "V1", "W1", "U3", "V3", "W3", "CDU", "CDV", "CDW", "X", "B", "F", "SRC",
              "ETA", "INFLOW"]
ADJ_FIELD = {name: i for i, name in enumerate(ADJ_FIELDS)}


class CfdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class CfdConfig(C.Structure):
    _fields_ = [("nx_cal", C.c_int), ("ny_cal", C.c_int), ("nz_cal", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("re", C.c_double), ("dt", C.c_double),
                ("method", C.c_int), ("solver", C.c_int), ("precision", C.c_int),
                ("p_criteria", C.c_double), ("p_iter_max", C.c_int),
                ("p_sor_omega", C.c_double), ("p_sor_iter_max", C.c_int),
                ("aligned_source", C.c_int), ("compat_rhs", C.c_int),
                ("bc_dir", (C.c_double * 3) * 6), ("bc_num", (C.c_double * 3) * 6),
                ("check_every", C.c_int), ("inner_tol", C.c_double), ("max_outer", C.c_int),
                ("inner_solver", C.c_int), ("les_smagorinsky", C.c_int), ("conv_outflow_uc", C.c_double),
                ("periodic_z", C.c_int)]


class CfdStepInfo(C.Structure):
    _fields_ = [("loop", C.c_longlong), ("time", C.c_double), ("iters", C.c_int * 4),
                ("relres", C.c_double * 4), ("outer", C.c_int * 4), ("cd", C.c_double),
                ("cl", C.c_double)]


class CfdSmlConfig(C.Structure):
    _fields_ = [("fine_fraction", C.c_double * 3), ("fine_cells", C.c_int * 3), ("offset", C.c_int * 3)]


class CfdCflInfo(C.Structure):
    _fields_ = [("cfl", C.c_double), ("cfl_max", C.c_double), ("u_max", C.c_double * 3),
                ("u_min", C.c_double * 3), ("dt_next", C.c_double)]


class CfdAdjStepInfo(C.Structure):
    _fields_ = [("iters", C.c_int * 4), ("relres", C.c_double * 4)]


class CfdAdjRunConfig(C.Structure):
    _fields_ = [("first", C.c_int), ("last", C.c_int), ("interval", C.c_int)]


class CfdAdjRunResult(C.Structure):
    _fields_ = [("J", C.c_double), ("forward_seconds", C.c_double), ("adjoint_seconds", C.c_double),
                ("forward_iters", C.c_longlong), ("adjoint_iters", C.c_longlong), ("checkpoints", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    """Load libcfdgpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run cfd_nssolver_forhpc_gb300.build.build() first")
    L = C.CDLL(str(LIB_PATH))
    vp, dp, ip, i, d, sz = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int, C.c_double, C.c_size_t
    proto = {
        "cfd_abi_version": ([], i),
        "cfd_last_error": ([], C.c_char_p),
        "cfd_config_default": ([C.POINTER(CfdConfig), i, i, i], i),
        "cfd_create": ([C.POINTER(CfdConfig), C.POINTER(vp)], i),
        "cfd_destroy": ([vp], i),
        "cfd_sync": ([vp], i),
        "cfd_grid_uniform": ([vp], i),
        "cfd_set_metrics": ([vp] + [dp] * 9, i),
        "cfd_upload": ([vp, i, dp, sz], i),
        "cfd_download": ([vp, i, dp, sz], i),
        "cfd_field_count": ([vp, i], sz),
        "cfd_host_register": ([vp, sz], i),
        "cfd_host_mapped": ([vp], i),
        "cfd_host_mapped_range": ([vp, sz], i),
        "cfd_set_test_limits": ([vp, i, C.c_longlong], i),
        "cfd_set_step_divergence_check": ([vp, i], i),
        "cfd_set_clock": ([vp, C.c_longlong, d], i),
        "cfd_get_clock": ([vp, C.POINTER(C.c_longlong), dp], i),
        "cfd_step_divergence": ([vp, dp], i),
        "cfd_host_unregister": ([vp], i),
        "cfd_init_uniform": ([vp, d, d, d], i),
        "cfd_start": ([vp], i),
        "cfd_convection_diffusion": ([vp, i, i], i),
        "cfd_add_source": ([vp, i], i),
        "cfd_accumulate_source": ([vp], i),
        "cfd_clear_source": ([vp], i),
        "cfd_create_b": ([vp, i, dp], i),
        "cfd_bicgstab": ([vp, ip, dp], i),
        "cfd_apply_operator": ([vp], i),
        "cfd_pressure_transform": ([vp], i),
        "cfd_sor": ([vp, i, ip, dp], i),
        "cfd_update_uf": ([vp, i, i], i),
        "cfd_cdcl": ([vp, dp, dp], i),
        "cfd_bc_main": ([vp, i], i),
        "cfd_bc_copy": ([vp, i, i], i),
        "cfd_copy_velocity": ([vp, i, i], i),
        "cfd_sync_periodic_z": ([vp, i], i),
        "cfd_eta_cylinder_z": ([vp, d, d, d, i], i),
        "cfd_step": ([vp, C.POINTER(CfdStepInfo)], i),
        "cfd_div_inf": ([vp, i, dp], i),
        "cfd_div_projected": ([vp, i, dp, dp], i),
        "cfd_stream": ([vp, C.POINTER(vp)], i),
        "cfd_launch_count": ([vp, C.POINTER(C.c_longlong)], i),
        "cfd_cdcl_noalloc": ([i, i, i, d, vp, vp, vp, vp, dp, dp, vp], i),
        "cfd_time_kernels": ([vp, i, dp, i], i),
        "cfd_set_inflow_profile": ([vp, dp, sz], i),
        "cfd_adj_enable": ([vp, i], i),
        "cfd_adj_zero": ([vp], i),
        "cfd_adj_field_count": ([vp, i], sz),
        "cfd_adj_upload": ([vp, i, dp, sz], i),
        "cfd_adj_download": ([vp, i, dp, sz], i),
        "cfd_adj_convection_diffusion": ([vp, i], i),
        "cfd_adj_update_uf": ([vp, i, d, d], i),
        "cfd_adj_create_b": ([vp], i),
        "cfd_adj_pressure_solve": ([vp, ip, dp], i),
        "cfd_adj_add_source": ([vp], i),
        "cfd_adj_bc_main": ([vp], i),
        "cfd_adj_bc_copy": ([vp], i),
        "cfd_step_record": ([vp, i, C.POINTER(CfdStepInfo)], i),
        "cfd_adj_step": ([vp, i, d, d, C.POINTER(CfdAdjStepInfo)], i),
        "cfd_adj_finish": ([vp], i),
        "cfd_checkpoint_alloc": ([vp, i], i),
        "cfd_checkpoint_save": ([vp, i], i),
        "cfd_checkpoint_load": ([vp, i], i),
        "cfd_adj_forward": ([vp, C.POINTER(CfdAdjRunConfig), C.POINTER(CfdAdjRunResult)], i),
        "cfd_adj_reverse": ([vp, C.POINTER(CfdAdjRunResult)], i),
        "cfd_adj_mean_drag": ([vp, C.POINTER(CfdAdjRunConfig), C.POINTER(CfdAdjRunResult)], i),
        "cfd_cfl": ([vp, i, C.POINTER(CfdCflInfo)], i),
        "cfd_smagorinsky": ([vp, i], i),
        "cfd_sml_default": ([C.POINTER(CfdSmlConfig)], i),
        "cfd_sml_metrics": ([i, i, i, d, d, d, C.POINTER(CfdSmlConfig)] + [dp] * 9, i),
        "cfd_grid_sml": ([vp, C.POINTER(CfdSmlConfig)], i),
        "cfd_steady_max": ([vp, i, i, dp], i),
        "cfd_write_plot3d_x": ([vp, C.c_char_p], i),
        "cfd_write_plot3d_q": ([vp, i, C.c_char_p], i),
        "cfd_plot3d_q_host": ([C.c_char_p, i, i, i, d, d, dp, dp, dp, dp, dp], i),
        "cfd_read_plot3d_q": ([C.c_char_p, i, i, i, dp, dp, dp, dp, dp, dp], i),
        "cfd_save_state": ([vp, C.c_char_p], i),
        "cfd_load_state": ([vp, C.c_char_p], i),
    }
    for name, (args, res) in proto.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(status: int, allow=()) -> int:
    if status != CFD_OK and status not in allow:
        msg = lib().cfd_last_error()
        raise CfdError(status, msg.decode() if msg else "")
    return status


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def exported_symbols() -> list[str]:
    """Names declared in include/cfdgpu.h (for the load/export test)."""
    hdr = Path(__file__).resolve().parent.parent / "include" / "cfdgpu.h"
    import re
    return sorted(set(re.findall(r"\b(cfd_[a-z0-9_]+)\s*\(", hdr.read_text())))


def library_path() -> str:
    return os.fspath(LIB_PATH)
