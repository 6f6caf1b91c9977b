"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, exports
every entry point declared in include/cfdgpu.h, and validates arguments on
the host before touching the GPU (no compute call is made here)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.build import build

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def L():
    build()
    return capi.lib()


def test_header_symbols_exported(L):
    names = capi.exported_symbols()
    assert len(names) >= 30
    nm = subprocess.run(["nm", "-D", "--defined-only", str(capi.LIB_PATH)], capture_output=True,
                        text=True, check=True).stdout
    exported = set(re.findall(r"\bT (cfd_[a-z0-9_]+)", nm))
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared in cfdgpu.h but not exported: {missing}"
    for n in names:
        assert hasattr(L, n)


def test_abi_version(L):
    assert L.cfd_abi_version() == 1


def test_config_defaults_follow_reference(L):
    cfg = capi.CfdConfig()
    assert L.cfd_config_default(C.byref(cfg), 128, 64, 8) == 0
    assert (cfg.nx_cal, cfg.ny_cal, cfg.nz_cal) == (128, 64, 8)
    assert cfg.p_criteria == 1e-3        # simuClass.hpp:74
    assert cfg.p_iter_max == 5000        # bicgstabRe2.hpp:57
    assert cfg.p_sor_omega == 1.8        # simuClass.hpp:78
    assert cfg.p_sor_iter_max == 5000    # simuClass.hpp:80
    assert cfg.re == 40.0 and cfg.dt == 0.002  # src/CFD_MX.cpp:37-39
    assert cfg.method == capi.METHOD_PC and cfg.solver == capi.SOLVER_BICG_SPE
    assert L.cfd_config_default(None, 1, 1, 1) == -1


def _cfg(L, **kw):
    cfg = capi.CfdConfig()
    L.cfd_config_default(C.byref(cfg), 16, 12, 6)
    cfg.lx, cfg.ly, cfg.lz = 4.0, 3.0, 0.75
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


@pytest.mark.parametrize("kw,needle", [
    (dict(nx_cal=3), "at least 4"),
    (dict(dt=0.0), "dt"),
    (dict(re=-1.0), "dt and re"),
    (dict(lz=0.0), "lengths"),
    (dict(p_criteria=0.0), "tolerance"),
    (dict(solver=2), "unknown solver"),
    (dict(method=7), "unknown method"),
    (dict(precision=5), "unknown precision"),
    (dict(check_every=0), "check_every"),
    (dict(precision=1, inner_tol=2.0), "inner_tol"),
    (dict(conv_outflow_uc=-1.0), "conv_outflow_uc"),
    (dict(conv_outflow_uc=float("nan")), "conv_outflow_uc"),
    (dict(conv_outflow_uc=float("inf")), "conv_outflow_uc"),
])
def test_create_rejects_bad_config(L, kw, needle):
    cfg = _cfg(L, **kw)
    h = C.c_void_p()
    st = L.cfd_create(C.byref(cfg), C.byref(h))
    assert st == -1
    assert not h.value
    assert needle in L.cfd_last_error().decode()


def test_null_arguments_rejected(L):
    h = C.c_void_p()
    assert L.cfd_create(None, C.byref(h)) == -1
    assert L.cfd_step(None, None) == -1
    assert L.cfd_upload(None, 0, None, 0) == -1
    assert L.cfd_destroy(None) == 0
    assert L.cfd_host_register(None, 0) == -1
    assert L.cfd_host_mapped(None) == 0


def test_build_is_sm103a_only():
    """The library is compiled for sm_103a and nothing else."""
    from cfd_nssolver_forhpc_gb300.build import ARCH, _flags
    assert ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-lineinfo" in _flags()


def test_kernel_timing_names_follow_the_header_enum():
    """capi.KERNELS names the slots of cfd_time_kernels in the order of the
    CFD_KERNEL_* enum of include/cfdgpu.h."""
    import re
    from pathlib import Path

    from cfd_nssolver_forhpc_gb300 import capi
    hdr = (Path(__file__).resolve().parent.parent / "include" / "cfdgpu.h").read_text()
    body = hdr[hdr.index("CFD_KERNEL_BICG_AP"):hdr.index("CFD_KERNEL_COUNT")]
    names = re.findall(r"CFD_KERNEL_([A-Z0-9_]+)", body)
    assert [n.lower() for n in names] == capi.KERNELS
