"""cfd_cdcl_noalloc against cfd_cdcl (GPU).

cfd_cdcl_noalloc computes the drag and lift coefficients without allocating
any device memory, for callers that cannot: an application whose own memory
pool owns the GPU and forbids allocations outside it, or a time-critical loop
that cannot afford the device-wide synchronisation a cudaMalloc may cause.
Its only scratch is a file-scope device array shared by every call, so this
test checks two calls in a row (the second must not see the first's partial
sums) against the context-based cfd_cdcl, which allocates its scratch in
cfd_create.  The input arrays here come from PyTorch's allocator: the caller
owns its memory, the entry point adds none, which the free device memory
before and after a call shows.

This file is collected last so that a run stopping at the first failure has
run every other test already; it does not depend on them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.capi import check, lib
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import seeded_field
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu

# the tolerance the drag/lift comparisons of the other GPU tests use
CDCL_RTOL = 1e-12


def _uniform_widths(w):
    """grid::init_uniform cell widths (structureGrid.hpp:411-437)."""
    return [np.full(n + 4, L / (n + 4 - 4.0)) for n, L in ((w.nxc, w.lx), (w.nyc, w.ly), (w.nzc, w.lz))]


def _random_widths(w, seed):
    """Positive, different widths on every axis (a swapped axis would show)."""
    return [0.5 + seeded_field(n + 4, seed + a, 0.0, 1.0) for a, n in enumerate((w.nxc, w.nyc, w.nzc))]


def _metrics(widths):
    """cfd_set_metrics arrays for ghosted cell widths: nodes as cumulative
    sums, staggered widths as the mean of neighbouring cells."""
    out = {}
    for name, d in zip("xyz", widths):
        out[name.upper()] = np.concatenate([[0.0], np.cumsum(d)])
        out["D" + name] = d
        out["D" + name + "s"] = np.concatenate([0.5 * (d[:-1] + d[1:]), d[-1:]])
    return out


def _noalloc(w, widths_dev, f_dev, stream):
    cd, cl = C.c_double(), C.c_double()
    check(lib().cfd_cdcl_noalloc(w.nxc, w.nyc, w.nzc, w.lz, widths_dev[0].data_ptr(), widths_dev[1].data_ptr(),
                                 widths_dev[2].data_ptr(), f_dev.data_ptr(), C.byref(cd), C.byref(cl),
                                 C.c_void_p(stream.cuda_stream)))
    return cd.value, cl.value


@pytest.mark.parametrize("name,widths", [("g1", "uniform"), ("c1", "uniform"), ("g1", "random"),
                                         ("c1", "random")])
def test_noalloc_cdcl_matches_cfd_cdcl_twice(name, widths):
    import torch

    w = WORKLOADS[name]
    n = w.n_cells
    dev = torch.device("cuda", 0)
    host_widths = _uniform_widths(w) if widths == "uniform" else _random_widths(w, 700)
    widths_dev = [torch.from_numpy(a).to(dev) for a in host_widths]
    stream = torch.cuda.current_stream(dev)
    with Simulation(w) as S:
        if widths == "uniform":
            S.grid_uniform()
        else:
            S.set_metrics(_metrics(host_widths))
        fs = [seeded_field(3 * n, 500 + call, -10.0, 10.0) for call in range(2)]
        f_devs = [torch.from_numpy(f).to(dev) for f in fs]
        torch.cuda.synchronize()
        for call in range(2):
            S.upload("F", fs[call])
            cd_ref, cl_ref = S.Delay_IO_CD_CL()
            free0 = torch.cuda.mem_get_info(dev)[0]
            cd, cl = _noalloc(w, widths_dev, f_devs[call], stream)
            free1 = torch.cuda.mem_get_info(dev)[0]
            assert cd == pytest.approx(cd_ref, rel=CDCL_RTOL, abs=1e-12), call
            assert cl == pytest.approx(cl_ref, rel=CDCL_RTOL, abs=1e-12), call
            if call == 1:
                # the first call may load the library's device code on this
                # device (and with it the scratch array); later calls take
                # no device memory at all
                assert free1 == free0


def test_noalloc_rejects_grids_beyond_its_scratch():
    """Sizes above CFD_NOALLOC_MAX_CELLS are refused before any device work
    (the pointers below are never dereferenced)."""
    cd, cl = C.c_double(), C.c_double()
    dummy = C.c_void_p(16)
    st = lib().cfd_cdcl_noalloc(1024, 1024, 257, 1.0, dummy, dummy, dummy, dummy, C.byref(cd),
                                C.byref(cl), None)
    assert st == -1
    assert "scratch limit" in lib().cfd_last_error().decode()
