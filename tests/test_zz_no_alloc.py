"""cfd_cdcl_noalloc against cfd_cdcl (GPU).

cfd_cdcl_noalloc computes the drag and lift coefficients without allocating
any device memory, for callers that cannot: an application whose own memory
pool owns the GPU and forbids allocations outside it, or a time-critical loop
that cannot afford the device-wide synchronisation a cudaMalloc may cause.
Its only scratch is a file-scope device array shared by every call, so this
test checks two calls in a row (the second must not see the first's partial
sums) against the context-based cfd_cdcl, which allocates its scratch in
cfd_create.  The input arrays here come from PyTorch's allocator: the caller
owns its memory, the entry point adds none.

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


@pytest.mark.parametrize("name", ["g1", "c1"])
def test_noalloc_cdcl_matches_cfd_cdcl_twice(name):
    import torch

    w = WORKLOADS[name]
    n = w.n_cells
    dev = torch.device("cuda", 0)
    widths = [torch.from_numpy(a).to(dev) for a in _uniform_widths(w)]
    stream = torch.cuda.current_stream(dev)
    with Simulation(w) as S:
        S.grid_uniform()
        for call in range(2):
            f = seeded_field(3 * n, 500 + call, -10.0, 10.0)
            S.upload("F", f)
            cd_ref, cl_ref = S.Delay_IO_CD_CL()
            f_dev = torch.from_numpy(f).to(dev)
            stream.synchronize()
            cd, cl = C.c_double(), C.c_double()
            check(lib().cfd_cdcl_noalloc(w.nxc, w.nyc, w.nzc, w.lz, widths[0].data_ptr(),
                                         widths[1].data_ptr(), widths[2].data_ptr(), f_dev.data_ptr(),
                                         C.byref(cd), C.byref(cl), C.c_void_p(stream.cuda_stream)))
            assert cd.value == pytest.approx(cd_ref, rel=CDCL_RTOL, abs=1e-12), call
            assert cl.value == pytest.approx(cl_ref, rel=CDCL_RTOL, abs=1e-12), call


def test_noalloc_rejects_grids_beyond_its_scratch():
    """Sizes above CFD_NOALLOC_MAX_CELLS are refused before any device work
    (the pointers below are never dereferenced)."""
    cd, cl = C.c_double(), C.c_double()
    dummy = C.c_void_p(16)
    st = lib().cfd_cdcl_noalloc(1024, 1024, 257, 1.0, dummy, dummy, dummy, dummy, C.byref(cd),
                                C.byref(cl), None)
    assert st == -1
    assert "scratch limit" in lib().cfd_last_error().decode()
