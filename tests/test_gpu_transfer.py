"""Host transfers through the C ABI: an upload from a host buffer the GPU can
address (registered and mapped) is read by one kernel over the host link,
other uploads and all downloads go through copies.  Both must move identical
bits, for FP32 velocity fields (mixed precision) and FP64 fields alike."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.capi import check, lib
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu


def _registered(n):
    a = np.empty(n)
    check(lib().cfd_host_register(a.ctypes.data_as(C.c_void_p), a.nbytes))
    return a


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_registered_and_plain_transfers_move_identical_bits(precision):
    w = WORKLOADS["g1"]
    rng = np.random.default_rng(3)
    with Simulation(w, precision=precision) as S:
        S.grid_uniform()
        for name in ("U0", "V0", "W0", "P", "X"):
            n = S.count(name)
            src = rng.standard_normal(n)
            reg = _registered(n)
            try:
                assert lib().cfd_host_mapped(reg.ctypes.data_as(C.c_void_p)) == 1
                # upload from a registered buffer, download into a plain one
                reg[:] = src
                S.upload(name, reg)
                plain = np.empty(n)
                S.download(name, plain)
                # upload from a plain buffer, download into a registered one
                S.upload(name, src)
                reg[:] = np.nan
                S.download(name, reg)
                np.testing.assert_array_equal(reg, plain)
                if precision == capi.PREC_MIXED and name in ("U0", "V0", "W0"):
                    np.testing.assert_array_equal(plain, src.astype(np.float32).astype(np.float64))
                else:
                    np.testing.assert_array_equal(plain, src)
            finally:
                check(lib().cfd_host_unregister(reg.ctypes.data_as(C.c_void_p)))


def test_unaligned_registered_buffer_falls_back_to_copies():
    """A registered buffer that does not start on a 16-byte boundary takes the
    copy path and still moves the right data."""
    w = WORKLOADS["g1"]
    with Simulation(w, precision=capi.PREC_MIXED) as S:
        S.grid_uniform()
        n = S.count("U0")
        raw = np.empty(n + 2)
        check(lib().cfd_host_register(raw.ctypes.data_as(C.c_void_p), raw.nbytes))
        try:
            view = raw[1:n + 1]  # 8-byte offset
            src = np.linspace(-1.0, 1.0, n)
            view[:] = src
            S.upload("U0", view)
            out = np.empty(n)
            S.download("U0", out)
            np.testing.assert_array_equal(out, src.astype(np.float32).astype(np.float64))
        finally:
            check(lib().cfd_host_unregister(raw.ctypes.data_as(C.c_void_p)))
