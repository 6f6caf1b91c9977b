"""Plot3D files and the state file written from a device context (GPU).

The host writer is pinned byte for byte against the reference's own writer
on the CPU (test_plot3d_host.py); here the context's GPU writer must give the
same bytes as the host writer fed with the downloaded fields, the grid file
must hold the cell centres of the uniform grid, and a run restarted from a
state file must continue bitwise like the run that wrote it."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation, plot3d_q_host

pytestmark = pytest.mark.gpu


def _run(w, steps, **kw):
    S = Simulation(w, **kw)
    S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
    hist = [S.step() for _ in range(steps)]
    return S, hist


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_q_file_from_device_equals_host_writer(tmp_path, prec):
    w = WORKLOADS["g2"]
    S, _ = _run(w, 3, tol=1e-8, precision=prec)
    with S:
        dev = tmp_path / "dev.q"
        S.OutputPLOT3D_Qfile(dev, S.T0)
        f = [S.download(k) for k in ("P", "U0", "V0", "W0", "ETA")]
        host = tmp_path / "host.q"
        plot3d_q_host(host, w, w.re, 3 * w.dt, *f)
    assert dev.read_bytes() == host.read_bytes()


def test_x_file_holds_cell_centres(tmp_path):
    w = WORKLOADS["g2"]
    with Simulation(w) as S:
        S.grid_uniform()
        path = tmp_path / "g.x"
        S.OutputPlot3D_Xfile(path)
    raw = path.read_bytes()
    nb, nx, ny, nz = struct.unpack("4i", raw[:16])
    assert (nb, nx, ny, nz) == (1, w.nxc, w.nyc, w.nzc)
    xyz = np.frombuffer(raw[16:], dtype=np.float32).reshape(3, nz, ny, nx)
    for a, (n, L) in enumerate(((w.nxc, w.lx), (w.nyc, w.ly), (w.nzc, w.lz))):
        c = ((np.arange(n) + 0.5) * (L / n)).astype(np.float32)
        got = np.moveaxis(xyz[a], (0, 1, 2), (2, 1, 0))  # (nx, ny, nz)
        line = got[:, 0, 0] if a == 0 else got[0, :, 0] if a == 1 else got[0, 0, :]
        np.testing.assert_allclose(line, c, rtol=2e-7, atol=1e-6)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_state_file_restart_is_bitwise(tmp_path, prec):
    w = WORKLOADS["g1"]
    prof = 1.0 + 0.02 * np.sin(np.arange(w.nyc))
    S, _ = _run(w, 0, tol=1e-10, precision=prec)
    with S:
        S.set_inflow_profile(prof)
        for _ in range(3):
            S.step()
        state = tmp_path / "s.bin"
        S.save_state(state)
        a = [S.step()["cd"] for _ in range(3)]
        ua = S.download("U0")
    with Simulation(w, tol=1e-10, precision=prec) as R:
        R.grid_uniform()
        R.load_state(state)
        b = [R.step()["cd"] for _ in range(3)]
        ub = R.download("U0")
    assert a == b
    np.testing.assert_array_equal(ua, ub)
