"""Plot3D files on the host (CPU): the library's q writer and reader against
the reference's own OutputPLOT3D_Qfile and QfileRead (io/Plot3D/qfile.hpp:7,
qfileRead.hpp:6), compiled from the reference headers by oracle/build_ref.py.
The writer must produce the same bytes; the reader the same ghosted arrays.
Skipped where the reference sources are unavailable."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.build import build
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import seeded_field
from cfd_nssolver_forhpc_gb300.simulation import QfileRead, plot3d_q_host


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref
    from oracle.oracle import RefHarness
    w = WORKLOADS["g1"]
    try:
        build_ref.build(w.name)
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference sources unavailable: {e}")
    build()
    R = RefHarness(w.name, build=False)
    R.set_threads(1)
    R.setup(w.dt, w.re, 1e-8, True)
    return w, R


def fields(w, seed):
    ng = w.n_ghosted
    return [seeded_field(ng, seed + k, lo, hi) for k, (lo, hi) in
            enumerate([(-2.0, 2.0), (0.5, 1.5), (-0.3, 0.3), (-0.3, 0.3), (0.0, 1.0)])]


def test_q_writer_bytes_equal_reference(ref, tmp_path):
    w, R = ref
    f = fields(w, 40)
    theirs = R.plot3d_q(tmp_path, 7, 0.375, *f)
    ours = tmp_path / "ours.q"
    plot3d_q_host(ours, w, w.re, 0.375, *f)
    a, b = theirs.read_bytes(), ours.read_bytes()
    assert len(a) == 32 + 5 * 4 * w.n_cells
    assert a == b


def test_q_reader_equals_reference_reader(ref, tmp_path):
    w, R = ref
    f = fields(w, 50)
    path = R.plot3d_q(tmp_path, 3, 1.25, *f)
    cond_r, *theirs = R.plot3d_read(path)
    cond_o, *ours = QfileRead(path, w)
    assert cond_o == pytest.approx(cond_r, abs=0)
    for a, b in zip(theirs, ours):
        np.testing.assert_array_equal(a, b)


def test_q_roundtrip_keeps_centred_values(ref, tmp_path):
    """Writing then reading keeps p and eta at interior cells to float
    rounding and rebuilds faces from the centred velocities."""
    w, _ = ref
    f = fields(w, 60)
    path = tmp_path / "rt.q"
    plot3d_q_host(path, w, w.re, 2.0, *f)
    cond, p, u, v, ww, eta = QfileRead(path, w)
    assert cond == (0.0, 0.0, pytest.approx(w.re), 2.0)
    shape = (w.nxc + 4, w.nyc + 4, w.nzc + 4)
    inner = (slice(2, -2),) * 3
    for got, want in ((p, f[0]), (eta, f[4])):
        np.testing.assert_allclose(got.reshape(shape)[inner], want.reshape(shape)[inner].astype(np.float32),
                                   rtol=0, atol=0)
    # u face i = average of the centred values of cells i and i+1 (float sum)
    uc = 0.5 * (f[1].reshape(shape)[1:-3, 2:-2, 2:-2] + f[1].reshape(shape)[2:-2, 2:-2, 2:-2])
    uc = uc.astype(np.float32)
    want = uc.astype(np.float64)
    want[:-1] = (uc[:-1] + uc[1:]).astype(np.float64) / 2.0
    np.testing.assert_allclose(u.reshape(shape)[inner], want, rtol=0, atol=0)


def test_reader_rejects_grid_mismatch(ref, tmp_path):
    w, _ = ref
    f = fields(w, 70)
    path = tmp_path / "m.q"
    plot3d_q_host(path, w, w.re, 0.0, *f)
    from cfd_nssolver_forhpc_gb300.capi import CfdError
    with pytest.raises(CfdError, match="header does not match"):
        QfileRead(path, w.with_(nxc=w.nxc + 1))
