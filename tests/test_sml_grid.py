"""The stretched SML grid (host): the library's generator against the
reference's own grid::init_nonuniform_SML (structureGrid.hpp:326-405),
compiled from the reference headers with Gridder = "non_uniform-SML";
every node coordinate and width must be bitwise equal.  Skipped where the
reference sources are unavailable."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.build import build
from cfd_nssolver_forhpc_gb300.capi import CfdError
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.simulation import sml_default, sml_metrics


def test_sml_metrics_bitwise_equal_reference():
    from oracle import build_ref
    from oracle.oracle import RefHarness
    w = WORKLOADS["s1"]
    try:
        build_ref.build(w.name, gridder="non_uniform-SML")
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference sources unavailable: {e}")
    build()
    R = RefHarness(w.name, build=False)
    R.setup(w.dt, w.re, 1e-8, False)
    ref = R.grid_metrics()
    ours = sml_metrics(w)
    for k in ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs"):
        np.testing.assert_array_equal(ours[k], ref[k], err_msg=k)
    # the grid is stretched: fine cells in the middle of x and y
    assert ours["Dx"].max() / ours["Dx"].min() > 1.5
    assert np.ptp(ours["Dz"]) == 0.0


def test_sml_rejects_odd_split():
    build()
    w = WORKLOADS["s1"].with_(nxc=121)
    with pytest.raises(CfdError, match="even"):
        sml_metrics(w)
    cfg = sml_default()
    cfg.fine_cells[0] = 0
    m = sml_metrics(w, cfg)
    assert np.allclose(m["Dx"], w.lx / w.nxc)
