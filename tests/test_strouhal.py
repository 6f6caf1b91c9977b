"""The Strouhal estimator on synthetic lift histories (no GPU): a shedding
signal after a decaying transient, with noise and a slow drift, and a run too
short to hold enough periods."""
from __future__ import annotations

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300.strouhal import strouhal


@pytest.mark.parametrize("f", [0.12, 0.165, 0.2])
def test_recovers_the_shedding_frequency(f):
    rng = np.random.default_rng(2)
    dt = 2e-3
    t = np.arange(1, 30001) * dt  # 60 time units, ~10 periods
    transient = 2.0 * np.exp(-t / 3.0)
    cl = 0.3 * np.sin(2 * np.pi * f * t + 0.4) + transient + 1e-3 * t / 60 + 1e-3 * rng.standard_normal(t.size)
    est = strouhal(t, cl, diameter=1.0, velocity=1.0)
    assert est["st"] == pytest.approx(f, rel=2e-3)
    assert est["st_fft"] == pytest.approx(f, rel=2e-2)
    assert est["periods"] >= 3
    assert est["period_spread"] < 0.01


def test_scales_with_diameter_and_velocity():
    t = np.arange(1, 30001) * 2e-3
    cl = np.sin(2 * np.pi * 0.2 * t)
    est = strouhal(t, cl, diameter=2.0, velocity=4.0)
    assert est["st"] == pytest.approx(0.2 * 2.0 / 4.0, rel=1e-3)


def test_too_short_a_run_gives_no_estimate():
    t = np.arange(1, 1001) * 2e-3  # 2 time units
    est = strouhal(t, np.sin(2 * np.pi * 0.165 * t))
    assert est["st"] is None and "periods" in est["reason"]
