"""Strouhal number of the cylinder wake.  The reference only logs Cd and Cl
(RUN_CPU_PC_METHOD.hpp:416-435); the shedding frequency is derived here from
the lift history.

    python -m cfd_nssolver_forhpc_gb300.strouhal --workload c1 --time 60 --precision mixed

runs the cylinder workload for the given number of time units, records Cl
every step and prints one JSON line: St from the mean interval between upward
zero crossings of Cl - mean(Cl) (with hysteresis) over the window after the transient, the
peak of the windowed spectrum of the same samples as a cross-check, the
spread of the periods and the mean Cd.  St = f D / U with D = 2 radius and U
the inflow velocity.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def strouhal(t, cl, diameter: float = 1.0, velocity: float = 1.0, settle: float = 0.5,
             min_periods: int = 3) -> dict:
    """Shedding frequency of a lift history.  `settle` is the fraction of the
    run treated as transient; at least `min_periods` full periods must remain
    in the window, else st is None with the reason."""
    t = np.asarray(t, dtype=np.float64)
    cl = np.asarray(cl, dtype=np.float64)
    if t.size < 8 or t.size != cl.size:
        return {"st": None, "reason": "too few samples"}
    w = t >= t[0] + settle * (t[-1] - t[0])
    tw, x = t[w], cl[w] - cl[w].mean()
    # upward zero crossings with hysteresis: a crossing counts only after the
    # signal has been below -h (h a tenth of the window's amplitude), so noise
    # around zero cannot add crossings
    h = 0.1 * np.abs(x).max()
    tcs, armed = [], False
    for i in range(x.size - 1):
        if x[i] < -h:
            armed = True
        if armed and x[i] < 0.0 <= x[i + 1]:
            tcs.append(tw[i] + (tw[i + 1] - tw[i]) * (-x[i]) / (x[i + 1] - x[i]))
            armed = False
    tc = np.asarray(tcs)
    if tc.size < min_periods + 1:
        return {"st": None, "reason": f"{max(tc.size - 1, 0)} periods in the window, {min_periods} needed"}
    periods = np.diff(tc)
    f = 1.0 / periods.mean()
    # windowed spectrum of the same samples (uniform step), peak refined by a parabola
    dt = float(np.median(np.diff(tw)))
    spec = np.abs(np.fft.rfft(x * np.hanning(x.size)))
    freqs = np.fft.rfftfreq(x.size, dt)
    k = int(np.argmax(spec[1:])) + 1
    if 1 <= k < spec.size - 1:
        a, b, c = np.log(spec[k - 1:k + 2] + 1e-300)
        shift = 0.5 * (a - c) / (a - 2 * b + c) if (a - 2 * b + c) != 0 else 0.0
    else:
        shift = 0.0
    f_fft = (k + shift) * (freqs[1] - freqs[0])
    scale = diameter / velocity
    return {"st": f * scale, "st_fft": f_fft * scale, "periods": int(periods.size),
            "period_spread": float(periods.std() / periods.mean()), "window_start": float(tw[0]),
            "cl_amplitude": float(0.5 * (x.max() - x.min()))}


def _run(S, steps: int, hist: dict) -> float:
    """steps steps of S, recording time, Cd and Cl; returns wall seconds."""
    t0 = time.perf_counter()
    for _ in range(steps):
        h = S.step()
        hist["t"].append(h["time"])
        hist["cd"].append(h["cd"])
        hist["cl"].append(h["cl"])
    return time.perf_counter() - t0


def _summary(hist: dict, w, settle: float, wall: float) -> dict:
    est = strouhal(hist["t"], hist["cl"], diameter=2.0 * w.radius, velocity=w.bc_dir[0][0], settle=settle)
    cd = np.asarray(hist["cd"])
    start = int(settle * cd.size)
    return {"steps": len(hist["t"]), "wall_s": round(wall, 2), "cd_mean": float(cd[start:].mean()), **est}


def main(argv=None):
    from . import capi
    from .configs import WORKLOADS
    from .initial import initial_velocity
    from .simulation import Simulation

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c1")
    ap.add_argument("--time", type=float, default=60.0, help="time units to run")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--solver", default="spe", choices=["spe", "ell", "sor"])
    ap.add_argument("--tol", type=float, default=None)
    ap.add_argument("--settle", type=float, default=0.5, help="fraction of the run treated as transient")
    ap.add_argument("--compare", type=float, default=0.0,
                    help="after the run, continue it for this many time units in both precisions from "
                         "the same state and compare the shedding of the two continuations")
    ap.add_argument("--history", default=None, help="write the Cd/Cl histories to this .npz")
    a = ap.parse_args(argv)
    w = WORKLOADS[a.workload]
    solver = {"spe": capi.SOLVER_BICG_SPE, "ell": capi.SOLVER_BICG_ELL, "sor": capi.SOLVER_SOR_RB}[a.solver]
    prec = {"mixed": capi.PREC_MIXED, "fp64": capi.PREC_FP64}
    tol = w.tol if a.tol is None else a.tol
    out = {"workload": a.workload, "solver": a.solver, "tol": tol, "dt": w.dt}
    hists = {}
    with Simulation(w, solver=solver, precision=prec[a.precision], tol=tol) as S:
        S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
        h = {"t": [], "cd": [], "cl": []}
        wall = _run(S, int(round(a.time / w.dt)), h)
        hists["run"] = h
        out["run"] = {"precision": a.precision, "time_units": a.time, **_summary(h, w, a.settle, wall)}
        state = S.state() if a.compare > 0 else None
    if state is not None:
        # both continuations start from the same fields and clock
        steps = int(round(a.compare / w.dt))
        for name in ("mixed", "fp64"):
            with Simulation(w, solver=solver, precision=prec[name], tol=tol,
                            maxit=5000 if name == "mixed" else 50000) as S:
                S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
                S.restore(state)
                h = {"t": [], "cd": [], "cl": []}
                wall = _run(S, steps, h)
                hists[name] = h
                out[name] = {"time_units": a.compare, **_summary(h, w, 0.0, wall)}
        m, f = out["mixed"], out["fp64"]
        if m.get("st") and f.get("st"):
            out["st_rel_diff_mixed_vs_fp64"] = abs(m["st"] / f["st"] - 1.0)
        out["cd_mean_rel_diff_mixed_vs_fp64"] = abs(m["cd_mean"] / f["cd_mean"] - 1.0)
    if a.history:
        np.savez_compressed(a.history, **{f"{k}_{q}": np.asarray(v[q]) for k, v in hists.items() for q in v})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
