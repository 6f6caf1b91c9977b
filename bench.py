"""Benchmark of the GB300 time step: Mcell-steps/s of the predictor-corrector
step of the flow-past-a-cylinder workload at 512x256x32 (4.19 M cells),
Poisson solves to relative residual 1e-10.  The headline is the mixed-precision
step (FP32 fields and inner CG, FP64 defect correction); the FP64 step
(BiCGSTAB over the matrix-free Jacobi-scaled operator) is timed beside it and
ratio_mixed_vs_fp64 is their ratio at the same tolerance.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  A "step" is one iteration of the reference's main
loop (three predictor passes and the final pass, four Poisson solves).

* value      -- device time: K steps bracketed by CUDA events on the library's
                stream, inputs resident in HBM; the working set (~1.5 GB) is far
                larger than L2, so no flush is needed between steps.
* e2e        -- the same K steps through the C ABI with the state crossing the
                boundary every step: upload of T0 (u, v, w) and p from pinned
                host buffers, the step, download of T0 and p.
* roofline   -- the dominant kernel (largest share of the step's device time),
                timed alone with CUDA events on the library stream; bytes are
                the algorithmic bytes of one launch.
* adjoint    -- gradient of the mean drag w.r.t. the inflow profile and eta on
                the 256x128x16 workload (bounded sample of steps): forward run
                with checkpoints, then recompute + reverse sweep; ratio =
                adjoint seconds / forward seconds, FP64 and mixed forward.
* cpu_baseline / --impl reference -- the reference's own CPU code for the step
                (oracle/_ref/<workload>/libref.so, its headers compiled from a
                patched copy), else the oracle's C restatement, on the host's
                cores; see the `sample` field for what was timed.

With --gpus N under torchrun each rank runs an independent replica (the step
is not sharded); value is the sum over ranks, time the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell-steps/s mixed vs FP64 on GPU at ||div u||<1e-10; adjoint/forward time ratio"
UNIT = "Mcell-steps/s"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
# FP64 FMA instructions per second of one GB300, measured with a register-
# resident DFMA loop (2 FP64 FMA per SM per clock)
FP64_PEAK_TOPS = 0.599

# Algorithmic bytes per row (compact cell) of one launch of each kernel, FP64
# fields (8 B); the FP32 inner kernels of the mixed path move half of the
# vector bytes (jp included).
KERNEL_BYTES_PER_ROW = {
    "bicg_ap": 4,   # read p1, r0, jp; write ap
    "bicg_s": 3,    # read r1, ap; write s
    "bicg_as": 3,   # read s, jp; write as
    "bicg_xr": 7,   # read x, p1, s, as, r0; write x, r1
    "bicg_p": 4,    # read r1, p1, ap; write p1
}
KERNEL_BYTES_PER_CELL_FLOW = {
    "convdiff": 6,   # read u, v, w; write u*, v*, w*
    "update_uf": 13,  # read u*, v*, w*, p, eta; write u, v, w, f (3)
    "rhs": 6,        # read u*, v*, w*, jp; write b (+ mean pass reads jp, b, writes b)
}
# the fused predictor-corrector pass kernels: (field words, extra FP64 bytes)
# per cell; a word is the field type (FP32 in the mixed path)
KERNEL_BYTES_PASS = {
    "pass": (9, 16),         # read C (3), src (3); write T1 (3); read jp, write b (FP64 or a float pair)
    "update_pass": (13, 8),  # read T1 (3), eta; write T3 (3); src += dt f (read, write 3 each); read p
}
# one red-black SOR sweep (both colours) per cell: seven FP64 coefficients
# and the right-hand side read, p read and written once
SOR_BYTES_PER_CELL = 80
# FP64 operations per cell of a sweep: six products and six sums of the
# neighbour term, the right-hand side, the scale, the change, its product
# with omega and the update
SOR_FP64_OPS_PER_CELL = 16
# the FP32 sweeps of the mixed path (two colour passes of the level-0
# smoother): per pass the correction read, half of it and half of the
# right-hand side written / read
SOR32_BYTES_PER_CELL = 16
SOR32_PER_BODY = 4 * 16  # FP32 sweeps per loop body (4 x check_every)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--solver", default="spe", choices=["spe", "ell", "sor"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="precision of the headline step (the other one is timed beside it)")
    ap.add_argument("--spinup", type=int, default=None,
                    help="untimed steps from the seeded start before the warm-up (past the impulsive-start "
                         "transient; the comparison legs start from the state they reach); default 60 for "
                         "the mixed step, 0 for the FP64 one (seconds a step)")
    ap.add_argument("--inner-tol", type=float, default=1e-3,
                    help="relative tolerance of each FP32 inner solve of the mixed defect correction")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the other-precision comparison leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward ratio leg")
    ap.add_argument("--adj-workload", default="c4")
    ap.add_argument("--adj-steps", type=int, default=20, help="steps of the bounded adjoint sample")
    ap.add_argument("--fp64-maxit", type=int, default=20000,
                    help="BiCGSTAB iteration cap per solve of the FP64 leg (the reference's is 5000; "
                         "at tolerance 1e-10 some of its solves need more)")
    ap.add_argument("--leg", default=None, choices=["c3", "c5"],
                    help="run one of the large-workload legs instead of the headline: c3 = mixed vs FP64 "
                         "at 1024x512x64 (bounded steps, per-field errors); c5 = memory plan and one "
                         "forward + adjoint segment at 1536x768x96")
    ap.add_argument("--leg-steps", type=int, default=3, help="steps of the large-workload leg")
    ap.add_argument("--cpu-worker", default=None, help=argparse.SUPPRESS)
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def whole_job_rate(n_cells: int, steps: int, world: int, seconds_max: float) -> float:
    """Mcell-steps/s of the whole job: every rank advances its own replica of
    n_cells by `steps`, the job takes as long as its slowest rank."""
    return n_cells * steps * world / seconds_max / 1e6


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(workload: str, kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    f = ROOT / "profiles" / "ncu_traffic.json"
    try:
        d = json.loads(f.read_text())
        return d[workload][kernel]["dram_bytes_per_launch"]
    except Exception:
        return None


# ---------------------------------------------------------------------------
def build_sim(args, w, precision):
    from cfd_nssolver_forhpc_gb300 import capi
    from cfd_nssolver_forhpc_gb300.initial import initial_velocity
    from cfd_nssolver_forhpc_gb300.simulation import Simulation
    solver = {"spe": capi.SOLVER_BICG_SPE, "ell": capi.SOLVER_BICG_ELL, "sor": capi.SOLVER_SOR_RB}[args.solver]
    prec = {"mixed": capi.PREC_MIXED, "fp64": capi.PREC_FP64, "fp64_dc": capi.PREC_FP64_DC}[precision]
    maxit = args.fp64_maxit if precision == "fp64" else 5000
    S = Simulation(w, solver=solver, precision=prec, tol=w.tol, check_every=16, maxit=maxit,
                   inner_tol=args.inner_tol)
    S.setup_cylinder(*initial_velocity(w.nxc, w.nyc, w.nzc))
    return S


def timed_steps(S, K, dist):
    """K steps bracketed by barrier + synchronize; CUDA events on the
    library's stream.  Returns (seconds, step infos)."""
    import torch
    stream = torch.cuda.ExternalStream(S.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    S.sync()
    n0 = S.launch_count()
    e0.record(stream)
    infos = [S.step(allow_noconv=True) for _ in range(K)]
    e1.record(stream)
    S.sync()
    torch.cuda.synchronize()
    dist.barrier()
    return e0.elapsed_time(e1) / 1e3, infos, S.launch_count() - n0


def e2e_steps(S, K, dist):
    """K steps through the C ABI with the state crossing the host boundary."""
    import ctypes as C

    import numpy as np
    import torch

    from cfd_nssolver_forhpc_gb300.capi import check, lib
    bufs = {k: np.empty(S.count(k)) for k in ("U0", "V0", "W0", "P")}
    for k, a in bufs.items():
        S.download(k, a)
        check(lib().cfd_host_register(a.ctypes.data_as(C.c_void_p), a.nbytes))
    stream = torch.cuda.ExternalStream(S.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    S.sync()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(K):
        for k, a in bufs.items():
            S.upload(k, a)
        S.step(allow_noconv=True)
        for k, a in bufs.items():
            S.download(k, a)
    e1.record(stream)
    S.sync()
    wall = time.perf_counter() - t0
    dist.barrier()
    for a in bufs.values():
        lib().cfd_host_unregister(a.ctypes.data_as(C.c_void_p))
    nbytes = sum(a.nbytes for a in bufs.values())
    return max(e0.elapsed_time(e1) / 1e3, 0.0), wall, nbytes


# FP32 kernels of the mixed-precision inner solve (bytes per row) and the
# FP64 residual of its defect correction
KERNEL_BYTES_MIXED = {
    "cg_pq": 16,       # read z (or h), p; write p', q (FP32)
    "cg_upd": 24,      # read e, p, h, q; write e, h (FP32; 1/P from the axis tables)
    "residual64": 28,  # read b, x, jp (FP64); write r (FP32)
    "mg_smooth": 8,    # one colour on the finest level: read x (all), b (half); write x (half)
    "mg_restrict": 8,  # read b, x of the finest level (coarse writes 1/8)
    "mg_prolong": 8,   # read and write x of the finest level
    "mg_upd": 24,      # read e, p, h, q; write e, h
    "mg_rho": 8,       # read h, z
}
MG_SWEEPS = 2  # smoothing sweeps per level before and after the coarse correction


def roofline(S, w, infos, precision, ms_step):
    """Dominant kernel by share of the step's device time (count per step x
    its CUDA-event time per launch / the measured ms per step), its achieved
    GB/s.  "other" is the rest of the step: the coarser multigrid levels,
    small kernels and launch gaps."""
    ms = S.time_kernels(reps=20)
    iters = sum(sum(i["iters"]) for i in infos) / len(infos)
    outer = sum(sum(i["outer"]) for i in infos) / len(infos)
    npass = 4
    if precision == "mixed" and "mg_smooth" in ms:
        # multigrid-preconditioned CG: one V-cycle per inner iteration and one
        # per inner solve (its start); per V-cycle 4 * sweeps colour passes,
        # one restriction and one prolongation on the finest level and the
        # coarse solve (the separable solve of the coarsest level)
        v = iters + outer
        counts = {"mg_smooth": 4 * MG_SWEEPS * v, "mg_restrict": v, "mg_prolong": v, "mg_coarse": v,
                  "cg_pq": iters, "mg_upd": iters, "mg_rho": v, "residual64": outer + npass}
        per_row = dict(KERNEL_BYTES_MIXED)
    elif precision == "mixed":
        counts = {"cg_pq": iters, "cg_upd": iters, "residual64": outer + npass}
        per_row = dict(KERNEL_BYTES_MIXED)
    else:
        counts = {k: iters for k in KERNEL_BYTES_PER_ROW}
        per_row = {k: v * 8 for k, v in KERNEL_BYTES_PER_ROW.items()}
    word = 4 if precision == "mixed" else 8
    per_row.update({k: v * word for k, v in KERNEL_BYTES_PER_CELL_FLOW.items()})
    if "pass" in ms:
        # fused predictor-corrector step: one convection-diffusion, then per
        # pass the pass kernel and the fused projection
        counts.update({"convdiff": 1, "pass": npass, "update_pass": npass})
        per_row.update({k: a * word + b for k, (a, b) in KERNEL_BYTES_PASS.items()})
    else:
        counts.update({"convdiff": npass, "update_uf": npass, "rhs": npass})
    if "sor_sweep" in ms:
        counts = {k: v for k, v in counts.items() if k in ("convdiff", "pass", "update_pass", "update_uf")}
        # sweeps per step: iterations + 1 per solve (the timed steps all solve)
        sweeps = [n + 1 for i in infos for n in i["iters"]]
        if "sor32_sweep" in ms:
            # mixed precision: one FP64 sweep per loop body of 4 x 16 FP32 sweeps
            fp64 = [-(-n // (SOR32_PER_BODY + 1)) for n in sweeps]
            counts["sor_sweep"] = sum(fp64) / len(infos)
            counts["sor32_sweep"] = (sum(sweeps) - sum(fp64)) / len(infos)
            per_row["sor32_sweep"] = SOR32_BYTES_PER_CELL
        else:
            counts["sor_sweep"] = sum(sweeps) / len(infos)
        per_row["sor_sweep"] = SOR_BYTES_PER_CELL
    shares = {k: ms[k] * counts[k] for k in ms if k in counts}
    total = ms_step if ms_step > 0 else (sum(shares.values()) or 1.0)
    top = max((k for k in shares if k in per_row), key=shares.get)
    bytes_launch = per_row[top] * w.n_cells
    peak, how = peaks()
    achieved = bytes_launch / (ms[top] * 1e-3) / 1e9
    out = {
        "kernel": top, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4), "peak_source": f"{how} hbm_gbs",
        "traffic": ncu_traffic(w.name, top),
        "algorithmic_bytes_per_launch": bytes_launch,
        "ms_per_launch": round(ms[top], 5),
        "share_of_step": round(shares[top] / total, 3),
        "kernels_ms": {k: round(v, 5) for k, v in ms.items()},
        "shares": {k: round(v / total, 3) for k, v in shares.items()},
    }
    out["shares"]["other"] = round(max(0.0, 1.0 - sum(shares.values()) / total), 3)
    if "mg_vcycle" in ms:
        out["mg_vcycle_ms"] = round(ms["mg_vcycle"], 5)
    if top == "mg_smooth":
        out["note"] = ("launch time from back-to-back launches on the finest level, whose x and b "
                       "(8 B/cell) stay in L2 between passes as they do inside the V-cycle; an ncu "
                       "capture with caches flushed gives the cold figure")
    if top == "sor_sweep":
        # the sweeps are bound by the FP64 pipe (one rounding per operation)
        rate = SOR_FP64_OPS_PER_CELL * w.n_cells / (ms[top] * 1e-3) / 1e12
        out["bound"] = "fp64"
        out["fp64_pipe"] = {"achieved_tops": round(rate, 4), "peak_tops": FP64_PEAK_TOPS,
                            "frac": round(rate / FP64_PEAK_TOPS, 3),
                            "peak_source": "register-resident DFMA loop on GB300 (0.599 T FMA/s)"}
    if precision != "mixed" and top != "sor_sweep":
        # the FP64 Krylov kernels are bound by the FP64 pipe: FP64 operations
        # per row (SpMV 7, each dot 1, updates as written) / measured DFMA rate
        fp64_ops = {"bicg_ap": 8, "bicg_s": 1, "bicg_as": 9, "bicg_xr": 6, "bicg_p": 2}
        if top in fp64_ops:
            rate = fp64_ops[top] * w.n_cells / (ms[top] * 1e-3) / 1e12
            out["fp64_pipe"] = {"achieved_tops": round(rate, 4), "peak_tops": FP64_PEAK_TOPS,
                                "frac": round(rate / FP64_PEAK_TOPS, 3),
                                "peak_source": "register-resident DFMA loop on GB300 (0.599 T FMA/s)"}
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the reference's own functions (or the oracle restatement)
def cpu_worker(spec: str):
    """Runs in a subprocess (its own OpenMP runtime and thread count)."""
    d = json.loads(spec)
    from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
    from cfd_nssolver_forhpc_gb300.initial import initial_velocity
    w = WORKLOADS[d["workload"]]
    solver = {"spe": 0, "ell": 1, "sor": 2}[d["solver"]]
    warm, steps = d["warmup"], d["steps"]
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    kind = None
    try:
        from oracle.oracle import RefHarness
        R = RefHarness(w.name, build=False, fast=True)
        flags = R.flags
        R.setup(w.dt, w.re, w.tol, True)
        R.pc_start(u0, v0, w0)
        kind = "reference"

        def run(n):
            cd, cl, it, wall = R.pc_run(n, 0, solver, True)
            return list(wall), it.tolist()
    except (FileNotFoundError, OSError):
        from oracle.oracle import Grid, Oracle
        O = Oracle()
        g = Grid.of(w, O)
        eta = O.eta_cylinder_z(g, w.cx, w.center_y)
        sim = O.sim(g, method=0, solver=solver if solver < 2 else 3, compat=True, dt=w.dt, nu=1.0 / w.re,
                    tol=w.tol, omega=w.omega, bc_dir=w.bc_dir, bc_num=w.bc_num, eta=eta)
        sim.init()
        sim.field("u0")[:] = u0
        sim.field("v0")[:] = v0
        sim.field("w0")[:] = w0
        sim.start()
        kind = "port"
        flags = "-O2 -ffp-contract=off"

        def run(n):
            walls, its = [], []
            for _ in range(n):
                t = time.perf_counter()
                r = sim.step()
                walls.append(time.perf_counter() - t)
                its.append(r[2])
            return walls, its
    run(warm)
    walls, its = run(steps)
    print(json.dumps({"kind": kind, "walls": walls, "iters": its, "flags": flags}))


def cpu_baseline(args, w, warmup, steps, budget_s=600):
    threads = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PLACES="cores", OMP_PROC_BIND="close",
               OMP_SCHEDULE="STATIC")
    spec = json.dumps({"workload": w.name, "solver": args.solver, "warmup": warmup, "steps": steps})
    try:
        r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--cpu-worker", spec], env=env,
                           capture_output=True, text=True, timeout=budget_s)
        line = [x for x in r.stdout.splitlines() if x.startswith("{")][-1]
        d = json.loads(line)
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": UNIT, "cores": threads, "kind": "unavailable",
                "sample": f"CPU run failed: {type(e).__name__}"}
    t = sum(d["walls"])
    value = w.n_cells * len(d["walls"]) / t / 1e6
    its = [sum(x) for x in d["iters"]]
    return {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": d["kind"],
            "sample": (f"{w.name} {w.nxc}x{w.nyc}x{w.nzc} predictor-corrector steps "
                       f"{warmup + 1}..{warmup + steps} (after {warmup} untimed), BiCGSTAB tol {w.tol:g}, "
                       f"{its} solver iterations per step, {t:.1f} s, g++ {d.get('flags', '?')}"),
            "s_per_step": round(t / len(d["walls"]), 3)}


# ---------------------------------------------------------------------------
def adjoint_leg(args, dist):
    """Gradient of the mean drag (steps n/2..n of an n-step cylinder run on the
    adjoint workload) w.r.t. the inflow profile and eta, by checkpointed reverse
    time stepping: forward run with checkpoints, then recompute + reverse
    sweep.  ratio = (recompute + reverse) seconds / forward seconds, for the
    FP64 forward and for the FP32 forward with FP64-refined solves."""
    import numpy as np

    from cfd_nssolver_forhpc_gb300 import capi
    from cfd_nssolver_forhpc_gb300.adjoint import MeanDrag
    from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
    wa = WORKLOADS[args.adj_workload]
    n = max(4, args.adj_steps)
    first, interval = n // 2, max(1, n // 4)
    out = {"workload": f"{wa.name}: cylinder wake {wa.nxc}x{wa.nyc}x{wa.nzc}, Re {wa.re:g}, dt {wa.dt:g}, "
                       f"tol {wa.tol:g}",
           "objective": f"mean Cd over steps {first}..{n} (bounded sample of the {wa.steps}-step run)",
           "parameters": f"inflow profile ({wa.nyc}) + eta ({wa.n_ghosted})",
           "checkpoint_interval": interval}
    out["legs"] = {"fp64": "FP64 fields, FP64 BiCGSTAB forward; the adjoint solves run the FP64 defect "
                           "correction around the FP32 multigrid-CG (not the same solver family)",
                   "fp64_dc": "FP64 fields, the FP64 defect correction around the FP32 multigrid-CG in "
                              "both directions (like for like)",
                   "mixed": "FP32 fields, the same defect-correction solver in both directions"}
    for prec_name, prec in (("fp64", capi.PREC_FP64), ("fp64_dc", capi.PREC_FP64_DC), ("mixed", capi.PREC_MIXED)):
        m = MeanDrag(wa, first, n, interval, precision=prec, tol=wa.tol)
        try:
            eta = m.default_eta().numpy()
            prof = np.full(wa.nyc, float(wa.bc_dir[0][0]))
            dist.barrier()
            J = m.objective(prof, eta)
            g_in, g_eta = m.gradient()
            run = m.last_run
            out[prec_name] = {
                "J": J, "forward_seconds": round(run["forward_seconds"], 4),
                "adjoint_seconds": round(run["adjoint_seconds"], 4),
                "ratio": round(run["adjoint_seconds"] / run["forward_seconds"], 3),
                "forward_iters": run["forward_iters"], "adjoint_iters": run["adjoint_iters"],
                "grad_inflow_norm": float(np.linalg.norm(g_in)), "grad_eta_norm": float(np.linalg.norm(g_eta)),
            }
        finally:
            m.close()
    out["ratio"] = out["mixed"]["ratio"] if args.precision == "mixed" else out["fp64"]["ratio"]
    return out


def div_check(S, tol):
    """Divergence of the last projection of the last step, measured inside
    the step (after the solve, before the boundary update): T2 = u* - dt grad p
    (updateUandF.hpp:136, 158, 179).  dev_inf = max |div T2 + dt m| (m: the RHS
    mean the compatibility projection removed) is the part a converged solve
    answers for; dev_rel divides it by max |div u*|, the divergence the
    projection had to remove."""
    S.divergence_check(True)
    S.step(allow_noconv=True)
    d = S.step_divergence()
    S.divergence_check(False)
    dev, du = d["dev_inf"], d["div_ustar_inf"]
    return {"dev_inf": dev, "div_T2_inf": d["div_T2_inf"], "div_ustar_inf": du,
            "dev_rel": dev / du if du > 0 else 0.0, "dev_inf_below_1e-10": bool(dev < 1e-10),
            "dev_rel_below_1e-10": bool(dev < 1e-10 * du), "solver_tol": tol,
            "measured": "one extra step after the timed ones"}


def snapshot(S):
    return {k: S.download(k) for k in ("U0", "V0", "W0", "P")}


def field_errors(a: dict, b: dict, w) -> dict:
    """Per-field max and L2 error of a against b, relative to b's max / L2.
    The pressure of the all-Neumann problem is defined up to a constant, so
    p is compared over the interior cells with its mean removed (the edge
    and corner ghost cells, which no boundary condition updates, keep
    values that do not follow the solution's constant)."""
    import numpy as np
    gc = 2
    out = {}
    for k in a:
        if k == "P":
            def interior(p):
                q = p.reshape(w.nxc + 2 * gc, w.nyc + 2 * gc, w.nzc + 2 * gc)[gc:-gc, gc:-gc, gc:-gc]
                return q - q.mean()
            a = dict(a, P=interior(a[k]))
            b = dict(b, P=interior(b[k]))
        d = a[k] - b[k]
        out[k] = {"max_rel": float(np.abs(d).max() / max(np.abs(b[k]).max(), 1e-300)),
                  "l2_rel": float(np.linalg.norm(d) / max(np.linalg.norm(b[k]), 1e-300))}
    return out


def cap_hits(infos, tol):
    """Solves whose final relative residual did not reach the tolerance (the
    first step solves nothing)."""
    return sum(1 for i in infos[1:] for r in i["relres"] if not r < tol)


def leg_c3(args):
    """Mixed precision against FP64 on the GPU at 1024x512x64 (Re 150, dt
    5e-4, tolerance 1e-10): the same seeded start, leg-steps steps each, the
    per-field max/L2 errors of u, v, w, p (p without its mean), drag and lift,
    the projected divergence of the last step, and both step rates."""
    from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
    w = WORKLOADS["c3"]
    K = max(2, args.leg_steps)
    out = {"leg": "c3", "workload": f"{w.name}: cylinder wake {w.nxc}x{w.nyc}x{w.nzc} ({w.n_cells} cells), Re {w.re:g}, "
                                    f"dt {w.dt:g}, tol {w.tol:g}, {K} steps (the first solves no Poisson equation)"}
    fields, legs = {}, {}
    for prec in ("mixed", "fp64"):
        S = build_sim(args, w, prec)
        t0 = time.perf_counter()
        infos = [S.step(allow_noconv=True) for _ in range(K - 1)]
        S.divergence_check(True)
        infos.append(S.step(allow_noconv=True))
        wall = time.perf_counter() - t0
        fields[prec] = snapshot(S)
        legs[prec] = {"s_per_solved_step": round(wall / max(1, K - 1), 3),
                      "iters_per_step": [sum(i["iters"]) for i in infos],
                      "outer_per_step": [sum(i["outer"]) for i in infos],
                      "max_relres": max(r for i in infos[1:] for r in i["relres"]),
                      "solves_above_tol": cap_hits(infos, w.tol),
                      "cd": [i["cd"] for i in infos], "cl": [i["cl"] for i in infos],
                      "divergence": S.step_divergence()}
        S.close()
    out.update(legs)
    cd_m, cd_f = legs["mixed"]["cd"][-1], legs["fp64"]["cd"][-1]
    out["cd_rel_mixed_vs_fp64"] = abs(cd_m / cd_f - 1.0)
    out["cl_diff_rel_to_cd"] = abs(legs["mixed"]["cl"][-1] - legs["fp64"]["cl"][-1]) / abs(cd_f)
    out["fields_mixed_vs_fp64"] = field_errors(fields["mixed"], fields["fp64"], w)
    return out


def leg_c5(args):
    """Memory plan and one bounded forward + adjoint segment at 1536x768x96
    (Re 200, dt 5e-4, mixed forward): device memory of the context with the
    adjoint state and a tape of `interval` steps, of each checkpoint, and the
    checkpoint interval that fits the full 400-step run (J over its last 200
    steps, every step reversed) in the GPU's memory."""
    import torch

    import numpy as np

    from cfd_nssolver_forhpc_gb300 import capi
    from cfd_nssolver_forhpc_gb300.adjoint import MeanDrag
    from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
    w = WORKLOADS["c5"]
    n = max(4, args.leg_steps)
    interval = max(1, n // 2)
    dev = torch.device("cuda", 0)
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info(dev)
    m = MeanDrag(w, n // 2, n, interval, precision=capi.PREC_MIXED, tol=w.tol)
    try:
        eta = m.default_eta().numpy()
        prof = np.full(w.nyc, float(w.bc_dir[0][0]))
        free1 = torch.cuda.mem_get_info(dev)[0]
        J = m.objective(prof, eta)
        free2 = torch.cuda.mem_get_info(dev)[0]
        g_in, g_eta = m.gradient()
        free3 = torch.cuda.mem_get_info(dev)[0]
        run = m.last_run
    finally:
        m.close()
    ng, nc = w.n_ghosted, w.n_cells
    tape_step = 3 * ng * 4 + 4 * nc * 8  # T0 (FP32) and the pressure of the four passes (FP64)
    nck = run.get("checkpoints") or -(-n // interval)
    ck_bytes = (free1 - free2) / max(1, nck) if free2 < free1 else None
    base = (free0 - free1) - interval * tape_step
    # the full run: 400 steps, J over the last 200; only the reversed window
    # needs checkpoints (one at its start, then one per interval) and a tape
    # of one interval
    full_steps, reversed_steps = 400, 200
    plan = None
    if ck_bytes:
        budget = 0.92 * total
        best = None
        for I in range(1, reversed_steps + 1):
            nck_full = -(-reversed_steps // I)
            tot = base + I * tape_step + nck_full * ck_bytes
            # fewest recomputed steps (one forward of the window) first, then memory
            if tot <= budget and (best is None or tot < best[1]):
                best = (I, tot, nck_full)
        if best:
            plan = {"steps": full_steps, "reversed_steps": reversed_steps, "interval": best[0],
                    "checkpoints": best[2], "device_bytes": int(best[1]), "of_total": round(best[1] / total, 3)}
    return {"leg": "c5",
            "workload": f"{w.name}: cylinder wake {w.nxc}x{w.nyc}x{w.nzc} ({w.n_cells} cells), Re {w.re:g}, "
                        f"dt {w.dt:g}, tol {w.tol:g}, mixed forward",
            "segment": {"steps": n, "objective": f"mean Cd over steps {n // 2}..{n}", "interval": interval,
                        "J": J, "forward_seconds": round(run["forward_seconds"], 3),
                        "adjoint_seconds": round(run["adjoint_seconds"], 3),
                        "ratio": round(run["adjoint_seconds"] / run["forward_seconds"], 3),
                        "grad_inflow_norm": float(np.linalg.norm(g_in)),
                        "grad_eta_norm": float(np.linalg.norm(g_eta))},
            "memory": {"gpu_total_bytes": int(total),
                       "context_adjoint_and_tape_bytes": int(free0 - free1),
                       "tape_step_bytes": int(tape_step), "checkpoint_bytes": int(ck_bytes) if ck_bytes else None,
                       "base_bytes": int(base), "peak_used_bytes": int(free0 - min(free2, free3))},
            "plan_400_steps": plan}


def main():
    args = parse()
    if args.cpu_worker:
        cpu_worker(args.cpu_worker)
        return
    if args.leg:
        from cfd_nssolver_forhpc_gb300.build import build
        build()
        import torch
        torch.cuda.init()
        print(json.dumps(leg_c3(args) if args.leg == "c3" else leg_c5(args)))
        return
    from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
    w = WORKLOADS[args.workload]
    dist = Dist()
    K, W = args.steps, max(args.warmup, 0)

    if args.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        # each step of the reference arm is one full reference step; the
        # number of steps is bounded so the run ends within a few minutes
        k_ref = max(1, min(K, 2))
        w_ref = max(1, min(W, 3))
        cb = cpu_baseline(args, w, w_ref, k_ref, budget_s=1500)
        v = cb["value"]
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": k_ref, "warmup": w_ref, "ms_per_step": (cb.get("s_per_step") or 0) * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded 1e-3 perturbation of u=1, v=w=0)",
                "config": {"workload": f"{w.name}: cylinder wake {w.nxc}x{w.nyc}x{w.nzc}, Re {w.re:g}, "
                                       f"dt {w.dt:g}, PC step, BiCGSTAB {args.solver} tol {w.tol:g}"},
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if cb["value"] is None:
            line = {"impl": "reference", "unavailable": cb["sample"]}
        print(json.dumps(line))
        dist.close()
        return

    from cfd_nssolver_forhpc_gb300.build import build
    build()
    import torch
    torch.cuda.init()
    if args.spinup is None:
        args.spinup = 60 if args.precision == "mixed" else 0
    S = build_sim(args, w, args.precision)
    # spin-up: the first ~20 steps from the impulsive start are a transient
    # in which every Poisson solve starts far from its solution; the timed
    # steps come after it, and every leg of the comparison starts from the
    # state the spin-up reaches
    for _ in range(args.spinup):
        S.step(allow_noconv=True)
    spun = S.state() if args.spinup > 0 else None
    for _ in range(W):
        S.step(allow_noconv=True)
    with ClockSampler(dist.local) as clk:
        sec, infos, launches = timed_steps(S, K, dist)
    clocks = clk.summary()
    sec_max = dist.max(sec)
    value = whole_job_rate(w.n_cells, K, dist.world, sec_max)
    mixed = args.precision == "mixed"
    rl = roofline(S, w, infos, args.precision, sec_max / K * 1e3)
    cd64 = infos[-1]["cd"]
    cl64 = infos[-1]["cl"]
    fields = snapshot(S) if not args.no_compare and args.solver != "sor" else None
    div = div_check(S, w.tol)
    e2e = None
    if not args.no_e2e:
        dev_s, wall_s, nbytes = e2e_steps(S, K, dist)
        wall_s = dist.max(wall_s)
        e2e = {"value": round(whole_job_rate(w.n_cells, K, dist.world, wall_s), 4), "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "seconds": round(wall_s, 4)}
    S.close()
    # the other precision on the same workload: the mixed / FP64 ratio at the
    # same tolerance, and the drag difference
    other = None
    other_prec = "fp64" if mixed else "mixed"
    if not args.no_compare and args.solver != "sor":
        M = build_sim(args, w, other_prec)
        if spun:
            M.restore(spun)
        for _ in range(W):
            M.step(allow_noconv=True)
        msec, minfos, mlaunch = timed_steps(M, K, dist)
        msec = dist.max(msec)
        mval = whole_job_rate(w.n_cells, K, dist.world, msec)
        mixed_v, fp64_v = (value, mval) if mixed else (mval, value)
        mfields = snapshot(M)
        mixed_f, fp64_f = (fields, mfields) if mixed else (mfields, fields)
        mdiv = div_check(M, w.tol)
        other = {"precision": other_prec, "value": round(mval, 4), "unit": UNIT,
                 "dtype": "f64" if mixed else "f32+f64", "ms_per_step": round(msec / K * 1e3, 3),
                 "iters_per_step": [sum(i["iters"]) for i in minfos],
                 "max_relres": max(r for i in minfos[1:] or minfos for r in i["relres"]),
                 "solves_above_tol": cap_hits(minfos, w.tol),
                 "maxit": args.fp64_maxit if other_prec == "fp64" else 5000,
                 "cd_last": minfos[-1]["cd"], "cd_rel_vs_headline": abs(minfos[-1]["cd"] / cd64 - 1.0),
                 "cl_last": minfos[-1]["cl"],
                 "cl_diff_rel_to_cd": abs(minfos[-1]["cl"] - cl64) / abs(cd64),
                 "divergence": mdiv, "gpu_launches": mlaunch,
                 "fields_mixed_vs_fp64": field_errors(mixed_f, fp64_f, w),
                 "fields_after_steps": W + K, "from_step": args.spinup + 1,
                 "roofline": roofline(M, w, minfos, other_prec, msec / K * 1e3),
                 "ratio_mixed_vs_fp64": round(mixed_v / fp64_v, 3)}
        M.close()
    # FP64 fields with the mixed path's solver (the FP64 defect correction
    # around the FP32 multigrid CG): what the FP32 fields buy at the same
    # algorithm, beside what the algorithm buys against FP64 BiCGSTAB
    same_solver = None
    if mixed and not args.no_compare and args.solver != "sor":
        D = build_sim(args, w, "fp64_dc")
        if spun:
            D.restore(spun)
        for _ in range(W):
            D.step(allow_noconv=True)
        dsec, dinfos, dlaunch = timed_steps(D, K, dist)
        dsec = dist.max(dsec)
        dval = whole_job_rate(w.n_cells, K, dist.world, dsec)
        same_solver = {"precision": "fp64_dc", "value": round(dval, 4), "unit": UNIT, "dtype": "f64",
                       "ms_per_step": round(dsec / K * 1e3, 3),
                       "iters_per_step": [sum(i["iters"]) for i in dinfos],
                       "outer_per_step": [sum(i["outer"]) for i in dinfos],
                       "max_relres": max(r for i in dinfos[1:] or dinfos for r in i["relres"]),
                       "cd_rel_vs_headline": abs(dinfos[-1]["cd"] / cd64 - 1.0), "gpu_launches": dlaunch,
                       "ratio_mixed_vs_fp64_dc": round(value / dval, 3)}
        D.close()
    adjoint = None
    if not args.no_adjoint and args.solver != "sor":
        adjoint = adjoint_leg(args, dist)
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, w, 1, 1, budget_s=300)
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": dist.world, "steps": K,
            "warmup": W, "ms_per_step": round(sec_max / K * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
            "data": "synthetic (seeded 1e-3 perturbation of u=1, v=w=0)",
            "config": {"workload": f"{w.name}: cylinder wake {w.nxc}x{w.nyc}x{w.nzc} ({w.n_cells} cells), "
                                   f"Re {w.re:g}, dt {w.dt:g}, predictor-corrector step",
                       "solver": f"BiCGSTAB {args.solver}" if args.solver != "sor" else "red-black SOR",
                       "tol": w.tol, "precision": args.precision, "parallelism": f"replicas x{dist.world}",
                       "l2": "working set larger than L2 (no flush needed)",
                       "spinup_steps": args.spinup,
                       "timed_steps_start_at": args.spinup + W + 1},
            "iters_per_step": [sum(i["iters"]) for i in infos],
            "outer_per_step": [sum(i["outer"]) for i in infos],
            "max_relres": max(r for i in infos[1:] or infos for r in i["relres"]),
            "solves_above_tol": cap_hits(infos, w.tol),
            "cd_last": infos[-1]["cd"], "divergence": div,
            "roofline": rl, "cpu_baseline": cpu, "clocks": clocks, "e2e": e2e,
            "gpu_launches": launches,
        }
        if mixed:
            line["config"]["inner_tol"] = args.inner_tol
        if same_solver:
            line["fp64_dc"] = same_solver
        if other:
            line[other_prec] = other
            line["ratio_mixed_vs_fp64"] = other["ratio_mixed_vs_fp64"]
        if adjoint:
            line["adjoint"] = adjoint
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
