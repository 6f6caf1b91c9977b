"""The C++ drop-in branch runs (GPU).

tests/drop_in_driver.cpp is the reference's predictor-corrector main loop
(RUN_CPU_PC_METHOD.hpp:287-627) with every hot-path call switched to the
*_CUDA functions of include/cfdgpu_reference.hpp.  Compiled against the
reference's own headers (the patched copy for the 128x64x8 cylinder) and
linked to libcfdgpu.so, it runs 20 steps from the seeded initial state.  Its
drag and lift must match the reference's own run of the same 20 steps
(tests/golden/c1_run.npz) and the library's cfd_step on the same state.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cfd_nssolver_forhpc_gb300 import capi
from cfd_nssolver_forhpc_gb300.configs import WORKLOADS
from cfd_nssolver_forhpc_gb300.initial import initial_velocity
from cfd_nssolver_forhpc_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
STEPS = 20


def _build(tmp: Path) -> Path:
    from oracle import build_ref
    inc = build_ref.OUT / "c1" / "inc"
    if not inc.exists():
        try:
            build_ref.build("c1")
        except (FileNotFoundError, OSError) as e:
            pytest.skip(f"reference headers unavailable: {e}")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    libdir = Path(capi.library_path()).parent
    exe = tmp / "drop_in"
    r = subprocess.run([gxx, "-std=c++17", "-fopenmp", "-O2", "-w", "-DCFDGPU_DROP_IN_MAIN", "-I", str(inc),
                        "-I", str(ROOT / "include"), str(ROOT / "tests" / "drop_in_driver.cpp"),
                        "-L", str(libdir), "-lcfdgpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_drop_in_driver_runs_the_reference_loop_on_the_gpu(tmp_path, golden):
    w = WORKLOADS["c1"]
    tol = 1e-8
    exe = _build(tmp_path)
    u0, v0, w0 = initial_velocity(w.nxc, w.nyc, w.nzc)
    files = []
    for name, a in (("u0", u0), ("v0", v0), ("w0", w0)):
        f = tmp_path / f"{name}.bin"
        np.ascontiguousarray(a, dtype=np.float64).tofile(f)
        files.append(str(f))
    bc = tmp_path / "bc.txt"
    bc.write_text(" ".join(repr(float(x)) for row in w.bc_dir for x in row) + "\n"
                  + " ".join(repr(float(x)) for row in w.bc_num for x in row) + "\n")
    r = subprocess.run([str(exe), str(STEPS), repr(w.dt), repr(w.re), repr(tol), repr(w.cx), str(bc)] + files,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    rows = np.array([[float(x) for x in line.split()[1:]] for line in r.stdout.split("\n")
                     if line.startswith("CDCL ")])
    assert rows.shape == (STEPS, 3)
    cd, cl = rows[:, 1], rows[:, 2]
    G = golden("c1_run")
    np.testing.assert_allclose(cd, G["spe_cd"], rtol=1e-6)
    np.testing.assert_allclose(cl, G["spe_cl"], rtol=1e-3, atol=1e-4)
    # the same steps through cfd_step (the library's fused step)
    with Simulation(w, tol=tol) as S:
        S.setup_cylinder(u0, v0, w0)
        hist = [S.step() for _ in range(STEPS)]
    np.testing.assert_allclose(cd, [h["cd"] for h in hist], rtol=1e-9)
    np.testing.assert_allclose(cl, [h["cl"] for h in hist], rtol=1e-6, atol=1e-9)
