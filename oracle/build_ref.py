"""Build recipe for the reference harness (test infrastructure only).

The reference fixes its grid size, domain lengths, grid type, boundary table
and cylinder centre at compile time (inc/grid/structureGrid.hpp:26,34,44-46,
inc/BoundaryCondition/Boundary_Condition.hpp:11, inc/dfib/setEta.hpp:145).
For each workload this script copies the reference's inc/ tree into
oracle/_ref/<name>/inc (git-ignored), rewrites exactly those lines, and
compiles oracle/ref_harness.cpp against the copy into
oracle/_ref/<name>/libref.so with plain g++ (no build system, no -march:
-O2 -fopenmp -ffp-contract=off, so no multiply-add is fused).  That build is
the parity checker.  build(name, fast=True) compiles the same sources with the
reference's own optimisation flags (-O3 -march=native, Makefile:18) into
libref_fast.so: the timed CPU baseline, never a checker (its fused multiply-
adds change the rounding).

When the reference tree is absent (e.g. on a machine that only received the
patched copy), an existing oracle/_ref/<name>/inc is compiled as is.

Usage: python oracle/build_ref.py g1 c1 ...
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))

from cfd_nssolver_forhpc_gb300.configs import WORKLOADS, Workload  # noqa: E402

REFERENCE = Path(os.environ.get("CFD_REFERENCE_ROOT", "/root/reference"))
OUT = HERE / "_ref"
# workloads whose reference run is also timed (bench.py's CPU baseline)
TIMED_WORKLOADS = ("c2",)


def _replace_once(path: Path, old: str, new: str) -> None:
    text = path.read_text()
    if text.count(old) != 1:
        raise RuntimeError(f"patch point not unique in {path}: {old!r}")
    path.write_text(text.replace(old, new))


def _bc_table(w: Workload) -> str:
    lines = ["// generated by oracle/build_ref.py: Dir/Num table of the workload"]
    for b in range(6):
        for c in range(3):
            lines.append(f"Dir[{b}][{c}] = {w.bc_dir[b][c]!r}; Num[{b}][{c}] = {w.bc_num[b][c]!r};")
    return "\n".join(lines) + "\n"


def patch_tree(w: Workload, gridder: str = "uniform", out_name: str | None = None) -> Path:
    dst = OUT / (out_name or w.name) / "inc"
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(REFERENCE / "inc", dst, ignore=shutil.ignore_patterns("amgcl", "yakutat"))
    sg = dst / "grid" / "structureGrid.hpp"
    _replace_once(sg, 'const std::string Gridder = "non_uniform-SML";',
                  f'const std::string Gridder = "{gridder}";')
    _replace_once(sg, "const double  lx = 17.0 ,      ly = 12.0 ,      lz = 3.0 ;",
                  f"const double  lx = {w.lx!r} , ly = {w.ly!r} , lz = {w.lz!r} ;")
    _replace_once(sg, "const int       nxCal = 190,     // nx should > 40\n"
                      "                        nyCal = 210,\n"
                      "                        nzCal = 40;",
                  f"const int nxCal = {w.nxc}, nyCal = {w.nyc}, nzCal = {w.nzc};")
    bc = dst / "BoundaryCondition" / "Boundary_Condition.hpp"
    _replace_once(bc, '#include "BC_Cavity_A.hpp"', '#include "BC_HARNESS_TABLE.hpp"')
    (dst / "BoundaryCondition" / "BC_HARNESS_TABLE.hpp").write_text(_bc_table(w))
    # the LES model does not compile as shipped (a misspelt `auto`,
    # source/smagorinskyModel.hpp:63); fixed here so the TERBULENCE_SMAGORINSKY
    # build used by the LES parity tests can be made
    _replace_once(dst / "source" / "smagorinskyModel.hpp", "const auot icelCal", "const auto icelCal")
    eta = dst / "dfib" / "setEta.hpp"
    _replace_once(eta, "double  center_x    = 6.5,", f"double  center_x    = {w.cx!r},")
    if abs(w.center_y - w.ly / 2.0) > 0.0:
        raise RuntimeError("the reference places the cylinder at y = ly/2")
    return dst


# the reference's own optimisation flags (Makefile:18), tried in this order
# where the host compiler does not take -march=native
FAST_FLAGS = (["-O3", "-march=native"], ["-O3", "-mcpu=native"], ["-O3"])


def build(name: str, gridder: str = "uniform", force: bool = False, les: bool = False,
          fast: bool = False) -> Path:
    """les: the reference's Smagorinsky model compiled in
    (TERBULENCE_SMAGORINSKY), output under oracle/_ref/<name>_les/.
    fast: the timing build (libref_fast.so, the reference's -O3 -march=native)."""
    w = WORKLOADS[name]
    out_name = name + ("_les" if les else "")
    lib = OUT / out_name / ("libref_fast.so" if fast else "libref.so")
    inc = OUT / out_name / "inc"
    if REFERENCE.exists() and (force or not inc.exists()):
        patch_tree(w, gridder, out_name)
    if not inc.exists():
        raise FileNotFoundError(f"no reference sources for {name}: {REFERENCE} absent")
    src = HERE / "ref_harness.cpp"
    if lib.exists() and lib.stat().st_mtime > max(src.stat().st_mtime, inc.stat().st_mtime) and not force:
        return lib
    base = ["g++", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-w", "-I", str(inc), str(src), "-o", str(lib)]
    if les:
        base[1:1] = ["-DTERBULENCE_SMAGORINSKY"]
    if not fast:
        subprocess.run(base[:1] + ["-O2", "-ffp-contract=off"] + base[1:], check=True)
        return lib
    err = None
    for flags in FAST_FLAGS:
        r = subprocess.run(base[:1] + flags + base[1:], capture_output=True, text=True)
        if r.returncode == 0:
            (OUT / out_name / "libref_fast.flags").write_text(" ".join(flags) + "\n")
            return lib
        err = r.stderr
    raise RuntimeError(f"reference timing build failed: {err}")


if __name__ == "__main__":
    names = sys.argv[1:] or ["g1"]
    for n in names:
        print(build(n, force=True))
        if n in TIMED_WORKLOADS:
            print(build(n, fast=True, force=True))
