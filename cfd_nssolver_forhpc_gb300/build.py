"""In-tree build of libcfdgpu.so (the C-ABI library) for sm_103a.

Each .cu file under csrc/ is compiled to an object in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a), then the objects are linked into
cfd_nssolver_forhpc_gb300/_lib/libcfdgpu.so.  Host code is compiled with
-ffp-contract=off so the host-side metric tables keep the reference's
rounding on every architecture.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libcfdgpu.so"
SOURCES = ["flow.cu", "poisson.cu", "adjoint.cu", "api.cu", "adjoint_api.cu", "plot3d.cu", "grid.cu", "multigrid.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise FileNotFoundError("nvcc not found")
    return exe


def _flags() -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                   "-I", str(PKG.parent / "include")]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "cfdgpu.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append((s, o))

    def run(job):
        s, o = job
        tmp = o.with_suffix(f".{os.getpid()}.o")
        cmd = [nvcc()] + _flags() + ["-c", str(s), "-o", str(tmp)]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s.name}:\n{r.stderr}")
        os.replace(tmp, o)
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for line in logs:
            print(line)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(f".{os.getpid()}.so")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
