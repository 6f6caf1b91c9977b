"""The C++ drop-in header (include/cfdgpu_reference.hpp) compiles inside the
reference's own translation unit: tests/drop_in_driver.cpp is the reference's
predictor-corrector loop with every hot-path call switched to its *_CUDA
counterpart, type-checked against a patched copy of the reference headers
(compile only; no GPU)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_drop_in_driver_compiles():
    from oracle import build_ref
    inc = build_ref.OUT / "g1" / "inc"
    if not inc.exists():
        try:
            build_ref.build("g1")
        except (FileNotFoundError, OSError) as e:
            pytest.skip(f"reference sources unavailable: {e}")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    r = subprocess.run([gxx, "-std=c++17", "-fopenmp", "-fsyntax-only", "-w", "-I", str(inc),
                        "-I", str(ROOT / "include"), str(ROOT / "tests" / "drop_in_driver.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
