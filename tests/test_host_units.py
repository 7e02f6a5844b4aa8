"""Host-side units of the GPU library (no GPU): the division magic numbers of
the multigrid levels, the level hierarchy of the large grid, the fine-level
tile choice and the FP64 dense inverse of a coarsest level, compiled from the
library's own sources with the host compiler (tests/host/host_units.cpp)."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "mag2d_gb300" / "csrc"


def test_host_units(tmp_path):
    gxx = shutil.which("g++")
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    if gxx is None or not (cuda / "cuda_runtime.h").exists():
        pytest.skip("needs g++ and the CUDA headers")
    exe = tmp_path / "host_units"
    cmd = [gxx, "-std=c++17", "-O1", f"-I{CSRC}", f"-I{cuda}", str(ROOT / "tests" / "host" / "host_units.cpp"),
           str(CSRC / "multigrid_host.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host units ok" in r.stdout
