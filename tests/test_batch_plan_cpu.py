"""The batched tensor-core launch plan (fft3dcl_gb300/csrc/f3d_batch_plan.hpp)
on the CPU: CTA prefixes, the filter's runs of one geometry and shifted
windows, refused batches. Compiles tests/batch_plan/check.cpp with the host
compiler against the CUDA runtime headers (no GPU needed)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_batch_plan():
    cxx = shutil.which("g++")
    if cxx is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA runtime headers")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "check")
        subprocess.run([cxx, "-std=c++17", "-O1", "-Wall",
                        "-I", os.path.join(ROOT, "fft3dcl_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                        "-I", CUDA_INC, os.path.join(ROOT, "tests", "batch_plan", "check.cpp"), "-o", exe],
                       check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout
