"""The search kernels' warp-free index math, compiled for the host from the
CUDA header itself (csrc/grand_device.cuh) and checked against plain
combinatorics and a brute-force search (tests/host_device_math.cpp): binomials,
colex unranking in closed form and by table, colex successors, lexicographic
ranks, the FP32 cost key, and whole run tiles lane by lane, first-hit and ML.
Runs without a GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


def test_device_index_math_on_host(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "device_math")
    subprocess.run([cxx, "-std=c++17", "-O2",
                    "-I", os.path.join(ROOT, "library_s_grand_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), "-I", inc,
                    os.path.join(HERE, "host_device_math.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("ok"), out.stdout
