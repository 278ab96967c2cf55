"""The search's device code, compiled for the host from the CUDA headers
themselves (csrc/grand_device.cuh, csrc/grand_lookup.cuh) and checked against plain combinatorics and a
brute-force search, without a GPU:
  tests/host_device_math.cpp  warp-free math: binomials, colex unranking in
      closed form and by table, colex successors, lexicographic ranks, the FP32
      cost key, whole run tiles lane by lane, first-hit and ML, and the
      solo-column table of the classification step (csrc/grand_solo.h) against
      its brute-force definition;
  tests/host_warp_math.cpp    warp-level code on an emulated warp (32 host
      threads whose collectives meet at a barrier): the warp minima, the result
      writer's warp-parallel unranking, whole masked colex tiles, the lookup
      tables (csrc/grand_lookup.cuh: filter and buckets hold every column, the
      filter's false-pass rate stays under its bound) and whole lookup tiles of
      weights 1-6 against brute force, first-hit and ML."""
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


def _build_and_run(tmp_path, source, std, extra=()):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / os.path.splitext(source)[0])
    subprocess.run([cxx, f"-std={std}", "-O2", *extra,
                    "-I", os.path.join(ROOT, "library_s_grand_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), "-I", inc,
                    os.path.join(HERE, source), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("ok"), out.stdout


def test_device_index_math_on_host(tmp_path):
    _build_and_run(tmp_path, "host_device_math.cpp", "c++17")


def test_warp_level_device_code_on_an_emulated_warp(tmp_path):
    _build_and_run(tmp_path, "host_warp_math.cpp", "c++20", ["-pthread"])
