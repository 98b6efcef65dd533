"""Chunk and copy ranges of the host-buffer pipelines (engine.cuh), checked
on the CPU: built from the header with the host compiler and run over fixed
and random splits (contiguity, 256-byte ends, every transform's input copied
before it, only finished output copied out, copy-out and later copy-in ranges
disjoint so in-place host buffers stay correct)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_pipeline_ranges(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = tmp_path / "host_ranges_check"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "kfft_gb300", "csrc"), "-I", inc,
                    os.path.join(ROOT, "tests", "host_ranges_check.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
