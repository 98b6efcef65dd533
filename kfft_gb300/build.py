"""Builds the GB300 FFT engine shared libraries with nvcc for sm_103a.

Two libraries come out of the same sources, mirroring the reference's
compile-time precision switch (KFFT_HALF_SCALAR, incs/kfft_types.h:21-25):

  kfft_gb300/lib/libkfft_gb300.so    double build (kfft_scalar = double)
  kfft_gb300/lib/libkfft_gb300_f.so  float build  (kfft_scalar = float)

Object files are compiled in parallel; a rebuild happens only when a source or
header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
SOURCES = ["pass_smem.cu", "pass_reg.cu", "persistent.cu", "tables.cu", "plan.cu", "api.cu",
           "uneven.cu", "noalloc.cu", "helpers.cu", "mlp.cu"]
HEADERS = ["engine.cuh", "fft_device.cuh", "plan_host.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
VARIANTS = {"libkfft_gb300.so": [], "libkfft_gb300_f.so": ["-DKFFT_HALF_SCALAR"]}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, defines: list[str]) -> None:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
           "-I", CSRC, *defines, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> dict[str, str]:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    deps += [os.path.join(ROOT, "include", h) for h in ("kfft.h", "kfft_gb300.h")]
    out = {}
    jobs = []
    for lib, defines in VARIANTS.items():
        target = os.path.join(LIB_DIR, lib)
        out[lib] = target
        if not force and not _stale(target, deps):
            continue
        tag = lib.replace(".so", "")
        objs = []
        for s in SOURCES:
            obj = os.path.join(OBJ_DIR, f"{tag}_{s.replace('.cu', '.o')}")
            objs.append(obj)
            jobs.append((os.path.join(CSRC, s), obj, defines))
        jobs.append(("LINK", target, objs))
    compile_jobs = [j for j in jobs if j[0] != "LINK"]
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda j: _compile(*j), compile_jobs))
    for j in jobs:
        if j[0] == "LINK":
            tmp = j[1] + f".tmp{os.getpid()}"
            cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *j[2], "-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
            os.replace(tmp, j[1])
            if verbose:
                print("built", j[1])
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
