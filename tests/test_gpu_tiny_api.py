"""The tiny API (include/kfft_tiny.h, the reference's kfft_tiny.h interface)
run on the GPU: tests/tiny_api_check.c is compiled with gcc against the
header and the engine library of each precision, run on the inputs written
here, and every output is compared with the FP64 oracle (FP64 build:
rel-L2 <= 1e-13*log2 N; FP32 build: 1e-6).  The program makes the calls of
the reference's docs/example/example_tiny.c (complex 1D inverse with
GENERIC_ONLY, scalar 1D, scalar and complex 2D convolution of 50 x 50) and
the other plan kinds.  A compile-only check of the same program, which needs
no GPU, is in test_abi.py."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import TOL32, rel_l2, tol64

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBS = {"double": "libkfft_gb300.so", "float": "libkfft_gb300_f.so"}
N1, NX, NY = 100, 50, 50


def build_tiny_program(out_dir, precision):
    """Compiles tests/tiny_api_check.c against include/ and one engine build."""
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("needs gcc")
    lib_dir = os.path.join(ROOT, "kfft_gb300", "lib")
    exe = os.path.join(out_dir, f"tiny_{precision}")
    cmd = [gcc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "tiny_api_check.c"), "-o", exe,
           os.path.join(lib_dir, LIBS[precision]), f"-Wl,-rpath,{lib_dir}"]
    if precision == "float":
        cmd.insert(2, "-DKFFT_HALF_SCALAR")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("precision", ["double", "float"])
def test_tiny_api_program_against_oracle(tmp_path, precision):
    cdt = np.complex128 if precision == "double" else np.complex64
    rdt = np.float64 if precision == "double" else np.float32
    exe = build_tiny_program(str(tmp_path), precision)
    rng = np.random.default_rng(11)
    n2 = NX * NY
    a = (rng.standard_normal(n2) + 1j * rng.standard_normal(n2)).astype(cdt)
    b = (rng.standard_normal(n2) + 1j * rng.standard_normal(n2)).astype(cdt)
    ra = rng.uniform(-1, 1, n2).astype(rdt)
    rb = rng.uniform(-1, 1, n2).astype(rdt)
    with open(tmp_path / "in.bin", "wb") as f:
        for v in (a, b, ra, rb):
            f.write(v.tobytes())
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "tiny api ok" in r.stdout

    def out(name, dt, count):
        v = np.fromfile(tmp_path / f"out_{name}.bin", dtype=dt)
        assert v.size == count, name
        return v.astype(np.complex128 if np.iscomplexobj(v) else np.float64)

    def tol(n):
        return tol64(n) if precision == "double" else TOL32

    a64, b64 = a.astype(np.complex128), b.astype(np.complex128)
    ra64, rb64 = ra.astype(np.float64), rb.astype(np.float64)
    x1 = a64[:N1]
    spec = O.rfft(ra64[:N1])
    checks = {
        "cpx_fwd": (out("cpx_fwd", cdt, N1), O.fft_cpx(x1), N1),
        "cpx_inv": (out("cpx_inv", cdt, N1), O.fft_cpx(x1, O.FLAG_INVERSE), N1),
        "sclr_fwd": (out("sclr_fwd", cdt, N1 // 2 + 1), spec, N1),
        # the inverse of the spectrum the program computed (the even-length
        # real inverse returns twice the input, as the reference's does)
        "sclr_inv": (out("sclr_inv", rdt, N1),
                     O.irfft(out("sclr_fwd", cdt, N1 // 2 + 1), N1), N1),
        "cpx2_fwd": (out("cpx2_fwd", cdt, n2), O.fft2_cpx(a64.reshape(NY, NX)).ravel(), n2),
        "sclr2_fwd": (out("sclr2_fwd", cdt, n2), O.rfft2(ra64.reshape(NY, NX)).ravel(), n2),
        "conv_cpx": (out("conv_cpx", cdt, N1), O.conv_cpx(x1, b64[:N1]), N1),
        "conv_sclr": (out("conv_sclr", rdt, N1), O.conv_scalar(ra64[:N1], rb64[:N1]), N1),
        "conv2_sclr": (out("conv2_sclr", rdt, n2),
                       O.conv2_scalar(ra64.reshape(NY, NX), rb64.reshape(NY, NX)).ravel(), n2),
        "conv2_cpx": (out("conv2_cpx", cdt, n2),
                      O.conv2_cpx(a64.reshape(NY, NX), b64.reshape(NY, NX), O.FLAG_GENERIC).ravel(), n2),
    }
    for name, (got, ref, n) in checks.items():
        assert rel_l2(got, ref) <= tol(n), (name, rel_l2(got, ref))
    assert rel_l2(checks["sclr_inv"][0], 2.0 * ra64[:N1]) <= 2 * tol(N1)
