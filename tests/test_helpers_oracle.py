"""Post-transform helpers (fftshift, the kfft_math API, the tiny API header):
the oracle's restatements pinned against the reference library built from
its own sources, and the engine's headers checked to compile the reference's
tiny API.  CPU only.

Reference defects found here (the oracle follows the intent, the tests pin
only what the reference gets right):
* kfft_shift_cpx / kfft_shift_scalar on an even length swap halves through a
  macro whose temporary aliases its operand, so the buffer comes back zeroed
  (kfft_shift.c:10-12); only odd lengths are compared.
* the inverse shift of a length-1 buffer counts k = c-1 down from 0 in
  unsigned arithmetic (kfft_shift.c:16-19) and runs off the buffer; it is not
  called.
* kfft_math_average sums into a shared variable from every OpenMP thread
  without a reduction (kfft_math.c:143-146); it is called with one thread.
* kfft_tiny.h closes the switch of kfft_tiny_eval inside its
  KFFT_SPARSE_ENABLE block (kfft_tiny.h:243-247), so it compiles only with the
  sparse extension, which neither library has; the compile test moves that
  brace out of the block in a temporary copy.
"""
import ctypes
import ctypes.util
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_SRC = os.environ.get("KFFT_REFERENCE_DIR", "/root/reference")


def _ref(precision="double"):
    if O.ref_library_path(precision) is None:
        pytest.skip("reference library not built here")
    lib = ctypes.CDLL(O.ref_library_path(precision))
    vp, u32, b = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_bool
    for n in ("kfft_shift_cpx", "kfft_shift_scalar"):
        getattr(lib, n).argtypes = [vp, u32, b, vp]
    for n in ("kfft_shift2_cpx", "kfft_shift2_scalar"):
        getattr(lib, n).argtypes = [vp, vp, u32, u32, b, vp]
    for n in ("kfft_math_hadamard_cpx", "kfft_math_hadamard_scalar", "kfft_math_magnitude"):
        getattr(lib, n).argtypes = [vp, vp, u32]
    for n in ("kfft_math_transpose_cpx", "kfft_math_transpose_scalar"):
        getattr(lib, n).argtypes = [vp, vp, u32, u32]
    for n in ("kfft_math_transpose_ip_cpx", "kfft_math_transpose_ip_scalar"):
        getattr(lib, n).argtypes = [vp, u32, u32]
    lib.kfft_math_magnitude_ip.argtypes = [vp, u32]
    lib.kfft_math_average.argtypes = [vp, u32]
    lib.kfft_math_average.restype = ctypes.c_double if precision == "double" else ctypes.c_float
    return lib


def _one_omp_thread():
    name = ctypes.util.find_library("gomp")
    if name:
        ctypes.CDLL(name).omp_set_num_threads(1)


@pytest.mark.parametrize("n", list(range(1, 40, 2)) + [101, 1023, 4097])
def test_shift_matches_reference_on_odd_lengths(n):
    ref = _ref()
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for inverse in (False, True):
        if inverse and n == 1:
            continue  # the reference's unsigned countdown runs off a length-1 buffer
        a = x.copy()
        ref.kfft_shift_cpx(a.ctypes.data, n, inverse, None)
        assert np.array_equal(a, O.shift(x, inverse)), (n, inverse)
        r = x.real.copy()
        ref.kfft_shift_scalar(r.ctypes.data, n, inverse, None)
        assert np.array_equal(r, O.shift(x.real, inverse)), (n, inverse)


def test_shift_is_numpy_fftshift():
    for n in range(1, 34):
        x = np.arange(n)
        assert np.array_equal(O.shift(x), np.fft.fftshift(x))
        assert np.array_equal(O.shift(x, True), np.fft.ifftshift(x))
        assert np.array_equal(O.shift(O.shift(x), True), x)


def test_reference_even_shift_defect_is_documented():
    ref = _ref()
    x = np.arange(1, 9, dtype=np.float64) + 0j
    a = x.copy()
    ref.kfft_shift_cpx(a.ctypes.data, 8, False, None)
    # the aliased swap leaves zeros where the shifted halves should be
    assert not np.array_equal(a, O.shift(x))


@pytest.mark.parametrize("shape", [(3, 5), (7, 9), (1, 13), (11, 1), (33, 17)])
def test_shift2_matches_reference_on_odd_shapes(shape):
    ref = _ref()
    y, x = shape
    rng = np.random.default_rng(x * 100 + y)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    for inverse in (False, True):
        if inverse and 1 in shape:
            continue  # length-1 axes hit the same unsigned countdown
        h = a.copy()
        tmp = np.empty_like(a)
        ref.kfft_shift2_cpx(h.ctypes.data, tmp.ctypes.data, x, y, inverse, None)
        assert np.array_equal(h, O.shift(a, inverse)), (shape, inverse)
        hr = a.real.copy()
        tr = np.empty_like(hr)
        ref.kfft_shift2_scalar(hr.ctypes.data, tr.ctypes.data, x, y, inverse, None)
        assert np.array_equal(hr, O.shift(a.real, inverse)), (shape, inverse)


def test_math_helpers_match_reference():
    ref = _ref()
    _one_omp_thread()
    rng = np.random.default_rng(5)
    n = 1001
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    w = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    h = w.copy()
    ref.kfft_math_hadamard_cpx(h.ctypes.data, z.ctypes.data, n)
    assert np.allclose(h, w * z, rtol=1e-15, atol=0)
    hr = w.real.copy()
    zr = np.ascontiguousarray(z.real)
    ref.kfft_math_hadamard_scalar(hr.ctypes.data, zr.ctypes.data, n)
    assert np.array_equal(hr, w.real * zr)
    m = np.empty(n)
    ref.kfft_math_magnitude(z.ctypes.data, m.ctypes.data, n)
    assert np.allclose(m, O.magnitude(z), rtol=2e-16, atol=0)
    zi = z.copy()
    ref.kfft_math_magnitude_ip(zi.ctypes.data, n)
    assert np.allclose(zi.view(np.float64)[:n], O.magnitude(z), rtol=2e-16, atol=0)
    v = rng.standard_normal(n)
    assert ref.kfft_math_average(v.ctypes.data, n) == pytest.approx(O.average(v), rel=1e-15)
    a = rng.standard_normal((37, 101)) + 1j * rng.standard_normal((37, 101))
    t = np.empty((101, 37), np.complex128)
    ref.kfft_math_transpose_cpx(a.ctypes.data, t.ctypes.data, 101, 37)
    assert np.array_equal(t, O.transpose(a))
    ip = a.copy()
    ref.kfft_math_transpose_ip_cpx(ip.ctypes.data, 101, 37)
    assert np.array_equal(ip.reshape(101, 37), O.transpose(a))
    ar = np.ascontiguousarray(a.real)
    tr = np.empty((101, 37))
    ref.kfft_math_transpose_scalar(ar.ctypes.data, tr.ctypes.data, 101, 37)
    assert np.array_equal(tr, O.transpose(a.real))
    ref.kfft_math_transpose_ip_scalar(ar.ctypes.data, 101, 37)
    assert np.array_equal(ar.reshape(101, 37), O.transpose(a.real))


TINY_PROGRAM = r"""
#include <stdio.h>
#include "kfft_tiny.h"
int main(void) {
    kfft_args_norm a = {64};
    kfft_plan p = kfft_configuration(KFFT_PLAN_COMPLEX, 0, &a);
    kfft_args_2d b = {8, 8};
    kfft_plan q = kfft_configuration(KFFT_PLAN_SCALAR_CONV2D, 0, &b);
    (void)q;
    kfft_finalization(p);
    return 0;
}
"""


def test_tiny_api_header_compiles_and_links_against_the_engine(tmp_path):
    src = os.path.join(REF_SRC, "kfft_tiny.h")
    lib = os.path.join(ROOT, "kfft_gb300", "lib", "libkfft_gb300.so")
    if not os.path.isfile(src):
        pytest.skip("reference headers not present")
    if not os.path.isfile(lib):
        pytest.skip("engine library not built")
    text = open(src).read()
    # move the misplaced switch brace out of the sparse-only block
    broken = "    };\n#endif /* KFFT_SPARSE_ENABLE */\n    return KFFT_RET_IMPROPER_PLAN;"
    fixed = "#endif /* KFFT_SPARSE_ENABLE */\n    };\n    return KFFT_RET_IMPROPER_PLAN;"
    assert broken in text
    (tmp_path / "kfft_tiny.h").write_text(text.replace(broken, fixed))
    (tmp_path / "t.c").write_text(TINY_PROGRAM)
    shutil.copy(os.path.join(ROOT, "include", "kfft.h"), tmp_path / "kfft.h")
    shutil.copy(os.path.join(ROOT, "include", "kfft_gb300.h"), tmp_path / "kfft_gb300.h")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", str(tmp_path),
                        str(tmp_path / "t.c"), "-o", str(tmp_path / "t"), lib],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
