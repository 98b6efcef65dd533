"""C-ABI boundary checks that need no GPU: the libraries load, export every
symbol the headers declare, keep the reference's pool and size-query protocol
(incs/kfft_algo.h:15-39, kfft_pool.c) and refuse to plan without a device."""
import ctypes
import os
import re

import pytest

import kfft_gb300
from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("kfft.h", "kfft_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        for m in re.finditer(r"KFFT_API\s+[^;(]*?\b(kfft_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module", params=["double", "float"])
def clib(request):
    if not os.path.exists(kfft_gb300.library_path(request.param)):
        kfft_gb300.build()
    return kfft_gb300.KfftLib(request.param)


def test_headers_declare_the_reference_api():
    names = declared_symbols()
    for n in ("kfft_config_cpx", "kfft_eval_cpx", "kfft_config_scalar", "kfft_eval_scalar",
              "kfft_evali_scalar", "kfft_config2_cpx", "kfft_eval2_cpx", "kfft_config2_scalar",
              "kfft_eval2_scalar", "kfft_evali2_scalar", "kfft_config_conv_cpx",
              "kfft_eval_conv_cpx", "kfft_config_conv_scalar", "kfft_eval_conv_scalar",
              "kfft_config2_conv_cpx", "kfft_eval2_conv_cpx", "kfft_config2_conv_scalar",
              "kfft_eval2_conv_scalar", "kfft_cleanup", "kfft_malloc", "kfft_free_null",
              "kfft_info", "kfft_strerr", "kfft_next_fast_size", "kfft_pool_create",
              "kfft_pool_alloc", "kfft_pool_clear", "kfft_pool_free", "kfft_pool_empty",
              "kfft_pool_zmem"):
        assert n in names, n
    assert names == set(kfft_gb300.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(clib):
    for n in declared_symbols():
        assert hasattr(clib.L, n), n


def test_pool_protocol(clib):
    L = clib.L
    P = L.kfft_pool_create(100)
    assert P
    pool = ctypes.cast(P, ctypes.POINTER(ctypes.c_size_t))
    assert L.kfft_pool_empty(P) == 100
    assert not L.kfft_pool_alloc(P, 0)
    assert not L.kfft_pool_alloc(P, 101)
    assert L.kfft_pool_empty(P) == 100
    a = L.kfft_pool_alloc(P, 25)
    b = L.kfft_pool_alloc(P, 25)
    assert a and b and b - a == 25
    assert L.kfft_pool_empty(P) == 50
    assert L.kfft_pool_alloc(P, 50)
    assert L.kfft_pool_empty(P) == 0
    assert not L.kfft_pool_alloc(P, 1)
    L.kfft_pool_clear(P)
    assert L.kfft_pool_empty(P) == 100
    assert pool[0] >= 100  # allocated = header + size
    L.kfft_pool_free(P)
    Z = L.kfft_pool_create(0)
    assert Z and L.kfft_pool_empty(Z) == 0 and not L.kfft_pool_alloc(Z, 1)
    L.kfft_pool_free(Z)


def test_size_query_protocol(clib):
    # N = 0 needs exactly one plan header (api_cpx1.c:26-36); N = 101 more (:38-48)
    s0 = clib.size_query("kfft_config_cpx", 0, 0)
    s101 = clib.size_query("kfft_config_cpx", 101, 0)
    assert s0 > 0 and s101 > s0
    assert clib.size_query("kfft_config_scalar", 100, 0) > 0
    assert clib.size_query("kfft_config2_cpx", 10, 11, 0) > s101
    assert clib.size_query("kfft_config_conv_cpx", 64, 0) > 0
    assert clib.size_query("kfft_config2_conv_scalar", 8, 8, 0) > 0
    # a real conv2d plan of even x also holds the two plans of its
    # half-spectrum inverse: its query exceeds the odd-x one by their sizes
    even = clib.size_query("kfft_config2_conv_scalar", 8, 7, 0)
    odd = clib.size_query("kfft_config2_conv_scalar", 9, 7, 0)
    extra = (clib.size_query("kfft_config_cpx", 7, 1) +
             clib.size_query("kfft_config_scalar", 8, 1))
    base_even = (clib.size_query("kfft_config2_scalar", 8, 7, 0) +
                 clib.size_query("kfft_config2_scalar", 8, 7, 1))
    base_odd = (clib.size_query("kfft_config2_scalar", 9, 7, 0) +
                clib.size_query("kfft_config2_scalar", 9, 7, 1))
    assert even - base_even == odd - base_odd + extra
    # a user pool smaller than the query refuses and reports the size
    n = ctypes.c_size_t(s101 - 1)
    P = clib.L.kfft_pool_create(s101)
    assert not clib.L.kfft_config_cpx(101, 0, P, ctypes.byref(n))
    assert n.value == s101
    clib.L.kfft_pool_free(P)


def test_service_functions(clib):
    L = clib.L
    assert [L.kfft_next_fast_size(n) for n in (1, 7, 11, 97, 1000)] == [1, 8, 12, 100, 1000]
    assert clib.strerr(0) == "Success operation result"
    assert clib.strerr(4) == "Use improper real function for this plan"
    assert clib.strerr(99) == "Unknown return code"
    i = clib.info()
    assert (i.vmajor, i.vminor, i.vpatch) == (0, 8, 1)
    assert bool(i.flags & (1 << 7)) == (clib.precision == "float")
    p = L.kfft_malloc(1000)
    assert p and p % 16 == 0
    pp = ctypes.c_void_p(p)
    L.kfft_free_null(ctypes.byref(pp))
    assert pp.value is None
    assert L.kfft_cleanup(None) == kfft_gb300.RET_FREE_NULL


def test_no_cpu_fallback_without_gpu(clib):
    if gpu_available():
        pytest.skip("a GPU is present")
    assert not clib.L.kfft_config_cpx(64, 0, None, None)
    assert "no CUDA device" in clib.last_error()
    assert clib.stats().device == -1


DYNAPI_NAMES = ["config_cpx", "eval_cpx", "config_scalar", "eval_scalar", "evali_scalar", "info",
                "next_fast_size", "malloc", "free_null", "cleanup", "strerr", "shift_cpx",
                "shift_scalar", "config2_cpx", "eval2_cpx", "shift2_cpx", "config2_scalar",
                "eval2_scalar", "evali2_scalar", "shift2_scalar", "config_conv_cpx",
                "eval_conv_cpx", "config_conv_scalar", "eval_conv_scalar", "config_conv2_cpx",
                "eval_conv2_cpx", "config_conv2_scalar", "eval_conv2_scalar"]
# callback name -> exported function, where the two differ
DYNAPI_TARGET = {"config_conv2_cpx": "config2_conv_cpx", "eval_conv2_cpx": "eval2_conv_cpx",
                 "config_conv2_scalar": "config2_conv_scalar",
                 "eval_conv2_scalar": "eval2_conv_scalar"}


@pytest.mark.parametrize("half", [False, True])
def test_dynapi_callback_types_match_the_functions(tmp_path, half):
    """Every DYNAPI callback typedef (the reference's function-pointer types for
    dynamic loading) is assignable from the engine's function without a cast,
    in both precision builds, and the program links."""
    import shutil
    import subprocess
    lines = ['#include "kfft.h"', "int main(void) {"]
    for n in DYNAPI_NAMES:
        f = "kfft_" + DYNAPI_TARGET.get(n, n)
        lines.append(f"    kfft_callback_{n} p_{n} = {f}; (void)p_{n};")
    lines += ["    return 0;", "}"]
    (tmp_path / "d.c").write_text("\n".join(lines) + "\n")
    lib = kfft_gb300.library_path("float" if half else "double")
    if not os.path.isfile(lib) or shutil.which("gcc") is None:
        pytest.skip("engine library or gcc missing")
    cmd = ["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(tmp_path / "d.c"), "-o", str(tmp_path / "d"), lib]
    if half:
        cmd.insert(1, "-DKFFT_HALF_SCALAR")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("precision", ["double", "float"])
def test_tiny_api_program_compiles_and_links(tmp_path, precision):
    """The tiny-API program (include/kfft_tiny.h) builds with -Wall -Werror
    against either engine build; running it needs a GPU (test_gpu_tiny_api.py)."""
    from tests.test_gpu_tiny_api import build_tiny_program
    lib = os.path.join(ROOT, "kfft_gb300", "lib",
                       "libkfft_gb300.so" if precision == "double" else "libkfft_gb300_f.so")
    if not os.path.isfile(lib):
        pytest.skip("engine library not built")
    exe = build_tiny_program(str(tmp_path), precision)
    assert os.path.isfile(exe)
