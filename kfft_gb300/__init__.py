"""GB300-native FFT engine with the reference kfft C API.

The product is the C-ABI shared library built from ``kfft_gb300/csrc`` (see
``include/kfft.h``).  This package builds it (``build()``) and exposes a thin
ctypes mirror of the C API (``KfftLib``) that the tests and the benchmark use.
There is no CPU fallback: loading fails loudly if the library or a CUDA device
is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB_DIR, build  # noqa: F401

FLAG_NORMAL = 0
FLAG_INVERSE = 1 << 0
FLAG_RENEW = 1 << 1
FLAG_GENERIC = 1 << 2
FLAG_GENERIC_ONLY = 1 << 3
FLAG_EXPAND_SCALAR = 1 << 4
FLAG_DISABLE_NORM = 1 << 5
FLAG_TENSOR_CORES = 1 << 8

RET_SUCCESS = 0
RET_ALLOC_FAIL = 1
RET_BUFFER_FAIL = 2
RET_FREE_NULL = 3
RET_IMPROPER_PLAN = 4
RET_BADARGUMENTS = 5

LIB_NAMES = {"double": "libkfft_gb300.so", "float": "libkfft_gb300_f.so"}

# Every symbol the C headers declare; the CPU tests check that each is exported.
EXPORTED_SYMBOLS = [
    "kfft_pool_create", "kfft_pool_alloc", "kfft_pool_empty", "kfft_pool_zmem",
    "kfft_pool_clear", "kfft_pool_free",
    "kfft_config_cpx", "kfft_eval_cpx",
    "kfft_config_scalar", "kfft_eval_scalar", "kfft_evali_scalar",
    "kfft_info", "kfft_next_fast_size", "kfft_malloc", "kfft_free_null", "kfft_cleanup",
    "kfft_strerr",
    "kfft_config2_cpx", "kfft_eval2_cpx", "kfft_config2_scalar", "kfft_eval2_scalar",
    "kfft_evali2_scalar",
    "kfft_config_conv_cpx", "kfft_eval_conv_cpx", "kfft_config_conv_scalar",
    "kfft_eval_conv_scalar",
    "kfft_config2_conv_cpx", "kfft_eval2_conv_cpx", "kfft_config2_conv_scalar",
    "kfft_eval2_conv_scalar",
    "kfft_eval_cpx_batch", "kfft_eval_cpx_async", "kfft_eval_scalar_batch",
    "kfft_evali_scalar_batch",
    "kfft_config_cpx_uneven", "kfft_eval_cpx_uneven", "kfft_eval_cpx_uneven_async",
    "kfft_uneven_total", "kfft_release_uneven",
    "kfft_gb300_stats", "kfft_gb300_last_error", "kfft_gb300_describe",
    "kfft_eval_cpx_noalloc", "kfft_noalloc_scratch_bytes", "kfft_noalloc_last_message",
    "kfft_shift_cpx", "kfft_shift_scalar", "kfft_shift2_cpx", "kfft_shift2_scalar",
    "kfft_math_hadamard_cpx", "kfft_math_hadamard_scalar", "kfft_math_transpose_cpx",
    "kfft_math_transpose_scalar", "kfft_math_transpose_ip_cpx", "kfft_math_transpose_ip_scalar",
    "kfft_math_magnitude", "kfft_math_magnitude_ip", "kfft_math_average",
    "kfft_variant_count", "kfft_config_cpx_variant", "kfft_tune_set", "kfft_tune_get",
    "kfft_tune_clear",
    "kfft_mlp_create", "kfft_mlp_release", "kfft_mlp_params", "kfft_mlp_get", "kfft_mlp_set",
    "kfft_mlp_predict", "kfft_mlp_loss_grad", "kfft_mlp_train", "kfft_gb300_queue_selftest",
    "kfft_gb300_check_waits", "kfft_gb300_set_bulk_wait_polls",
]


class KfftError(RuntimeError):
    pass


class Stats(ctypes.Structure):
    _fields_ = [("kernel_launches", ctypes.c_uint64), ("graph_launches", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("device", ctypes.c_int32),
                ("last_cuda_error", ctypes.c_int32)]


class InfoT(ctypes.Structure):
    _fields_ = [("vmajor", ctypes.c_uint16), ("vminor", ctypes.c_uint16),
                ("vpatch", ctypes.c_uint16), ("flags", ctypes.c_uint16)]


def library_path(precision: str = "double") -> str:
    """Path of one precision build; KFFT_GB300_LIB_DIR overrides the folder."""
    return os.path.join(os.environ.get("KFFT_GB300_LIB_DIR") or LIB_DIR, LIB_NAMES[precision])


def _ptr(a):
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class KfftLib:
    """ctypes view of one precision build of the engine's C API."""

    def __init__(self, precision: str = "double", path: str | None = None):
        self.precision = precision
        self.path = path or library_path(precision)
        if not os.path.exists(self.path):
            raise KfftError(f"engine library missing: {self.path} (run kfft_gb300.build())")
        self.L = ctypes.CDLL(self.path)
        self.real = np.float32 if precision == "float" else np.float64
        self.cpx = np.complex64 if precision == "float" else np.complex128
        vp, u32, u64, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
        L = self.L
        L.kfft_pool_create.restype = vp
        L.kfft_pool_create.argtypes = [sz]
        L.kfft_pool_alloc.restype = vp
        L.kfft_pool_alloc.argtypes = [vp, sz]
        L.kfft_pool_empty.restype = sz
        L.kfft_pool_empty.argtypes = [vp]
        L.kfft_pool_zmem.argtypes = [vp, vp, sz]
        L.kfft_pool_clear.argtypes = [vp]
        L.kfft_pool_free.argtypes = [vp]
        for n in ("kfft_config_cpx", "kfft_config_scalar", "kfft_config_conv_cpx",
                  "kfft_config_conv_scalar"):
            getattr(L, n).restype = vp
            getattr(L, n).argtypes = [u32, u32, vp, vp]
        for n in ("kfft_config2_cpx", "kfft_config2_scalar", "kfft_config2_conv_cpx",
                  "kfft_config2_conv_scalar"):
            getattr(L, n).restype = vp
            getattr(L, n).argtypes = [u32, u32, u32, vp, vp]
        for n in ("kfft_eval_cpx", "kfft_eval_scalar", "kfft_evali_scalar", "kfft_eval2_cpx",
                  "kfft_eval2_scalar", "kfft_evali2_scalar"):
            getattr(L, n).restype = ctypes.c_uint
            getattr(L, n).argtypes = [vp, vp, vp]
        for n in ("kfft_eval_conv_cpx", "kfft_eval_conv_scalar", "kfft_eval2_conv_cpx",
                  "kfft_eval2_conv_scalar"):
            getattr(L, n).restype = ctypes.c_uint
            getattr(L, n).argtypes = [vp, vp, vp, vp]
        for n in ("kfft_eval_cpx_batch", "kfft_eval_scalar_batch", "kfft_evali_scalar_batch"):
            getattr(L, n).restype = ctypes.c_uint
            getattr(L, n).argtypes = [vp, vp, vp, u32]
        L.kfft_eval_cpx_async.restype = ctypes.c_uint
        L.kfft_eval_cpx_async.argtypes = [vp, vp, vp, u32, vp]
        L.kfft_config_cpx_uneven.restype = vp
        L.kfft_config_cpx_uneven.argtypes = [u32, vp, u32]
        L.kfft_eval_cpx_uneven.restype = ctypes.c_uint
        L.kfft_eval_cpx_uneven.argtypes = [vp, vp, vp]
        L.kfft_eval_cpx_uneven_async.restype = ctypes.c_uint
        L.kfft_eval_cpx_uneven_async.argtypes = [vp, vp, vp, vp]
        L.kfft_uneven_total.restype = u64
        L.kfft_uneven_total.argtypes = [vp]
        L.kfft_release_uneven.argtypes = [vp]
        L.kfft_cleanup.restype = ctypes.c_uint
        L.kfft_cleanup.argtypes = [vp]
        L.kfft_strerr.restype = ctypes.c_char_p
        L.kfft_strerr.argtypes = [ctypes.c_uint]
        L.kfft_next_fast_size.restype = u32
        L.kfft_next_fast_size.argtypes = [u32]
        L.kfft_malloc.restype = vp
        L.kfft_malloc.argtypes = [u32]
        L.kfft_free_null.argtypes = [ctypes.POINTER(vp)]
        L.kfft_info.argtypes = [ctypes.POINTER(InfoT)]
        L.kfft_gb300_stats.argtypes = [ctypes.POINTER(Stats)]
        L.kfft_eval_cpx_noalloc.restype = ctypes.c_uint
        L.kfft_eval_cpx_noalloc.argtypes = [vp, vp, vp, u32, vp]
        L.kfft_noalloc_scratch_bytes.restype = sz
        L.kfft_noalloc_last_message.restype = ctypes.c_char_p
        for n in ("kfft_shift_cpx", "kfft_shift_scalar"):
            getattr(L, n).argtypes = [vp, u32, ctypes.c_bool, vp]
        for n in ("kfft_shift2_cpx", "kfft_shift2_scalar"):
            getattr(L, n).argtypes = [vp, vp, u32, u32, ctypes.c_bool, vp]
        for n in ("kfft_math_hadamard_cpx", "kfft_math_hadamard_scalar", "kfft_math_magnitude"):
            getattr(L, n).argtypes = [vp, vp, u32]
        for n in ("kfft_math_transpose_cpx", "kfft_math_transpose_scalar"):
            getattr(L, n).argtypes = [vp, vp, u32, u32]
        for n in ("kfft_math_transpose_ip_cpx", "kfft_math_transpose_ip_scalar"):
            getattr(L, n).argtypes = [vp, u32, u32]
        L.kfft_math_magnitude_ip.argtypes = [vp, u32]
        L.kfft_math_average.argtypes = [vp, u32]
        L.kfft_math_average.restype = ctypes.c_float if precision == "float" else ctypes.c_double
        L.kfft_variant_count.restype = u32
        L.kfft_config_cpx_variant.restype = vp
        L.kfft_config_cpx_variant.argtypes = [u32, u32, u32, vp, vp]
        L.kfft_tune_set.restype = ctypes.c_uint
        L.kfft_tune_set.argtypes = [u32, u32, u32]
        L.kfft_tune_get.restype = ctypes.c_int
        L.kfft_tune_get.argtypes = [u32, u32]
        fp = ctypes.POINTER(ctypes.c_float)
        L.kfft_mlp_create.restype = vp
        L.kfft_mlp_create.argtypes = [u32, ctypes.c_uint64]
        L.kfft_mlp_release.argtypes = [vp]
        L.kfft_mlp_params.restype = u32
        L.kfft_mlp_params.argtypes = [vp]
        for n in ("kfft_mlp_get", "kfft_mlp_set"):
            getattr(L, n).restype = ctypes.c_uint
            getattr(L, n).argtypes = [vp, vp]
        L.kfft_mlp_predict.restype = ctypes.c_uint
        L.kfft_mlp_predict.argtypes = [vp, vp, u32, vp]
        L.kfft_mlp_loss_grad.restype = ctypes.c_uint
        L.kfft_mlp_loss_grad.argtypes = [vp, vp, vp, u32, fp, vp]
        L.kfft_mlp_train.restype = ctypes.c_uint
        L.kfft_mlp_train.argtypes = [vp, vp, vp, u32, u32, u32, ctypes.c_float, ctypes.c_uint64,
                                     fp]
        L.kfft_gb300_queue_selftest.restype = ctypes.c_int
        L.kfft_gb300_queue_selftest.argtypes = [u32, ctypes.c_int]
        L.kfft_gb300_check_waits.restype = ctypes.c_int
        L.kfft_gb300_check_waits.argtypes = [vp]
        L.kfft_gb300_set_bulk_wait_polls.restype = None
        L.kfft_gb300_set_bulk_wait_polls.argtypes = [u32]
        L.kfft_gb300_last_error.restype = ctypes.c_char_p
        L.kfft_gb300_describe.restype = ctypes.c_char_p
        L.kfft_gb300_describe.argtypes = [vp]

    # ---- service --------------------------------------------------------
    def stats(self) -> Stats:
        s = Stats()
        self.L.kfft_gb300_stats(ctypes.byref(s))
        return s

    def last_error(self) -> str:
        return self.L.kfft_gb300_last_error().decode()

    def describe(self, plan) -> str:
        return self.L.kfft_gb300_describe(plan).decode()

    def info(self) -> InfoT:
        i = InfoT()
        self.L.kfft_info(ctypes.byref(i))
        return i

    def strerr(self, code: int) -> str:
        return self.L.kfft_strerr(code).decode()

    def cleanup(self, plan) -> int:
        return self.L.kfft_cleanup(plan)

    def size_query(self, config: str, *args) -> int:
        n = ctypes.c_size_t(0)
        getattr(self.L, config)(*args, None, ctypes.byref(n))
        return n.value

    def _check(self, r, what):
        if r != RET_SUCCESS:
            raise KfftError(f"{what} returned {r} ({self.strerr(r)}): {self.last_error()}")

    def _plan(self, config, *args):
        p = getattr(self.L, config)(*args, None, None)
        if not p:
            raise KfftError(f"{config}{args} failed: {self.last_error()}")
        return p

    # ---- one-shot helpers (create, eval, release) --------------------------
    def fft_cpx(self, x, flags=0):
        x = np.ascontiguousarray(x, self.cpx)
        p = self._plan("kfft_config_cpx", x.shape[-1], flags)
        try:
            y = np.empty_like(x)
            batch = x.size // max(x.shape[-1], 1)
            self._check(self.L.kfft_eval_cpx_batch(p, _ptr(x), _ptr(y), batch), "eval_cpx_batch")
            return y
        finally:
            self.cleanup(p)

    def rfft(self, x, flags=0):
        x = np.ascontiguousarray(x, self.real)
        n = x.shape[-1]
        batch = x.size // max(n, 1)
        bins = n if (n % 2 or flags & FLAG_EXPAND_SCALAR) else n // 2 + 1
        p = self._plan("kfft_config_scalar", n, flags)
        try:
            y = np.zeros(x.shape[:-1] + (bins,), self.cpx)
            self._check(self.L.kfft_eval_scalar_batch(p, _ptr(x), _ptr(y), batch), "eval_scalar")
            return y
        finally:
            self.cleanup(p)

    def irfft(self, X, n, flags=FLAG_INVERSE):
        X = np.ascontiguousarray(X, self.cpx)
        bins = X.shape[-1]
        batch = X.size // max(bins, 1)
        p = self._plan("kfft_config_scalar", n, flags)
        try:
            y = np.zeros(X.shape[:-1] + (n,), self.real)
            self._check(self.L.kfft_evali_scalar_batch(p, _ptr(X), _ptr(y), batch), "evali_scalar")
            return y
        finally:
            self.cleanup(p)

    def fft2_cpx(self, a, flags=0):
        a = np.ascontiguousarray(a, self.cpx)
        y, x = a.shape
        p = self._plan("kfft_config2_cpx", x, y, flags)
        try:
            out = np.empty_like(a)
            self._check(self.L.kfft_eval2_cpx(p, _ptr(a), _ptr(out)), "eval2_cpx")
            return out
        finally:
            self.cleanup(p)

    def rfft2(self, a, flags=0):
        a = np.ascontiguousarray(a, self.real)
        y, x = a.shape
        p = self._plan("kfft_config2_scalar", x, y, flags)
        try:
            out = np.zeros((y, x), self.cpx)
            self._check(self.L.kfft_eval2_scalar(p, _ptr(a), _ptr(out)), "eval2_scalar")
            return out
        finally:
            self.cleanup(p)

    def irfft2(self, A, flags=FLAG_INVERSE):
        A = np.ascontiguousarray(A, self.cpx)
        y, x = A.shape
        p = self._plan("kfft_config2_scalar", x, y, flags)
        try:
            out = np.zeros((y, x), self.real)
            self._check(self.L.kfft_evali2_scalar(p, _ptr(A), _ptr(out)), "evali2_scalar")
            return out
        finally:
            self.cleanup(p)

    def conv_cpx(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.cpx) for v in (a, b))
        p = self._plan("kfft_config_conv_cpx", a.size, flags)
        try:
            out = np.empty_like(a)
            self._check(self.L.kfft_eval_conv_cpx(p, _ptr(a), _ptr(b), _ptr(out)), "eval_conv_cpx")
            return out
        finally:
            self.cleanup(p)

    def conv_scalar(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.real) for v in (a, b))
        p = self._plan("kfft_config_conv_scalar", a.size, flags)
        try:
            out = np.zeros(a.size, self.real)
            self._check(self.L.kfft_eval_conv_scalar(p, _ptr(a), _ptr(b), _ptr(out)),
                        "eval_conv_scalar")
            return out
        finally:
            self.cleanup(p)

    def conv2_cpx(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.cpx) for v in (a, b))
        y, x = a.shape
        p = self._plan("kfft_config2_conv_cpx", x, y, flags)
        try:
            out = np.empty_like(a)
            self._check(self.L.kfft_eval2_conv_cpx(p, _ptr(a), _ptr(b), _ptr(out)),
                        "eval2_conv_cpx")
            return out
        finally:
            self.cleanup(p)

    def conv2_scalar(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.real) for v in (a, b))
        y, x = a.shape
        p = self._plan("kfft_config2_conv_scalar", x, y, flags)
        try:
            out = np.zeros((y, x), self.real)
            self._check(self.L.kfft_eval2_conv_scalar(p, _ptr(a), _ptr(b), _ptr(out)),
                        "eval2_conv_scalar")
            return out
        finally:
            self.cleanup(p)


_libs: dict[str, KfftLib] = {}


def load(precision: str = "double") -> KfftLib:
    """Returns the engine library of one precision, building it if needed."""
    if precision not in _libs:
        if not os.path.exists(library_path(precision)):
            build()
        _libs[precision] = KfftLib(precision)
    return _libs[precision]
