"""TEST INFRASTRUCTURE ONLY: numpy front end of the FP64 CPU oracle.

The oracle (``kfft_oracle.c``) restates the reference kfft transform path in
plain C.  This module compiles it with gcc when its shared object is missing
and exposes numpy-level calls.  Only the tests, the smoke check and the CPU
baseline leg of the benchmark import it; the product library never does.

It also wraps the reference library itself (``oracle/_ref/libkfft_ref*.so``)
when that was built by ``oracle/build_ref.sh`` (only possible where the
reference sources are present), for pinning the oracle and for fixtures.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
SO_PATH = os.path.join(BUILD_DIR, "libkfft_oracle.so")
# float flavour: the same source compiled with -DORACLE_FLOAT, following the
# reference's float build; only a timed baseline, never a checker
SO_PATH_F = os.path.join(BUILD_DIR, "libkfft_oracle_f.so")
REF_DIR = os.path.join(HERE, "_ref")

FLAG_NORMAL = 0
FLAG_INVERSE = 1 << 0
FLAG_RENEW = 1 << 1
FLAG_GENERIC = 1 << 2
FLAG_GENERIC_ONLY = 1 << 3
FLAG_EXPAND_SCALAR = 1 << 4
FLAG_DISABLE_NORM = 1 << 5

_lock = threading.Lock()
_libs = {}


def build(force: bool = False, precision: str = "double") -> str:
    """Compile the oracle C restatement into oracle/_build (gcc, OpenMP); the
    float flavour with -DORACLE_FLOAT."""
    src = os.path.join(HERE, "kfft_oracle.c")
    hdr = os.path.join(HERE, "kfft_oracle.h")
    so = SO_PATH_F if precision == "float" else SO_PATH
    if (not force and os.path.exists(so)
            and os.path.getmtime(so) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return so
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = so + f".tmp{os.getpid()}"
    cmd = ["gcc", "-std=gnu11", "-O3", "-fPIC", "-fopenmp", "-shared", "-o", tmp, src, "-lm"]
    if precision == "float":
        cmd.insert(1, "-DORACLE_FLOAT")
    subprocess.run(cmd, check=True)
    os.replace(tmp, so)
    return so


def build_all(force: bool = False) -> None:
    build(force, "double")
    build(force, "float")


def _load(precision: str = "double"):
    with _lock:
        if precision in _libs:
            return _libs[precision]
        lib = ctypes.CDLL(build(precision=precision))
        vp, u32, i32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64
        lib.oracle_plan_cpx.restype = vp
        lib.oracle_plan_cpx.argtypes = [u32, u32]
        lib.oracle_plan_free.argtypes = [vp]
        lib.oracle_exec_cpx_batch.argtypes = [vp, vp, vp, u64, i32]
        for name in ("oracle_fft_cpx", "oracle_rfft", "oracle_irfft", "oracle_conv_cpx",
                     "oracle_conv_scalar"):
            getattr(lib, name).restype = i32
        lib.oracle_fft_cpx.argtypes = [u32, u32, vp, vp]
        lib.oracle_rfft.argtypes = [u32, u32, vp, vp]
        lib.oracle_irfft.argtypes = [u32, u32, vp, vp]
        lib.oracle_fft2_cpx.argtypes = [u32, u32, u32, vp, vp]
        lib.oracle_rfft2.argtypes = [u32, u32, u32, vp, vp]
        lib.oracle_irfft2.argtypes = [u32, u32, u32, vp, vp]
        lib.oracle_conv_cpx.argtypes = [u32, u32, vp, vp, vp]
        lib.oracle_conv_scalar.argtypes = [u32, u32, vp, vp, vp]
        lib.oracle_conv2_cpx.argtypes = [u32, u32, u32, vp, vp, vp]
        lib.oracle_conv2_scalar.argtypes = [u32, u32, u32, vp, vp, vp]
        lib.oracle_dft_exact.argtypes = [u32, i32, vp, vp]
        lib.oracle_exec_uneven.argtypes = [u32, vp, u32, vp, vp, i32]
        lib.oracle_uneven_create.restype = vp
        lib.oracle_uneven_create.argtypes = [u32, vp, u32]
        lib.oracle_uneven_exec.argtypes = [vp, vp, vp, i32]
        lib.oracle_uneven_free.argtypes = [vp]
        _libs[precision] = lib
        return lib


def _c128(a, precision: str = "double"):
    return np.ascontiguousarray(a, dtype=np.complex64 if precision == "float" else np.complex128)


def _f64(a, precision: str = "double"):
    return np.ascontiguousarray(a, dtype=np.float32 if precision == "float" else np.float64)


def _check(r, what):
    if r != 0:
        raise RuntimeError(f"oracle {what} returned {r}")


class CpxPlan:
    """An oracle complex plan of one length, reusable over a batch."""

    def __init__(self, nfft: int, flags: int = 0, precision: str = "double"):
        self.lib = _load(precision)
        self.precision = precision
        self.nfft = nfft
        self.ptr = self.lib.oracle_plan_cpx(nfft, flags)
        if not self.ptr:
            raise MemoryError("oracle plan allocation failed")

    def __call__(self, x, threads: int = 0):
        x = _c128(x, self.precision)
        batch = x.size // max(self.nfft, 1)
        y = np.empty_like(x)
        _check(self.lib.oracle_exec_cpx_batch(self.ptr, x.ctypes.data, y.ctypes.data,
                                              batch, threads), "exec_cpx_batch")
        return y

    def close(self):
        if self.ptr:
            self.lib.oracle_plan_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fft_cpx(x, flags: int = 0, precision: str = "double"):
    """kfft_eval_cpx on one or more rows (last axis = sequence)."""
    x = _c128(x, precision)
    n = x.shape[-1]
    p = CpxPlan(n, flags, precision)
    try:
        return p(x).reshape(x.shape)
    finally:
        p.close()


def rfft(x, flags: int = 0, precision: str = "double"):
    lib = _load(precision)
    x = _f64(x, precision)
    n = x.size
    cdt = np.complex64 if precision == "float" else np.complex128
    out = np.zeros(n if (flags & FLAG_EXPAND_SCALAR or n % 2) else n // 2 + 1, cdt)
    if n % 2 == 0 and not flags & FLAG_EXPAND_SCALAR:
        buf = np.zeros(n // 2 + 1, cdt)
    else:
        buf = np.zeros(max(n, n // 2 + 1), cdt)
    _check(lib.oracle_rfft(n, flags, x.ctypes.data, buf.ctypes.data), "rfft")
    return buf[: out.size].copy()


def irfft(X, n: int, flags: int = FLAG_INVERSE, precision: str = "double"):
    lib = _load(precision)
    X = _c128(X, precision)
    need = n if n % 2 else n // 2 + 1
    if X.size < need:
        raise ValueError("spectrum too short")
    out = np.zeros(n + 2, np.float32 if precision == "float" else np.float64)
    _check(lib.oracle_irfft(n, flags, X.ctypes.data, out.ctypes.data), "irfft")
    return out[:n].copy()


def fft2_cpx(a, flags: int = 0, precision: str = "double"):
    """2D complex transform of a (y, x) row-major array (x contiguous)."""
    lib = _load(precision)
    a = _c128(a, precision)
    y, x = a.shape
    out = np.empty_like(a)
    _check(lib.oracle_fft2_cpx(x, y, flags, a.ctypes.data, out.ctypes.data), "fft2_cpx")
    return out


def rfft2(a, flags: int = 0):
    lib = _load()
    a = _f64(a)
    y, x = a.shape
    out = np.zeros((y, x), np.complex128)
    _check(lib.oracle_rfft2(x, y, flags, a.ctypes.data, out.ctypes.data), "rfft2")
    return out


def irfft2(A, flags: int = FLAG_INVERSE):
    lib = _load()
    A = _c128(A)
    y, x = A.shape
    out = np.zeros((y, x), np.float64)
    _check(lib.oracle_irfft2(x, y, flags, A.ctypes.data, out.ctypes.data), "irfft2")
    return out


def conv_cpx(a, b, flags: int = 0):
    lib = _load()
    a, b = _c128(a), _c128(b)
    out = np.empty_like(a)
    _check(lib.oracle_conv_cpx(a.size, flags, a.ctypes.data, b.ctypes.data, out.ctypes.data),
           "conv_cpx")
    return out


def conv_scalar(a, b, flags: int = 0):
    lib = _load()
    a, b = _f64(a), _f64(b)
    out = np.zeros(a.size + 2, np.float64)
    _check(lib.oracle_conv_scalar(a.size, flags, a.ctypes.data, b.ctypes.data,
                                  out.ctypes.data), "conv_scalar")
    return out[: a.size].copy()


def conv2_cpx(a, b, flags: int = 0):
    lib = _load()
    a, b = _c128(a), _c128(b)
    y, x = a.shape
    out = np.empty_like(a)
    _check(lib.oracle_conv2_cpx(x, y, flags, a.ctypes.data, b.ctypes.data, out.ctypes.data),
           "conv2_cpx")
    return out


def conv2_scalar(a, b, flags: int = 0, precision: str = "double"):
    lib = _load(precision)
    a, b = _f64(a, precision), _f64(b, precision)
    y, x = a.shape
    out = np.zeros((y, x), np.float32 if precision == "float" else np.float64)
    _check(lib.oracle_conv2_scalar(x, y, flags, a.ctypes.data, b.ctypes.data,
                                   out.ctypes.data), "conv2_scalar")
    return out


def fft_uneven(lengths, x, flags: int = 0, threads: int = 0):
    """Transforms sequences of the given lengths packed back to back."""
    lib = _load()
    lengths = np.ascontiguousarray(lengths, dtype=np.uint32)
    x = _c128(x)
    if x.size != int(lengths.sum(dtype=np.int64)):
        raise ValueError("input size does not match the lengths")
    y = np.empty_like(x)
    _check(lib.oracle_exec_uneven(lengths.size, lengths.ctypes.data, flags, x.ctypes.data,
                                  y.ctypes.data, threads), "exec_uneven")
    return y


class UnevenPlan:
    """Oracle plans for a packed batch of uneven lengths, built once."""

    def __init__(self, lengths, flags: int = 0, precision: str = "double"):
        self.lib = _load(precision)
        self.precision = precision
        self.lengths = np.ascontiguousarray(lengths, dtype=np.uint32)
        self.total = int(self.lengths.sum(dtype=np.int64))
        self.ptr = self.lib.oracle_uneven_create(self.lengths.size, self.lengths.ctypes.data, flags)
        if not self.ptr:
            raise MemoryError("oracle uneven plan failed")

    def __call__(self, x, threads: int = 0):
        x = _c128(x, self.precision)
        if x.size != self.total:
            raise ValueError("input size does not match the lengths")
        y = np.empty_like(x)
        _check(self.lib.oracle_uneven_exec(self.ptr, x.ctypes.data, y.ctypes.data, threads),
               "uneven_exec")
        return y

    def close(self):
        if self.ptr:
            self.lib.oracle_uneven_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dft_exact(x, inverse: bool = False):
    """O(N^2) long-double DFT with integer phase reduction (small N only)."""
    lib = _load()
    x = _c128(x)
    out = np.empty_like(x)
    lib.oracle_dft_exact(x.size, int(inverse), x.ctypes.data, out.ctypes.data)
    return out


# ---------------------------------------------------------------------------
# post-transform helpers: fftshift and the kfft_math API (index arithmetic,
# restated in numpy; no floating-point rounding beyond one operation each)
# ---------------------------------------------------------------------------
def shift(a, inverse: bool = False):
    """fftshift (forward) / ifftshift (inverse) of every axis of a 1D or 2D array.

    Follows kfft_shift.c:4-31 for one axis: an odd length n = 2c+1 moves
    element (i + c + 1) mod n to i going forward and (i + c) mod n going
    back; an even length swaps its halves both ways (the intent of
    kfft_shift.c:10-11, whose swap macro zeroes the data in the reference
    build).  2D arrays (sz_y rows of sz_x) are shifted along the rows, then
    along the columns, as ext/2d/kfft_cpx2.c:188-226 does through transposes.
    """
    a = np.asarray(a)
    out = a
    for ax in range(a.ndim):
        n = a.shape[ax]
        c = n // 2
        k = c if inverse else (n - c)
        # new[i] = old[(i + k) mod n]
        out = np.roll(out, -k, axis=ax)
    return out


def magnitude(z):
    """|z| = sqrt(re^2 + im^2) per element in the working precision (kfft_math.h:153-155)."""
    z = np.asarray(z)
    r = z.real
    i = z.imag
    return np.sqrt(r * r + i * i)


def average(v):
    """Sum of the elements in index order, divided by the count (kfft_math.c:139-148)."""
    v = np.asarray(v)
    acc = v.dtype.type(0)
    for e in v.tolist():
        acc = v.dtype.type(acc + e)
    return v.dtype.type(acc / v.dtype.type(len(v)))


def transpose(a):
    """Fout[i][j] = Fin[j][i] for Fin of y rows by x columns (kfft_math.c:60-78)."""
    return np.ascontiguousarray(np.asarray(a).T)


# ---------------------------------------------------------------------------
# The reference library itself (present only where oracle/build_ref.sh ran).
# ---------------------------------------------------------------------------
def ref_library_path(precision: str = "double") -> str | None:
    name = {"double": "libkfft_ref.so", "float": "libkfft_ref_f.so",
            "default": "libkfft_ref_default.so"}[precision]
    p = os.path.join(REF_DIR, name)
    if not os.path.exists(p):
        return None
    try:
        ctypes.CDLL(p)
    except OSError:
        return None
    return p


class RefLib:
    """ctypes view of the reference kfft C API (the upstream library built from source)."""

    def __init__(self, precision: str = "double"):
        path = ref_library_path(precision)
        if path is None:
            raise FileNotFoundError("reference library not built (oracle/build_ref.sh)")
        self.lib = ctypes.CDLL(path)
        self.real = np.float32 if precision == "float" else np.float64
        self.cpx = np.complex64 if precision == "float" else np.complex128
        vp, u32 = ctypes.c_void_p, ctypes.c_uint32
        L = self.lib
        for name in ("kfft_config_cpx", "kfft_config_scalar", "kfft_config_conv_cpx",
                     "kfft_config_conv_scalar"):
            getattr(L, name).restype = vp
            getattr(L, name).argtypes = [u32, u32, vp, vp]
        for name in ("kfft_config2_cpx", "kfft_config2_scalar", "kfft_config2_conv_cpx",
                     "kfft_config2_conv_scalar"):
            getattr(L, name).restype = vp
            getattr(L, name).argtypes = [u32, u32, u32, vp, vp]
        for name in ("kfft_eval_cpx", "kfft_eval_scalar", "kfft_evali_scalar", "kfft_eval2_cpx",
                     "kfft_eval2_scalar", "kfft_evali2_scalar"):
            getattr(L, name).argtypes = [vp, vp, vp]
        for name in ("kfft_eval_conv_cpx", "kfft_eval_conv_scalar", "kfft_eval2_conv_cpx",
                     "kfft_eval2_conv_scalar"):
            getattr(L, name).argtypes = [vp, vp, vp, vp]
        L.kfft_cleanup.argtypes = [vp]

    def _run(self, cfg, args, ev, ins, out):
        p = getattr(self.lib, cfg)(*args, None, None)
        if not p:
            raise MemoryError(cfg)
        try:
            r = getattr(self.lib, ev)(p, *[a.ctypes.data for a in ins], out.ctypes.data)
        finally:
            self.lib.kfft_cleanup(p)
        if r != 0:
            raise RuntimeError(f"{ev} returned {r}")
        return out

    def fft_cpx(self, x, flags=0):
        x = np.ascontiguousarray(x, self.cpx)
        return self._run("kfft_config_cpx", (x.size, flags), "kfft_eval_cpx", [x],
                         np.empty_like(x))

    def rfft(self, x, flags=0):
        x = np.ascontiguousarray(x, self.real)
        n = x.size
        out = np.zeros(max(n, n // 2 + 1), self.cpx)
        self._run("kfft_config_scalar", (n, flags), "kfft_eval_scalar", [x], out)
        return out if (flags & FLAG_EXPAND_SCALAR or n % 2) else out[: n // 2 + 1].copy()

    def irfft(self, X, n, flags=FLAG_INVERSE):
        X = np.ascontiguousarray(X, self.cpx)
        out = np.zeros(n + 2, self.real)
        self._run("kfft_config_scalar", (n, flags), "kfft_evali_scalar", [X], out)
        return out[:n].copy()

    def fft2_cpx(self, a, flags=0):
        a = np.ascontiguousarray(a, self.cpx)
        y, x = a.shape
        return self._run("kfft_config2_cpx", (x, y, flags), "kfft_eval2_cpx", [a],
                         np.empty_like(a))

    def rfft2(self, a, flags=0):
        a = np.ascontiguousarray(a, self.real)
        y, x = a.shape
        return self._run("kfft_config2_scalar", (x, y, flags), "kfft_eval2_scalar", [a],
                         np.zeros((y, x), self.cpx))

    def irfft2(self, A, flags=FLAG_INVERSE):
        A = np.ascontiguousarray(A, self.cpx)
        y, x = A.shape
        return self._run("kfft_config2_scalar", (x, y, flags), "kfft_evali2_scalar", [A],
                         np.zeros((y, x), self.real))

    def conv_cpx(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.cpx) for v in (a, b))
        return self._run("kfft_config_conv_cpx", (a.size, flags), "kfft_eval_conv_cpx", [a, b],
                         np.empty_like(a))

    def conv_scalar(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.real) for v in (a, b))
        out = np.zeros(a.size + 2, self.real)
        self._run("kfft_config_conv_scalar", (a.size, flags), "kfft_eval_conv_scalar", [a, b],
                  out)
        return out[: a.size].copy()

    def conv2_cpx(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.cpx) for v in (a, b))
        y, x = a.shape
        return self._run("kfft_config2_conv_cpx", (x, y, flags), "kfft_eval2_conv_cpx", [a, b],
                         np.empty_like(a))

    def conv2_scalar(self, a, b, flags=0):
        a, b = (np.ascontiguousarray(v, self.real) for v in (a, b))
        y, x = a.shape
        return self._run("kfft_config2_conv_scalar", (x, y, flags), "kfft_eval2_conv_scalar",
                         [a, b], np.zeros((y, x), self.real))
