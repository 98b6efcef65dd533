"""Benchmark of the GB300 FFT engine (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload uneven|learned_planner|c2c4096|...]

Metric: 5*N*log2(N) GFLOP/s summed over every transform of a step (forward and
inverse counted separately), the reference's own throughput convention
(test/bench/speed/*).  Workloads:

* uneven (default): 4096 complex FP32 sequences in one launch, lengths
  log-uniform in [16, 2^20] snapped to smooth / 11-13-smooth / prime classes,
  ~2^28 points, re/im iid N(0,1), seed 2; one step = forward transform of the
  whole batch.
* c2c4096: 256 complex FP64 sequences of N = 4096, re/im iid U[-1,1), seed 1;
  one step = forward + inverse.

Inputs are resident in HBM for `value`; `e2e` goes through the C ABI with
pinned host buffers (host->device and device->host copies inside the timed
region).  The CPU baseline is the FP64 oracle port (the reference kfft
algorithm restated in C, OpenMP over sequences) on this host's cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def _smooth_candidates(limit, primes):
    vals = {1}
    for p in primes:
        new = set()
        for v in vals:
            x = v
            while x <= limit:
                new.add(x)
                x *= p
        vals = new
    return np.array(sorted(vals))


def _is_prime(n):
    if n < 2:
        return False
    for p in range(2, int(math.isqrt(n)) + 1):
        if n % p == 0:
            return False
    return True


def uneven_lengths(seed=2, count=4096, lo=16, hi=1 << 20, target=1 << 28):
    """Lengths of the uneven-batch workload: log-uniform, snapped by class."""
    rng = np.random.default_rng(seed)
    smooth = _smooth_candidates(hi, [2, 3, 5, 7])
    s7 = smooth
    with1113 = np.array(sorted({int(v * f) for v in s7 for f in (11, 13) if v * f <= hi}))
    raw = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    cls = rng.permutation(np.array([0] * (count // 2) + [1] * (count // 4) +
                                   [2] * (count - count // 2 - count // 4)))
    out = []
    for r, c in zip(raw, cls):
        r = int(round(r))
        if c == 0:
            out.append(int(smooth[np.argmin(np.abs(smooth - r))]))
        elif c == 1:
            out.append(int(with1113[np.argmin(np.abs(with1113 - r))]))
        else:
            k = max(r, 17)
            while not _is_prime(k):
                k += 1
            out.append(k)
    out = np.array(out, dtype=np.int64)
    # rescale to ~target points by dropping the largest sequences
    order = np.argsort(out)
    while out.sum() > target * 1.05 and len(out) > 1:
        out = np.delete(out, np.argmax(out))
    return out.astype(np.uint32)


def uneven_input(total, precision="float", seed=2):
    """Input of the uneven batch, the same in both arms: re/im iid N(0,1) from
    numpy's default_rng(seed), drawn in float32 (complex64) or float64."""
    rng = np.random.default_rng(seed)
    dt = np.float32 if precision == "float" else np.float64
    x = np.empty(total, np.complex64 if precision == "float" else np.complex128)
    x.real = rng.standard_normal(total, dtype=dt)
    x.imag = rng.standard_normal(total, dtype=dt)
    return x


class Workload:
    name = ""
    precision = "double"

    def flops_per_step(self) -> float:
        raise NotImplementedError


class Uniform(Workload):
    """B complex sequences of one length N, forward then inverse per step."""

    def __init__(self, lib, N, B, precision, seed, dist_name, tc=False):
        self.lib = lib
        self.N, self.B, self.precision, self.seed = N, B, precision, seed
        self.dist_name = dist_name
        self.tc = tc and precision == "float"
        tag = "fp64" if precision == "double" else "fp32"
        self.name = f"c2c {tag} N={N} batch {B} forward+inverse" + (
            ", radix-16 stages on tensor cores (FP16 split hi+lo, FP32 accumulate)" if self.tc else "")
        if dist_name == "hdr":
            self.name += ", high-dynamic-range input"

    def _cdt(self):
        return np.complex128 if self.precision == "double" else np.complex64

    def _input(self):
        rng = np.random.default_rng(self.seed)
        shape = (self.B, self.N)
        if self.dist_name == "uniform":
            x = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        elif self.dist_name == "hdr":
            # 32 random tones, amplitudes log-uniform 1e-6..1, random phases, + N(0, 1e-7^2)
            n = np.arange(self.N)
            x = np.zeros(shape, np.complex128)
            for b_ in range(self.B):
                f = rng.integers(0, self.N, 32)
                amp = 10.0 ** rng.uniform(-6, 0, 32)
                ph = rng.uniform(0, 2 * np.pi, 32)
                for k in range(32):
                    x[b_] += amp[k] * np.exp(1j * (2 * np.pi * f[k] * n / self.N + ph[k]))
            x += 1e-7 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        else:
            x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        return x.astype(self._cdt())

    def setup(self, torch, dev, nbuf):
        x = self._input()
        self.host_in = x
        extra = (1 << 8) if self.tc else 0  # KFFT_FLAG_TENSOR_CORES
        self.fwd = self.lib.L.kfft_config_cpx(self.N, 0 | extra, None, None)
        self.inv = self.lib.L.kfft_config_cpx(self.N, 1 | extra, None, None)
        assert self.fwd and self.inv, self.lib.last_error()
        # rotating input buffers: together larger than the 129 MB L2
        self.ins = [torch.from_numpy(x).to(dev) for _ in range(nbuf)]
        self.mid = torch.empty_like(self.ins[0])
        self.out = torch.empty_like(self.ins[0])
        self.pin_in = torch.from_numpy(x).pin_memory()
        self.pin_mid = torch.empty_like(self.pin_in).pin_memory()
        self.pin_out = torch.empty_like(self.pin_in).pin_memory()

    def elem_bytes(self):
        return 16 if self.precision == "double" else 8

    def bytes_per_buffer(self):
        return self.N * self.B * self.elem_bytes()

    def flops_per_step(self):
        return 2 * 5.0 * self.N * math.log2(max(self.N, 2)) * self.B

    def launches_per_step(self):
        return None  # one or more passes per transform; see roofline()

    def algorithmic_bytes_per_launch(self):
        return None

    def algorithmic_bytes_per_step(self):
        return 2 * 2 * self.N * self.B * self.elem_bytes()  # fwd + inv, read + write once

    def step(self, i, stream):
        L = self.lib.L
        x = self.ins[i % len(self.ins)]
        s = ctypes.c_void_p(stream)
        r1 = L.kfft_eval_cpx_async(self.fwd, x.data_ptr(), self.mid.data_ptr(), self.B, s)
        r2 = L.kfft_eval_cpx_async(self.inv, self.mid.data_ptr(), self.out.data_ptr(), self.B, s)
        assert r1 == 0 and r2 == 0

    def step_e2e(self):
        L = self.lib.L
        r1 = L.kfft_eval_cpx_batch(self.fwd, self.pin_in.data_ptr(), self.pin_mid.data_ptr(), self.B)
        r2 = L.kfft_eval_cpx_batch(self.inv, self.pin_mid.data_ptr(), self.pin_out.data_ptr(), self.B)
        assert r1 == 0 and r2 == 0

    def e2e_bytes(self):
        b = self.bytes_per_buffer()
        return 2 * b, 2 * b

    def accuracy(self, oracle_mod, max_seq=4):
        """rel-L2 of the forward transform against the FP64 oracle on the same input."""
        k = min(self.B, max_seq)
        x = np.ascontiguousarray(self.host_in[:k])
        y = np.empty_like(x)
        assert self.lib.L.kfft_eval_cpx_batch(self.fwd, x.ctypes.data, y.ctypes.data, k) == 0
        ref = oracle_mod.fft_cpx(x.astype(np.complex128))
        return {"rel_l2_vs_fp64_oracle": float(np.linalg.norm(y - ref) / np.linalg.norm(ref)),
                "sequences_checked": int(k), "input": self.dist_name}

    def cpu_sample(self, oracle_mod, threads, budget_s=8.0):
        fwd = oracle_mod.CpxPlan(self.N, 0, precision=self.precision)
        inv = oracle_mod.CpxPlan(self.N, 1, precision=self.precision)
        x = self.host_in
        n_done, t0 = 0, time.perf_counter()
        while True:
            y = fwd(x, threads)
            inv(y, threads)
            n_done += 1
            el = time.perf_counter() - t0
            if el > budget_s:
                break
        fwd.close()
        inv.close()
        return self.flops_per_step() * n_done / el / 1e9, f"{n_done} steps of the full workload"


class Config4(Workload):
    """Real, 2D and 2D-convolution shapes through the synchronous C ABI (device buffers
    for `value`, pinned host buffers for `e2e`); one step = forward + inverse
    (real, 2D) or one circular 2D convolution.  These entry points queue on
    the calling thread's stream, so the bench times them there."""

    timing_stream_ptr = 2  # cudaStreamPerThread

    def __init__(self, lib, kind, precision, seed):
        self.lib, self.kind, self.precision, self.seed = lib, kind, precision, seed
        tag = "fp64" if precision == "double" else "fp32"
        if kind == "real":
            self.N, self.B = 1 << 22, 64
            self.name = f"real {tag} N=2^22 batch 64 forward+inverse, U[-1,1)"
        elif kind == "c2d":
            self.X = self.Y = 8192 if precision == "float" else 4096
            self.name = f"2D complex {tag} {self.X}x{self.Y} forward+inverse, N(0,1)"
        else:
            # image 4096^2 U[0,1) and a 63x63 Gaussian (sigma 8, sum 1), both
            # zero-padded to M >= 4096 + 63 - 1 = 4158 for a linear convolution
            self.M = 4160
            self.name = (f"conv2d {tag} image 4096^2 U[0,1) * Gaussian 63x63 sigma 8, "
                         f"zero-padded to {self.M}^2 (circular conv of padded arrays)")

    def _real_t(self):
        return np.float32 if self.precision == "float" else np.float64

    def _cpx_t(self):
        return np.complex64 if self.precision == "float" else np.complex128

    def make_inputs(self):
        """Seeded host inputs (also what the reference arm transforms)."""
        rng = np.random.default_rng(self.seed)
        if self.kind == "real":
            self.host_in = rng.uniform(-1, 1, (self.B, self.N)).astype(self._real_t())
        elif self.kind == "c2d":
            shape = (self.Y, self.X)
            self.host_in = (rng.standard_normal(shape) +
                            1j * rng.standard_normal(shape)).astype(self._cpx_t())
        else:
            M = self.M
            img = np.zeros((M, M), self._real_t())
            img[:4096, :4096] = rng.uniform(0, 1, (4096, 4096))
            g = np.arange(63) - 31
            k = np.exp(-(g[:, None] ** 2 + g[None, :] ** 2) / (2 * 8.0 ** 2))
            ker = np.zeros((M, M), self._real_t())
            ker[:63, :63] = k / k.sum()
            self.host_in, self.host_ker = img, ker

    def setup(self, torch, dev, nbuf):
        self.make_inputs()
        L = self.lib.L
        if self.kind == "real":
            x = self.host_in
            self.fwd = L.kfft_config_scalar(self.N, 0, None, None)
            self.inv = L.kfft_config_scalar(self.N, 1, None, None)
            bins = self.N // 2 + 1
            self.ins = [torch.from_numpy(x).to(dev)]
            self.mid = torch.empty((self.B, bins), dtype=torch.complex64 if self.precision == "float"
                                   else torch.complex128, device=dev)
            self.out = torch.empty_like(self.ins[0])
            self.pin_in = torch.from_numpy(x).pin_memory()
            self.pin_mid = torch.empty(tuple(self.mid.shape), dtype=self.mid.dtype).pin_memory()
            self.pin_out = torch.empty_like(self.pin_in).pin_memory()
        elif self.kind == "c2d":
            x = self.host_in
            self.fwd = L.kfft_config2_cpx(self.X, self.Y, 0, None, None)
            self.inv = L.kfft_config2_cpx(self.X, self.Y, 1, None, None)
            self.ins = [torch.from_numpy(x).to(dev)]
            self.mid = torch.empty_like(self.ins[0])
            self.out = torch.empty_like(self.ins[0])
            self.pin_in = torch.from_numpy(x).pin_memory()
            self.pin_mid = torch.empty_like(self.pin_in).pin_memory()
            self.pin_out = torch.empty_like(self.pin_in).pin_memory()
        else:
            M, img, ker = self.M, self.host_in, self.host_ker
            self.plan = L.kfft_config2_conv_scalar(M, M, 0, None, None)
            self.ins = [torch.from_numpy(img).to(dev)]
            self.ker = torch.from_numpy(ker).to(dev)
            self.out = torch.empty_like(self.ins[0])
            self.pin_in = torch.from_numpy(img).pin_memory()
            self.pin_ker = torch.from_numpy(ker).pin_memory()
            self.pin_out = torch.empty_like(self.pin_in).pin_memory()
        for p in ("fwd", "inv", "plan"):
            if hasattr(self, p):
                assert getattr(self, p), self.lib.last_error()

    def elem_bytes(self):
        return 4 if self.precision == "float" else 8  # one real value

    def flops_per_step(self):
        if self.kind == "real":
            return 2 * 2.5 * self.N * math.log2(self.N) * self.B
        if self.kind == "c2d":
            n = self.X * self.Y
            return 2 * 5.0 * n * math.log2(n)
        n = self.M * self.M
        return 3 * 2.5 * n * math.log2(n)  # two forward and one inverse real 2D transforms

    def algorithmic_bytes_per_step(self):
        s = self.elem_bytes()
        if self.kind == "real":
            return 2 * self.B * (self.N * s + (self.N // 2 + 1) * 2 * s)
        if self.kind == "c2d":
            return 2 * 2 * self.X * self.Y * 2 * s
        return 3 * self.M * self.M * s  # two images read, one written

    def step(self, i, stream):
        L = self.lib.L
        if self.kind == "real":
            r1 = L.kfft_eval_scalar_batch(self.fwd, self.ins[0].data_ptr(), self.mid.data_ptr(), self.B)
            r2 = L.kfft_evali_scalar_batch(self.inv, self.mid.data_ptr(), self.out.data_ptr(), self.B)
        elif self.kind == "c2d":
            r1 = L.kfft_eval2_cpx(self.fwd, self.ins[0].data_ptr(), self.mid.data_ptr())
            r2 = L.kfft_eval2_cpx(self.inv, self.mid.data_ptr(), self.out.data_ptr())
        else:
            r1 = L.kfft_eval2_conv_scalar(self.plan, self.ins[0].data_ptr(), self.ker.data_ptr(),
                                          self.out.data_ptr())
            r2 = 0
        assert r1 == 0 and r2 == 0, (r1, r2, self.lib.last_error())

    def step_e2e(self):
        L = self.lib.L
        if self.kind == "real":
            r1 = L.kfft_eval_scalar_batch(self.fwd, self.pin_in.data_ptr(), self.pin_mid.data_ptr(), self.B)
            r2 = L.kfft_evali_scalar_batch(self.inv, self.pin_mid.data_ptr(), self.pin_out.data_ptr(), self.B)
        elif self.kind == "c2d":
            r1 = L.kfft_eval2_cpx(self.fwd, self.pin_in.data_ptr(), self.pin_mid.data_ptr())
            r2 = L.kfft_eval2_cpx(self.inv, self.pin_mid.data_ptr(), self.pin_out.data_ptr())
        else:
            r1 = L.kfft_eval2_conv_scalar(self.plan, self.pin_in.data_ptr(), self.pin_ker.data_ptr(),
                                          self.pin_out.data_ptr())
            r2 = 0
        assert r1 == 0 and r2 == 0

    def e2e_bytes(self):
        if self.kind == "real":
            a = self.pin_in.numel() * self.elem_bytes()
            b = self.pin_mid.numel() * 2 * self.elem_bytes()
            return a + b, a + b
        if self.kind == "c2d":
            a = self.pin_in.numel() * 2 * self.elem_bytes()
            return 2 * a, 2 * a
        a = self.pin_in.numel() * self.elem_bytes()
        return 2 * a, a

    def accuracy(self, oracle_mod):
        """rel-L2 of the forward result against numpy's FP64 FFT on the same input."""
        L = self.lib.L
        if self.kind == "real":
            x = np.ascontiguousarray(self.host_in[:2])
            y = np.zeros((2, self.N // 2 + 1), self._cpx_t())
            assert L.kfft_eval_scalar_batch(self.fwd, x.ctypes.data, y.ctypes.data, 2) == 0
            ref = np.fft.rfft(x.astype(np.float64), axis=-1)
        elif self.kind == "c2d":
            x = self.host_in
            y = np.empty_like(x)
            assert L.kfft_eval2_cpx(self.fwd, x.ctypes.data, y.ctypes.data) == 0
            ref = np.fft.fft2(x.astype(np.complex128))
        else:
            y = np.empty_like(self.host_in)
            assert L.kfft_eval2_conv_scalar(self.plan, self.host_in.ctypes.data,
                                            self.host_ker.ctypes.data, y.ctypes.data) == 0
            a = self.host_in.astype(np.float64)
            b = self.host_ker.astype(np.float64)
            # the reference's even-length real inverse returns twice the input
            ref = 2.0 * np.fft.irfft2(np.fft.rfft2(a) * np.fft.rfft2(b), s=a.shape)
        return {"rel_l2_vs_fp64": float(np.linalg.norm(y - ref) / np.linalg.norm(ref)),
                "reference": "numpy.fft (FP64, pocketfft) on the same input"}

    def cpu_sample(self, oracle_mod, threads, budget_s=8.0):
        # bounded sample: the oracle's real / 2D / conv2d transforms in FP64 on
        # all host threads, repeated until the budget is spent
        t0 = time.perf_counter()
        calls, flops = 0, 0.0
        if self.kind == "real":
            # rows in parallel on host threads (the oracle's calls release the GIL)
            from concurrent.futures import ThreadPoolExecutor

            def row(b):
                p = self.precision
                oracle_mod.irfft(oracle_mod.rfft(self.host_in[b % self.B], precision=p), self.N,
                                 precision=p)

            with ThreadPoolExecutor(max_workers=threads) as ex:
                while time.perf_counter() - t0 < budget_s:
                    list(ex.map(row, range(calls, calls + threads)))
                    calls += threads
            flops = calls * 2 * 2.5 * self.N * math.log2(self.N)
            el = time.perf_counter() - t0
            return flops / el / 1e9, f"{calls} rows forward+inverse on {threads} threads, {el:.1f}s", threads
        while time.perf_counter() - t0 < budget_s:
            if self.kind == "c2d":
                oracle_mod.fft2_cpx(self.host_in, precision=self.precision)
                flops += 5.0 * self.X * self.Y * math.log2(self.X * self.Y)
            else:
                oracle_mod.conv2_scalar(self.host_in, self.host_ker, precision=self.precision)
                flops += self.flops_per_step()
            calls += 1
        el = time.perf_counter() - t0
        return flops / el / 1e9, f"{calls} oracle calls (OpenMP over rows and columns), {el:.1f}s", threads


CONFIG4_WORKLOADS = {
    "real_f32_2p22x64": lambda lib: Config4(lib, "real", "float", 5),
    "c2d_f32_8192": lambda lib: Config4(lib, "c2d", "float", 6),
    "c2d_f64_4096": lambda lib: Config4(lib, "c2d", "double", 6),
    "conv2d_f32_4096": lambda lib: Config4(lib, "conv2d", "float", 7),
}


def C2C4096(lib):
    return Uniform(lib, 4096, 256, "double", 1, "uniform")


UNIFORM_WORKLOADS = {
    "tc_f32_2p18x64": lambda lib: Uniform(lib, 1 << 18, 64, "float", 3, "normal", tc=True),
    "tc_f32_2p24": lambda lib: Uniform(lib, 1 << 24, 1, "float", 3, "normal", tc=True),
    "tc_f32_2p18x64_hdr": lambda lib: Uniform(lib, 1 << 18, 64, "float", 4, "hdr", tc=True),
    "c2c_f32_2p18x64_hdr": lambda lib: Uniform(lib, 1 << 18, 64, "float", 4, "hdr"),
    "c2c4096": lambda lib: Uniform(lib, 4096, 256, "double", 1, "uniform"),
    "c2c_f32_2p18x64": lambda lib: Uniform(lib, 1 << 18, 64, "float", 3, "normal"),
    "c2c_f32_2p24": lambda lib: Uniform(lib, 1 << 24, 1, "float", 3, "normal"),
    "c2c_f64_2p18x64": lambda lib: Uniform(lib, 1 << 18, 64, "double", 3, "normal"),
    "c2c_f32_4096x4096": lambda lib: Uniform(lib, 4096, 4096, "float", 1, "uniform"),
    "c2c_f32_2p20x16": lambda lib: Uniform(lib, 1 << 20, 16, "float", 3, "normal"),
    "c2c_f64_4096x4096": lambda lib: Uniform(lib, 4096, 4096, "double", 1, "uniform"),
}


class Uneven(Workload):
    precision = "float"

    def __init__(self, lib, precision="float", subset=1):
        self.lib = lib
        self.precision = precision
        self.lengths = np.ascontiguousarray(uneven_lengths()[::subset])
        self.total = int(self.lengths.sum(dtype=np.int64))
        self.name = (f"uneven batch: {len(self.lengths)} complex {'fp32' if precision == 'float' else 'fp64'}"
                     f" sequences, lengths log-uniform in [16, 2^20], {self.total} points, forward")

    def setup(self, torch, dev, nbuf):
        x = torch.from_numpy(uneven_input(self.total, self.precision))
        self.host_in = x
        self.plan = self.lib.L.kfft_config_cpx_uneven(len(self.lengths), self.lengths.ctypes.data, 0)
        assert self.plan, self.lib.last_error()
        self.ins = [x.to(dev)]
        self.out = torch.empty_like(self.ins[0])
        self.pin_in = x.pin_memory()
        self.pin_out = torch.empty_like(x).pin_memory()

    def flops_per_step(self):
        n = self.lengths.astype(np.float64)
        return float(np.sum(5.0 * n * np.log2(np.maximum(n, 2))))

    def launches_per_step(self):
        return None

    def algorithmic_bytes_per_launch(self):
        return None

    def step(self, i, stream):
        r = self.lib.L.kfft_eval_cpx_uneven_async(self.plan, self.ins[0].data_ptr(),
                                                  self.out.data_ptr(), ctypes.c_void_p(stream))
        assert r == 0, self.lib.last_error()

    def step_e2e(self):
        r = self.lib.L.kfft_eval_cpx_uneven(self.plan, self.pin_in.data_ptr(), self.pin_out.data_ptr())
        assert r == 0

    def e2e_bytes(self):
        b = self.total * (8 if self.precision == "float" else 16)
        return b, b

    def accuracy(self, oracle_mod):
        """rel-L2 against an FP64 FFT (numpy's: fast for any prime) on the
        longest sequence of each kind (direct, Rader, Bluestein), and the
        worst over them."""
        x = self.pin_in.numpy()
        y = self.pin_out.numpy()  # the last e2e step's output of this input
        offs = np.concatenate([[0], np.cumsum(self.lengths.astype(np.int64))])
        import kfft_gb300.tuner as T
        picks = {}
        for i, n in enumerate(self.lengths.tolist()):
            inner = T.inner_length(n, max_prime=13)
            kind = "direct" if inner == 0 else ("rader" if inner == n - 1 else "bluestein")
            if kind not in picks or n > self.lengths[picks[kind]]:
                picks[kind] = i
        out = {}
        for kind, i in picks.items():
            a, b = offs[i], offs[i + 1]
            ref = np.fft.fft(x[a:b].astype(np.complex128))
            out[f"{kind}_N{int(self.lengths[i])}"] = float(np.linalg.norm(y[a:b] - ref) / np.linalg.norm(ref))
        out["worst"] = max(out.values())
        out["against"] = "numpy.fft in FP64, longest sequence of each kind"
        return out

    def cpu_sample(self, oracle_mod, threads, budget_s=8.0, every=16):
        """The reference algorithm (oracle port, in the workload's precision)
        on the host cores, OpenMP over sequences, plans built outside the
        timer.  every=1 times the whole batch once; every=k > 1 times every
        k-th sequence, repeated until budget_s is spent."""
        idx = np.arange(0, len(self.lengths), every)
        cache = getattr(self, "_cpu_plans", None)
        if cache is None:
            cache = self._cpu_plans = {}
        if every not in cache:  # plans and sample input built once, outside the timer
            x = np.asarray(self.host_in.numpy())
            if every == 1:
                sub_len, sub = self.lengths, x
            else:
                offs = np.concatenate([[0], np.cumsum(self.lengths.astype(np.int64))])
                sub_len = self.lengths[idx]
                sub = np.concatenate([x[offs[i]:offs[i] + int(self.lengths[i])] for i in idx])
            cache[every] = (sub_len, sub, oracle_mod.UnevenPlan(sub_len, 0, precision=self.precision))
        sub_len, sub, plan = cache[every]
        n = sub_len.astype(np.float64)
        flops_call = float(np.sum(5.0 * n * np.log2(np.maximum(n, 2))))
        calls, t0 = 0, time.perf_counter()
        while True:
            plan(sub, threads)
            calls += 1
            el = time.perf_counter() - t0
            if every == 1 or el > budget_s:
                break
        what = ("the whole batch" if every == 1 else
                f"every {every}th sequence ({len(idx)} of {len(self.lengths)}, {int(n.sum())} points)")
        return flops_call * calls / el / 1e9, f"{what} x{calls}, {el:.2f}s"


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config(wl, ws, nbuf):
    """The `config` object of both arms' lines (the same workload, the same keys)."""
    return {"workload": wl.name, "parallelism": f"replicas x{ws}",
            "l2": "inputs rotate over buffers larger than the 129 MB L2"
            if nbuf > 1 else "working set larger than the 129 MB L2"}


def rotating_buffers(wl):
    if hasattr(wl, "bytes_per_buffer"):
        return max(1, int(math.ceil(268e6 / wl.bytes_per_buffer())))
    return 1


def run_reference(args, ws, rank):
    """The reference algorithm on the host cores: the oracle port in the
    workload's precision (its float flavour follows the reference's float
    build, KFFT_HALF_SCALAR), OpenMP over sequences, plans built outside the
    timer, on the same inputs and for the same metric and config as our arm.
    The uneven batch is timed whole, one batch per step, when the run fits
    about four minutes; otherwise every k-th sequence per step, which the
    line's cpu_baseline.sample states."""
    if rank != 0:
        return
    from oracle import oracle

    class _NoLib:
        L = None
    wl = make_workload(args.workload, _NoLib(), need_lib=False, subset=args.subset,
                       precision=args.precision, batch=args.batch)
    threads = os.cpu_count() or 1
    if isinstance(wl, Uneven):
        import types
        x = uneven_input(wl.total, wl.precision)
        wl.host_in = types.SimpleNamespace(numpy=lambda: x)
    elif hasattr(wl, "make_inputs"):
        wl.make_inputs()
    else:
        wl.host_in = wl._input()
    vals, samples = [], []
    cores = threads
    if isinstance(wl, Uneven):
        # first warm-up step: the whole batch (its plans are built before the timer)
        gf = wl.cpu_sample(oracle, threads, every=1)[0]
        t_batch = wl.flops_per_step() / (gf * 1e9)
        runs = args.steps + args.warmup
        every = 1 if t_batch * runs <= 240.0 else int(math.ceil(t_batch * runs / 240.0))
        for _ in range(args.warmup - 1):
            wl.cpu_sample(oracle, threads, budget_s=0.0, every=every)
        for _ in range(args.steps):
            res = wl.cpu_sample(oracle, threads, budget_s=0.0, every=every)
            vals.append(res[0])
            samples.append(res[1])
        v = statistics.median(vals)
        # the whole batch: the median step time; a sample: extrapolated by flops
        ms = wl.flops_per_step() / (v * 1e9) * 1e3
    else:
        budget = max(2.0, 20.0 / max(args.steps + args.warmup, 1))
        for _ in range(args.warmup):
            wl.cpu_sample(oracle, threads, budget_s=budget / 2)
        for _ in range(args.steps):
            res = wl.cpu_sample(oracle, threads, budget_s=budget)
            vals.append(res[0])
            samples.append(res[1])
            if len(res) > 2:
                cores = res[2]
        v = statistics.median(vals)
        ms = wl.flops_per_step() / (v * 1e9) * 1e3
    line = {"impl": "reference", "metric": "5N*log2N GFLOP/s", "value": round(v, 3),
            "unit": "GFLOP/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if wl.precision == "float" else "f64",
            "data": "synthetic", "config": workload_config(wl, ws, rotating_buffers(wl)),
            "implementation": (f"reference kfft algorithm (oracle port, "
                               f"{'float flavour of the float build' if wl.precision == 'float' else 'double build'}),"
                               f" OpenMP over sequences on {cores} host threads"),
            "cpu_baseline": {"value": round(v, 3), "unit": "GFLOP/s", "cores": cores,
                             "kind": "port", "sample": samples[0]},
            "e2e": {"value": round(v, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_learned_planner(args):
    """Learned-planner sweep: complex fp32 lengths N = 1, 102, 203, ... <= 10^6
    (every `--stride`-th of them), batch ceil(2^24 / N).  Every plan variant of
    every length is timed (the exhaustive tuner); the MLP cost model is trained
    on the timings of 20% of the lengths (chosen by seed) with the engine's own
    CUDA kernels and proposes a variant for each of the other lengths.  The
    line reports the throughput of the proposed plans, of the plain (default)
    plans and of the best measured plans on those lengths, and the regret."""
    import torch
    import kfft_gb300
    from kfft_gb300 import tuner as T

    torch.cuda.set_device(0)
    lib = kfft_gb300.load("float")
    lengths = list(range(1, 1_000_001, 101))[::max(1, args.stride)]
    t0 = time.perf_counter()
    recs = T.exhaustive(lib, lengths, points=1 << 24, reps=max(3, args.steps),
                        warmup=args.warmup)
    sweep_s = time.perf_counter() - t0
    train, test = T.split_lengths(recs, 0.2, seed=7)
    model = T.CostModel(lib, seed=3)
    t1 = time.perf_counter()
    loss = model.fit(train, epochs=300)
    train_s = time.perf_counter() - t1
    r = T.evaluate(model, test)
    if args.tune_db:
        db = T.TuneDB(args.tune_db)
        db.update("float", recs)
        db.save()
        model.save(args.tune_db + ".model.npz")
    model.close()
    n_test = r.lengths
    peak, peak_kind = measured_peaks()
    g = T.by_length(test)
    bytes_total = sum(2 * 8 * n * next(iter(v.values())).batch for n, v in g.items())
    achieved = bytes_total / (r.ms_chosen / 1e3) / 1e9
    line = {"metric": "5N*log2N GFLOP/s", "value": round(r.gflops_chosen, 2), "unit": "GFLOP/s",
            "n_gpus": 1, "steps": n_test, "warmup": args.warmup,
            "ms_per_step": round(r.ms_chosen / max(n_test, 1), 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"learned planner: complex fp32 N = 1 + 101 k <= 10^6, every "
                                   f"{max(1, args.stride)}-th ({len(lengths)} lengths), batch "
                                   f"ceil(2^24/N), one forward transform per length",
                       "l2": "2^24-point launches (128 MB) rotate through one buffer"},
            "learned_planner": {
                "lengths_train": len({x.n for x in train}), "lengths_test": n_test,
                "records": len(recs), "variants": lib.L.kfft_variant_count(),
                "regret_geomean": round(r.geomean_regret, 4), "regret_max": round(r.max_regret, 4),
                "hit_rate": round(r.hit_rate, 4), "gain_vs_plain_geomean": round(r.geomean_gain, 4),
                "gflops_plain": round(r.gflops_default, 2), "gflops_best": round(r.gflops_best, 2),
                "gflops_chosen": round(r.gflops_chosen, 2), "train_loss": round(loss, 5),
                "sweep_s": round(sweep_s, 1), "train_s": round(train_s, 2),
                "worst": [[round(a, 3), int(b), int(c)] for a, b, c in r.worst]},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                         "peak_source": peak_kind, "kernel": "k_pass_reg / k_pass (proposed plans)"}}
    print(json.dumps(line), flush=True)


def make_workload(name, lib, need_lib=True, subset=1, precision="float", batch=0):
    if name in UNIFORM_WORKLOADS:
        wl = UNIFORM_WORKLOADS[name](lib)
    elif name in CONFIG4_WORKLOADS:
        wl = CONFIG4_WORKLOADS[name](lib)
    else:
        return Uneven(lib, precision=precision, subset=subset)
    if batch and hasattr(wl, "B"):
        # profiling only: fewer sequences of the same length (a small ncu case)
        wl.name = wl.name.replace(f"batch {wl.B}", f"batch {batch}")
        wl.B = batch
    return wl


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("KFFT_BENCH_WORKLOAD", "uneven"),
                    choices=["uneven", "learned_planner"] + sorted(UNIFORM_WORKLOADS)
                    + sorted(CONFIG4_WORKLOADS))
    ap.add_argument("--stride", type=int, default=1,
                    help="learned_planner: keep every k-th length of the sweep")
    ap.add_argument("--tune-db", default="",
                    help="learned_planner: write the tuning table (JSON) and model here")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=0,
                    help="profiling only: sequences per step of a uniform or real workload")
    ap.add_argument("--subset", type=int, default=1,
                    help="profiling only: keep every k-th sequence of the uneven batch")
    ap.add_argument("--precision", default="float", choices=["float", "double"],
                    help="uneven workload precision")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.workload == "learned_planner":
        if rank == 0:
            run_learned_planner(args)
        return

    import torch
    import kfft_gb300

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    probe = make_workload(args.workload, None, subset=args.subset, precision=args.precision,
                          batch=args.batch)
    lib = kfft_gb300.load(probe.precision)
    wl = make_workload(args.workload, lib, subset=args.subset, precision=args.precision,
                       batch=args.batch)
    nbuf = rotating_buffers(wl)
    wl.setup(torch, dev, nbuf)
    stream = torch.cuda.Stream(device=dev)
    if getattr(wl, "timing_stream_ptr", None) is not None:
        # synchronous entry points queue on the thread's own stream: time there
        stream = torch.cuda.ExternalStream(wl.timing_stream_ptr, device=dev)
    sptr = stream.cuda_stream

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            wl.step(i, sptr)
    stream.synchronize()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    l0 = lib.stats().kernel_launches
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        start.record(stream)
        for i in range(args.steps):
            wl.step(i, sptr)
        end.record(stream)
        end.synchronize()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    launches = lib.stats().kernel_launches - l0
    ms_total = start.elapsed_time(end)
    ms, value = aggregate_over_ranks(ms_total, wl.flops_per_step(), args.steps, ws, pg, dev)

    # end to end through the C ABI with pinned host buffers.  Each step is
    # timed on its own and the line reports the median: on the shared hosts
    # this runs on, plain pinned copies of the same buffers stall now and
    # then for 20-130 ms (seen with torch's pinned buffers and with
    # registered huge-page buffers alike), which one step in a short mean
    # would carry; the mean and the slowest step are reported beside it.
    for _ in range(max(2, min(args.warmup, 3))):
        wl.step_e2e()
    e2e_steps = max(5, min(args.steps, 10))
    e2e_times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        wl.step_e2e()
        e2e_times.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = float(np.median(e2e_times))
    h2d, d2h = wl.e2e_bytes()
    e2e_val = ws * wl.flops_per_step() / (e2e_ms / 1e3) / 1e9

    peak, peak_kind = measured_peaks()
    roof = dominant_kernel_roofline(wl, ms, lib, peak, peak_kind,
                                    launches_per_step=launches / max(args.steps, 1),
                                    workload=args.workload)
    line = {"metric": "5N*log2N GFLOP/s", "value": round(value, 2), "unit": "GFLOP/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if wl.precision == "float" else "f64",
            "data": "synthetic",
            "config": workload_config(wl, ws, nbuf),
            "e2e": {"value": round(e2e_val, 2), "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 3),
                    "steps": e2e_steps, "stat": "median of per-step wall times",
                    "ms_per_step_mean": round(float(np.mean(e2e_times)), 3),
                    "ms_per_step_max": round(float(np.max(e2e_times)), 3)},
            "gpu_launches": int(launches), "roofline": roof, "clocks": clk.summary()}
    if rank == 0 and hasattr(wl, "accuracy"):
        from oracle import oracle as _oracle
        line["accuracy"] = wl.accuracy(_oracle)
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle
        threads = os.cpu_count() or 1
        res = wl.cpu_sample(oracle, threads)
        v, sample = res[0], res[1]
        cores = res[2] if len(res) > 2 else threads  # the threads the sample really used
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "GFLOP/s", "cores": cores,
                                "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


def aggregate_over_ranks(ms_total, flops_per_step, steps, world, dist=None, device="cpu"):
    """Max step time over ranks and the whole-job throughput (weak scaling:
    every rank runs the full per-GPU workload, replicas only)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(ms_total)], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    ms = ms_total / steps
    return ms, world * flops_per_step / (ms / 1e3) / 1e9


# DRAM bytes per launch of the dominant kernel from ncu captures
# (dram__bytes_read.sum + dram__bytes_write.sum, averaged over the captured
# pass launches).  The uneven batch is too large for a full-set capture:
# every 8th sequence was captured (37.47 M points, 2.708 GB) and scaled by
# points, which the same length mix allows.
NCU_DRAM_BYTES_PER_POINT = {"uneven_float": 2.708141e9 / 37465227,
                            "uneven_double": 5.925791e9 / 37465227}
NCU_DRAM_BYTES_PER_LAUNCH = {"c2c_f32_4096x4096": 217.3e6, "c2c_f32_2p18x64": 216.7e6,
                             "c2c_f32_2p20x16": 215.7e6, "c2c_f32_2p24": 215.9e6,
                             "c2c4096": 18.7e6}


def dominant_kernel_roofline(wl, ms_step, lib, peak, peak_kind, launches_per_step=None,
                             workload=""):
    """Roofline of the dominant kernel: algorithmic bytes of one launch (read +
    write every point it transforms once) over the average launch time."""
    es = 8 if wl.precision == "float" else 16
    if isinstance(wl, Config4):
        # several kernels per step (passes, real pre/post, transposes,
        # spectrum product): the algorithmic bytes of the step over its time
        achieved = wl.algorithmic_bytes_per_step() / (ms_step / 1e3) / 1e9
        return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                "kernel": "all launches of the step (per step, not per launch)",
                "launches_per_step": launches_per_step}
    if hasattr(wl, "algorithmic_bytes_per_step"):
        # uniform batches: every pass launch reads and writes every point once
        n = max(1, int(round(launches_per_step or 1)))
        per_launch = 2 * wl.N * wl.B * es
        dur = ms_step / n
        achieved = per_launch / (dur / 1e3) / 1e9
        per_transform = wl.algorithmic_bytes_per_step() / (ms_step / 1e3) / 1e9
        traffic = NCU_DRAM_BYTES_PER_LAUNCH.get(workload)
        generic = wl.precision == "double" or getattr(wl, "tc", False)
        kernel = ("k_pass_reg (one launch per pass)" if generic else
                  "k_pass_bulk / k_pass_pipe / k_pass_pipe_wide (one launch per pass)")
        return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": kernel,
                "launches_per_step": n, "launch_ms": round(dur, 4),
                "per_transform_gbs": round(per_transform, 1)}
    # the uneven batch: one k_persistent launch runs every pass of every sequence
    total_bytes = wl.total * es * 2
    achieved = total_bytes / (ms_step / 1e3) / 1e9
    ratio = NCU_DRAM_BYTES_PER_POINT.get(f"uneven_{wl.precision}")
    traffic = round(ratio * wl.total) if ratio else None
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "peak_source": peak_kind, "kernel": "k_persistent (all passes of the batch)"}


if __name__ == "__main__":
    main()
