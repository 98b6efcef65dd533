"""Plan tuner of the GB300 FFT engine: exhaustive timing and a learned cost model.

The reference plans every length one way (kfft_generic.c:129-151 picks the
factorisation, kfft_cpx.c:315-366 builds the plan).  The engine can build
each length several ways (``kfft_variant_count()`` plan variants: largest
pass length, lanes per tile, fused register tiles or shared-memory tiles,
tensor-core radix-16 stages) and every variant computes the same transform.
This module chooses between them.

* ``exhaustive`` times every distinct variant of every length on the GPU (CUDA
  events on the launching stream, device-resident buffers, median of a few
  launches) and returns the records.  It is the fallback of the learned model
  and the yardstick its regret is measured against.
* ``CostModel`` is a 3-layer 64-wide MLP trained by the engine's own CUDA
  kernels (``kfft_mlp_train``) on the log launch time of (length, variant)
  records.  Features: log2 N, log2 batch, precision, the exponents of the
  primes 2..13 in N, the count of larger prime factors, log2 of the largest
  prime, the same block for the inner length of a Rader/Bluestein plan, and
  the variant (one-hot).  It proposes a variant for lengths it has never
  timed; it only ranks plans and never touches the transform arithmetic.
* ``TuneDB`` persists the winners as JSON and installs them into the
  library's tuning table (``kfft_tune_set``), after which plain
  ``kfft_config_cpx`` calls use them.
* ``evaluate`` measures the model's regret (time of the proposed plan over
  the best measured time) and its gain over the built-in default plan.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

SMALL_PRIMES = (2, 3, 5, 7, 11, 13)
FLAG_TENSOR_CORES = 1 << 8
MAX_DIRECT_PRIME = 31


# ---------------------------------------------------------------------------
# features
# ---------------------------------------------------------------------------
def factorize(n: int) -> dict[int, int]:
    f: dict[int, int] = {}
    d = 2
    while d * d <= n:
        while n % d == 0:
            f[d] = f.get(d, 0) + 1
            n //= d
        d += 1
    if n > 1:
        f[n] = f.get(n, 0) + 1
    return f


def _smooth7(m: int) -> bool:
    for p in (2, 3, 5, 7):
        while m % p == 0:
            m //= p
    return m == 1


def inner_length(n: int, max_prime: int = MAX_DIRECT_PRIME) -> int:
    """Length of the nested transform a non-direct plan runs (0 for direct plans).

    Follows the engine's planner: a length whose prime factors are all at most
    ``max_prime`` is direct; a prime whose p-1 is direct runs Rader on p-1;
    anything else runs Bluestein on a 7-smooth M >= 2n-1.  The feature uses
    the smallest such M; the planner may take a slightly longer one that needs
    fewer or cheaper passes, which changes the feature's scale very little.
    """
    def direct(m):
        return m <= 1 or all(q <= max_prime for q in factorize(m))

    if direct(n):
        return 0
    f = factorize(n)
    if len(f) == 1 and next(iter(f.values())) == 1 and direct(n - 1):
        return n - 1
    m = 2 * n - 1
    while not _smooth7(m):
        m += 1
    return m


def _prime_block(n: int) -> list[float]:
    f = factorize(n) if n > 1 else {}
    exps = [float(f.get(p, 0)) for p in SMALL_PRIMES]
    larger = float(sum(e for p, e in f.items() if p > SMALL_PRIMES[-1]))
    big = max(f) if f else 1
    return exps + [larger, math.log2(big)]


N_BASE_FEATURES = 3 + 2 * (len(SMALL_PRIMES) + 2)


def features(n: int, batch: int, precision: str, variant: int, n_variants: int) -> np.ndarray:
    inner = inner_length(n)
    v = [math.log2(max(n, 1)), math.log2(max(batch, 1)), 1.0 if precision == "float" else 0.0]
    v += _prime_block(n)
    v += _prime_block(inner) if inner else [0.0] * (len(SMALL_PRIMES) + 2)
    onehot = [0.0] * n_variants
    onehot[variant] = 1.0
    return np.asarray(v + onehot, dtype=np.float32)


# ---------------------------------------------------------------------------
# exhaustive timing
# ---------------------------------------------------------------------------
@dataclass
class Record:
    n: int
    batch: int
    variant: int
    plan: str
    ms: float


def batch_for(n: int, points: int) -> int:
    return max(1, -(-points // n))


def exhaustive(lib, lengths, points: int = 1 << 24, reps: int = 5, warmup: int = 2,
               allow_tc: bool = False, flags: int = 0, progress=None) -> list[Record]:
    """Time every distinct plan variant of every length (batch = ceil(points/n)).

    Variants whose plans describe identically share one measurement.  Inputs
    are device-resident; for the default 2^24 points they exceed the L2.
    """
    import torch

    cdt = torch.complex64 if lib.precision == "float" else torch.complex128
    cap = max(batch_for(int(n), points) * int(n) for n in lengths)
    gen = torch.Generator(device="cuda").manual_seed(11)
    xbuf = torch.randn(cap, dtype=cdt, device="cuda", generator=gen)
    ybuf = torch.empty_like(xbuf)
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    L = lib.L
    nvar = L.kfft_variant_count()
    vflags = flags | (FLAG_TENSOR_CORES if (allow_tc and lib.precision == "float") else 0)
    out: list[Record] = []
    for i, n in enumerate(lengths):
        n = int(n)
        batch = batch_for(n, points)
        seen: dict[str, float] = {}
        for v in range(nvar):
            plan = L.kfft_config_cpx_variant(n, vflags, v, None, None)
            if not plan:
                continue  # variant not allowed for these flags
            try:
                desc = lib.describe(plan)
                if desc not in seen:
                    seen[desc] = _time_plan(lib, plan, xbuf, ybuf, batch, n, stream, sp,
                                            reps, warmup)
                out.append(Record(n, batch, v, desc, seen[desc]))
            finally:
                lib.cleanup(plan)
        if progress:
            progress(i, n)
    return out


def _time_plan(lib, plan, xbuf, ybuf, batch, n, stream, sp, reps, warmup) -> float:
    import torch

    x = xbuf[: batch * n]
    y = ybuf[: batch * n]
    L = lib.L
    for _ in range(warmup):
        r = L.kfft_eval_cpx_async(plan, x.data_ptr(), y.data_ptr(), batch, sp)
        if r != 0:
            raise RuntimeError(f"eval failed for n={n}: {lib.strerr(r)} {lib.last_error()}")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    stream.synchronize()
    for a, b in ev:
        a.record(stream)
        L.kfft_eval_cpx_async(plan, x.data_ptr(), y.data_ptr(), batch, sp)
        b.record(stream)
    stream.synchronize()
    times = sorted(a.elapsed_time(b) for a, b in ev)
    return float(times[len(times) // 2])


# ---------------------------------------------------------------------------
# learned cost model
# ---------------------------------------------------------------------------
class CostModel:
    """MLP over (length, variant) features predicting log launch time."""

    def __init__(self, lib, seed: int = 1):
        self.lib = lib
        self.nvar = lib.L.kfft_variant_count()
        self.d_in = N_BASE_FEATURES + self.nvar
        self.h = lib.L.kfft_mlp_create(self.d_in, seed)
        if not self.h:
            raise RuntimeError("kfft_mlp_create failed: " + lib.last_error())
        self.mu = np.zeros(self.d_in, np.float32)
        self.sd = np.ones(self.d_in, np.float32)
        self.ymu = 0.0
        self.ysd = 1.0
        self.loss = float("nan")

    def close(self):
        if getattr(self, "h", None):
            self.lib.L.kfft_mlp_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _raw(self, recs) -> np.ndarray:
        p = self.lib.precision
        return np.stack([features(r.n, r.batch, p, r.variant, self.nvar) for r in recs])

    def _norm(self, X: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray((X - self.mu) / self.sd, dtype=np.float32)

    def fit(self, recs: list[Record], epochs: int = 300, minibatch: int = 64,
            lr: float = 2e-3, seed: int = 5) -> float:
        """Trains on the records; returns the final loss on standardised targets."""
        X = self._raw(recs)
        self.mu = X.mean(0).astype(np.float32)
        sd = X.std(0)
        self.sd = np.where(sd > 1e-6, sd, 1.0).astype(np.float32)
        t = np.log(np.asarray([r.ms for r in recs], dtype=np.float64))
        self.ymu, self.ysd = float(t.mean()), float(max(t.std(), 1e-6))
        y = np.ascontiguousarray((t - self.ymu) / self.ysd, dtype=np.float32)
        Xn = self._norm(X)
        loss = ctypes.c_float(0.0)
        r = self.lib.L.kfft_mlp_train(self.h, Xn.ctypes.data, y.ctypes.data, len(y), epochs,
                                      minibatch, lr, seed, ctypes.byref(loss))
        if r != 0:
            raise RuntimeError("kfft_mlp_train failed: " + self.lib.last_error())
        self.loss = float(loss.value)
        return self.loss

    def predict_ms(self, n: int, batch: int, variants) -> np.ndarray:
        p = self.lib.precision
        X = np.stack([features(n, batch, p, v, self.nvar) for v in variants])
        Xn = self._norm(X)
        out = np.empty(len(variants), np.float32)
        r = self.lib.L.kfft_mlp_predict(self.h, Xn.ctypes.data, len(variants), out.ctypes.data)
        if r != 0:
            raise RuntimeError("kfft_mlp_predict failed: " + self.lib.last_error())
        return np.exp(out.astype(np.float64) * self.ysd + self.ymu)

    def propose(self, n: int, batch: int, variants=None) -> int:
        variants = list(range(self.nvar)) if variants is None else list(variants)
        return int(variants[int(np.argmin(self.predict_ms(n, batch, variants)))])

    def save(self, path: str) -> None:
        P = np.empty(self.lib.L.kfft_mlp_params(self.h), np.float32)
        self.lib.L.kfft_mlp_get(self.h, P.ctypes.data)
        np.savez(path, params=P, mu=self.mu, sd=self.sd, y=np.array([self.ymu, self.ysd]),
                 d_in=np.array([self.d_in]))

    def load(self, path: str) -> None:
        z = np.load(path)
        if int(z["d_in"][0]) != self.d_in:
            raise ValueError("cost model saved for another feature width")
        P = np.ascontiguousarray(z["params"], dtype=np.float32)
        self.lib.L.kfft_mlp_set(self.h, P.ctypes.data)
        self.mu, self.sd = z["mu"], z["sd"]
        self.ymu, self.ysd = float(z["y"][0]), float(z["y"][1])


# ---------------------------------------------------------------------------
# evaluation and the tuning database
# ---------------------------------------------------------------------------
def by_length(recs: list[Record]) -> dict[int, dict[int, Record]]:
    g: dict[int, dict[int, Record]] = {}
    for r in recs:
        g.setdefault(r.n, {})[r.variant] = r
    return g


def split_lengths(recs: list[Record], train_frac: float = 0.2, seed: int = 0):
    """Splits the records by length: all variants of a length land on one side."""
    lengths = sorted(by_length(recs))
    rng = np.random.default_rng(seed)
    k = max(1, int(round(train_frac * len(lengths))))
    pick = set(int(v) for v in rng.choice(lengths, size=k, replace=False))
    train = [r for r in recs if r.n in pick]
    test = [r for r in recs if r.n not in pick]
    return train, test


@dataclass
class Regret:
    lengths: int = 0
    geomean_regret: float = 1.0      # chosen / best, geometric mean over lengths
    max_regret: float = 1.0
    hit_rate: float = 0.0            # share of lengths where the chosen plan is the best
    geomean_gain: float = 1.0        # default / chosen
    ms_best: float = 0.0
    ms_chosen: float = 0.0
    ms_default: float = 0.0
    gflops_chosen: float = 0.0       # 5 N log2 N per sequence over the summed times
    gflops_default: float = 0.0
    gflops_best: float = 0.0
    worst: list = field(default_factory=list)


def evaluate(model, test: list[Record]) -> Regret:
    g = by_length(test)
    lr, lg = [], []
    out = Regret()
    flops = 0.0
    for n, vs in g.items():
        rec0 = next(iter(vs.values()))
        choice = model.propose(n, rec0.batch, sorted(vs))
        best = min(r.ms for r in vs.values())
        chosen = vs[choice].ms
        default = vs[0].ms if 0 in vs else chosen
        lr.append(chosen / best)
        lg.append(default / chosen)
        out.ms_best += best
        out.ms_chosen += chosen
        out.ms_default += default
        out.hit_rate += 1.0 if chosen <= best * (1 + 1e-9) else 0.0
        flops += 5.0 * n * math.log2(max(n, 2)) * rec0.batch
        out.worst.append((chosen / best, n, choice))
    out.lengths = len(g)
    if out.lengths:
        out.geomean_regret = float(np.exp(np.mean(np.log(lr))))
        out.max_regret = float(max(lr))
        out.geomean_gain = float(np.exp(np.mean(np.log(lg))))
        out.hit_rate /= out.lengths
        out.gflops_chosen = flops / (out.ms_chosen * 1e6)
        out.gflops_default = flops / (out.ms_default * 1e6)
        out.gflops_best = flops / (out.ms_best * 1e6)
    out.worst = sorted(out.worst, reverse=True)[:5]
    return out


class TuneDB:
    """Best measured variant per (length, precision), persisted as JSON.

    The path defaults to the KFFT_TUNE_DB environment variable.
    """

    def __init__(self, path: str | None = None):
        self.path = path or os.environ.get("KFFT_TUNE_DB", "")
        self.best: dict[str, dict[int, int]] = {"double": {}, "float": {}}
        if self.path and os.path.exists(self.path):
            with open(self.path) as f:
                raw = json.load(f)
            for prec, table in raw.items():
                self.best[prec] = {int(k): int(v) for k, v in table.items()}

    def update(self, precision: str, recs: list[Record]) -> None:
        for n, vs in by_length(recs).items():
            self.best[precision][n] = min(vs.values(), key=lambda r: r.ms).variant

    def save(self, path: str | None = None) -> None:
        path = path or self.path
        with open(path, "w") as f:
            json.dump({p: {str(k): v for k, v in t.items()} for p, t in self.best.items()}, f,
                      indent=0, sort_keys=True)

    def install(self, lib, flags: int = 0) -> int:
        """Writes the table into the library's tuning table; returns the entries set."""
        count = 0
        for n, v in self.best.get(lib.precision, {}).items():
            if lib.L.kfft_tune_set(n, flags, v) == 0:
                count += 1
        return count
