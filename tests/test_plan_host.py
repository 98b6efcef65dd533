"""Host planning arithmetic (plan_host.h, FP32 build), built with the host
compiler and checked on the CPU against an independent restatement here:
the power-of-two pass splits (a search over pass lengths 16..rmax with
per-pass costs 1 up to 256 points, 1.44 at 512, 1.65 at 1024; ties to fewer
passes, then the more even split), the shared-memory bank model that picks a
register tile's lane stride (wavefronts per 128-byte request, the skew with
the fewest), the balanced multi-pass split of other lengths, and the
Bluestein convolution length (the 7-smooth M >= 2N-1, up to twice that,
with the least M * passes * (1 + 0.15 * odd factors))."""
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


@pytest.fixture(scope="module")
def printed(tmp_path_factory):
    cxx, inc = shutil.which("g++"), _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = tmp_path_factory.mktemp("plan_host") / "plan_host_check"
    subprocess.run([cxx, "-std=c++17", "-O1", "-DKFFT_HALF_SCALAR", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "kfft_gb300", "csrc"), "-I", inc,
                    os.path.join(ROOT, "tests", "plan_host_check.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    return [line.split() for line in out.splitlines()]


# ---- restatement -----------------------------------------------------------

def split(L, rmax):
    emax = min(10, rmax.bit_length() - 1)
    cost = {9: 1.44, 10: 1.65}
    best = [None, None]
    cur = []

    def walk(left, top, c):
        if left == 0:
            b = best
            if (b[0] is None or c < b[0] - 1e-9 or
                    (c < b[0] + 1e-9 and (len(cur) < len(b[1]) or (len(cur) == len(b[1]) and cur < b[1])))):
                best[0], best[1] = c, list(cur)
            return
        for e in range(min(top, left), 3, -1):
            cur.append(e)
            walk(left - e, e, c + cost.get(e, 1.0))
            cur.pop()

    walk(L, emax, 0.0)
    return [1 << e for e in best[1]]


# butterfly flops of each register radix, plus r-1 twiddle products, per point
BFLY = {2: 4, 3: 16, 4: 16, 5: 40, 6: 44, 7: 72, 8: 52, 9: 120, 10: 100, 11: 140, 12: 112,
        13: 190, 14: 172, 15: 200, 16: 144}


def _flops(r):
    return (BFLY.get(r, 4.0 * r * r) + 6.0 * (r - 1)) / r


def radices(R):
    """Inner stages of a tile of R points: powers of two as 16s then 8/4/2;
    otherwise the fewest stages from radices 2..16 (ties: least estimated
    flops), largest first, with prime factors 17..31 as stages of their own."""
    if R >= 2 and R & (R - 1) == 0:
        e2 = R.bit_length() - 1
        return [16] * (e2 // 4) + ([1 << (e2 % 4)] if e2 % 4 else [])
    big, rest, p = [], R, 2
    while p * p <= rest:
        while rest % p == 0:
            if p > 16:
                big.append(p)
            rest //= p
        p += 1
    # `rest` now holds at most one prime left over; recompute the small part
    small = R
    for q in big:
        small //= q
    if rest > 16:
        big.append(rest)
        small //= rest

    from functools import lru_cache

    @lru_cache(maxsize=None)
    def best(d):
        if d == 1:
            return (0, 0.0, ())
        out = None
        for q in range(16, 1, -1):
            if d % q == 0:
                s, f, seq = best(d // q)
                cand = (s + 1, f + _flops(q), seq + (q,))
                if out is None or cand[0] < out[0] or (cand[0] == out[0] and cand[1] < out[1] - 1e-9):
                    out = cand
        return out

    return sorted(best(small)[2], reverse=True) + big


def pad(i):
    return i + i // 16


def wavefronts(idx):
    tot = 0
    for h in (idx[:16], idx[16:]):
        slots = {}
        for x in set(v for v in h if v is not None):
            slots.setdefault(x % 16, set()).add(x)
        tot += max((len(v) for v in slots.values()), default=0)
    return tot


def cost(R, C, stride, load_lane, store_lane, threads):
    rad = radices(R)
    tot, NS = 0, 1
    for s, P in enumerate(rad):
        M, last = R // P, s == len(rad) - 1
        items = C * M
        cfast = (s == 0 and load_lane) or (last and store_lane)
        for w in range(min(threads // 32, (items + 31) // 32)):
            maps = []
            for t in range(32):
                it = w * 32 + t
                if it >= items:
                    maps.append(None)
                else:
                    maps.append(divmod(it, C)[::-1] if cfast else divmod(it, M))
            for q in range(P):
                if s > 0:
                    tot += wavefronts([None if m is None else m[0] * stride + pad(m[1] + q * M) for m in maps])
                if not last:
                    tot += wavefronts([None if m is None else
                                       m[0] * stride + pad((m[1] // NS) * NS * P + m[1] % NS + q * NS) for m in maps])
        NS *= P
    return tot


def test_pow2_splits_match_restatement(printed):
    rows = [r for r in printed if r[0] == "split"]
    assert len(rows) == 16 * 3
    for r in rows:
        L, rmax = int(r[1]), int(r[2])
        assert [int(v) for v in r[3:]] == split(L, rmax), r
    got = {(int(r[1]), int(r[2])): [int(v) for v in r[3:]] for r in rows}
    assert got[(18, 1024)] == [1024, 256]
    assert got[(20, 1024)] == [128, 128, 64]
    assert got[(24, 1024)] == [256, 256, 256]


def test_lane_strides_match_restatement(printed):
    rows = [r for r in printed if r[0] == "stride"]
    assert len(rows) == 16
    for r in rows:
        R, C, ll, sl, T, s, c_best, c_base = (int(v) for v in r[1:])
        base = pad(R)
        costs = [cost(R, C, base + k, ll, sl, T) for k in range(16)]
        if C > 1 and len(radices(R)) > 1:
            assert s == base + costs.index(min(costs)), r
        else:
            assert s == base
        assert c_best == cost(R, C, s, ll, sl, T) and c_base == costs[0], r
        assert c_best <= c_base
    # the lane-major multi-lane cases the skew exists for
    by = {(int(r[1]), int(r[2]), int(r[3]), int(r[4]), int(r[5])): (int(r[7]), int(r[8])) for r in rows}
    assert by[(512, 8, 1, 1, 256)][0] * 2 < by[(512, 8, 1, 1, 256)][1]
    assert by[(64, 64, 1, 1, 256)][0] * 2 < by[(64, 64, 1, 1, 256)][1]


def factors(n):
    f, p = [], 2
    while p * p <= n:
        while n % p == 0:
            f.append(p)
            n //= p
        p += 1
    if n > 1:
        f.append(n)
    return f


def balanced(n, rmax):
    f = sorted(factors(n), reverse=True)
    for m in range(1, 33):
        g = [1] * m
        ok = True
        for p in f:
            cand = [i for i in range(m) if g[i] * p <= rmax]
            if not cand:
                ok = False
                break
            i = min(cand, key=lambda i: (g[i], i))
            g[i] *= p
        if ok:
            out = sorted((v for v in g if v > 1), reverse=True)
            return out or [1]
    return []


def bluestein(m, rmax=1024, single=4096):
    best, best_cost = None, None
    a = 1
    while a <= 2 * m:
        b = a
        while b <= 2 * m:
            c = b
            while c <= 2 * m:
                d = c
                while d <= 2 * m:
                    if d >= m:
                        odd, r = 0, d
                        for q in (3, 5, 7):
                            while r % q == 0:
                                r //= q
                                odd += 1
                        passes = 1 if d <= single else max(1, len(balanced(d, rmax)))
                        cost = d * passes * (1.0 + 0.15 * odd)
                        if best_cost is None or cost < best_cost:
                            best, best_cost = d, cost
                    d *= 7
                c *= 5
            b *= 3
        a *= 2
    return best


def test_balanced_splits_match_restatement(printed):
    rows = [r for r in printed if r[0] == "balanced"]
    assert len(rows) == 15
    for r in rows:
        assert [int(v) for v in r[3:]] == balanced(int(r[1]), int(r[2])), r


def test_bluestein_lengths_match_restatement(printed):
    rows = [r for r in printed if r[0] == "bluestein"]
    assert len(rows) == 9
    got = {int(r[1]): int(r[2]) for r in rows}
    for n, m in got.items():
        assert m == bluestein(2 * n - 1), (n, m)
        assert m >= 2 * n - 1
    assert got[999983] == 1 << 21  # over the nearest 7-smooth length, 2,000,000


def test_bluestein_lengths_for_queue_plans(printed):
    """The uneven batch's plans (2048-point tiles, 512-point passes) size
    their Bluestein convolutions for those limits."""
    rows = [r for r in printed if r[0] == "bluestein_q"]
    assert len(rows) == 9
    for r in rows:
        n, m = int(r[1]), int(r[2])
        assert m == bluestein(2 * n - 1, 512, 2048), (n, m)
        assert m >= 2 * n - 1


def test_inner_radix_schedules_match_restatement(printed):
    rows = [r for r in printed if r[0] == "radices"]
    assert len(rows) >= 40
    for r in rows:
        R = int(r[1])
        got = [int(v) for v in r[2:]]
        assert got == radices(R), r
        prod = 1
        for q in got:
            prod *= q
        assert prod == R
    got = {int(r[1]): [int(v) for v in r[2:]] for r in rows}
    assert got[729] == [9, 9, 9]           # six radix-3 stages before
    assert got[4096] == [16, 16, 16]       # the compile-time bodies' schedule
    assert got[2048] == [16, 16, 8]
    assert len(got[756]) == 3              # 4 * 27 * 7: five stages before
    assert got[31 * 16] == [16, 31]
