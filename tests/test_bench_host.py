"""Host-side checks of the benchmark's uneven-batch workload (no GPU): the
length mix the batched configuration describes and the shared input."""
import numpy as np

import bench


def _prime_factors(n):
    out, p = [], 2
    while p * p <= n:
        while n % p == 0:
            out.append(p)
            n //= p
        p += 1
    if n > 1:
        out.append(n)
    return out


def test_uneven_lengths_follow_the_configuration():
    L = bench.uneven_lengths().astype(np.int64)
    # 4096 drawn, the largest dropped until the batch is within 5% of 2^28
    assert len(L) == 3968
    assert int(L.sum()) == 281598199
    assert L.sum() <= 1.05 * (1 << 28)
    # log-uniform draws from [16, 2^20], snapped by class (the 11/13 class
    # snaps the shortest draws to 11 or 13 themselves)
    assert L.min() >= 11 and L.max() <= 1 << 20
    kinds = {"smooth": 0, "11/13": 0, "prime": 0}
    for n in L.tolist():
        f = _prime_factors(n)
        if len(f) == 1 and n > 16:
            kinds["prime"] += 1
        elif max(f) <= 7:
            kinds["smooth"] += 1
        else:
            assert set(f) - {2, 3, 5, 7} <= {11, 13}, n
            kinds["11/13"] += 1
    # about half 7-smooth, a quarter with one 11 or 13, a quarter prime
    # (the dropped largest sequences shift the shares by a few percent)
    assert abs(kinds["smooth"] / len(L) - 0.5) < 0.05, kinds
    assert abs(kinds["11/13"] / len(L) - 0.25) < 0.05, kinds
    assert abs(kinds["prime"] / len(L) - 0.25) < 0.05, kinds
    # log-uniform: every octave from 2^4 to 2^20 holds sequences
    octaves = np.floor(np.log2(L)).astype(int)
    assert set(range(4, 20)) <= set(octaves.tolist())


def test_uneven_input_is_seeded_and_shared():
    a = bench.uneven_input(1000, "float")
    b = bench.uneven_input(1000, "float")
    assert a.dtype == np.complex64 and np.array_equal(a, b)
    d = bench.uneven_input(1000, "double")
    assert d.dtype == np.complex128
    assert abs(float(np.std(d.real)) - 1.0) < 0.1 and abs(float(np.mean(d.imag))) < 0.1
