"""Host-side arithmetic of the planner, restated and checked on the CPU."""
import numpy as np


def fastdiv(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return m, l


def apply(n, m, l):
    return ((n * m >> 32) + n) >> l


def test_fastdiv_magic_matches_integer_division():
    rng = np.random.default_rng(0)
    ds = [1, 2, 3, 5, 7, 16, 25, 100, 1000, 4096, 4099, 65535, 65537, 999983, 2**31 - 1,
          2**31, 2**32 - 1] + list(rng.integers(1, 2**32 - 1, 200))
    ns = [0, 1, 2, 3, 1000, 2**31 - 1, 2**31, 2**32 - 2, 2**32 - 1] + list(
        rng.integers(0, 2**32 - 1, 300))
    for d in ds:
        d = int(d)
        m, l = fastdiv(d)
        assert 0 <= m < 2**32
        for n in ns:
            n = int(n)
            assert apply(n, m, l) == n // d, (n, d)


def test_chirp_phase_reduction_is_exact():
    # k^2 mod 2N in integers keeps the Bluestein chirp phase exact for large k
    n = 999983
    for k in (0, 1, 12345, n - 1, 2 * n - 1):
        e = (k * k) % (2 * n)
        ph = np.pi * e / n
        assert abs(np.exp(-1j * ph) - np.exp(-1j * np.pi * (k * k) / n)) < 1e-6 or k * k < 2**52
