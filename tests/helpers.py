import numpy as np


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def tol64(n):
    """FP64 parity bound against the reference double build: 1e-13 * log2(N)."""
    return 1e-13 * max(np.log2(max(n, 2)), 1.0)


# FP32 builds are compared with the FP64 oracle; the reference float build
# itself reaches ~1.2e-6 on Rader primes.
TOL32 = 5e-6
