"""Regenerates the committed golden fixtures from the reference kfft itself.

Run in a checkout where the reference sources are available:

    oracle/build_ref.sh /path/to/kfft && python tests/golden/make_golden.py /path/to/kfft

It writes two files next to this script:
  * ``defs_cpx1.json`` -- the reference unit-test golden ramps (N = 2, 3, 5, 7,
    330), read as text from ``test/unit/suites/defs_cpx1.h`` (tolerance 1e-3 as
    in ``test/unit/suites/api_cpx1.c:10``);
  * ``ref_vectors.npz`` -- seeded inputs and the outputs of the reference's
    double build (SYSMATH, Rader, RADER_LIMIT=25) and float build for every
    transform family of the path, at sizes that run in milliseconds.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

CPX_SIZES = [1, 2, 3, 4, 5, 7, 8, 11, 13, 16, 25, 27, 49, 97, 121, 128, 169, 330, 1000, 1024,
             2879, 4096, 4099]
REAL_SIZES = [1, 2, 3, 4, 7, 8, 30, 101, 128, 330, 1000, 4096]
SHAPES_2D = [(10, 11), (11, 10), (8, 8), (16, 6), (7, 9), (5, 1), (12, 30)]  # (y, x)
CONV_SIZES = [1, 2, 3, 8, 9, 100, 101, 1024]


def parse_defs(ref_root):
    text = open(os.path.join(ref_root, "test/unit/suites/defs_cpx1.h")).read()
    out = {}
    for m in re.finditer(r"const kfft_cpx fft(\d+)_(in|out)\[[^\]]*\]\s*=\s*\{(.*?)\};", text, re.S):
        n, kind, body = int(m.group(1)), m.group(2), m.group(3)
        vals = [float(v) for v in re.findall(r"-?\d+\.\d+", body)]
        pairs = [[vals[2 * i], vals[2 * i + 1]] for i in range(len(vals) // 2)]
        out.setdefault(str(n), {})[kind] = pairs
    return out


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    with open(os.path.join(HERE, "defs_cpx1.json"), "w") as f:
        json.dump({"tolerance": 1e-3, "vectors": parse_defs(ref_root)}, f)

    R = O.RefLib("double")
    Rf = O.RefLib("float")
    rng = np.random.default_rng(20240601)
    z = {}

    def cx(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    for n in CPX_SIZES:
        x = cx(n)
        z[f"cpx_in_{n}"] = x
        z[f"cpx_fwd_{n}"] = R.fft_cpx(x, 0)
        z[f"cpx_inv_{n}"] = R.fft_cpx(x, O.FLAG_INVERSE)
        z[f"cpx_invnn_{n}"] = R.fft_cpx(x, O.FLAG_INVERSE | O.FLAG_DISABLE_NORM)
        z[f"cpxf_fwd_{n}"] = Rf.fft_cpx(x.astype(np.complex64), 0)
    for n in REAL_SIZES:
        x = rng.uniform(-1, 1, n)
        z[f"real_in_{n}"] = x
        z[f"real_fwd_{n}"] = R.rfft(x, 0)
        z[f"real_fwdx_{n}"] = R.rfft(x, O.FLAG_EXPAND_SCALAR)
        spec = np.fft.rfft(x) if n % 2 == 0 else np.fft.fft(x)
        z[f"real_spec_{n}"] = spec
        z[f"real_inv_{n}"] = R.irfft(spec, n, O.FLAG_INVERSE)
    for (y, x) in SHAPES_2D:
        a = cx(y, x)
        z[f"c2_in_{y}x{x}"] = a
        z[f"c2_fwd_{y}x{x}"] = R.fft2_cpx(a, 0)
        z[f"c2_inv_{y}x{x}"] = R.fft2_cpx(a, O.FLAG_INVERSE)
        ar = rng.uniform(-1, 1, (y, x))
        z[f"s2_in_{y}x{x}"] = ar
        z[f"s2_fwd_{y}x{x}"] = R.rfft2(ar, 0)
        spec = np.fft.fft2(ar)
        z[f"s2_spec_{y}x{x}"] = spec
        z[f"s2_inv_{y}x{x}"] = R.irfft2(spec, O.FLAG_INVERSE)
        br = rng.uniform(-1, 1, (y, x))
        z[f"s2c_b_{y}x{x}"] = br
        z[f"s2c_out_{y}x{x}"] = R.conv2_scalar(ar, br, 0)
        if x == y:  # the reference's complex conv2d plans x*x (ext/conv2d/kfft_cpx_conv.c:67)
            b = cx(y, x)
            z[f"c2c_b_{y}x{x}"] = b
            z[f"c2c_out_{y}x{x}"] = R.conv2_cpx(a, b, 0)
    for n in CONV_SIZES:
        a, b = cx(n), cx(n)
        z[f"cc_a_{n}"], z[f"cc_b_{n}"] = a, b
        z[f"cc_out_{n}"] = R.conv_cpx(a, b, 0)
        ar, br = a.real.copy(), b.real.copy()
        z[f"sc_out_{n}"] = R.conv_scalar(ar, br, 0)
    np.savez_compressed(os.path.join(HERE, "ref_vectors.npz"), **z)
    print("wrote", len(z), "arrays")


if __name__ == "__main__":
    main()
