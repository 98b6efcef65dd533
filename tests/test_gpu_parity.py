"""GPU parity of the engine through its C ABI against the reference fixtures
and the FP64 oracle.  FP64: rel-L2 <= 1e-13*log2(N); FP32: rel-L2 <= 1e-6."""
import json
import os

import numpy as np
import pytest

import kfft_gb300 as K
from oracle import oracle as O
from tests.helpers import TOL32, rel_l2, tol64

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def cx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_defs_cpx1_golden(lib):
    d = json.load(open(os.path.join(GOLD, "defs_cpx1.json")))
    for n, v in d["vectors"].items():
        x = np.array([complex(*p) for p in v["in"]])
        y = np.array([complex(*p) for p in v["out"]])
        out = lib.fft_cpx(x)
        assert np.max(np.abs(out - y)) <= 2 * d["tolerance"], n
        back = lib.fft_cpx(y, K.FLAG_INVERSE)
        assert np.max(np.abs(back - x)) <= 2 * d["tolerance"], n


@pytest.mark.parametrize("kind", ["fwd", "inv", "invnn"])
def test_complex_fixtures(lib, golden, kind):
    flags = {"fwd": 0, "inv": K.FLAG_INVERSE, "invnn": K.FLAG_INVERSE | K.FLAG_DISABLE_NORM}[kind]
    sizes = sorted(int(k.split("_")[-1]) for k in golden.files if k.startswith("cpx_in_"))
    for n in sizes:
        got = lib.fft_cpx(golden[f"cpx_in_{n}"], flags)
        assert rel_l2(got, golden[f"cpx_{kind}_{n}"]) <= tol64(n), n


SWEEP = (list(range(1, 130)) + [243, 256, 330, 343, 625, 1000, 1001, 1024, 2048, 2310, 2879,
                               3125, 4096, 4099, 5000, 6561, 8191, 8192, 10201, 12288, 16384,
                               65536, 65537, 100000, 131072, 262144, 1 << 20, 999983, 1009 * 2,
                               4158, 4320])


@pytest.mark.parametrize("n", SWEEP)
def test_complex_sweep_vs_oracle(lib, n):
    rng = np.random.default_rng(n)
    x = cx(rng, n)
    ref = O.fft_cpx(x)
    got = lib.fft_cpx(x)
    assert rel_l2(got, ref) <= tol64(n), n
    back = lib.fft_cpx(got, K.FLAG_INVERSE)
    assert rel_l2(back, x) <= tol64(n)


def test_config1_batch_round_trip(lib):
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (256, 4096)) + 1j * rng.uniform(-1, 1, (256, 4096))
    y = lib.fft_cpx(x)
    ref = O.fft_cpx(x)
    assert rel_l2(y, ref) <= tol64(4096)
    z = lib.fft_cpx(y, K.FLAG_INVERSE)
    assert rel_l2(z, x) <= tol64(4096)


@pytest.mark.parametrize("n", [16, 330, 4096, 4099, 8191, 65536, 1 << 20])
def test_batched_matches_single(lib, n):
    rng = np.random.default_rng(n + 7)
    x = cx(rng, 3, n)
    y = lib.fft_cpx(x)
    for b in range(3):
        assert rel_l2(y[b], O.fft_cpx(x[b])) <= tol64(n)


@pytest.mark.parametrize("n", [7, 64, 4096, 8191, 4099, 1 << 18])
def test_in_place(lib, n):
    import ctypes
    rng = np.random.default_rng(n)
    x = cx(rng, n).astype(np.complex128)
    ref = O.fft_cpx(x)
    p = lib.L.kfft_config_cpx(n, 0, None, None)
    buf = x.copy()
    assert lib.L.kfft_eval_cpx(p, buf.ctypes.data, buf.ctypes.data) == 0
    lib.cleanup(p)
    assert rel_l2(buf, ref) <= tol64(n)


def test_real_fixtures(lib, golden):
    sizes = sorted(int(k.split("_")[-1]) for k in golden.files if k.startswith("real_in_"))
    for n in sizes:
        x = golden[f"real_in_{n}"]
        assert rel_l2(lib.rfft(x), golden[f"real_fwd_{n}"]) <= tol64(n), n
        assert rel_l2(lib.rfft(x, K.FLAG_EXPAND_SCALAR), golden[f"real_fwdx_{n}"]) <= tol64(n), n
        assert rel_l2(lib.irfft(golden[f"real_spec_{n}"], n), golden[f"real_inv_{n}"]) <= tol64(n), n


@pytest.mark.parametrize("n", [2, 5, 6, 97, 98, 1000, 4098, 8190, 1 << 16, 1 << 22, 999983 * 2])
def test_real_vs_oracle(lib, n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n)
    assert rel_l2(lib.rfft(x), O.rfft(x)) <= tol64(n)
    X = O.rfft(x)
    assert rel_l2(lib.irfft(X, n), O.irfft(X, n)) <= tol64(n)


@pytest.mark.parametrize("n,batch,flags", [(1 << 14, 6, 0), (1 << 14, 3, K.FLAG_EXPAND_SCALAR),
                                           (1 << 17, 5, K.FLAG_EXPAND_SCALAR), (1 << 20, 2, 0),
                                           (1 << 22, 2, 0), (8192, 4, 0), (3 << 12, 2, 0)])
def test_real_fp32_batches_vs_oracle(libf, n, batch, flags):
    """FP32 real transforms in batches, forward (with and without EXPAND) and
    inverse, against the oracle sequence by sequence: single-pass (8192),
    multi-pass power-of-two (2^14 - 2^22) and mixed-radix (3 * 2^12)
    half lengths."""
    rng = np.random.default_rng(n + batch)
    x = rng.uniform(-1, 1, (batch, n)).astype(np.float32)
    X = libf.rfft(x, flags)
    for b in range(batch):
        assert rel_l2(X[b], O.rfft(x[b].astype(np.float64), flags)) <= TOL32, b
    spec = np.stack([O.rfft(x[b].astype(np.float64)) for b in range(batch)]).astype(np.complex64)
    y = libf.irfft(spec, n)
    for b in range(batch):
        assert rel_l2(y[b], O.irfft(spec[b].astype(np.complex128), n)) <= TOL32, b


@pytest.mark.parametrize("n", [1 << 16, 6000])
def test_real_conv_fp32_product_in_the_forward_store(libf, n):
    """A real convolution multiplies the two spectra inside the second
    operand's post-twiddle kernel instead of a separate product sweep."""
    rng = np.random.default_rng(n)
    a, b = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    got = libf.conv_scalar(a.astype(np.float32), b.astype(np.float32))
    ref = O.conv_scalar(a.astype(np.float32).astype(np.float64), b.astype(np.float32).astype(np.float64))
    assert rel_l2(got, ref) <= TOL32


def test_real_improper_plan(lib):
    p = lib.L.kfft_config_scalar(64, K.FLAG_INVERSE, None, None)
    x = np.zeros(64)
    y = np.zeros(33, np.complex128)
    assert lib.L.kfft_eval_scalar(p, x.ctypes.data, y.ctypes.data) == K.RET_IMPROPER_PLAN
    lib.cleanup(p)
    p = lib.L.kfft_config_scalar(64, 0, None, None)
    assert lib.L.kfft_evali_scalar(p, y.ctypes.data, x.ctypes.data) == K.RET_IMPROPER_PLAN
    lib.cleanup(p)


def test_2d_fixtures(lib, golden):
    shapes = sorted({k.split("_")[-1] for k in golden.files if k.startswith("c2_in_")})
    for s in shapes:
        a = golden[f"c2_in_{s}"]
        y, x = a.shape
        t = tol64(x * y)
        assert rel_l2(lib.fft2_cpx(a), golden[f"c2_fwd_{s}"]) <= t, s
        assert rel_l2(lib.fft2_cpx(a, K.FLAG_INVERSE), golden[f"c2_inv_{s}"]) <= t, s
        assert rel_l2(lib.rfft2(golden[f"s2_in_{s}"]), golden[f"s2_fwd_{s}"]) <= t, s
        assert rel_l2(lib.irfft2(golden[f"s2_spec_{s}"]), golden[f"s2_inv_{s}"]) <= t, s
        assert rel_l2(lib.conv2_scalar(golden[f"s2_in_{s}"], golden[f"s2c_b_{s}"]),
                      golden[f"s2c_out_{s}"]) <= t, s
        if f"c2c_out_{s}" in golden.files:
            assert rel_l2(lib.conv2_cpx(a, golden[f"c2c_b_{s}"]), golden[f"c2c_out_{s}"]) <= t


@pytest.mark.parametrize("shape", [(1, 5), (5, 1), (64, 48), (128, 4096), (4096, 64), (37, 101),
                                   (1024, 1024), (101, 4099)])
def test_2d_vs_oracle(lib, shape):
    rng = np.random.default_rng(sum(shape))
    a = cx(rng, *shape)
    t = tol64(shape[0] * shape[1])
    assert rel_l2(lib.fft2_cpx(a), O.fft2_cpx(a)) <= t
    assert rel_l2(lib.fft2_cpx(a, K.FLAG_INVERSE), O.fft2_cpx(a, O.FLAG_INVERSE)) <= t
    ar = a.real.copy()
    assert rel_l2(lib.rfft2(ar), O.rfft2(ar)) <= t
    S = np.fft.fft2(ar)
    assert rel_l2(lib.irfft2(S), O.irfft2(S)) <= t


@pytest.mark.parametrize("shape", [(6, 10), (64, 48), (2, 7), (9, 8), (256, 100), (8192, 16),
                                   (4096, 33)])
def test_irfft2_any_spectrum_vs_oracle(lib, libf, shape):
    """The real 2D inverse of a spectrum that is not Hermitian: the result
    depends on which bins the transform reads, so it must read the same ones
    as the reference (rows 0..y/2 of the row transforms for an even y, every
    row for an odd y), normalised and not.  The shapes take both the
    column path and the transposes (y = 8192 in FP32, y = 4096 in FP64)."""
    rng = np.random.default_rng(sum(shape) + 5)
    S = cx(rng, *shape)
    t = tol64(shape[0] * shape[1])
    for flags in (0, K.FLAG_DISABLE_NORM):
        ref = O.irfft2(S, flags | O.FLAG_INVERSE) if flags else O.irfft2(S)
        assert rel_l2(lib.irfft2(S, K.FLAG_INVERSE | flags), ref) <= t, flags
        assert rel_l2(libf.irfft2(S.astype(np.complex64), K.FLAG_INVERSE | flags), ref) <= TOL32, flags


def test_conv_fixtures(lib, golden):
    sizes = sorted(int(k.split("_")[-1]) for k in golden.files if k.startswith("cc_a_"))
    for n in sizes:
        a, b = golden[f"cc_a_{n}"], golden[f"cc_b_{n}"]
        assert rel_l2(lib.conv_cpx(a, b), golden[f"cc_out_{n}"]) <= tol64(n), n
        assert rel_l2(lib.conv_scalar(a.real, b.real), golden[f"sc_out_{n}"]) <= tol64(n), n


@pytest.mark.parametrize("shape", [(12, 30), (64, 64), (100, 33), (33, 100), (31, 2), (1, 8)])
def test_conv2_vs_oracle(lib, shape):
    rng = np.random.default_rng(11)
    a, b = cx(rng, *shape), cx(rng, *shape)
    t = tol64(shape[0] * shape[1])
    assert rel_l2(lib.conv2_cpx(a, b), O.conv2_cpx(a, b)) <= t
    assert rel_l2(lib.conv2_scalar(a.real, b.real), O.conv2_scalar(a.real, b.real)) <= t


@pytest.mark.parametrize("shape", [(12, 30), (33, 100), (100, 33)])
def test_conv2_scalar_unnormalised(lib, libf, shape):
    """Real conv2d without normalisation (KFFT_FLAG_DISABLE_NORM): an even
    row length runs through half spectra, an odd one through the expanded
    spectra; both must give the reference's unnormalised sums."""
    rng = np.random.default_rng(12)
    a, b = rng.uniform(-1, 1, shape), rng.uniform(-1, 1, shape)
    ref = O.conv2_scalar(a, b, O.FLAG_DISABLE_NORM)
    t = tol64(shape[0] * shape[1])
    assert rel_l2(lib.conv2_scalar(a, b, K.FLAG_DISABLE_NORM), ref) <= t
    assert rel_l2(libf.conv2_scalar(a, b, K.FLAG_DISABLE_NORM), ref) <= TOL32


@pytest.mark.parametrize("n", [1, 2, 3, 7, 64, 330, 4096, 4099, 8191, 1 << 16])
def test_float_build_vs_oracle(libf, n):
    rng = np.random.default_rng(n)
    x = cx(rng, n)
    got = libf.fft_cpx(x.astype(np.complex64))
    assert rel_l2(got, O.fft_cpx(x.astype(np.complex64).astype(np.complex128))) <= TOL32
    xr = rng.uniform(-1, 1, n)
    got = libf.rfft(xr.astype(np.float32))
    assert rel_l2(got, O.rfft(xr.astype(np.float32).astype(np.float64))) <= TOL32


def test_float_fixtures(libf, golden):
    sizes = sorted(int(k.split("_")[-1]) for k in golden.files if k.startswith("cpx_in_"))
    for n in sizes:
        got = libf.fft_cpx(golden[f"cpx_in_{n}"].astype(np.complex64))
        # against the reference double build; the reference float build is also stored
        assert rel_l2(got, golden[f"cpx_fwd_{n}"]) <= TOL32, n
        assert rel_l2(golden[f"cpxf_fwd_{n}"], golden[f"cpx_fwd_{n}"]) <= 2e-5, n


def test_device_pointers_and_async(lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    x = cx(rng, 8, 1024)
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    p = lib.L.kfft_config_cpx(1024, 0, None, None)
    assert lib.L.kfft_eval_cpx_batch(p, xt.data_ptr(), yt.data_ptr(), 8) == 0
    assert rel_l2(yt.cpu().numpy(), O.fft_cpx(x)) <= tol64(1024)
    s = torch.cuda.Stream()
    zt = torch.empty_like(xt)
    assert lib.L.kfft_eval_cpx_async(p, xt.data_ptr(), zt.data_ptr(), 8, s.cuda_stream) == 0
    s.synchronize()
    assert rel_l2(zt.cpu().numpy(), O.fft_cpx(x)) <= tol64(1024)
    lib.cleanup(p)


def test_uneven_batch(lib):
    import ctypes
    rng = np.random.default_rng(9)
    lengths = np.array([16, 17, 4096, 97, 1000, 4099, 8191, 1, 65536, 30, 4096, 12345],
                       dtype=np.uint32)
    total = int(lengths.sum())
    x = cx(rng, total)
    p = lib.L.kfft_config_cpx_uneven(len(lengths), lengths.ctypes.data, 0)
    assert p
    assert lib.L.kfft_uneven_total(p) == total
    y = np.empty_like(x)
    for _ in range(2):
        assert lib.L.kfft_eval_cpx_uneven(p, x.ctypes.data, y.ctypes.data) == 0
    off = 0
    for n in lengths:
        n = int(n)
        assert rel_l2(y[off:off + n], O.fft_cpx(x[off:off + n])) <= tol64(n), n
        off += n
    lib.L.kfft_release_uneven(p)


def test_user_pool_and_renew(lib):
    import ctypes
    s1, s2 = lib.size_query("kfft_config_cpx", 101, K.FLAG_INVERSE), lib.size_query("kfft_config_cpx", 78, 0)
    P = lib.L.kfft_pool_create(s1 + s2)
    a = lib.L.kfft_config_cpx(78, 0, P, None)
    b = lib.L.kfft_config_cpx(101, K.FLAG_INVERSE, P, None)
    assert a and b
    x = cx(np.random.default_rng(1), 78)
    y = np.empty_like(x)
    assert lib.L.kfft_eval_cpx(a, x.ctypes.data, y.ctypes.data) == 0
    assert rel_l2(y, O.fft_cpx(x)) <= tol64(78)
    # overflow of the user pool returns NULL (api_cpx1.c:77-102)
    assert not lib.L.kfft_config_cpx(107, K.FLAG_INVERSE, P, None)
    # RENEW clears the pool and builds a new plan in it
    c = lib.L.kfft_config_cpx(78, K.FLAG_INVERSE | K.FLAG_RENEW, P, None)
    assert c
    z = np.empty_like(x)
    assert lib.L.kfft_eval_cpx(c, y.ctypes.data, z.ctypes.data) == 0
    assert rel_l2(z, x) <= tol64(78)
    lib.L.kfft_pool_free(P)


def test_release_frees_device_memory(lib):
    before = lib.stats().device_bytes
    p = lib.L.kfft_config_cpx(1 << 20, 0, None, None)
    assert lib.stats().device_bytes > before
    assert lib.cleanup(p) == 0
    assert lib.stats().device_bytes == before


@pytest.mark.parametrize("precision", ["double", "float"])
def test_uneven_workload_subset(precision):
    """Every 8th sequence of the uneven-batch benchmark workload, both builds."""
    import bench
    lib = K.load(precision)
    lengths = np.ascontiguousarray(bench.uneven_lengths()[::8])
    total = int(lengths.sum(dtype=np.int64))
    rng = np.random.default_rng(2)
    x = cx(rng, total)
    cdt = np.complex128 if precision == "double" else np.complex64
    xin = x.astype(cdt)
    p = lib.L.kfft_config_cpx_uneven(len(lengths), lengths.ctypes.data, 0)
    assert p, lib.last_error()
    y = np.empty_like(xin)
    assert lib.L.kfft_eval_cpx_uneven(p, xin.ctypes.data, y.ctypes.data) == 0
    lib.L.kfft_release_uneven(p)
    ref = O.fft_uneven(lengths, xin.astype(np.complex128))
    off = 0
    worst = 0.0
    for n in lengths:
        n = int(n)
        e = rel_l2(y[off:off + n], ref[off:off + n])
        worst = max(worst, e / (tol64(n) if precision == "double" else TOL32))
        off += n
    assert worst <= 1.0, worst


@pytest.mark.parametrize("n,batch", [(16, 64), (256, 16), (4096, 8), (65536, 2), (1 << 18, 1),
                                     (1 << 20, 1), (3 * 4096, 2), (1000, 4)])
def test_tensor_core_radix16_path(libf, n, batch):
    """FP32 build with KFFT_FLAG_TENSOR_CORES: FP16 split hi+lo radix-16
    stages, held to the plain FP32 bound at these sizes (up to 2^20; the
    larger benchmark sizes are in test_gpu_config_sizes.py)."""
    rng = np.random.default_rng(n)
    x = cx(rng, batch, n).astype(np.complex64)
    ref = O.fft_cpx(x.astype(np.complex128))
    p = libf.L.kfft_config_cpx(n, 1 << 8, None, None)
    y = np.empty_like(x)
    assert libf.L.kfft_eval_cpx_batch(p, x.ctypes.data, y.ctypes.data, batch) == 0
    libf.cleanup(p)
    assert rel_l2(y, ref) <= TOL32
    pi = libf.L.kfft_config_cpx(n, 1 | (1 << 8), None, None)
    z = np.empty_like(x)
    assert libf.L.kfft_eval_cpx_batch(pi, y.ctypes.data, z.ctypes.data, batch) == 0
    libf.cleanup(pi)
    assert rel_l2(z, x) <= 2 * TOL32
