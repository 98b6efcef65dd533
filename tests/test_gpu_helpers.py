"""fftshift and the kfft_math helpers on the GPU through the C ABI, against the
oracle: bit-exact for the index work (shifts, transposes), within an ulp or
two for the Hadamard products and magnitudes (the kernels may fuse a
multiply-add), 1e-13 absolute for the FP64 average, whose summation order
differs from the reference's."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n", [1, 2, 7, 8, 1000, 1001, 1 << 20, (1 << 20) + 1])
def test_shift_1d(lib, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for inverse in (False, True):
        h = x.copy()
        lib.L.kfft_shift_cpx(h.ctypes.data, n, inverse, None)
        assert np.array_equal(h, O.shift(x, inverse)), (n, inverse)
        d = torch.from_numpy(x.real.copy()).cuda()
        lib.L.kfft_shift_scalar(d.data_ptr(), n, inverse, None)
        assert np.array_equal(d.cpu().numpy(), O.shift(x.real, inverse)), (n, inverse)


@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (8, 8), (7, 12), (1024, 999), (33, 1)])
def test_shift_2d(lib, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    y, x = shape
    for inverse in (False, True):
        h = a.copy()
        lib.L.kfft_shift2_cpx(h.ctypes.data, None, x, y, inverse, None)
        assert np.array_equal(h, O.shift(a, inverse))
        d = torch.from_numpy(a.real.copy()).cuda()
        lib.L.kfft_shift2_scalar(d.data_ptr(), None, x, y, inverse, None)
        assert np.array_equal(d.cpu().numpy(), O.shift(a.real, inverse))


def test_math_helpers(lib):
    rng = np.random.default_rng(7)
    n = 10007
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    m = np.empty(n)
    lib.L.kfft_math_magnitude(z.ctypes.data, m.ctypes.data, n)
    assert np.allclose(m, O.magnitude(z), rtol=1e-15, atol=0)
    zi = z.copy()
    lib.L.kfft_math_magnitude_ip(zi.ctypes.data, n)
    assert np.allclose(zi.view(np.float64)[:n], O.magnitude(z), rtol=1e-15, atol=0)
    v = rng.standard_normal(n)
    assert abs(lib.L.kfft_math_average(v.ctypes.data, n) - O.average(v)) < 1e-13
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    h = b.copy()
    lib.L.kfft_math_hadamard_cpx(h.ctypes.data, z.ctypes.data, n)
    assert np.allclose(h, b * z, rtol=1e-15)
    hr = b.real.copy()
    zr = np.ascontiguousarray(z.real)
    lib.L.kfft_math_hadamard_scalar(hr.ctypes.data, zr.ctypes.data, n)
    assert np.array_equal(hr, b.real * zr)
    a = rng.standard_normal((37, 101)) + 1j * rng.standard_normal((37, 101))
    t = np.empty((101, 37), np.complex128)
    lib.L.kfft_math_transpose_cpx(a.ctypes.data, t.ctypes.data, 101, 37)
    assert np.array_equal(t, O.transpose(a))
    ip = a.copy()
    lib.L.kfft_math_transpose_ip_cpx(ip.ctypes.data, 101, 37)
    assert np.array_equal(ip.reshape(101, 37), a.T)
    ar = np.ascontiguousarray(a.real)
    tr = np.empty((101, 37))
    lib.L.kfft_math_transpose_scalar(ar.ctypes.data, tr.ctypes.data, 101, 37)
    assert np.array_equal(tr, a.real.T)
    lib.L.kfft_math_transpose_ip_scalar(ar.ctypes.data, 101, 37)
    assert np.array_equal(ar.reshape(101, 37), a.real.T)


def test_math_helpers_fp32_device_buffers(libf):
    rng = np.random.default_rng(8)
    n = 1 << 20
    z = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    zd = torch.from_numpy(z).cuda()
    md = torch.empty(n, dtype=torch.float32, device="cuda")
    libf.L.kfft_math_magnitude(zd.data_ptr(), md.data_ptr(), n)
    # one rounding each way; the kernel may contract r*r + i*i into an FMA
    assert np.allclose(md.cpu().numpy(), O.magnitude(z), rtol=3e-7, atol=0)
    v = rng.standard_normal(n).astype(np.float32)
    vd = torch.from_numpy(v).cuda()
    avg = libf.L.kfft_math_average(vd.data_ptr(), n)
    assert abs(avg - float(np.mean(v.astype(np.float64)))) < 1e-6
