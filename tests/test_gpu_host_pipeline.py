"""Host-buffer calls large enough to be split into overlapping chunks (copy in,
transform, copy out of neighbouring chunks on separate streams).  Splitting
changes no arithmetic: results equal the device-buffer path bit for bit, and
spot checks against the FP64 oracle hold the usual tolerances."""
import ctypes

import numpy as np
import pytest

import kfft_gb300 as K
from oracle import oracle as O
from tests.helpers import TOL32, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _device_result_batch(lib, plan, x, batch):
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    assert lib.L.kfft_eval_cpx_async(plan, xd.data_ptr(), yd.data_ptr(), batch, None) == 0
    torch.cuda.synchronize()
    return yd.cpu().numpy()


@pytest.mark.parametrize("inplace", [False, True])
@pytest.mark.parametrize("n,batch", [(1 << 16, 160),   # 80 MiB each way: split into chunks
                                     (3000, 3000)])    # 72 MB; chunk ends off 256-byte boundaries
def test_chunked_host_batch_matches_device_path(libf, inplace, n, batch):
    rng = np.random.default_rng(21)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    p = libf._plan("kfft_config_cpx", n, 0)
    try:
        ref = _device_result_batch(libf, p, x, batch)
        if inplace:
            y = x.copy()
            assert libf.L.kfft_eval_cpx_batch(p, y.ctypes.data, y.ctypes.data, batch) == 0
        else:
            y = np.empty_like(x)
            assert libf.L.kfft_eval_cpx_batch(p, x.ctypes.data, y.ctypes.data, batch) == 0
        assert np.array_equal(y, ref)
        for b in (0, 77, batch // 2, batch - 1):
            assert rel_l2(y[b], O.fft_cpx(x[b])) <= TOL32
    finally:
        libf.cleanup(p)


@pytest.mark.parametrize("precision,x,y,inplace", [("float", 1024, 4096, False),
                                                   ("float", 2048, 1536, True),
                                                   ("double", 4096, 1024, False),
                                                   ("float", 8192, 8192, False)])
def test_2d_host_pipeline_matches_device_path(lib, libf, precision, x, y, inplace):
    """2D complex transforms between host buffers copy rows in by chunks, each
    chunk's row passes starting once its copy lands.  Splitting changes no
    arithmetic: the result equals the device-buffer call bit for bit, and
    matches the FP64 oracle; in place too."""
    L = libf if precision == "float" else lib
    cdt = np.complex64 if precision == "float" else np.complex128
    rng = np.random.default_rng(x + y)
    a = (rng.standard_normal((y, x)) + 1j * rng.standard_normal((y, x))).astype(cdt)
    p = L._plan("kfft_config2_cpx", x, y, 0)
    try:
        ad = torch.from_numpy(a).cuda()
        od = torch.empty_like(ad)
        torch.cuda.synchronize()
        assert L.L.kfft_eval2_cpx(p, ad.data_ptr(), od.data_ptr()) == 0
        ref = od.cpu().numpy()
        if inplace:
            out = a.copy()
            assert L.L.kfft_eval2_cpx(p, out.ctypes.data, out.ctypes.data) == 0
        else:
            out = np.empty_like(a)
            assert L.L.kfft_eval2_cpx(p, a.ctypes.data, out.ctypes.data) == 0
        assert np.array_equal(out, ref)
        if x * y <= 1 << 22:
            tol = TOL32 if precision == "float" else 1e-13 * np.log2(x * y)
            assert rel_l2(out, O.fft2_cpx(a.astype(np.complex128))) <= tol
    finally:
        L.cleanup(p)


def test_grouped_host_uneven_matches_device_path(libf):
    rng = np.random.default_rng(22)
    lengths = [1 << 20, 999983, 65537, 3 * 5 * 7 * 11 * 13 * 16, 4096, 17, 1]
    lengths += [int(v) for v in rng.integers(2, 1 << 20, 80)]
    lengths = np.ascontiguousarray(np.array(lengths, dtype=np.uint32))
    total = int(lengths.sum())
    assert total >= 2 << 24  # enough points to be split into groups
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    p = libf.L.kfft_config_cpx_uneven(len(lengths), lengths.ctypes.data, 0)
    assert p, libf.last_error()
    try:
        xd = torch.from_numpy(x).cuda()
        yd = torch.empty_like(xd)
        torch.cuda.synchronize()
        assert libf.L.kfft_eval_cpx_uneven_async(p, xd.data_ptr(), yd.data_ptr(), None) == 0
        torch.cuda.synchronize()
        ref = yd.cpu().numpy()
        y = np.empty_like(x)
        for _ in range(2):  # the second call replays the recorded groups
            y[:] = 0
            assert libf.L.kfft_eval_cpx_uneven(p, x.ctypes.data, y.ctypes.data) == 0
            assert np.array_equal(y, ref)
        offs = np.concatenate([[0], np.cumsum(lengths.astype(np.int64))])
        for i in (0, 1, 2, 3, len(lengths) - 1):
            a, b = offs[i], offs[i + 1]
            assert rel_l2(y[a:b], O.fft_cpx(x[a:b])) <= TOL32, int(lengths[i])
    finally:
        libf.L.kfft_release_uneven(p)


def test_queue_wait_gives_up_and_reports(libf, lib):
    """A dependency that is never met (a counter nothing increments) makes the
    queue kernel's bounded wait give up, set its error word and return; the
    context stays usable.  The control queue, whose dependency is met,
    reports no error."""
    for L in (libf, lib):
        assert L.L.kfft_gb300_queue_selftest(1 << 12, 1) == 0
        assert L.L.kfft_gb300_queue_selftest(1 << 12, 0) == 1
        assert L.L.kfft_gb300_queue_selftest(1 << 12, 1) == 0  # still usable
    x = np.arange(64, dtype=np.complex128)
    assert rel_l2(lib.fft_cpx(x), O.fft_cpx(x)) <= 1e-13 * 6


def test_bulk_copy_wait_gives_up_and_reports(libf):
    """The FP32 single-pass kernel that receives its tiles by bulk copy waits
    on each copy with a bounded poll loop.  With the limit lowered to one
    non-blocking poll, the first wait of every CTA runs out on a valid copy
    still in flight: the CTA records the failure, waits (with the default
    limit) for that copy to land and stops.  The synchronous call must then
    return KFFT_RET_BUFFER_FAIL, the asynchronous one must report it through
    kfft_gb300_check_waits, and with the default limit restored the same
    calls succeed and match the FP64 oracle in the same context."""
    n, batch = 4096, 4096  # 2^24 points: more tiles than resident CTAs, so the bulk path runs
    rng = np.random.default_rng(31)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    p = libf._plan("kfft_config_cpx", n, 0)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    try:
        torch.cuda.synchronize()
        libf.L.kfft_gb300_set_bulk_wait_polls(1)
        try:
            assert libf.L.kfft_eval_cpx_batch(p, xd.data_ptr(), yd.data_ptr(), batch) == K.RET_BUFFER_FAIL
            assert "wait" in libf.last_error()
            assert libf.L.kfft_eval_cpx_async(p, xd.data_ptr(), yd.data_ptr(), batch, None) == 0
            assert libf.L.kfft_gb300_check_waits(None) == 1
            assert libf.L.kfft_gb300_check_waits(None) == 0  # the record was cleared
        finally:
            libf.L.kfft_gb300_set_bulk_wait_polls(0)
        yd.zero_()
        torch.cuda.synchronize()
        assert libf.L.kfft_eval_cpx_batch(p, xd.data_ptr(), yd.data_ptr(), batch) == 0
        assert libf.L.kfft_eval_cpx_async(p, xd.data_ptr(), yd.data_ptr(), batch, None) == 0
        assert libf.L.kfft_gb300_check_waits(None) == 0
        y = yd.cpu().numpy()
        for b in (0, 1, batch // 2, batch - 1):
            assert rel_l2(y[b], O.fft_cpx(x[b])) <= TOL32
    finally:
        libf.cleanup(p)


@pytest.mark.parametrize("logn", list(range(4, 13)) + [13, 16, 20, 22])
def test_pipelined_power_of_two_passes(libf, logn):
    """FP32 power-of-two passes run as resident CTAs that loop over many
    tiles (2^22 points per call: more tiles than the GPU holds at once).
    Forward and inverse against numpy's FP64 FFT, round trip, both directions
    and in place."""
    n = 1 << logn
    batch = max(1, (1 << 22) // n)
    rng = np.random.default_rng(logn)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    fwd = libf._plan("kfft_config_cpx", n, 0)
    inv = libf._plan("kfft_config_cpx", n, K.FLAG_INVERSE)
    try:
        torch.cuda.synchronize()
        assert libf.L.kfft_eval_cpx_async(fwd, xd.data_ptr(), yd.data_ptr(), batch, None) == 0
        torch.cuda.synchronize()
        y = yd.cpu().numpy()
        rows = sorted({0, batch // 2, batch - 1})
        ref = np.fft.fft(x[rows].astype(np.complex128), axis=-1)
        assert rel_l2(y[rows], ref) <= TOL32
        # inverse in place on the device
        assert libf.L.kfft_eval_cpx_async(inv, yd.data_ptr(), yd.data_ptr(), batch, None) == 0
        torch.cuda.synchronize()
        assert rel_l2(yd.cpu().numpy(), x) <= TOL32
    finally:
        libf.cleanup(fwd)
        libf.cleanup(inv)


def test_device_buffers_on_a_fresh_plan_need_no_workspace(lib, libf):
    """A fresh 2D or real plan whose passes need no scratch, called first with
    device buffers (nothing to stage), runs instead of failing for want of a
    workspace allocation of zero bytes."""
    for L, cdt, rdt, tol in ((lib, torch.complex128, torch.float64, 1e-13 * 12),
                             (libf, torch.complex64, torch.float32, TOL32)):
        rng = np.random.default_rng(5)
        a = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
        p = L.L.kfft_config2_cpx(64, 64, 0, None, None)
        ad = torch.from_numpy(a.astype(L.cpx)).cuda()
        od = torch.empty_like(ad)
        torch.cuda.synchronize()
        assert L.L.kfft_eval2_cpx(p, ad.data_ptr(), od.data_ptr()) == 0, L.last_error()
        assert rel_l2(od.cpu().numpy(), np.fft.fft2(a)) <= tol
        L.cleanup(p)
        x = rng.standard_normal(4096)
        p = L.L.kfft_config_scalar(4096, 0, None, None)
        xd = torch.from_numpy(x.astype(L.real)).cuda()
        yd = torch.empty(2049, dtype=cdt, device="cuda")
        torch.cuda.synchronize()
        assert L.L.kfft_eval_scalar(p, xd.data_ptr(), yd.data_ptr()) == 0, L.last_error()
        assert rel_l2(yd.cpu().numpy(), np.fft.rfft(x)) <= tol
        L.cleanup(p)


def test_2d_rows_through_bulk_copies(libf):
    """Rows of 4096 contiguous points, 1024 of them: the row pass runs on
    bulk-copied tiles; the 2D result against numpy's FP64 FFT."""
    rng = np.random.default_rng(23)
    a = (rng.standard_normal((1024, 4096)) + 1j * rng.standard_normal((1024, 4096))).astype(np.complex64)
    p = libf.L.kfft_config2_cpx(4096, 1024, 0, None, None)
    try:
        ad = torch.from_numpy(a).cuda()
        od = torch.empty_like(ad)
        torch.cuda.synchronize()
        assert libf.L.kfft_eval2_cpx(p, ad.data_ptr(), od.data_ptr()) == 0, libf.last_error()
        assert rel_l2(od.cpu().numpy(), np.fft.fft2(a.astype(np.complex128))) <= TOL32
    finally:
        libf.cleanup(p)


@pytest.mark.parametrize("n,batch", [(1 << 16, 300),   # 78 MB in: split into chunks; 262152-byte spectra
                                     (4095, 5000)])    # odd length: full complex transforms, 80 MB in
def test_chunked_host_real_batch_matches_device_path(libf, n, batch):
    """Real forward and inverse batches with host buffers run in overlapping
    chunks whose copies start on 256-byte boundaries; results equal the
    device-buffer path bit for bit."""
    rng = np.random.default_rng(23)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    bins = n if n % 2 else n // 2 + 1  # an odd length gives all n bins, as in the reference
    fwd = libf.L.kfft_config_scalar(n, 0, None, None)
    inv = libf.L.kfft_config_scalar(n, K.FLAG_INVERSE, None, None)
    assert fwd and inv, libf.last_error()
    try:
        xd = torch.from_numpy(x).cuda()
        Xd = torch.empty((batch, bins), dtype=torch.complex64, device="cuda")
        yd = torch.empty_like(xd)
        torch.cuda.synchronize()
        assert libf.L.kfft_eval_scalar_batch(fwd, xd.data_ptr(), Xd.data_ptr(), batch) == 0
        assert libf.L.kfft_evali_scalar_batch(inv, Xd.data_ptr(), yd.data_ptr(), batch) == 0
        torch.cuda.synchronize()
        X_ref, y_ref = Xd.cpu().numpy(), yd.cpu().numpy()
        X = np.zeros((batch, bins), dtype=np.complex64)
        y = np.zeros_like(x)
        assert libf.L.kfft_eval_scalar_batch(fwd, x.ctypes.data, X.ctypes.data, batch) == 0
        assert libf.L.kfft_evali_scalar_batch(inv, X_ref.ctypes.data, y.ctypes.data, batch) == 0
        assert np.array_equal(X, X_ref)
        assert np.array_equal(y, y_ref)
        spectrum = np.fft.fft if n % 2 else np.fft.rfft
        for b in (0, batch // 3, batch - 1):
            assert rel_l2(X[b], spectrum(x[b].astype(np.float64))) <= TOL32
    finally:
        libf.cleanup(fwd)
        libf.cleanup(inv)
