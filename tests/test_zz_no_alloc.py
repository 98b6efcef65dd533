"""kfft_eval_cpx_noalloc: the complex transform for callers that cannot call
cudaMalloc (graph-capture regions, allocator-free real-time loops, hosts whose
framework owns every allocation).

It must give the same result as the allocating entry point
(kfft_eval_cpx_async) on two calls in a row, allocate no device memory while
doing it, and reject what does not fit its fixed 32 MiB scratch array.  This
file sorts last so that a run stopping at the first failure has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import kfft_gb300 as K
from oracle import oracle as O
from tests.helpers import TOL32, rel_l2, tol64

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _run_pair(lib, n, batch, flags, cdt, seed):
    """Two calls of each entry point in a row on fresh inputs; returns the worst error."""
    L = lib.L
    plan = L.kfft_config_cpx(n, flags, None, None)
    assert plan, lib.last_error()
    try:
        rng = np.random.default_rng(seed)
        stream = torch.cuda.Stream()
        worst = 0.0
        for call in range(2):
            x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(cdt)
            xd = torch.from_numpy(x).cuda()
            ref = torch.empty_like(xd)
            out = torch.empty_like(xd)
            torch.cuda.synchronize()
            assert L.kfft_eval_cpx_async(plan, xd.data_ptr(), ref.data_ptr(), batch,
                                         ctypes.c_void_p(stream.cuda_stream)) == 0
            stream.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            bytes_before = lib.stats().device_bytes
            r = L.kfft_eval_cpx_noalloc(plan, xd.data_ptr(), out.data_ptr(), batch,
                                        ctypes.c_void_p(stream.cuda_stream))
            assert r == 0, L.kfft_noalloc_last_message()
            stream.synchronize()
            # the first call on a device may load the module that holds the
            # scratch array; from then on free device memory does not move
            if call == 1:
                assert torch.cuda.mem_get_info()[0] == free_before
            assert lib.stats().device_bytes == bytes_before
            y = out.cpu().numpy()
            worst = max(worst, rel_l2(y, ref.cpu().numpy()))
            # and against the FP64 oracle on the first and last sequence
            for b in sorted({0, batch - 1}):
                worst = max(worst, rel_l2(y[b], O.fft_cpx(x[b].astype(np.complex128), flags)))
        return worst
    finally:
        lib.cleanup(plan)


@pytest.mark.parametrize("precision,n,batch", [("double", 1 << 18, 2), ("float", 3 * 5 * 7 * 16 * 64, 3)])
def test_noalloc_in_place(lib, libf, precision, n, batch):
    """fin == fout: every pass writes scratch or the output only after its
    own reads of the same elements, so the transform may run in place."""
    L = lib if precision == "double" else libf
    cdt = np.complex128 if precision == "double" else np.complex64
    plan = L.L.kfft_config_cpx(n, 0, None, None)
    assert plan, L.last_error()
    try:
        rng = np.random.default_rng(n)
        x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(cdt)
        xd = torch.from_numpy(x).cuda()
        stream = torch.cuda.Stream()
        torch.cuda.synchronize()
        for _ in range(2):  # two calls in a row, each on fresh input
            xd.copy_(torch.from_numpy(x))
            torch.cuda.synchronize()
            r = L.L.kfft_eval_cpx_noalloc(plan, xd.data_ptr(), xd.data_ptr(), batch,
                                          ctypes.c_void_p(stream.cuda_stream))
            assert r == 0, L.L.kfft_noalloc_last_message()
            assert L.L.kfft_gb300_check_waits(ctypes.c_void_p(stream.cuda_stream)) == 0
            y = xd.cpu().numpy()
            tol = tol64(n) if precision == "double" else TOL32
            for b in range(batch):
                assert rel_l2(y[b], O.fft_cpx(x[b].astype(np.complex128))) <= tol
    finally:
        L.cleanup(plan)


@pytest.mark.parametrize("n,batch,flags", [(1 << 20, 1, 0), (1 << 16, 8, K.FLAG_INVERSE),
                                           (3 * 5 * 7 * 11 * 13 * 16, 2, 0), (4096, 16, 0)])
def test_noalloc_matches_allocating_entry_fp64(lib, n, batch, flags):
    assert _run_pair(lib, n, batch, flags, np.complex128, seed=n) <= tol64(n)


@pytest.mark.parametrize("n,batch", [(1 << 21, 1), (1 << 18, 4)])
def test_noalloc_matches_allocating_entry_fp32(libf, n, batch):
    assert _run_pair(libf, n, batch, 0, np.complex64, seed=n) <= TOL32


def test_noalloc_limits(lib):
    L = lib.L
    assert L.kfft_noalloc_scratch_bytes() == 32 << 20
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # too much scratch: 2^22 fp64 needs 64 MiB
    p = L.kfft_config_cpx(1 << 22, 0, None, None)
    x = torch.zeros(1 << 22, dtype=torch.complex128, device="cuda")
    y = torch.empty_like(x)
    assert L.kfft_eval_cpx_noalloc(p, x.data_ptr(), y.data_ptr(), 1, stream) == K.RET_BADARGUMENTS
    assert b"scratch" in L.kfft_noalloc_last_message()
    lib.cleanup(p)
    # a prime length is not a direct mixed-radix plan
    p = L.kfft_config_cpx(4099, 0, None, None)
    x = torch.zeros(4099, dtype=torch.complex128, device="cuda")
    y = torch.empty_like(x)
    assert L.kfft_eval_cpx_noalloc(p, x.data_ptr(), y.data_ptr(), 1, stream) == K.RET_BADARGUMENTS
    lib.cleanup(p)
    # host buffers would need staging memory
    p = L.kfft_config_cpx(64, 0, None, None)
    h = np.zeros(64, np.complex128)
    assert L.kfft_eval_cpx_noalloc(p, h.ctypes.data, h.ctypes.data, 1, stream) == K.RET_BADARGUMENTS
    lib.cleanup(p)
