"""Concurrent evaluation of one shared plan from several host threads.

The reference lets threads evaluate one plan at once (the 2D extension calls
kfft_eval_cpx on a shared plan from an OpenMP loop, ext/2d/kfft_cpx2.c:100-104).
Here each calling thread gets its own device workspace and its own stream, so
calls on one plan overlap instead of taking turns: 8 threads each run 12
synchronous calls on one FP32 plan (device and host buffers, complex and
real) and every result equals the single-threaded result bit for bit; and a
short call made while another thread's long call on the same plan is in
flight returns first (a per-plan lock would make it wait)."""
import threading
import time

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import TOL32, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

THREADS, CALLS = 8, 12


@pytest.mark.parametrize("where", ["device", "host"])
def test_threads_share_one_complex_plan(libf, where):
    n, batch = 1 << 16, 32
    plan = libf._plan("kfft_config_cpx", n, 0)
    rng = np.random.default_rng(5)
    xs = [(rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
          for _ in range(THREADS)]
    try:
        # single-threaded results first
        expect = []
        for x in xs:
            y = np.empty_like(x)
            assert libf.L.kfft_eval_cpx_batch(plan, x.ctypes.data, y.ctypes.data, batch) == 0
            expect.append(y)
        if where == "device":
            ins = [torch.from_numpy(x).cuda() for x in xs]
            outs = [torch.empty_like(t) for t in ins]
            torch.cuda.synchronize()
            ptrs = [(a.data_ptr(), b.data_ptr()) for a, b in zip(ins, outs)]
        else:
            outs = [np.empty_like(x) for x in xs]
            ptrs = [(a.ctypes.data, b.ctypes.data) for a, b in zip(xs, outs)]
        errors = []

        def work(t):
            try:
                for _ in range(CALLS):
                    r = libf.L.kfft_eval_cpx_batch(plan, ptrs[t][0], ptrs[t][1], batch)
                    if r != 0:
                        errors.append((t, r))
            except Exception as e:  # pragma: no cover - reported below
                errors.append((t, repr(e)))

        th = [threading.Thread(target=work, args=(t,)) for t in range(THREADS)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errors, errors
        for t in range(THREADS):
            got = outs[t].cpu().numpy() if where == "device" else outs[t]
            assert np.array_equal(got, expect[t]), t
        assert rel_l2(expect[0][0], O.fft_cpx(xs[0][0])) <= TOL32
    finally:
        libf.cleanup(plan)


def test_short_call_does_not_wait_for_a_long_one_on_the_same_plan(libf):
    """Thread A transforms 2^26 points from pinned host memory (copies of
    512 MiB each way: several milliseconds); thread B starts a 2^16-point
    device-buffer call on the same plan once A is under way.  B must return
    before A does."""
    n = 1 << 16
    plan = libf._plan("kfft_config_cpx", n, 0)
    big_batch = 1 << 10
    rng = np.random.default_rng(8)
    xa = torch.from_numpy((rng.standard_normal((big_batch, n)) +
                           1j * rng.standard_normal((big_batch, n))).astype(np.complex64)).pin_memory()
    ya = torch.empty_like(xa).pin_memory()
    xb = torch.randn(n, dtype=torch.complex64, device="cuda")
    yb = torch.empty_like(xb)
    torch.cuda.synchronize()
    ends, rets = {}, []
    warm = threading.Barrier(2)
    started = threading.Event()

    def long_call():
        # each thread first warms its own workspace and the kernels it uses
        rets.append(libf.L.kfft_eval_cpx_batch(plan, xa.data_ptr(), ya.data_ptr(), big_batch))
        warm.wait()
        started.set()
        rets.append(libf.L.kfft_eval_cpx_batch(plan, xa.data_ptr(), ya.data_ptr(), big_batch))
        ends["a"] = time.perf_counter()

    def short_call():
        rets.append(libf.L.kfft_eval_cpx_batch(plan, xb.data_ptr(), yb.data_ptr(), 1))
        warm.wait()
        started.wait()
        time.sleep(0.001)
        rets.append(libf.L.kfft_eval_cpx_batch(plan, xb.data_ptr(), yb.data_ptr(), 1))
        ends["b"] = time.perf_counter()

    try:
        ta, tb = threading.Thread(target=long_call), threading.Thread(target=short_call)
        ta.start()
        tb.start()
        ta.join()
        tb.join()
        assert rets == [0, 0, 0, 0] and set(ends) == {"a", "b"}
        assert ends["b"] < ends["a"]
        assert rel_l2(yb.cpu().numpy(), O.fft_cpx(xb.cpu().numpy())) <= TOL32
    finally:
        libf.cleanup(plan)


def test_threads_share_one_real_plan(lib):
    n, batch = 1 << 14, 16
    plan = lib._plan("kfft_config_scalar", n, 0)
    rng = np.random.default_rng(6)
    xs = [rng.uniform(-1, 1, (batch, n)) for _ in range(THREADS)]
    bins = n // 2 + 1
    outs = [np.zeros((batch, bins), np.complex128) for _ in range(THREADS)]
    errors = []

    def work(t):
        for _ in range(CALLS):
            r = lib.L.kfft_eval_scalar_batch(plan, xs[t].ctypes.data, outs[t].ctypes.data, batch)
            if r != 0:
                errors.append((t, r))

    try:
        th = [threading.Thread(target=work, args=(t,)) for t in range(THREADS)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errors, errors
        for t in range(THREADS):
            for b in (0, batch - 1):
                assert rel_l2(outs[t][b], O.rfft(xs[t][b])) <= 1e-13 * 14
    finally:
        lib.cleanup(plan)
