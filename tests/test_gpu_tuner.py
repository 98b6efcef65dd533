"""Plan variants, the tuning table and the learned cost model on the GPU.

* Every plan variant computes the same transform: parity with the FP64 oracle
  (FP64 build: rel-L2 <= 1e-13*log2 N; FP32 build: 1e-6, also for the
  opt-in tensor-core variant except inside Rader and Bluestein plans, where
  its two-term FP16 split is held to 1.5e-6).
* kfft_tune_set steers plain kfft_config_cpx calls.
* The MLP kernels: forward, loss and gradient against the FP64 numpy
  restatement (FP32 kernels: relative error <= 1e-4), one Adam step against
  the restatement, and training that fits.
* A small end-to-end tuning run: exhaustive timings, a model trained on 20%
  of the lengths, its regret and its gain over the default plan on the rest.
"""
import ctypes
import math

import numpy as np
import pytest

import kfft_gb300 as K
from kfft_gb300 import tuner as T
from oracle import mlp_ref
from oracle import oracle as O
from tests.helpers import TOL32, TOL32_TC, TOL32_TC_CONV, rel_l2, tol64

pytestmark = pytest.mark.gpu

LENGTHS = [4096, 1 << 18, 1 << 20, 3 * 5 * 7 * 11 * 13 * 16, 65537, 4099, 2 ** 10 * 3 ** 7]


def _eval_variant(lib, n, variant, x, flags=0):
    p = lib.L.kfft_config_cpx_variant(n, flags, variant, None, None)
    assert p, lib.last_error()
    try:
        x = np.ascontiguousarray(x, lib.cpx)
        y = np.empty_like(x)
        batch = x.size // n
        lib._check(lib.L.kfft_eval_cpx_batch(p, x.ctypes.data, y.ctypes.data, batch), "eval")
        return y, lib.describe(p)
    finally:
        lib.cleanup(p)


@pytest.mark.parametrize("n", LENGTHS)
def test_every_variant_matches_oracle_fp64(lib, n):
    rng = np.random.default_rng(n)
    batch = 2 if n <= (1 << 18) else 1
    x = rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))
    ref = np.stack([O.fft_cpx(r) for r in x])
    plans = set()
    for v in range(lib.L.kfft_variant_count()):
        y, desc = _eval_variant(lib, n, v, x)
        plans.add(desc)
        assert rel_l2(y, ref) <= tol64(n), (n, v, desc)
        back, _ = _eval_variant(lib, n, v, y, K.FLAG_INVERSE)
        assert rel_l2(back, x) <= tol64(n), (n, v)
    if n >= 1 << 18:
        assert len(plans) >= 3, plans  # the variants really are different plans


@pytest.mark.parametrize("n", LENGTHS)
def test_every_variant_matches_oracle_fp32(libf, n):
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal((1, n)) + 1j * rng.standard_normal((1, n))
    ref = O.fft_cpx(x[0])
    nvar = libf.L.kfft_variant_count()
    for v in range(nvar):
        tc = v == nvar - 1
        y, desc = _eval_variant(libf, n, v, x, K.FLAG_TENSOR_CORES if tc else 0)
        # the tensor-core variant is held to its own documented bounds
        conv = "rader" in desc or "bluestein" in desc
        tol = (TOL32_TC_CONV if conv else TOL32_TC) if tc else TOL32
        assert rel_l2(y[0], ref) <= tol, (n, v, desc)


def test_tensor_core_variant_needs_the_flag(libf, lib):
    v = libf.L.kfft_variant_count() - 1
    assert not libf.L.kfft_config_cpx_variant(4096, 0, v, None, None)
    assert lib.L.kfft_variant_count() == v  # no tensor-core variant in the double build
    assert not lib.L.kfft_config_cpx_variant(4096, 0, v, None, None)


def test_tuning_table_steers_config(lib):
    L = lib.L
    n = 1 << 18
    L.kfft_tune_clear()
    p = lib._plan("kfft_config_cpx", n, 0)
    default = lib.describe(p)
    lib.cleanup(p)
    try:
        assert L.kfft_tune_get(n, 0) == -1
        assert L.kfft_tune_set(n, 0, 3) == 0
        assert L.kfft_tune_get(n, 0) == 3
        assert L.kfft_tune_get(n, K.FLAG_INVERSE) == -1   # the direction is part of the key
        p = lib._plan("kfft_config_cpx", n, 0)
        tuned = lib.describe(p)
        lib.cleanup(p)
        p = L.kfft_config_cpx_variant(n, 0, 3, None, None)
        assert tuned == lib.describe(p) and tuned != default
        lib.cleanup(p)
        rng = np.random.default_rng(4)
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        assert rel_l2(lib.fft_cpx(x), O.fft_cpx(x)) <= tol64(n)
        assert L.kfft_tune_set(n, 0, 99) == K.RET_BADARGUMENTS
    finally:
        L.kfft_tune_clear()
    p = lib._plan("kfft_config_cpx", n, 0)
    assert lib.describe(p) == default
    lib.cleanup(p)


# ---------------------------------------------------------------------------
# MLP kernels against the FP64 restatement
# ---------------------------------------------------------------------------
def _model(lib, d, seed=3):
    h = lib.L.kfft_mlp_create(d, seed)
    assert h, lib.last_error()
    return h


def _params(lib, h):
    P = np.empty(lib.L.kfft_mlp_params(h), np.float32)
    assert lib.L.kfft_mlp_get(h, P.ctypes.data) == 0
    return P


def test_mlp_forward_and_gradient_match_cpu(lib):
    d = 23
    rng = np.random.default_rng(7)
    X = rng.standard_normal((1000, d)).astype(np.float32)
    y = rng.standard_normal(1000).astype(np.float32)
    h = _model(lib, d)
    try:
        P = _params(lib, h)
        assert len(P) == mlp_ref.n_params(d)
        out = np.empty(len(X), np.float32)
        assert lib.L.kfft_mlp_predict(h, X.ctypes.data, len(X), out.ctypes.data) == 0
        ref = mlp_ref.forward(P, X)
        assert np.max(np.abs(out - ref)) <= 1e-4 * max(1.0, np.max(np.abs(ref)))
        loss = ctypes.c_float()
        g = np.empty_like(P)
        assert lib.L.kfft_mlp_loss_grad(h, X.ctypes.data, y.ctypes.data, len(X),
                                        ctypes.byref(loss), g.ctypes.data) == 0
        rl, rg = mlp_ref.loss_grad(P, X, y)
        assert abs(loss.value - rl) <= 1e-4 * rl
        assert np.linalg.norm(g - rg) <= 1e-4 * np.linalg.norm(rg)
    finally:
        lib.L.kfft_mlp_release(h)


def test_mlp_one_adam_step_matches_cpu(libf):
    d = 9
    rng = np.random.default_rng(8)
    X = rng.standard_normal((128, d)).astype(np.float32)
    y = rng.standard_normal(128).astype(np.float32)
    h = _model(libf, d, seed=9)
    try:
        P0 = _params(libf, h)
        # one epoch with the whole set as one minibatch is exactly one Adam step
        assert libf.L.kfft_mlp_train(h, X.ctypes.data, y.ctypes.data, 128, 1, 128,
                                     ctypes.c_float(1e-2), 1, None) == 0
        P1 = _params(libf, h)
        _, g = mlp_ref.loss_grad(P0, X, y)
        ref, _, _ = mlp_ref.adam_step(P0.astype(np.float64), g, 0 * g, 0 * g, 1, lr=1e-2)
        # parameters whose gradient is clearly nonzero move by lr against its sign
        big = np.abs(g) > 1e-3 * np.max(np.abs(g))
        assert np.max(np.abs(P1[big] - ref[big])) <= 1e-5
    finally:
        libf.L.kfft_mlp_release(h)


def test_mlp_training_fits_a_smooth_function(lib):
    d = 5
    rng = np.random.default_rng(10)
    X = rng.uniform(-1, 1, (4000, d)).astype(np.float32)
    y = (np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] - 0.5 * X[:, 3] ** 2).astype(np.float32)
    h = _model(lib, d, seed=11)
    try:
        l0 = ctypes.c_float()
        assert lib.L.kfft_mlp_loss_grad(h, X.ctypes.data, y.ctypes.data, len(y),
                                        ctypes.byref(l0), None) == 0
        l1 = ctypes.c_float()
        assert lib.L.kfft_mlp_train(h, X.ctypes.data, y.ctypes.data, len(y), 40, 64,
                                    ctypes.c_float(2e-3), 5, ctypes.byref(l1)) == 0
        assert l1.value < 0.05 * float(np.var(y)) and l1.value < 0.1 * l0.value
        # the reported loss is the CPU loss of the trained parameters
        P = _params(lib, h)
        assert abs(mlp_ref.loss_grad(P, X, y)[0] - l1.value) <= 1e-3 * max(l1.value, 1e-3)
    finally:
        lib.L.kfft_mlp_release(h)


def test_mlp_rejects_bad_arguments(lib):
    assert not lib.L.kfft_mlp_create(0, 1)
    assert not lib.L.kfft_mlp_create(65, 1)
    assert lib.L.kfft_mlp_train(None, None, None, 0, 1, 1, ctypes.c_float(1e-3), 0,
                                None) == K.RET_BADARGUMENTS


# ---------------------------------------------------------------------------
# a small tuning run end to end
# ---------------------------------------------------------------------------
def test_small_tuning_run_reports_regret(libf, tmp_path):
    lengths = list(range(1000, 262144, 4357))  # 60 lengths: primes, smooth and mixed
    recs = T.exhaustive(libf, lengths, points=1 << 20, reps=3, warmup=1)
    assert {r.n for r in recs} == set(lengths)
    train, test = T.split_lengths(recs, 0.2, seed=1)
    model = T.CostModel(libf, seed=2)
    try:
        loss = model.fit(train, epochs=200)
        assert math.isfinite(loss) and loss < 1.0   # standardised targets have variance 1
        r = T.evaluate(model, test)
        assert r.lengths == len({x.n for x in test})
        assert 1.0 <= r.geomean_regret < 2.0 and r.max_regret >= r.geomean_regret
        assert r.gflops_chosen > 0 and r.gflops_default > 0
        print(f"regret geomean {r.geomean_regret:.3f} max {r.max_regret:.3f} "
              f"hit {r.hit_rate:.2f} gain {r.geomean_gain:.3f}")
        path = str(tmp_path / "model.npz")
        model.save(path)
        m2 = T.CostModel(libf, seed=99)
        m2.load(path)
        n0 = test[0].n
        assert np.allclose(m2.predict_ms(n0, test[0].batch, [0, 1]),
                           model.predict_ms(n0, test[0].batch, [0, 1]), rtol=1e-5)
        m2.close()
        db = T.TuneDB(str(tmp_path / "tune.json"))
        db.update("float", recs)
        db.save()
        assert db.install(libf) == len(lengths)
    finally:
        model.close()
        libf.L.kfft_tune_clear()


def test_uneven_batch_uses_tuned_variants(libf):
    """The uneven-batch planner takes the tuning table's variant per length
    (when it keeps register tiles); results stay within the FP32 bound."""
    lengths = np.ascontiguousarray(np.array([1 << 18, 1 << 20, 3 << 16, 1000], dtype=np.uint32))
    rng = np.random.default_rng(31)
    total = int(lengths.sum())
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    L = libf.L
    try:
        assert L.kfft_tune_set(1 << 18, 0, 2) == 0
        assert L.kfft_tune_set(1 << 20, 0, 1) == 0
        assert L.kfft_tune_set(1000, 0, 3) == 0  # shared-memory tiles: not used by the queue
        p = L.kfft_config_cpx_uneven(len(lengths), lengths.ctypes.data, 0)
        assert p, libf.last_error()
        y = np.empty_like(x)
        assert L.kfft_eval_cpx_uneven(p, x.ctypes.data, y.ctypes.data) == 0
        L.kfft_release_uneven(p)
        offs = np.concatenate([[0], np.cumsum(lengths.astype(np.int64))])
        for i in range(len(lengths)):
            a, b = offs[i], offs[i + 1]
            assert rel_l2(y[a:b], O.fft_cpx(x[a:b])) <= TOL32, int(lengths[i])
    finally:
        L.kfft_tune_clear()
