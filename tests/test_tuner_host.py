"""Host side of the plan tuner: features, the regret arithmetic, the tuning
database, and the FP64 restatement of the cost model that the GPU training
kernels are checked against (pinned here by finite differences)."""
import json
import math

import numpy as np
import pytest

from kfft_gb300 import tuner as T
from oracle import mlp_ref


def test_factorize_and_inner_length():
    assert T.factorize(2 ** 10 * 3 ** 2 * 13) == {2: 10, 3: 2, 13: 1}
    assert T.factorize(999983) == {999983: 1}
    assert T.inner_length(4096) == 0                 # direct
    assert T.inner_length(31 * 29 * 16) == 0         # direct: primes up to 31
    assert T.inner_length(65537) == 65536            # Rader on a direct p-1
    assert T.inner_length(4099) == 8232              # 4098 = 2*3*683: Bluestein
    assert T.inner_length(37 * 2) == 147             # composite with a large prime
    m = T.inner_length(999983)
    assert m >= 2 * 999983 - 1 and T._smooth7(m)


def test_feature_vector_layout():
    nvar = 10
    f = T.features(4096, 4096, "float", 3, nvar)
    assert f.dtype == np.float32 and f.shape == (T.N_BASE_FEATURES + nvar,)
    assert f[0] == 12 and f[1] == 12 and f[2] == 1.0
    assert f[3] == 12                                  # exponent of 2
    assert list(f[-nvar:]) == [0, 0, 0, 1, 0, 0, 0, 0, 0, 0]
    g = T.features(65537, 256, "double", 0, nvar)
    assert g[2] == 0.0
    inner = g[3 + len(T.SMALL_PRIMES) + 2:]
    assert inner[0] == 16                              # the Rader length 2^16


def _fd_grad(p, X, y, idx, h=1e-6):
    out = []
    for i in idx:
        a = p.copy()
        a[i] += h
        b = p.copy()
        b[i] -= h
        out.append((mlp_ref.loss_grad(a, X, y)[0] - mlp_ref.loss_grad(b, X, y)[0]) / (2 * h))
    return np.asarray(out)


def test_mlp_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    d = 7
    X = rng.standard_normal((40, d))
    y = rng.standard_normal(40)
    p = rng.standard_normal(mlp_ref.n_params(d)) * 0.3
    loss, g = mlp_ref.loss_grad(p, X, y)
    assert g.shape == p.shape and math.isfinite(loss)
    assert loss == pytest.approx(np.mean((mlp_ref.forward(p, X) - y) ** 2))
    idx = rng.choice(len(p), size=60, replace=False)
    fd = _fd_grad(p, X, y, idx)
    assert np.allclose(g[idx], fd, rtol=1e-5, atol=1e-7)


def test_adam_reference_step():
    p = np.array([1.0, -2.0])
    g = np.array([0.5, -0.25])
    p1, m, v = mlp_ref.adam_step(p, g, np.zeros(2), np.zeros(2), 1, lr=0.1)
    # the first bias-corrected step moves each parameter by lr against its gradient's sign
    assert np.allclose(p1, p - 0.1 * np.sign(g), atol=1e-6)


class _FixedModel:
    """Stand-in for CostModel.propose with a fixed answer per length."""

    def __init__(self, answers):
        self.answers = answers

    def propose(self, n, batch, variants):
        return self.answers[n]


def _recs():
    R = T.Record
    return [R(64, 8, 0, "a", 2.0), R(64, 8, 1, "b", 1.0), R(64, 8, 2, "c", 4.0),
            R(128, 4, 0, "a", 1.0), R(128, 4, 1, "b", 3.0)]


def test_regret_and_gain_arithmetic():
    recs = _recs()
    r = T.evaluate(_FixedModel({64: 1, 128: 0}), recs)
    assert r.lengths == 2 and r.geomean_regret == 1.0 and r.hit_rate == 1.0
    assert r.geomean_gain == pytest.approx(math.sqrt(2.0))
    r = T.evaluate(_FixedModel({64: 2, 128: 1}), recs)
    assert r.geomean_regret == pytest.approx(math.sqrt(4.0 * 3.0))
    assert r.max_regret == 4.0 and r.hit_rate == 0.0
    assert r.ms_chosen == 7.0 and r.ms_best == 2.0 and r.ms_default == 3.0


def test_split_is_by_length_and_seeded():
    recs = [T.Record(n, 1, v, str(v), 1.0) for n in range(10, 60) for v in range(3)]
    a, b = T.split_lengths(recs, 0.2, seed=3)
    la, lb = {r.n for r in a}, {r.n for r in b}
    assert len(la) == 10 and not (la & lb) and len(la | lb) == 50
    assert {r.n for r in T.split_lengths(recs, 0.2, seed=3)[0]} == la


def test_tune_db_roundtrip(tmp_path):
    path = tmp_path / "tune.json"
    db = T.TuneDB(str(path))
    db.update("float", _recs())
    assert db.best["float"] == {64: 1, 128: 0}
    db.save()
    raw = json.loads(path.read_text())
    assert raw["float"] == {"64": 1, "128": 0}
    assert T.TuneDB(str(path)).best["float"] == {64: 1, 128: 0}
