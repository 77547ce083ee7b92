"""The estimators' device="cuda" route on the GPU, against the direct API and the oracle.

A fit through an estimator must give exactly the trees of the same fit through the
device-binned dataset and the trainer (its bins equal the host's QuantizeDense), and those
trees are the oracle's fixed-point replica's. Predictions from raw matrices equal the
training predictions (up to the float32 output type of the reference's predict).
"""

from __future__ import annotations

import numpy as np
import pytest

import mpsboost_gb300 as mb
import oracle
from conftest import seeded_matrix

pytestmark = pytest.mark.gpu


def _data(seed, n=6000, f=8, nan=0.05):
    x = seeded_matrix(seed, n, f, nan, 2)
    rng = np.random.default_rng(seed + 1)
    xs = np.nan_to_num(x)
    y = np.sin(xs[:, 0]) + xs[:, 1] * xs[:, 2] + rng.normal(size=n) * 0.1
    return x, y, rng.uniform(0.5, 1.5, n)


@pytest.mark.parametrize("max_bins", [255, 256, 1024])
def test_regressor_equals_direct_fit_and_replica(backend, port, max_bins):
    """255 bins: u8; 256 (the reference's default) with missing values and 1024: u16 bins."""
    x, y, w = _data(61)
    model = mb.GradientBoostingRegressor(n_estimators=4, max_depth=5, learning_rate=0.2, max_bins=max_bins)
    assert model.fit(x, y, sample_weight=w) is model
    assert model.device_ == "cuda" and model.n_estimators_ == 4
    assert model.device_decision_["selected"] == "cuda"
    binned = mb.quantize_dense(x, max_bins)
    params = dict(n_estimators=4, max_depth=5, learning_rate=0.2, min_samples_leaf=20, min_child_weight=1.0)
    direct = mb.train_regressor(backend, binned, y, w, **params)
    trees = model.model_.model.trees
    assert [t.tobytes() for t in trees] == [t.tobytes() for t in direct.trees]
    want = port.train_regressor(port.quantize_dense(x, max_bins), y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert [t.tobytes() for t in trees] == [t.tobytes() for t in want.trees]
    pred = model.predict(x)
    assert pred.dtype == np.float32
    assert np.array_equal(pred, direct.train_predictions.astype(np.float32))
    assert model.score(x, y) > 0.5


def test_poisson_predictions_are_exponentiated(backend):
    x, y, _ = _data(62)
    y = np.floor(np.exp(np.clip(y, -2, 2)))
    model = mb.GradientBoostingRegressor(n_estimators=3, max_depth=4, max_bins=255, loss="poisson").fit(x, y)
    raw = model.model_.predict(x).astype(np.float64)
    assert np.allclose(model.predict(x), np.exp(raw), rtol=1e-6)


def test_binary_classifier(backend):
    x, y, _ = _data(63)
    labels = np.where(y > np.median(y), 7, 3)  # any two class values
    clf = mb.GradientBoostingClassifier(n_estimators=4, max_depth=5, max_bins=255).fit(x, labels)
    assert list(clf.classes_) == [3, 7]
    binned = mb.quantize_dense(x, 255)
    direct = mb.train_regressor(backend, binned, (labels == 7).astype(float), None, n_estimators=4,
                                max_depth=5, min_samples_leaf=20, min_child_weight=1.0,
                                objective="binary_logistic")
    assert [t.tobytes() for t in clf.model_.model.trees] == [t.tobytes() for t in direct.trees]
    proba = clf.predict_proba(x)
    assert proba.shape == (x.shape[0], 2) and np.allclose(proba.sum(axis=1), 1.0, atol=1e-6)
    assert set(np.unique(clf.predict(x))) <= {3, 7}
    assert clf.score(x, labels) > 0.7


@pytest.mark.parametrize("strategy", ["ovr", "softmax"])
def test_multiclass_classifier(backend, strategy):
    x, y, _ = _data(64, n=8000)
    labels = np.digitize(y, np.quantile(y, [0.25, 0.5, 0.75]))  # four classes
    clf = mb.GradientBoostingClassifier(n_estimators=3, max_depth=4, max_bins=255,
                                        multi_strategy=strategy).fit(x, labels)
    assert list(clf.classes_) == [0, 1, 2, 3]
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=3, max_depth=4, min_samples_leaf=20, min_child_weight=1.0)
    if strategy == "ovr":
        direct = mb.train_ovr(backend, binned, labels.astype(float), 4, **params)
        assert [t.tobytes() for m in direct for t in m.trees] == \
               [t.tobytes() for e in clf.estimators_ for t in e.model.trees]
    else:
        direct = mb.train_softmax(backend, binned, labels.astype(float), 4, **params)
        assert [t.tobytes() for t in direct.trees] == [t.tobytes() for t in clf.model_.trees]
    proba = clf.predict_proba(x)
    assert proba.shape == (x.shape[0], 4) and np.allclose(proba.sum(axis=1), 1.0, atol=1e-5)
    assert clf.score(x, labels) > 0.5


def test_random_forest_regressor(backend):
    x, y, _ = _data(65, n=20000, f=10)
    rf = mb.RandomForestRegressor(n_estimators=16, max_depth=6, max_features=0.5, random_state=3,
                                  max_bins=255, device="auto").fit(x, y)
    assert rf.n_estimators_ == 16 and len(rf.feature_subsets_) == 16
    counts, subsets, seeds = mb.forest_samples(x.shape[0], x.shape[1], 16, random_state=3, max_features=0.5)
    binned = mb.quantize_dense(x, 255)
    trees = mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=[np.sort(s) for s in subsets],
                            seeds=seeds, max_depth=6, min_samples_leaf=20, min_child_weight=1.0)
    assert [t.trees[0].tobytes() for t in trees] == [t.tobytes() for t in rf.model_.model.trees]
    per_tree = np.mean([t.predict(backend, binned) for t in trees], axis=0)
    np.testing.assert_allclose(rf.predict(x), per_tree, rtol=1e-5, atol=1e-5)
    assert rf.score(x, y) > 0.3
