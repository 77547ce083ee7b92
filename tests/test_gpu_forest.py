"""Forest training (every tree of a batch built in the same launches) against the oracle.

A forest tree fits the reference's single-tree trainer on its sample,
matrix[rows][:, features] (forest_sampling.py:42-63), here with this dataset's bins. The
oracle materializes that sample (``dataset_subset``) and trains one fixed-point round on
it; the GPU tree must equal it bit for bit once the sample's local feature indices are
mapped back to the dataset's.
"""

from __future__ import annotations

import numpy as np
import pytest

import mpsboost_gb300 as mb
import oracle
from conftest import seeded_matrix

pytestmark = pytest.mark.gpu


def _data(seed, rows, feats, nan=0.0, ints=0, objective="squared_error"):
    x = seeded_matrix(seed, rows, feats, nan, ints)
    rng = np.random.default_rng(seed + 1)
    xs = np.nan_to_num(x)
    y = np.sin(xs[:, 0]) + xs[:, 1] * xs[:, 2] + 0.5 * xs[:, 3] ** 2 + rng.normal(size=rows) * 0.1
    if objective == "binary_logistic":
        y = (y > np.median(y)).astype(np.float64)
    return x, y, rng.uniform(0.5, 1.5, rows)


def _oracle_tree(port, ds, y, w, counts, subset, params, seed=None):
    rows = np.repeat(np.arange(y.size), counts)
    feats = np.sort(np.asarray(subset))
    sub = port.dataset_subset(ds, rows, feats)
    p = dict(params, n_estimators=1, learning_rate=1.0)
    if seed is not None:
        p["random_seed"] = int(seed)
    model = port.train_regressor(sub, y[rows], None if w is None else w[rows],
                                 hist_mode=oracle.HIST_FIXED, **p)
    nodes = model.trees[0].copy()
    split = (nodes["flags"] & 1) == 0
    nodes["feature_index"][split] = feats[nodes["feature_index"][split]]
    return model.base_score, nodes


CASES = {
    "bootstrap": dict(seed=51, rows=3000, feats=10, nan=0.0, ints=2, trees=6, max_features=0.4,
                      params=dict(max_depth=5, min_samples_leaf=3)),
    "missing": dict(seed=52, rows=2500, feats=8, nan=0.1, ints=1, trees=5, max_features=0.5,
                    params=dict(max_depth=6, min_samples_leaf=2, min_child_weight=0.5)),
    "no_bootstrap": dict(seed=53, rows=2000, feats=6, nan=0.0, ints=0, trees=4, max_features=1.0,
                         bootstrap=False, sample_fraction=0.7, params=dict(max_depth=4)),
    "extra_trees": dict(seed=54, rows=2000, feats=7, nan=0.05, ints=0, trees=5, max_features=0.6,
                        params=dict(max_depth=5, min_samples_leaf=2, split_strategy="random_threshold")),
    "logistic": dict(seed=55, rows=3000, feats=8, nan=0.0, ints=2, trees=4, max_features=0.5,
                     objective="binary_logistic", params=dict(max_depth=4, min_samples_leaf=4)),
    # u16 bins (1000 per feature, missing values): the wide kernels under ragged forests.
    "wide_bins": dict(seed=56, rows=4000, feats=9, nan=0.05, ints=1, trees=5, max_features=0.6,
                      max_bins=1000, params=dict(max_depth=5, min_samples_leaf=3)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_forest_trees_bit_exact_to_replica(backend, port, name):
    c = CASES[name]
    objective = c.get("objective", "squared_error")
    x, y, w = _data(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"], objective)
    counts, subsets, seeds = mb.forest_samples(
        c["rows"], c["feats"], c["trees"], random_state=c["seed"], bootstrap=c.get("bootstrap", True),
        sample_fraction=c.get("sample_fraction", 1.0), max_features=c["max_features"])
    params = dict(c["params"], objective=objective)
    max_bins = c.get("max_bins", 64)
    binned = mb.quantize_dense(x, max_bins)
    models = mb.train_forest(backend, binned, y, w, row_counts=counts, feature_subsets=subsets,
                             seeds=seeds, **dict(params, max_bins=max_bins))
    ds = port.quantize_dense(x, max_bins)
    assert len(models) == c["trees"]
    for t, m in enumerate(models):
        base, nodes = _oracle_tree(port, ds, y, w, counts[t], subsets[t], dict(params, max_bins=max_bins), seeds[t])
        assert float(m.base_score).hex() == float(base).hex()
        assert m.learning_rate == 1.0 and len(m.trees) == 1
        assert m.trees[0].tobytes() == nodes.tobytes(), f"tree {t}"


def test_forest_batches_agree(backend, monkeypatch):
    """Trees do not depend on how many share a launch."""
    x, y, w = _data(56, 4000, 12, 0.02, 2)
    counts, subsets, seeds = mb.forest_samples(4000, 12, 7, random_state=3, max_features=0.5)
    binned = mb.quantize_dense(x, 255)
    params = dict(max_depth=6, min_samples_leaf=2)
    a = mb.train_forest(backend, binned, y, w, row_counts=counts, feature_subsets=subsets, seeds=seeds, **params)
    monkeypatch.setenv("MPSB_FOREST_BATCH", "3")
    b = mb.train_forest(backend, binned, y, w, row_counts=counts, feature_subsets=subsets, seeds=seeds, **params)
    for m1, m2 in zip(a, b):
        assert m1.base_score == m2.base_score
        assert m1.trees[0].tobytes() == m2.trees[0].tobytes()


def test_forest_errors(backend):
    x, y, w = _data(57, 300, 4)
    binned = mb.quantize_dense(x, 16)
    counts, subsets, _ = mb.forest_samples(300, 4, 2, random_state=1)
    empty = counts.copy()
    empty[1] = 0
    with pytest.raises(mb.TrainingError, match="sample"):
        mb.train_forest(backend, binned, y, row_counts=empty, feature_subsets=subsets, max_depth=2)
    with pytest.raises(mb.TrainingError, match="repeat"):
        mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=[[0, 0], [1]], max_depth=2)
    with pytest.raises(mb.TrainingError, match="range"):
        mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=[[0], [9]], max_depth=2)
    with pytest.raises(mb.UnsupportedError, match="interaction"):
        mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=subsets, max_depth=2,
                        interaction_constraints=[[0, 1]])


def test_forest_scale_properties(backend):
    """1M rows x 100 features, depth 12, max_features = sqrt (10): the ragged Poisson(1)
    samples of 16 trees built in the same launches. Deterministic; every split uses the
    tree's own features; base scores are the samples' means; every tree lowers the squared
    error on its own sample."""
    n, f, trees = 1_000_000, 100, 16
    rng = np.random.default_rng(58)
    x = rng.normal(size=(n, f)).astype(np.float32)
    y = (10 * np.sin(np.pi * x[:, 0] * x[:, 1]) + 20 * (x[:, 2] - 0.5) ** 2 + 10 * x[:, 3] + 5 * x[:, 4]
         + rng.normal(size=n))
    counts = np.random.default_rng(59).poisson(1.0, size=(trees, n)).astype(np.uint8)
    subsets = [np.random.default_rng(60 + t).choice(f, size=10, replace=False) for t in range(trees)]
    binned = mb.quantize_dense(x, 255)
    params = dict(max_depth=12, min_samples_leaf=20)
    a = mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=subsets, **params)
    b = mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=subsets, **params)
    for t in range(trees):
        assert a[t].trees[0].tobytes() == b[t].trees[0].tobytes()
        nodes = a[t].trees[0]
        split = (nodes["flags"] & 1) == 0
        assert set(nodes["feature_index"][split]) <= set(subsets[t].tolist())
        rows = np.repeat(np.arange(n), counts[t])
        assert a[t].base_score == pytest.approx(y[rows].mean(), rel=1e-12)
        pred = a[t].predict(backend, binned)
        assert np.mean((y[rows] - pred[rows]) ** 2) < np.mean((y[rows] - a[t].base_score) ** 2)
