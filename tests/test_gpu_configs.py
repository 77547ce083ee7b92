"""Each benchmark configuration at its own shape, against the oracle's fixed-point replica.

The device path must build the replica's trees bit for bit (feature, threshold, missing
direction, children, gain, leaf value) on the configuration's full row and feature counts,
depth and bins; for the logistic objective the leaf values and margins agree to 1e-9
relative (the device's FP64 exp may differ from the host's by an ulp). The oracle is
handed the device's own bins (``Oracle.dataset_from_bins``), which keeps its quantile
binning (a sort per feature) out of the test's time, and trains one round per
configuration except the small CPU-runnable one (all 50 trees). Independent oracle fits
run in threads (the oracle holds no shared state; ctypes releases the interpreter lock).

Configurations (the reference's benchmark suite, seeded synthetic data of its shapes):
  0  regression 100,000 x 32, depth 6, 50 trees, lr 0.1, unit weights, FP32 histograms
  1  regression 10,000,000 x 128, depth 8, lr 0.05, U(0.5, 1.5) weights (the headline)
  2  binary logistic 4,000,000 x 256 (200 continuous, 56 with 2-16 values), 10 % missing,
     depth 10, lr 0.1
  3  one-vs-rest K = 10, 2,000,000 x 64, depth 6
  4  random forest 1,000,000 x 100, depth 12, sqrt features, Poisson(1) row counts
"""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import mpsboost_gb300 as mb
import oracle

pytestmark = pytest.mark.gpu


def _binned(bins, missing, bin_counts):
    """A binned dataset over given feature-major u8 bins with an identity schema."""
    feats, rows = bins.shape
    cnt = np.asarray(bin_counts, np.uint32) - 1
    off = np.concatenate([[0], np.cumsum(cnt, dtype=np.uint64)[:-1]]).astype(np.uint64)
    bounds = np.concatenate([np.arange(c, dtype=np.float32) + 0.5 for c in cnt])
    miss = missing.sum(axis=1, dtype=np.uint64)
    return mb.BinnedDataset(rows, feats, 255, bins, missing, bounds, off, cnt,
                            np.asarray(bin_counts, np.uint32), miss)


def _structure(trees):
    return [[(int(n["feature_index"]), int(n["threshold_bin"]), int(n["default_left"]),
              int(n["left_child"]), int(n["right_child"]), int(n["flags"])) for n in t] for t in trees]


def test_config0_small_regression(backend, port):
    """100K x 32 N(0,1); y = sin(x0) + x1 x2 + 0.5 x3^2 + N(0, 0.1); 255 bins, depth 6,
    50 trees, lr 0.1, unit weights. Fixed point: all 50 trees and the predictions
    bit-exact, and the device's bins equal the oracle's own quantile binning. Against the
    FP64 reference, both the fixed-point and the FP32-histogram path (the configuration's
    plain path) end within 1e-4 training RMSE. The trees themselves part from the FP64
    reference's at a tie: on these inputs the first tree's node 45 has two candidates
    (feature 9 bin <= 253 and feature 20 bin <= 8) whose FP64 gains agree to 1e-8
    relative, the same rows summed in two orders; fixed point takes the smaller feature,
    FP64 whichever rounding favours."""
    n, f = 100_000, 32
    rng = np.random.default_rng(20260719)
    x = rng.standard_normal((n, f), dtype=np.float32)
    y = np.sin(x[:, 0]) + x[:, 1] * x[:, 2] + 0.5 * x[:, 3].astype(np.float64) ** 2 + rng.normal(0, 0.1, n)
    params = dict(n_estimators=50, max_depth=6, learning_rate=0.1)
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    assert np.array_equal(binned.bins, ds.bins)
    model = mb.train_regressor(backend, binned, y, **params)
    want = port.train_regressor(ds, y, None, hist_mode=oracle.HIST_FIXED, **params)
    assert float(model.base_score).hex() == float(want.base_score).hex()
    assert [t.tobytes() for t in model.trees] == [t.tobytes() for t in want.trees]
    assert model.train_predictions.tobytes() == want.predict(ds).tobytes()

    plain = mb.train_regressor(backend, binned, y, hist_mode="float", **params)
    exact = port.train_regressor(ds, y, None, hist_mode=oracle.HIST_FP64, **params)
    rmse = lambda p: float(np.sqrt(np.mean((p - y) ** 2)))  # noqa: E731
    assert abs(rmse(plain.train_predictions) - rmse(exact.predict(ds))) <= 1e-4
    assert abs(rmse(model.train_predictions) - rmse(exact.predict(ds))) <= 1e-4
    first = next(i for i, (p, q) in enumerate(zip(_structure(model.trees)[0], _structure(exact.trees)[0]))
                 if p != q)
    g_fixed, g_exact = model.trees[0]["gain"][first], exact.trees[0]["gain"][first]
    assert abs(g_fixed - g_exact) <= 1e-7 * abs(g_exact)  # a tie, not a different choice


def test_config1_headline_regression(backend, port):
    """10M x 128 (64 normal, 32 lognormal, 32 integer features), y = 16 pairwise
    products + N(0, 0.5), U(0.5, 1.5) weights, 255 bins, depth 8, lr 0.05: the
    benchmark's own data and parameters; the first round bit-exact."""
    import bench

    xf, y, w = bench.make_data(bench.ROWS)
    binned = mb.quantize_dense(xf.T, bench.BINS)
    del xf
    params = dict(bench.PARAMS, n_estimators=1)
    model = mb.train_regressor(backend, binned, y, w, **params)
    ds = port.dataset_from_bins(binned)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert float(model.base_score).hex() == float(want.base_score).hex()
    assert model.trees[0].tobytes() == want.trees[0].tobytes()
    assert int((model.trees[0]["flags"] & 1).sum()) > 128  # a deep tree
    assert model.train_predictions.tobytes() == want.predict(ds).tobytes()


def test_config2_logistic_with_missing(backend, port):
    """4M x 256: 200 continuous features (255 bins) and 56 with 2-16 values, 10 % of
    cells missing; labels ~ Bernoulli(sigmoid(w . x[:32] + 0.5 x0 x1)), w ~ N(0, 1/32);
    depth 10, lr 0.1, logistic loss (non-constant hessians)."""
    n, f_cont, f_int = 4_000_000, 200, 56
    rng = np.random.default_rng(20260719 + 3)
    counts = np.concatenate([np.full(f_cont, 255), rng.integers(2, 17, f_int)]).astype(np.uint32)
    bins = np.empty((f_cont + f_int, n), np.uint8)
    bins[:f_cont] = rng.integers(0, 255, (f_cont, n), dtype=np.uint8)
    for j in range(f_int):
        bins[f_cont + j] = rng.integers(0, counts[f_cont + j], n, dtype=np.uint8)
    missing = rng.integers(0, 10, bins.shape, dtype=np.uint8) == 0
    bins[missing] = 0
    x = (bins[:32].astype(np.float32) - 127.0) / 64.0
    x[missing[:32]] = 0.0
    logit = rng.normal(0.0, np.sqrt(1.0 / 32), 32).astype(np.float32) @ x + 0.5 * x[0] * x[1]
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-logit.astype(np.float64)))).astype(np.float64)
    del x, logit
    binned = _binned(bins, missing, counts)
    params = dict(n_estimators=1, max_depth=10, learning_rate=0.1, objective="binary_logistic")
    model = mb.train_regressor(backend, binned, y, **params)
    ds = port.dataset_from_bins(binned)
    want = port.train_regressor(ds, y, None, hist_mode=oracle.HIST_FIXED, **params)
    assert float(model.base_score).hex() == float(want.base_score).hex()
    assert _structure(model.trees) == _structure(want.trees)
    assert int((model.trees[0]["flags"] & 1).sum()) > 256
    np.testing.assert_allclose(model.trees[0]["leaf_value"], want.trees[0]["leaf_value"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(model.train_predictions, want.predict(ds), rtol=1e-9, atol=1e-12)


def test_config3_one_vs_rest(backend, port):
    """2M x 64 N(0,1), class = argmax of 10 random linear scores + Gumbel noise; K = 10
    one-vs-rest logistic trees of depth 6 per round, all built in the same launches: the
    first round's ten trees against ten independent oracle binary fits."""
    n, f, k = 2_000_000, 64, 10
    rng = np.random.default_rng(20260719 + 4)
    x = rng.standard_normal((n, f), dtype=np.float32)
    scores = x @ rng.standard_normal((f, k), dtype=np.float32) + rng.gumbel(size=(n, k)).astype(np.float32)
    labels = scores.argmax(axis=1).astype(np.float64)
    del scores
    binned = mb.quantize_dense(x, 255)
    del x
    params = dict(n_estimators=1, max_depth=6, learning_rate=0.1)
    models = mb.train_ovr(backend, binned, labels, k, **params)
    ds = port.dataset_from_bins(binned)

    def fit(c):
        return port.train_regressor(ds, (labels == c).astype(np.float64), None, hist_mode=oracle.HIST_FIXED,
                                    objective="binary_logistic", **params)

    with ThreadPoolExecutor(max_workers=k) as pool:
        wants = list(pool.map(fit, range(k)))
    assert len(models) == k
    for c, (m, want) in enumerate(zip(models, wants)):
        assert float(m.base_score).hex() == float(want.base_score).hex(), c
        assert _structure(m.trees) == _structure(want.trees), c
        np.testing.assert_allclose(m.trees[0]["leaf_value"], want.trees[0]["leaf_value"], rtol=1e-9, atol=1e-12)


def test_config4_forest(backend, port):
    """1M x 100 N(0,1), Friedman-1 target on x0..x4 + N(0,1); Poisson(1) row counts per
    tree, 10 = sqrt(100) features per tree, depth 12, min_samples_leaf 20: 16 trees built
    in the same launches, each bit-exact to the oracle's fit on its own sample."""
    n, f, trees = 1_000_000, 100, 16
    rng = np.random.default_rng(20260719 + 5)
    x = rng.standard_normal((n, f), dtype=np.float32)
    u = (x[:, :5] - x[:, :5].min(0)) / (x[:, :5].max(0) - x[:, :5].min(0))
    y = (10 * np.sin(np.pi * u[:, 0] * u[:, 1]) + 20 * (u[:, 2] - 0.5) ** 2 + 10 * u[:, 3] + 5 * u[:, 4]
         + rng.normal(size=n))
    counts = rng.poisson(1.0, size=(trees, n)).astype(np.uint8)
    subsets = [np.sort(rng.choice(f, size=10, replace=False)) for _ in range(trees)]
    binned = mb.quantize_dense(x, 255)
    del x
    params = dict(max_depth=12, min_samples_leaf=20)
    models = mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=subsets, **params)
    ds = port.dataset_from_bins(binned)

    def fit(t):
        rows = np.repeat(np.arange(n), counts[t])
        sub = port.dataset_subset(ds, rows, subsets[t])
        m = port.train_regressor(sub, y[rows], None, hist_mode=oracle.HIST_FIXED, n_estimators=1,
                                 learning_rate=1.0, **params)
        nodes = m.trees[0].copy()
        split = (nodes["flags"] & 1) == 0
        nodes["feature_index"][split] = subsets[t][nodes["feature_index"][split]]
        return m.base_score, nodes

    with ThreadPoolExecutor(max_workers=8) as pool:
        wants = list(pool.map(fit, range(trees)))
    for t, (m, (base, nodes)) in enumerate(zip(models, wants)):
        assert float(m.base_score).hex() == float(base).hex(), t
        assert m.trees[0].tobytes() == nodes.tobytes(), t
