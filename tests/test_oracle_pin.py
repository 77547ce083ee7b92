"""The plain-C oracle against the reference's own compiled core on seeded inputs (CPU).

Skipped where the reference sources are absent; ``test_golden.py`` carries the same pin
through committed fixtures there.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import seeded_matrix

CASES = [
    dict(rows=2000, feats=6, nan=0.0, ints=2, max_bins=255, objective="squared_error",
         params=dict(max_depth=6, min_samples_leaf=1)),
    dict(rows=1500, feats=5, nan=0.1, ints=1, max_bins=64, objective="squared_error",
         params=dict(max_depth=5, min_samples_leaf=5, reg_alpha=0.2, max_delta_step=0.5)),
    dict(rows=1200, feats=4, nan=0.05, ints=0, max_bins=256, objective="binary_logistic",
         params=dict(max_depth=4, min_samples_leaf=2, min_child_weight=0.1)),
    dict(rows=800, feats=3, nan=0.0, ints=0, max_bins=16, objective="quantile",
         params=dict(max_depth=3, objective_alpha=0.8)),
    dict(rows=900, feats=3, nan=0.0, ints=0, max_bins=32, objective="poisson",
         params=dict(max_depth=3)),
    dict(rows=900, feats=3, nan=0.0, ints=0, max_bins=32, objective="tweedie",
         params=dict(max_depth=3, tweedie_variance_power=1.3)),
    dict(rows=1000, feats=4, nan=0.0, ints=0, max_bins=32, objective="squared_error",
         params=dict(max_depth=4, monotonic_constraints=[1, -1, 0, 1])),
    dict(rows=1000, feats=5, nan=0.0, ints=0, max_bins=32, objective="squared_error",
         params=dict(max_depth=5, interaction_constraints=[[0, 1, 2], [2, 3], [4]])),
    dict(rows=700, feats=3, nan=0.0, ints=0, max_bins=32, objective="squared_error",
         params=dict(max_depth=4, split_strategy="random_threshold", random_seed=7)),
    dict(rows=700, feats=3, nan=0.0, ints=0, max_bins=32, objective="squared_error",
         params=dict(max_depth=6, max_leaves=9, gamma=0.001, min_gain_to_split=0.0001)),
    dict(rows=300, feats=2, nan=0.3, ints=0, max_bins=300, objective="squared_error",
         params=dict(max_depth=3)),
    # u16 storage with most features near max_bins and missing values in each.
    dict(rows=4000, feats=4, nan=0.05, ints=1, max_bins=1500, objective="squared_error",
         params=dict(max_depth=5, min_samples_leaf=3)),
    dict(rows=3000, feats=3, nan=0.1, ints=0, max_bins=4096, objective="binary_logistic",
         params=dict(max_depth=4, min_samples_leaf=2)),
]


def _labels(x, objective, rng):
    base = np.nan_to_num(x[:, 0]) + 0.5 * np.nan_to_num(x[:, 1]) ** 2 + rng.normal(size=len(x)) * 0.1
    if objective == "binary_logistic":
        return (base > np.median(base)).astype(float)
    if objective in ("poisson", "tweedie"):
        return np.floor(np.exp(np.clip(base, -3, 2)))
    return base


@pytest.mark.parametrize("case", range(len(CASES)))
def test_port_matches_reference(port, reference, case):
    c = CASES[case]
    x = seeded_matrix(1000 + case, c["rows"], c["feats"], c["nan"], c["ints"])
    rng = np.random.default_rng(2000 + case)
    y = _labels(x, c["objective"], rng)
    w = rng.uniform(0.5, 1.5, c["rows"])
    dp, dr = port.quantize_dense(x, c["max_bins"]), reference.quantize_dense(x, c["max_bins"])
    assert np.array_equal(dp.bins, dr.bins) and np.array_equal(dp.missing, dr.missing)
    assert dp.boundaries_flat.tobytes() == dr.boundaries_flat.tobytes()
    assert np.array_equal(dp.bin_counts, dr.bin_counts)
    kw = dict(n_estimators=3, learning_rate=0.3, objective=c["objective"], **c["params"])
    mp = port.train_regressor(dp, y, w, hist_mode=oracle.HIST_FP64, **kw)
    mr = reference.train_regressor(dr, y, w, **kw)
    assert float(mp.base_score).hex() == float(mr.base_score).hex()
    assert len(mp.trees) == len(mr.trees)
    for tp, tr in zip(mp.trees, mr.trees):
        assert tp.tobytes() == tr.tobytes()
    assert mp.predict(dp).tobytes() == mr.predict(dr).tobytes()


@pytest.mark.parametrize("objective", ["squared_error", "binary_logistic"])
def test_port_matches_reference_at_scale(port, reference, objective):
    """The pin at the sizes the GPU parity tests rely on: 120,000 rows x 32 features (the
    small benchmark configuration's shape, with 2 % missing cells and integer columns),
    depth 8, U(0.5, 1.5) weights, three rounds; bins, every tree node and the predictions
    bit for bit. The port runs its feature-parallel loops on every core."""
    n, f = 120_000, 32
    x = seeded_matrix(4242, n, f, 0.02, 4)
    rng = np.random.default_rng(4243)
    x0, x1, x2, x3 = (np.nan_to_num(x[:, i]).astype(np.float64) for i in range(4))
    y = np.sin(x0) + x1 * x2 + 0.5 * x3 ** 2 + rng.normal(0.0, 0.1, n)
    if objective == "binary_logistic":
        y = (y > np.median(y)).astype(np.float64)
    w = rng.uniform(0.5, 1.5, n)
    dp, dr = port.quantize_dense(x, 255), reference.quantize_dense(x, 255)
    assert np.array_equal(dp.bins, dr.bins) and np.array_equal(dp.missing, dr.missing)
    assert dp.boundaries_flat.tobytes() == dr.boundaries_flat.tobytes()
    kw = dict(n_estimators=3, learning_rate=0.1, objective=objective, max_depth=8,
              min_samples_leaf=20, min_child_weight=1.0, reg_lambda=1.0)
    port.set_threads(0)
    mp = port.train_regressor(dp, y, w, hist_mode=oracle.HIST_FP64, **kw)
    mr = reference.train_regressor(dr, y, w, **kw)
    assert float(mp.base_score).hex() == float(mr.base_score).hex()
    assert [t.tobytes() for t in mp.trees] == [t.tobytes() for t in mr.trees]
    assert int((mp.trees[0]["flags"] & 1).sum()) > 32  # deep trees
    assert mp.predict(dp).tobytes() == mr.predict(dr).tobytes()


def test_port_threads_do_not_change_results(port):
    """The port's feature-parallel loops give the same trees on one thread and on all."""
    x = seeded_matrix(4244, 40_000, 24, 0.05, 3)
    rng = np.random.default_rng(4245)
    y = np.nan_to_num(x[:, 0]) * np.nan_to_num(x[:, 1]) + rng.normal(0.0, 0.1, len(x))
    w = rng.uniform(0.5, 1.5, len(x))
    ds = port.quantize_dense(x, 255)
    kw = dict(n_estimators=2, learning_rate=0.1, max_depth=7, min_samples_leaf=5)
    out = []
    for threads in (1, 0):
        port.set_threads(threads)
        for mode in (oracle.HIST_FP64, oracle.HIST_FIXED):
            m = port.train_regressor(ds, y, w, hist_mode=mode, **kw)
            out.append(b"".join(t.tobytes() for t in m.trees) + m.predict(ds).tobytes())
    port.set_threads(0)
    assert out[0] == out[2] and out[1] == out[3]


def test_histograms_and_transform_match_reference(port, reference):
    x = seeded_matrix(77, 3000, 7, 0.1, 3)
    dp, dr = port.quantize_dense(x, 255), reference.quantize_dense(x, 255)
    rng = np.random.default_rng(5)
    pairs = np.column_stack([rng.normal(size=3000), rng.uniform(0, 2, 3000)])
    rows = np.sort(rng.choice(3000, 1700, replace=False)).astype(np.uint64)
    for a, b in zip(port.histograms(dp, pairs, rows), reference.histograms(dr, pairs, rows)):
        assert a.tobytes() == b.tobytes()
    x2 = seeded_matrix(78, 500, 7, 0.2)
    tp, tr = port.transform_dense(dp, x2), reference.transform_dense(dr, x2)
    assert np.array_equal(tp.bins, tr.bins) and np.array_equal(tp.missing, tr.missing)


def test_gradients_match_reference(port, reference):
    rng = np.random.default_rng(9)
    y = rng.integers(0, 2, 500).astype(float)
    p = rng.normal(size=500) * 3
    for obj in ("squared_error", "binary_logistic", "quantile", "poisson", "tweedie"):
        assert port.gradients(obj, y, p, 0.3, 1.4).tobytes() == reference.gradients(obj, y, p, 0.3, 1.4).tobytes()


@pytest.mark.parametrize("nan,weighted,max_leaves,max_bins", [(0.0, False, 0, 32), (0.08, True, 0, 32),
                                                             (0.03, True, 5, 32), (0.05, True, 0, 400)])
def test_softmax_port_matches_reference(port, reference, nan, weighted, max_leaves, max_bins):
    """TrainMulticlassSoftmaxModel: base scores, every (round, class) tree and the margins
    bit for bit (both sides take exp and log from the same libm); 400 bins: u16 storage."""
    rng = np.random.default_rng(int(nan * 100) + max_leaves)
    x = rng.normal(size=(500, 5)).astype(np.float32)
    x[rng.random(x.shape) < nan] = np.nan
    scores = np.nan_to_num(x) @ rng.normal(size=(5, 3)) + rng.gumbel(size=(500, 3))
    y = scores.argmax(axis=1).astype(np.float64)
    w = rng.uniform(0.5, 1.5, 500) if weighted else None
    params = dict(n_estimators=3, learning_rate=0.3, max_depth=4, min_samples_leaf=2, max_leaves=max_leaves,
                  max_bins=max_bins)
    a = port.train_softmax(port.quantize_dense(x, max_bins), y, 3, w, **params)
    ds = reference.quantize_dense(x, max_bins)
    b = reference.train_softmax(ds, y, 3, w, **params)
    assert a.base_scores.tobytes() == b.base_scores.tobytes()
    assert len(a.trees) == len(b.trees) == 9
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert a.predict_margins(port.quantize_dense(x, max_bins)).tobytes() == b.predict_margins(ds).tobytes()


LEAFWISE = [dict(max_depth=6, max_leaves=12), dict(max_depth=4), dict(max_depth=8, max_leaves=20, min_samples_leaf=5),
            dict(max_depth=6, max_leaves=9, monotonic_constraints=[1, 0, -1, 0, 0, 0]),
            dict(max_depth=6, max_leaves=16, max_active_leaves=16, interaction_constraints=[[0, 1], [1, 2, 3], [4, 5]])]


@pytest.mark.parametrize("max_bins", [32, 600])
@pytest.mark.parametrize("case", range(len(LEAFWISE)))
def test_leafwise_port_matches_reference(port, reference, case, max_bins):
    """TrainLeafWiseRegressionTree in FP64, bit for bit (including the reference's rebuild
    of a histogram whose step-best candidate was superseded); 600 bins: u16 storage."""
    rng = np.random.default_rng(5)
    x = rng.normal(size=(800, 6)).astype(np.float32)
    x[rng.random(x.shape) < 0.05] = np.nan
    y = np.nan_to_num(x[:, 0]) * 2 + np.nan_to_num(x[:, 1]) * np.nan_to_num(x[:, 2]) + rng.normal(size=800) * 0.1
    w = rng.uniform(0.5, 1.5, 800)
    params = dict(LEAFWISE[case], n_estimators=3, learning_rate=0.3, growth_strategy="leaf_wise", max_bins=max_bins)
    a = port.train_regressor(port.quantize_dense(x, max_bins), y, w, **params)
    ds = reference.quantize_dense(x, max_bins)
    b = reference.train_regressor(ds, y, w, **params)
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert a.predict(port.quantize_dense(x, max_bins)).tobytes() == b.predict(ds).tobytes()


def test_dataset_from_bins_equals_quantized(port):
    """The oracle's dataset over given bins (how tests hand it the device's bins) trains
    exactly as the dataset of its own quantile binning, and rejects a bin past its
    feature's count."""
    x = seeded_matrix(61, 3000, 5, 0.1, 1)
    y = np.nan_to_num(x[:, 0]) + np.nan_to_num(x[:, 1]) ** 2
    own = port.quantize_dense(x, 64)

    class Given:  # the fields of a binned dataset, as the package lays them out
        bins = own.bins.astype(np.uint8)
        missing = own.missing
        max_bins = own.max_bins
        boundaries_flat = own.boundaries_flat
        boundary_offsets = own.boundary_offsets
        boundary_counts = own.boundary_counts
        bin_counts = own.bin_counts

    given = port.dataset_from_bins(Given)
    assert np.array_equal(given.bins, own.bins) and np.array_equal(given.missing, own.missing)
    assert list(given.missing_counts) == list(own.missing_counts)
    params = dict(n_estimators=2, max_depth=4, learning_rate=0.3)
    for mode in (oracle.HIST_FP64, oracle.HIST_FIXED):
        a = port.train_regressor(own, y, None, hist_mode=mode, **params)
        b = port.train_regressor(given, y, None, hist_mode=mode, **params)
        assert [t.tobytes() for t in a.trees] == [t.tobytes() for t in b.trees]
    Given.bins = Given.bins.copy()
    f = 2
    row = int(np.flatnonzero(~Given.missing[f])[0])
    Given.bins[f, row] = Given.bin_counts[f]
    with pytest.raises(oracle.OracleError, match="exceeds"):
        port.dataset_from_bins(Given)


def test_fp64_missing_check_trips_on_logistic_configuration(port, reference):
    """On the binary-logistic configuration's data (256 features, 10 % missing cells, depth
    10), the reference's FP64 trainer stops with its own consistency check
    (tree_split.cpp:186-189: a node's missing-row hessian sum, added in another order than
    the node's total, exceeds it by rounding), and the port stops the same way. The
    fixed-point path sums exactly and trains this configuration (the GPU tests compare it
    with the fixed-point replica)."""
    import bench

    x, y = bench.make_logistic_data(200_000)
    params = dict(n_estimators=2, max_depth=10, learning_rate=0.1, objective="binary_logistic")
    for o, kw in ((reference, {}), (port, dict(hist_mode=oracle.HIST_FP64))):
        with pytest.raises(oracle.OracleError, match="missing statistics exceed parent"):
            o.train_regressor(o.quantize_dense(x, 255), y, None, **kw, **params)
    model = port.train_regressor(port.quantize_dense(x, 255), y, None, hist_mode=oracle.HIST_FIXED, **params)
    assert len(model.trees) == 2
