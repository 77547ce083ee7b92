"""Wide datasets on the GPU: u16 bins (max_bins 257..65536, or 256 bins with missing values)
against the oracle through the C ABI.

The reference stores bins as u16 above 256 (src/core/binned_dataset.cpp:132) and its Metal
histogram test runs max_bins 257 (tests/metal/test_mps_histogram.py:31-77). Here:
* per-node histograms bit-exact to the oracle's fixed-point replica, for features whose
  slots fit the shared-memory cells (several features per pass, one per pass) and for
  features too wide for them (global atomics);
* training bit-exact to the replica (every tree node, every training prediction), with
  missing values, weights, unit hessians, logistic loss and deep trees;
* against the FP64 oracle: identical tree structures, training RMSE within 1e-4;
* the split scan and the partition entries against the oracle.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

import mpsboost_gb300 as mb
import oracle
from conftest import seeded_matrix

pytestmark = pytest.mark.gpu


def _labels(x, seed, objective="squared_error"):
    rng = np.random.default_rng(seed)
    xs = np.nan_to_num(x)
    f = x.shape[1]
    y = np.sin(xs[:, 0]) + xs[:, 1 % f] * xs[:, 2 % f] + 0.5 * xs[:, 3 % f] ** 2 + rng.normal(size=len(x)) * 0.1
    if objective == "binary_logistic":
        y = (y > np.median(y)).astype(np.float64)
    return y, rng.uniform(0.5, 1.5, len(x))


@pytest.mark.parametrize("max_bins,rows", [(300, 20000), (1024, 20000), (8192, 40000), (20000, 60000)])
def test_wide_histograms_bit_exact_to_replica(backend, port, max_bins, rows):
    """Slots 512 (16 features per shared-memory pass), 1280 (6), 8448 (1) and 20224 (one
    feature's cells exceed the shared-memory budget: global atomics)."""
    x = seeded_matrix(40 + max_bins, rows, 37, 0.1, 3)
    binned = mb.quantize_dense(x, max_bins)
    assert binned.bins.dtype == np.uint16
    ds = port.quantize_dense(x, max_bins)
    rng = np.random.default_rng(max_bins)
    pairs = np.column_stack([rng.normal(size=rows) * 3, rng.uniform(0.2, 2.0, rows)])
    sel = np.sort(rng.choice(rows, rows * 2 // 3, replace=False))
    got = backend.histograms_from_pairs(binned, pairs, sel)
    p32 = pairs.astype(np.float32)
    kg, kh = port.fixed_scales(p32)
    bins, miss = port.fixed_histograms(ds, p32, kg, kh, sel)
    for f, (gf, wf) in enumerate(zip(got, bins)):
        qg = wf["gradient_q"].copy()
        qh = wf["hessian_q"].copy()
        cnt = wf["count"].copy()
        qg[0] += miss[f]["gradient_q"]
        qh[0] += miss[f]["hessian_q"]
        cnt[0] += miss[f]["count"]
        assert np.array_equal(gf["count"], cnt), f
        assert np.array_equal(gf["gradient_sum"], qg.astype(np.float64) * 2.0 ** -kg), f
        assert np.array_equal(gf["hessian_sum"], qh.astype(np.float64) * 2.0 ** -kh), f


def test_wide_layer_histograms_equal_node_histograms(backend):
    x = seeded_matrix(41, 30000, 45, 0.05, 2)
    binned = mb.quantize_dense(x, 700)
    rng = np.random.default_rng(5)
    pairs = np.column_stack([rng.normal(size=30000), rng.uniform(0.5, 1.5, 30000)])
    perm = rng.permutation(30000)
    nodes = [np.sort(perm[:9000]), np.sort(perm[9000:9100]), np.sort(perm[9100:])]
    layer = backend.layer_histograms(binned, pairs, nodes)
    for rows, hist in zip(nodes, layer):
        single = backend.histograms_from_pairs(binned, pairs, rows)
        for a, b in zip(hist, single):
            assert a.tobytes() == b.tobytes()
    assert sum(int(h[0]["count"].sum()) for h in layer) == 30000


WIDE_CASES = {
    # 1024 bins with missing values in every column: slots 1280, weighted.
    "weighted_missing": dict(seed=51, rows=30000, feats=10, nan=0.08, ints=2, max_bins=1024,
                             params=dict(n_estimators=3, learning_rate=0.2, max_depth=6, min_samples_leaf=3)),
    # No weights: count and gradient cells only, and the roots' count/hessian cells reused.
    "unweighted": dict(seed=52, rows=40000, feats=33, nan=0.02, ints=3, max_bins=2048, unweighted=True,
                       params=dict(n_estimators=3, learning_rate=0.2, max_depth=7, min_samples_leaf=2)),
    # 256 bins and missing values: the u8 layout has no slot left, the wide one has.
    "bins256_missing": dict(seed=53, rows=20000, feats=6, nan=0.1, ints=0, max_bins=256,
                            params=dict(n_estimators=3, learning_rate=0.3, max_depth=5, min_samples_leaf=5)),
    # Features too wide for the shared-memory cells: global atomics, scan over 40+ pages.
    "very_wide": dict(seed=54, rows=60000, feats=5, nan=0.03, ints=0, max_bins=12000,
                      params=dict(n_estimators=2, learning_rate=0.3, max_depth=5, min_samples_leaf=4)),
    "logistic": dict(seed=55, rows=20000, feats=8, nan=0.05, ints=1, max_bins=600, objective="binary_logistic",
                     params=dict(n_estimators=3, learning_rate=0.3, max_depth=5, min_child_weight=0.1)),
    "regularized_monotone": dict(seed=56, rows=15000, feats=4, nan=0.0, ints=0, max_bins=900,
                                 params=dict(n_estimators=3, learning_rate=0.3, max_depth=4, reg_lambda=2.0,
                                             reg_alpha=0.3, max_delta_step=0.4, gamma=0.001,
                                             monotonic_constraints=[1, -1, 0, 1])),
    "random_threshold": dict(seed=57, rows=8000, feats=4, nan=0.05, ints=0, max_bins=500,
                             params=dict(n_estimators=3, learning_rate=0.5, max_depth=4,
                                         split_strategy="random_threshold", random_seed=13)),
}


@pytest.mark.parametrize("name", sorted(WIDE_CASES))
def test_wide_training_bit_exact_to_replica(backend, port, name):
    c = WIDE_CASES[name]
    objective = c.get("objective", "squared_error")
    x = seeded_matrix(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"])
    y, w = _labels(x, c["seed"] + 1, objective)
    if c.get("unweighted"):
        w = None
    params = dict(c["params"], objective=objective)
    binned = mb.quantize_dense(x, c["max_bins"])
    model = mb.train_regressor(backend, binned, y, w, **params)
    ds = port.quantize_dense(x, c["max_bins"])
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert float(model.base_score).hex() == float(want.base_score).hex()
    assert len(model.trees) == len(want.trees)
    for got, exp in zip(model.trees, want.trees):
        assert got.tobytes() == exp.tobytes()
    assert model.train_predictions.tobytes() == want.predict(ds).tobytes()
    assert model.predict(backend, binned).tobytes() == want.predict(ds).tobytes()
    # Thresholds beyond the u8 range are in use (the bins are really wide).
    if c["max_bins"] > 256:
        assert max(int(t["threshold_bin"][(t["flags"] & 1) == 0].max(initial=0)) for t in model.trees) > 255


_FIELDS = ("feature_index", "threshold_bin", "default_left", "left_child", "right_child", "flags")


def test_wide_training_against_fp64_oracle(backend, port):
    """Identical structures and training RMSE within 1e-4 of the FP64 oracle, 2048 bins."""
    x = seeded_matrix(58, 50000, 12, 0.03, 1)
    y, w = _labels(x, 59)
    params = dict(n_estimators=4, learning_rate=0.2, max_depth=6, min_samples_leaf=10)
    binned = mb.quantize_dense(x, 2048)
    model = mb.train_regressor(backend, binned, y, w, **params)
    ds = port.quantize_dense(x, 2048)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **params)
    # Structures equal, except after an exact tie (two candidates whose FP64 gains agree
    # to 1e-7 relative), which fixed point resolves by (feature, threshold) and FP64 by
    # rounding.
    for t, (got, exp) in enumerate(zip(model.trees, want.trees)):
        a = [tuple(int(n[k]) for k in _FIELDS) for n in got]
        b = [tuple(int(n[k]) for k in _FIELDS) for n in exp]
        if a == b:
            continue
        node = next(i for i, (p, q) in enumerate(zip(a, b)) if p != q)
        ga, gb = float(got["gain"][node]), float(exp["gain"][node])
        assert abs(ga - gb) <= 1e-7 * abs(gb), (t, node, a[node], b[node], ga, gb)
        break
    p_gpu, p_ref = model.train_predictions, want.predict(ds)
    rmse_gpu = math.sqrt(float(np.mean((p_gpu - y) ** 2)))
    rmse_ref = math.sqrt(float(np.mean((p_ref - y) ** 2)))
    assert abs(rmse_gpu - rmse_ref) <= 1e-4


def test_wide_split_scan_matches_oracle(backend, port):
    x = seeded_matrix(60, 6000, 5, 0.15, 1)
    binned = mb.quantize_dense(x, 3000)
    ds = port.quantize_dense(x, 3000)
    rng = np.random.default_rng(61)
    labels = np.nan_to_num(x[:, 2]) * 2 + np.isnan(x[:, 3]) * 3 + rng.normal(size=6000) * 0.1
    pairs = port.gradients("squared_error", labels, np.zeros(6000))
    rows = np.arange(6000)
    kw = dict(min_samples_leaf=5, min_child_weight=1.0, reg_lambda=0.7, reg_alpha=0.3,
              gamma=0.01, max_delta_step=2.0, monotonic_constraints=[1, -1, 0, 0, 1])
    got = backend.split_candidates_from_pairs(binned, pairs, rows, **kw)
    want = port.scan_splits(ds, pairs, rows, **kw)
    for g, w in zip(got, want):
        assert g["valid"] == w["valid"]
        if w["valid"]:
            assert (g["threshold_bin"], g["default_left"], g["left_count"]) == (w["threshold_bin"], w["default_left"], w["left_count"])
            assert g["gain"] == pytest.approx(w["gain"], rel=2e-5, abs=2e-5)


def test_wide_partition_matches_oracle(backend, port):
    x = seeded_matrix(62, 100000, 3, 0.2, 0)
    binned = mb.quantize_dense(x, 5000)
    ds = port.quantize_dense(x, 5000)
    sel = np.sort(np.random.default_rng(63).choice(100000, 77777, replace=False))
    for thr in (100, 2500, 4990):
        for dl in (True, False):
            gl, gr = backend.partition_rows(binned, sel, 1, thr, default_left=dl)
            wl, wr = port.partition_rows(ds, sel, 1, thr, default_left=dl)
            assert gl == wl.tolist() and gr == wr.tolist()


def test_wide_launch_shapes_build_the_same_trees(backend, monkeypatch):
    """512 and 1024 threads per CTA (MPSB_WIDE_THREADS) give byte-identical models."""
    x = seeded_matrix(64, 30000, 40, 0.05, 2)
    y, w = _labels(x, 65)
    binned = mb.quantize_dense(x, 1500)
    params = dict(n_estimators=2, learning_rate=0.2, max_depth=6, min_samples_leaf=3)
    models = []
    for threads in ("1024", "512"):
        monkeypatch.setenv("MPSB_WIDE_THREADS", threads)
        models.append(mb.train_regressor(backend, binned, y, w, **params))
    assert [t.tobytes() for t in models[0].trees] == [t.tobytes() for t in models[1].trees]
    assert models[0].train_predictions.tobytes() == models[1].train_predictions.tobytes()


def test_wide_float_path_against_fp64_oracle(backend, port):
    """The plain FP32 path on u16 bins (FP32 shared atomics, FP64 slot adds): the first
    tree's structure matches the FP64 reference and the training RMSE is within 1e-4.
    Leaves within 1e-3: a cell's FP32 sum over a work item's rows (thousands here) carries
    relative errors near 1e-4 of the bin's absolute sum, which a leaf's cancelling
    gradients can enlarge; the fixed-point path has no such error."""
    x = seeded_matrix(66, 20000, 8, 0.05, 1)
    y, w = _labels(x, 67)
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=5, min_samples_leaf=5)
    binned = mb.quantize_dense(x, 1024)
    ds = port.quantize_dense(x, 1024)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **params)
    model = mb.train_regressor(backend, binned, y, w, hist_mode="float", **params)
    a = [tuple(int(n[k]) for k in _FIELDS) for n in model.trees[0]]
    b = [tuple(int(n[k]) for k in _FIELDS) for n in want.trees[0]]
    assert a == b
    np.testing.assert_allclose(model.trees[0]["leaf_value"], want.trees[0]["leaf_value"], rtol=1e-3, atol=1e-7)
    rmse = lambda p: float(np.sqrt(np.mean((p - y) ** 2)))  # noqa: E731
    assert abs(rmse(model.train_predictions) - rmse(want.predict(ds))) <= 1e-4


def test_wide_launch_paths_agree(backend):
    """Batched graph, batched without graph and per-node launches give identical trees."""
    x = seeded_matrix(68, 30000, 20, 0.05, 2)
    y, w = _labels(x, 69)
    binned = mb.quantize_dense(x, 700)
    params = dict(n_estimators=3, learning_rate=0.1, max_depth=7, min_samples_leaf=2)
    a = mb.train_regressor(backend, binned, y, w, **params)
    b = mb.train_regressor(backend, binned, y, w, graph=False, **params)
    c = mb.train_regressor(backend, binned, y, w, batched=False, **params)
    for t1, t2, t3 in zip(a.trees, b.trees, c.trees):
        assert t1.tobytes() == t2.tobytes() == t3.tobytes()
    assert a.train_predictions.tobytes() == c.train_predictions.tobytes()
