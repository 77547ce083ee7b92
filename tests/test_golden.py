"""The plain-C oracle against the reference's golden vectors (CPU).

Two sources of truth, both from the reference project:
* hand-computed known answers restated from its unit tests
  (tests/unit/test_cpu_tree.py:25-143, tests/unit/test_cpu_tree_missing.py:23-34,
  tests/unit/test_quantization.py:16-75);
* ``golden/reference_cases.json``: quantization, histograms, trees, models and
  predictions produced by the reference's own compiled core (make_golden.py).
"""

from __future__ import annotations

import json
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_cases.json")


def _hex(v):
    return float.fromhex(v)


def _train(port, matrix, labels, max_bins=16, **params):
    ds = port.quantize_dense(np.asarray(matrix, dtype=np.float32), max_bins)
    pairs = port.gradients("squared_error", labels, np.zeros(len(labels)))
    params.setdefault("reg_lambda", 0.0)
    nodes, pred = port.train_single_tree(ds, pairs, **params)
    return ds, nodes, pred


# ---- hand-computed known answers (tests/unit/test_cpu_tree.py) ---------------------------
def test_hand_histogram(port):
    ds = port.quantize_dense(np.array([[0, 10], [1, 10], [2, 20], [3, 20]], np.float32), 16)
    pairs = port.gradients("squared_error", [0.0, 1.0, 2.0, 3.0], [0.0] * 4)
    h = port.histograms(ds, pairs, [1, 2, 3])
    assert [(int(b["count"]), b["gradient_sum"], b["hessian_sum"]) for b in h[0]] == [
        (0, 0.0, 0.0), (1, -1.0, 1.0), (1, -2.0, 1.0), (1, -3.0, 1.0)]
    assert [(int(b["count"]), b["gradient_sum"], b["hessian_sum"]) for b in h[1]] == [
        (1, -1.0, 1.0), (2, -5.0, 2.0)]


def test_hand_root_split(port):
    ds, nodes, pred = _train(port, [[0.0], [1.0], [2.0], [3.0]], [0.0, 0.0, 2.0, 2.0], max_depth=1)
    assert len(nodes) == 3
    root = nodes[0]
    assert (root["feature_index"], root["threshold_bin"], root["left_child"], root["right_child"]) == (0, 1, 1, 2)
    assert root["gain"] == 2.0 and root["flags"] == 0 and root["default_left"] == 1
    assert nodes[1]["leaf_value"] == 0.0 and nodes[2]["leaf_value"] == 2.0
    assert pred.tolist() == [0.0, 0.0, 2.0, 2.0]


def test_hand_depth_two(port):
    labels = [0.0, 0.0, 1.0, 1.0, 2.0, 2.0, 3.0, 3.0]
    _, nodes, pred = _train(port, [[float(v)] for v in range(8)], labels, max_depth=2)
    assert len(nodes) == 7
    assert [(int(n["feature_index"]), int(n["threshold_bin"])) for n in nodes[:3]] == [(0, 3), (0, 1), (0, 5)]
    assert [(int(n["left_child"]), int(n["right_child"])) for n in nodes[:3]] == [(1, 2), (3, 4), (5, 6)]
    assert [n["leaf_value"] for n in nodes[3:]] == [0.0, 1.0, 2.0, 3.0]
    assert pred.tolist() == labels


def test_hand_tie_break(port):
    _, nodes, _ = _train(port, [[0, 0], [1, 1], [2, 2], [3, 3]], [0.0, 1.0, 1.0, 0.0], max_depth=1)
    assert (nodes[0]["feature_index"], nodes[0]["threshold_bin"]) == (0, 0)


def test_hand_random_threshold_seeded(port):
    ds = port.quantize_dense(np.array([[float(v)] for v in range(8)], np.float32), 8)
    labels = [0.0, 0.0, 1.0, 1.0, 2.0, 2.0, 3.0, 3.0]
    pairs = port.gradients("squared_error", labels, [0.0] * 8)
    kw = dict(max_depth=1, reg_lambda=0.0, split_strategy="random_threshold")
    a, _ = port.train_single_tree(ds, pairs, random_seed=101, **kw)
    b, _ = port.train_single_tree(ds, pairs, random_seed=101, **kw)
    c, _ = port.train_single_tree(ds, pairs, random_seed=202, **kw)
    assert a.tobytes() == b.tobytes()
    assert a[0]["threshold_bin"] != c[0]["threshold_bin"]


def test_hand_depth_zero_and_gamma(port):
    _, nodes, pred = _train(port, [[1.0], [1.0]], [2.0, 4.0], max_depth=0)
    assert len(nodes) == 1 and nodes[0]["leaf_value"] == 3.0 and pred.tolist() == [3.0, 3.0]
    _, nodes, _ = _train(port, [[0.0], [1.0], [2.0], [3.0]], [0.0, 0.0, 2.0, 2.0], max_depth=2, gamma=3.0)
    assert len(nodes) == 1 and nodes[0]["leaf_value"] == 1.0


def test_hand_min_child_constraints(port):
    _, nodes, _ = _train(port, [[0.0], [1.0], [2.0], [3.0]], [0.0, 0.0, 0.0, 10.0], max_bins=4,
                         max_depth=1, min_samples_leaf=2, min_child_weight=2.0)
    assert nodes[0]["threshold_bin"] == 1


def test_hand_missing_default_direction(port):
    """tests/unit/test_cpu_tree_missing.py:23-34."""
    ds = port.quantize_dense(np.array([[0.0], [1.0], [2.0], [np.nan]], np.float32), 4)
    pairs = port.gradients("squared_error", [0.0, 0.0, 10.0, 10.0], [0.0] * 4)
    nodes, pred = port.train_single_tree(ds, pairs, max_depth=1, min_samples_leaf=1,
                                         min_child_weight=0.0, reg_lambda=0.0)
    assert nodes[0]["flags"] == 0 and nodes[0]["default_left"] == 0
    assert pred.tolist() == [0.0, 0.0, 10.0, 10.0]
    assert ds.missing.tolist() == [[False, False, False, True]]


def test_contract_errors(port):
    one = port.quantize_dense(np.ones((2, 1), np.float32), 4)
    with pytest.raises(oracle.OracleError, match="min_samples_leaf"):
        port.train_single_tree(one, [[1.0, 1.0], [1.0, 1.0]], max_depth=1, min_samples_leaf=0)
    with pytest.raises(oracle.OracleError, match="reg_lambda"):
        port.train_single_tree(one, [[1.0, 1.0], [1.0, 1.0]], max_depth=1, reg_lambda=-1.0)
    with pytest.raises(oracle.OracleError, match="min_gain_to_split"):
        port.train_single_tree(one, [[1.0, 1.0], [1.0, 1.0]], max_depth=1, min_gain_to_split=-1.0)
    with pytest.raises(oracle.OracleError, match="Inf"):
        port.quantize_dense(np.array([[np.inf]], np.float32), 4)


# ---- hand-computed binning (tests/unit/test_quantization.py) -----------------------------
def test_quantization_lower_bound(port):
    ds = port.quantize_dense(np.array([[1, 10], [2, 10], [3, 20], [4, 20]], np.float32), 2)
    assert ds.boundaries == [[2.0], [10.0]]
    assert ds.bins.tolist() == [[0, 0, 1, 1], [0, 0, 1, 1]]


def test_quantization_constant_and_duplicates(port):
    ds = port.quantize_dense(np.array([[5, 1], [5, 1], [5, 2], [5, 2]], np.float64), 16)
    assert ds.boundaries[0] == [] and ds.bins[0].tolist() == [0, 0, 0, 0]
    assert ds.boundaries[1] == [1.0]


def test_quantization_nan(port):
    x = np.array([[1.0, np.nan], [2.0, 10.0], [np.nan, 20.0], [4.0, np.nan]], np.float32)
    ds = port.quantize_dense(x, 3)
    assert ds.boundaries == [[1.0, 2.0], [10.0]]
    assert ds.missing.tolist() == [[False, False, True, False], [True, False, False, True]]
    assert ds.bins[0][2] == 0 and ds.bins[1][0] == 0


def test_quantization_skew(port):
    x = np.concatenate([np.zeros((999, 1), np.float32), np.ones((1, 1), np.float32)])
    ds = port.quantize_dense(x, 256)
    assert ds.boundaries == [[0.0]]
    assert int((ds.bins[0] == 0).sum()) == 999 and int((ds.bins[0] == 1).sum()) == 1


# ---- golden cases produced by the compiled reference --------------------------------------
def _cases():
    with open(GOLDEN) as fh:
        return json.load(fh)["cases"]


@pytest.mark.parametrize("index", range(9))
def test_reference_cases(port, index):
    case = _cases()[index]
    x = np.array([[np.nan if v is None else _hex(v) for v in row] for row in case["x"]], np.float32)
    y = np.array([_hex(v) for v in case["y"]])
    w = np.array([_hex(v) for v in case["w"]])
    ds = port.quantize_dense(x, case["max_bins"])
    assert ds.bins.tolist() == case["bins"]
    assert ds.missing.astype(int).tolist() == case["missing"]
    assert ds.bin_counts.tolist() == case["bin_counts"]
    assert [[float(v).hex() for v in b] for b in ds.boundaries] == case["boundaries"]
    pairs = port.gradients("squared_error", y, np.zeros_like(y))
    hist = port.histograms(ds, pairs, np.array(case["hist_rows"], np.uint64))
    got = [[[int(b["count"]), float(b["gradient_sum"]).hex(), float(b["hessian_sum"]).hex()] for b in f] for f in hist]
    assert got == case["hist"]

    def nodes(arr):
        return [[int(n["feature_index"]), int(n["threshold_bin"]), int(n["left_child"]),
                 int(n["right_child"]), float(n["leaf_value"]).hex(), float(n["gain"]).hex(),
                 int(n["default_left"]), int(n["flags"])] for n in arr]

    tree, tree_pred = port.train_single_tree(ds, pairs, **case["tree_params"])
    assert nodes(tree) == case["tree"]
    assert [float(v).hex() for v in tree_pred] == case["tree_pred"]
    model = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **case["params"])
    assert float(model.base_score).hex() == case["base_score"]
    assert [nodes(t) for t in model.trees] == case["trees"]
    assert [float(v).hex() for v in model.predict(ds)] == case["pred"]
