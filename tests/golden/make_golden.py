"""Generate ``reference_cases.json`` from the reference's own C++ core.

Run where the reference sources exist (``python tests/golden/make_golden.py``): it builds
``oracle/_ref/libmpsb_ref.so`` from those sources (oracle/Makefile) and records, for small
seeded inputs stored verbatim in the file, the reference's quantization, histograms,
single trees, boosted models and predictions. ``tests/test_golden.py`` replays every case
against the plain-C oracle, so the oracle stays pinned where the reference is absent;
each case also keeps the reference's model file bytes (SerializeModel), which
``tests/test_model_io.py`` reads and rewrites.
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def nodes_json(nodes):
    return [
        [int(n["feature_index"]), int(n["threshold_bin"]), int(n["left_child"]),
         int(n["right_child"]), float(n["leaf_value"]).hex(), float(n["gain"]).hex(),
         int(n["default_left"]), int(n["flags"])]
        for n in nodes
    ]


def matrix(seed, rows, feats, nan=0.0, ints=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(rows, feats)).astype(np.float32)
    for c in range(ints):
        x[:, c] = rng.integers(0, 3 + 2 * c, rows)
    if nan:
        x[rng.random((rows, feats)) < nan] = np.nan
    return x


def main():
    oracle.build(reference=True)
    ref = oracle.Oracle("reference")
    cases = []
    configs = [
        dict(seed=1, rows=64, feats=3, nan=0.0, ints=1, max_bins=16,
             params=dict(n_estimators=3, learning_rate=0.3, max_depth=3, min_samples_leaf=2)),
        dict(seed=2, rows=120, feats=4, nan=0.1, ints=2, max_bins=8,
             params=dict(n_estimators=2, learning_rate=0.5, max_depth=4, min_samples_leaf=1,
                         reg_lambda=0.5, reg_alpha=0.05)),
        dict(seed=3, rows=200, feats=5, nan=0.05, ints=0, max_bins=255,
             params=dict(n_estimators=2, learning_rate=0.1, max_depth=5, min_samples_leaf=3,
                         min_child_weight=0.5, max_delta_step=0.7, gamma=0.01)),
        dict(seed=4, rows=150, feats=3, nan=0.0, ints=1, max_bins=32,
             params=dict(n_estimators=2, learning_rate=0.2, max_depth=3, min_samples_leaf=2,
                         monotonic_constraints=[1, -1, 0])),
        dict(seed=5, rows=150, feats=4, nan=0.0, ints=0, max_bins=32,
             params=dict(n_estimators=2, learning_rate=0.2, max_depth=4,
                         interaction_constraints=[[0, 1], [2, 3]])),
        dict(seed=6, rows=100, feats=3, nan=0.0, ints=0, max_bins=16,
             params=dict(n_estimators=2, learning_rate=1.0, max_depth=3,
                         split_strategy="random_threshold", random_seed=101)),
        dict(seed=7, rows=160, feats=3, nan=0.1, ints=0, max_bins=64,
             params=dict(n_estimators=2, learning_rate=0.3, max_depth=3,
                         objective="binary_logistic", min_samples_leaf=2)),
        dict(seed=8, rows=90, feats=2, nan=0.0, ints=0, max_bins=16,
             params=dict(n_estimators=2, learning_rate=0.3, max_depth=6, max_leaves=5)),
        # u16 storage (max_bins above 256) with missing values.
        dict(seed=9, rows=420, feats=3, nan=0.05, ints=0, max_bins=300,
             params=dict(n_estimators=2, learning_rate=0.3, max_depth=4, min_samples_leaf=2)),
    ]
    for cfg in configs:
        x = matrix(cfg["seed"], cfg["rows"], cfg["feats"], cfg["nan"], cfg["ints"])
        rng = np.random.default_rng(100 + cfg["seed"])
        y = np.nan_to_num(x[:, 0]).astype(np.float64) * 2 + rng.normal(size=cfg["rows"]) * 0.1
        if cfg["params"].get("objective") == "binary_logistic":
            y = (y > np.median(y)).astype(np.float64)
        w = rng.uniform(0.5, 1.5, cfg["rows"])
        ds = ref.quantize_dense(x, cfg["max_bins"])
        pairs = ref.gradients("squared_error", y, np.zeros_like(y))
        rows = np.arange(1, cfg["rows"], 2, dtype=np.uint64)
        hist = ref.histograms(ds, pairs, rows)
        tree_params = {k: v for k, v in cfg["params"].items() if k not in ("n_estimators", "learning_rate", "objective")}
        tree_nodes, tree_pred = ref.train_single_tree(ds, pairs, **tree_params)
        model = ref.train_regressor(ds, y, w, **cfg["params"])
        cases.append(
            dict(
                x=[[None if np.isnan(v) else float(v).hex() for v in row] for row in x.tolist()],
                y=[float(v).hex() for v in y], w=[float(v).hex() for v in w],
                max_bins=cfg["max_bins"], params=cfg["params"],
                bins=ds.bins.tolist(), missing=ds.missing.astype(int).tolist(),
                boundaries=[[float(v).hex() for v in b] for b in ds.boundaries],
                bin_counts=ds.bin_counts.tolist(),
                hist_rows=rows.tolist(),
                hist=[[[int(b["count"]), float(b["gradient_sum"]).hex(), float(b["hessian_sum"]).hex()] for b in f] for f in hist],
                tree_params=tree_params, tree=nodes_json(tree_nodes),
                tree_pred=[float(v).hex() for v in tree_pred],
                base_score=float(model.base_score).hex(),
                trees=[nodes_json(t) for t in model.trees],
                pred=[float(v).hex() for v in model.predict(ds)],
                model_file=ref.model_to_bytes(model).hex(),
            )
        )
    out = os.path.join(HERE, "reference_cases.json")
    with open(out, "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, fh, separators=(",", ":"))
    print(out, os.path.getsize(out), "bytes,", len(cases), "cases")


if __name__ == "__main__":
    main()
