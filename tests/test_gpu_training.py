"""The device-resident trainer against the oracle through the C ABI.

* Fixed-point mode is bit-exact to the oracle's fixed-point replica: every tree node
  (feature, threshold, missing direction, children, leaf value, gain) and every training
  prediction, round after round.
* Against the FP64 reference restatement: identical tree structures on these seeded
  inputs, leaf values and predictions within 1e-5 relative (a floor of 1e-9 absolute for
  values near zero), training RMSE within 1e-4.
* The plain float path: same structures on well-separated data, predictions within 1e-4.
"""

from __future__ import annotations

import math

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
    y = np.sin(xs[:, 0]) + xs[:, 1] * xs[:, 2 % feats] + 0.5 * xs[:, 3 % feats] ** 2 + rng.normal(size=rows) * 0.1
    if objective == "binary_logistic":
        y = (y > np.median(y)).astype(np.float64)
    elif objective in ("poisson", "tweedie"):
        y = np.floor(np.exp(np.clip(y, -3.0, 2.0)))  # non-negative counts
    w = rng.uniform(0.5, 1.5, rows)
    return x, y, w


def _structure(trees):
    return [[(int(n["feature_index"]), int(n["threshold_bin"]), int(n["default_left"]),
              int(n["left_child"]), int(n["right_child"]), int(n["flags"])) for n in t] for t in trees]


FIXED_CASES = {
    "weighted": dict(seed=21, rows=5000, feats=8, nan=0.0, ints=2, max_bins=255,
                     params=dict(n_estimators=4, learning_rate=0.1, max_depth=6, min_samples_leaf=3)),
    "missing": dict(seed=22, rows=4000, feats=6, nan=0.1, ints=1, max_bins=128,
                    params=dict(n_estimators=3, learning_rate=0.2, max_depth=5, min_samples_leaf=5,
                                min_child_weight=0.5)),
    "regularized": dict(seed=23, rows=3000, feats=5, nan=0.05, ints=0, max_bins=64,
                        params=dict(n_estimators=3, learning_rate=0.3, max_depth=4, reg_lambda=2.0,
                                    reg_alpha=0.3, max_delta_step=0.4, gamma=0.001)),
    "monotone": dict(seed=24, rows=3000, feats=4, nan=0.0, ints=0, max_bins=64,
                     params=dict(n_estimators=3, learning_rate=0.3, max_depth=4,
                                 monotonic_constraints=[1, -1, 0, 1])),
    "interaction": dict(seed=25, rows=3000, feats=5, nan=0.0, ints=0, max_bins=64,
                        params=dict(n_estimators=3, learning_rate=0.3, max_depth=5,
                                    interaction_constraints=[[0, 1, 2], [2, 3], [4]])),
    "random_threshold": dict(seed=26, rows=2000, feats=4, nan=0.0, ints=0, max_bins=32,
                             params=dict(n_estimators=3, learning_rate=0.5, max_depth=4,
                                         split_strategy="random_threshold", random_seed=11)),
    "max_leaves": dict(seed=27, rows=2000, feats=4, nan=0.0, ints=0, max_bins=32,
                       params=dict(n_estimators=2, learning_rate=0.5, max_depth=6, max_leaves=7)),
    "depth0": dict(seed=28, rows=500, feats=3, nan=0.0, ints=0, max_bins=16,
                   params=dict(n_estimators=2, learning_rate=0.5, max_depth=0)),
    "depth1": dict(seed=29, rows=500, feats=3, nan=0.2, ints=0, max_bins=16,
                   params=dict(n_estimators=2, learning_rate=0.5, max_depth=1)),
    "deep": dict(seed=30, rows=20000, feats=33, nan=0.02, ints=3, max_bins=255,
                 params=dict(n_estimators=2, learning_rate=0.1, max_depth=10, min_samples_leaf=2)),
    "quantile": dict(seed=31, rows=2000, feats=4, nan=0.0, ints=0, max_bins=64, objective="quantile",
                     params=dict(n_estimators=3, learning_rate=0.3, max_depth=4, objective_alpha=0.7)),
    # No sample weights: squared error and quantile have h = 1 on every row, so the
    # histograms build count and gradient limbs only (the hessian is count x unit).
    "unweighted": dict(seed=32, rows=20000, feats=40, nan=0.03, ints=2, max_bins=255, unweighted=True,
                       params=dict(n_estimators=3, learning_rate=0.2, max_depth=8, min_samples_leaf=2)),
    "unweighted_quantile": dict(seed=33, rows=6000, feats=12, nan=0.0, ints=1, max_bins=128, unweighted=True,
                                objective="quantile",
                                params=dict(n_estimators=3, learning_rate=0.3, max_depth=6, objective_alpha=0.3)),
}


@pytest.mark.parametrize("name", sorted(FIXED_CASES))
def test_fixed_point_bit_exact_to_replica(backend, port, name):
    c = FIXED_CASES[name]
    objective = c.get("objective", "squared_error")
    x, y, w = _data(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"], objective)
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


def first_divergence(a_trees, b_trees):
    """(tree, node) of the first structural difference, or None."""
    for t, (a, b) in enumerate(zip(_structure(a_trees), _structure(b_trees))):
        for i, (x, y) in enumerate(zip(a, b)):
            if x != y:
                return t, i
        if len(a) != len(b):
            return t, min(len(a), len(b))
    return None


@pytest.mark.parametrize("name", ["weighted", "missing", "regularized", "monotone", "interaction"])
def test_against_fp64_reference(backend, port, name):
    c = FIXED_CASES[name]
    x, y, w = _data(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"])
    binned = mb.quantize_dense(x, c["max_bins"])
    ds = port.quantize_dense(x, c["max_bins"])
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **c["params"])
    model = mb.train_regressor(backend, binned, y, w, **c["params"])
    assert first_divergence(model.trees, want.trees) is None
    for got, exp in zip(model.trees, want.trees):
        np.testing.assert_allclose(got["leaf_value"], exp["leaf_value"], rtol=1e-5, atol=1e-9)
    ref_pred = want.predict(ds)
    np.testing.assert_allclose(model.train_predictions, ref_pred, rtol=1e-5, atol=1e-9)
    rmse = lambda p: float(np.sqrt(np.mean((p - y) ** 2)))  # noqa: E731
    assert abs(rmse(model.train_predictions) - rmse(ref_pred)) <= 1e-4


def test_exact_ties_against_fp64_reference(backend, port):
    """Integer features at depth 10 make different features yield identical partitions:
    mathematically equal gains. The fixed-point path resolves them exactly by (feature,
    threshold) order; the FP64 reference by rounding noise. Trees may then diverge at a
    tie; training RMSE stays within 1e-4."""
    c = FIXED_CASES["deep"]
    x, y, w = _data(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"])
    binned = mb.quantize_dense(x, c["max_bins"])
    ds = port.quantize_dense(x, c["max_bins"])
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **c["params"])
    model = mb.train_regressor(backend, binned, y, w, **c["params"])
    div = first_divergence(model.trees, want.trees)
    if div is not None:
        print("first divergent (tree, node):", div)
    rmse = lambda p: float(np.sqrt(np.mean((p - y) ** 2)))  # noqa: E731
    assert abs(rmse(model.train_predictions) - rmse(want.predict(ds))) <= 1e-4


def test_float_path_against_reference(backend, port):
    """FP32 atomics: the first tree matches the FP64 reference on this seeded input;
    later trees see FP32-rounded predictions, so near-ties may flip. RMSE within 1e-4."""
    c = FIXED_CASES["weighted"]
    x, y, w = _data(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"])
    binned = mb.quantize_dense(x, c["max_bins"])
    ds = port.quantize_dense(x, c["max_bins"])
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **c["params"])
    model = mb.train_regressor(backend, binned, y, w, hist_mode="float", **c["params"])
    assert _structure(model.trees[:1]) == _structure(want.trees[:1])
    np.testing.assert_allclose(model.trees[0]["leaf_value"], want.trees[0]["leaf_value"], rtol=1e-4, atol=1e-7)
    rmse = lambda p: float(np.sqrt(np.mean((p - y) ** 2)))  # noqa: E731
    assert abs(rmse(model.train_predictions) - rmse(want.predict(ds))) <= 1e-4


def test_paths_agree(backend):
    """Batched graph, batched without graph and per-node launches give identical trees."""
    x, y, w = _data(40, 30000, 20, 0.05, 2)
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=3, learning_rate=0.1, max_depth=7, min_samples_leaf=2)
    a = mb.train_regressor(backend, binned, y, w, **params)
    b = mb.train_regressor(backend, binned, y, w, graph=False, **params)
    c = mb.train_regressor(backend, binned, y, w, batched=False, **params)
    for t1, t2, t3 in zip(a.trees, b.trees, c.trees):
        assert t1.tobytes() == t2.tobytes() == t3.tobytes()
    assert a.train_predictions.tobytes() == c.train_predictions.tobytes()


@pytest.mark.parametrize("objective", ["squared_error", "quantile"])
def test_root_reuse_is_exact(backend, monkeypatch, objective):
    """Rounds that restore the roots' count/hessian histograms from the first round give
    the same trees as rounds that build them in full."""
    x, y, w = _data(45, 20000, 12, 0.05, 2, objective)
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=4, learning_rate=0.2, max_depth=6, min_samples_leaf=2,
                  objective=objective)
    a = mb.train_regressor(backend, binned, y, w, **params)
    monkeypatch.setenv("MPSB_ROOT_REUSE", "0")
    b = mb.train_regressor(backend, binned, y, w, **params)
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert a.train_predictions.tobytes() == b.train_predictions.tobytes()


def test_unit_hessian_builds_equal_full_builds(backend, monkeypatch):
    """Count-and-gradient histograms (unweighted squared error and quantile) give the same
    trees as five-limb histograms, depth-wise, leaf-wise and for a forest."""
    x, y, _ = _data(48, 30000, 45, 0.02, 3)
    binned = mb.quantize_dense(x, 255)
    cases = [dict(n_estimators=3, learning_rate=0.2, max_depth=8, min_samples_leaf=3),
             dict(n_estimators=3, learning_rate=0.3, max_depth=6, objective="quantile", objective_alpha=0.6),
             dict(n_estimators=2, learning_rate=0.3, max_depth=8, growth_strategy="leaf_wise", max_leaves=40)]
    fast = [mb.train_regressor(backend, binned, y, None, **p) for p in cases]
    counts, subsets, seeds = mb.forest_samples(30000, 45, 4, random_state=5, max_features=0.5)
    forest_fast = mb.train_forest(backend, binned, y, None, row_counts=counts, feature_subsets=subsets,
                                  seeds=seeds, max_depth=9, min_samples_leaf=2)
    monkeypatch.setenv("MPSB_UNIT_HESS", "0")
    full = [mb.train_regressor(backend, binned, y, None, **p) for p in cases]
    forest_full = mb.train_forest(backend, binned, y, None, row_counts=counts, feature_subsets=subsets,
                                  seeds=seeds, max_depth=9, min_samples_leaf=2)
    for a, b in zip(fast + forest_fast, full + forest_full):
        assert a.base_score == b.base_score
        for t1, t2 in zip(a.trees, b.trees):
            assert t1.tobytes() == t2.tobytes()


def test_autotuned_shape_gives_the_same_trees(backend):
    """The autotuner's shape is used by later fits of the same shape and changes nothing
    in the trees."""
    x, y, w = _data(49, 60000, 40, 0.02, 2)
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=7, min_samples_leaf=2)
    backend.autotune_clear()
    plain = mb.train_regressor(backend, binned, y, w, **params)
    tuned = backend.autotune(binned, y, w, rounds_per_trial=2, **params)
    assert tuned["trials"] >= 1 and tuned["ms_per_round"] <= tuned["default_ms_per_round"]
    assert tuned["hist_threads"] in (512, 640, 768) and tuned["scan_threads"] in (128, 256)
    again = mb.train_regressor(backend, binned, y, w, **params)
    backend.autotune_clear()
    for t1, t2 in zip(plain.trees, again.trees):
        assert t1.tobytes() == t2.tobytes()
    assert plain.train_predictions.tobytes() == again.train_predictions.tobytes()


@pytest.mark.parametrize("rows", [20_000, 20_003])
def test_dataset_upload_layouts(backend, rows):
    """The per-block upload and pack gives the same trees from u8 and from u16 bins, with
    and without missing values, on row counts that take the 16-byte and the byte load
    paths of the pack (70 features: a partial last feature block)."""
    import dataclasses

    x, y, w = _data(47, rows, 70, 0.03, 2)
    params = dict(n_estimators=2, learning_rate=0.3, max_depth=6, min_samples_leaf=2)
    narrow = mb.quantize_dense(x, 200)
    wide = dataclasses.replace(narrow, bins=narrow.bins.astype(np.uint16), _device={})
    a = mb.train_regressor(backend, narrow, y, w, **params)
    b = mb.train_regressor(backend, wide, y, w, **params)
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert a.train_predictions.tobytes() == b.train_predictions.tobytes()


def _c_dataset(lib, backend, binned, create):
    import ctypes as C

    from mpsboost_gb300 import _lib

    ds = C.c_void_p()
    bins = np.ascontiguousarray(binned.bins)
    miss = np.ascontiguousarray(binned.missing, dtype=np.uint8)
    counts = np.ascontiguousarray(binned.bin_counts, np.uint32)
    rc = create(backend.handle, _lib.ptr(bins), bins.itemsize, _lib.ptr(miss), binned.rows, binned.features,
                _lib.ptr(counts), C.byref(ds))
    return rc, ds, (bins, miss, counts)


def _c_fit(lib, backend, ds, y, w, **params):
    import ctypes as C

    from mpsboost_gb300 import _lib

    p, keep = mb.make_params(**params)
    model = C.c_void_p()
    rc = lib.mpsb_cuda_train_regressor(backend.handle, ds, _lib.ptr(y), _lib.ptr(w), y.size, C.byref(p), 0,
                                       C.byref(model))
    del keep
    if rc:
        return rc, None
    trees = []
    for t in range(lib.mpsb_cuda_model_tree_count(model)):
        out = np.empty(lib.mpsb_cuda_model_tree_node_count(model, t), _lib.NODE_DTYPE)
        _lib.check(lib.mpsb_cuda_model_tree_nodes(model, t, _lib.ptr(out)))
        trees.append(out)
    preds = np.empty(y.size)
    _lib.check(lib.mpsb_cuda_model_train_predictions(model, _lib.ptr(preds)))
    lib.mpsb_cuda_model_destroy(model)
    return 0, (trees, preds)


def test_async_dataset_upload(backend):
    """mpsb_cuda_dataset_create_async: training on a dataset whose upload is still in
    flight (the host checks labels and weights meanwhile) gives the trees and predictions
    of the synchronous upload; a bin past its feature's count is reported by the wait
    and by every later entry, not by the create."""
    from mpsboost_gb300 import _lib

    lib = _lib.load()
    x, y, w = _data(48, 300_000, 70, 0.03, 2)
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=3, learning_rate=0.3, max_depth=6, min_samples_leaf=2)
    results = []
    bins = np.ascontiguousarray(binned.bins)
    pinned = mb.BinnedDataset(**{**{f: getattr(binned, f) for f in (
        "rows", "features", "max_bins", "missing", "boundaries_flat", "boundary_offsets",
        "boundary_counts", "bin_counts", "missing_counts")}, "bins": bins})
    _lib.check(lib.mpsb_cuda_host_register(_lib.ptr(bins), bins.nbytes))  # copies run async
    try:
        for create in (lib.mpsb_cuda_dataset_create, lib.mpsb_cuda_dataset_create_async):
            rc, ds, keep = _c_dataset(lib, backend, pinned, create)
            assert rc == 0
            rc, res = _c_fit(lib, backend, ds, y, w, **params)
            assert rc == 0
            assert lib.mpsb_cuda_dataset_wait(ds) == 0
            lib.mpsb_cuda_dataset_destroy(ds)
            del keep
            results.append(res)
    finally:
        lib.mpsb_cuda_host_unregister(_lib.ptr(bins))
    (ta, pa), (tb, pb) = results
    assert [t.tobytes() for t in ta] == [t.tobytes() for t in tb]
    assert pa.tobytes() == pb.tobytes()

    import dataclasses

    bad = dataclasses.replace(binned, bins=binned.bins.copy(), _device={})
    row = int(np.flatnonzero(~bad.missing[5])[0])
    bad.bins[5, row] = bad.bin_counts[5]  # one past the feature's last bin
    rc, ds, keep = _c_dataset(lib, backend, bad, lib.mpsb_cuda_dataset_create_async)
    assert rc == 0
    assert lib.mpsb_cuda_dataset_wait(ds) == _lib.MPSB_ERR_DATA
    assert b"exceeds" in lib.mpsb_cuda_last_error()
    rc, _ = _c_fit(lib, backend, ds, y, w, **params)
    assert rc == _lib.MPSB_ERR_DATA
    lib.mpsb_cuda_dataset_destroy(ds)
    rc, ds, keep = _c_dataset(lib, backend, bad, lib.mpsb_cuda_dataset_create)
    assert rc == _lib.MPSB_ERR_DATA and not ds.value


@pytest.mark.parametrize("threads", ["768", "512"])
def test_tma_staging_equals_cp_async(backend, monkeypatch, threads):
    """Row-major levels whose gathered rows arrive by TMA gather4 copies give the same
    trees as cp.async staging: depth 9 (levels 2-8 read the row-major bins), 70 features
    (a partial third feature block), small nodes with partial tiles."""
    x, y, w = _data(46, 40000, 70, 0.05, 3)
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=9, min_samples_leaf=1)
    monkeypatch.setenv("MPSB_HIST_THREADS", threads)
    monkeypatch.setenv("MPSB_HIST_TMA", "1")
    tma_bins = mb.quantize_dense(x, 255)
    a = mb.train_regressor(backend, tma_bins, y, w, **params)
    assert backend.dataset(tma_bins).uses_tma
    monkeypatch.setenv("MPSB_HIST_TMA", "0")
    plain_bins = mb.quantize_dense(x, 255)
    b = mb.train_regressor(backend, plain_bins, y, w, **params)
    assert not backend.dataset(plain_bins).uses_tma
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert a.train_predictions.tobytes() == b.train_predictions.tobytes()


@pytest.mark.parametrize("threads", ["768", "640", "512"])
@pytest.mark.parametrize("weighted", [True, False])
def test_direct_loads_equal_staged_builds(backend, port, monkeypatch, threads, weighted):
    """Register-direct histogram builds (the trainer's default: each lane loads its row's
    32 bin bytes with one 256-bit load, no shared-memory staging, flush by TMA bulk
    reductions) give the staged kernel's trees bit for bit (MPSB_HIST_DIRECT=0), and the
    replica's. Weighted squared error builds five limbs and, from the second boosting round, gradient-only
    roots; unweighted builds count and gradient limbs (unit hessian). Depth 9 with 70
    features (a partial feature block), 40,000 rows (dense and sparse nodes, partial row
    groups) and missing values."""
    x, y, w = _data(47, 40000, 70, 0.05, 3)
    w = w if weighted else None
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=9, min_samples_leaf=1)
    monkeypatch.setenv("MPSB_HIST_THREADS", threads)
    monkeypatch.setenv("MPSB_ROOT_THREADS", threads)
    monkeypatch.setenv("MPSB_HIST_DIRECT", "1")
    binned = mb.quantize_dense(x, 255)
    a = mb.train_regressor(backend, binned, y, w, **params)
    monkeypatch.setenv("MPSB_HIST_DIRECT", "0")
    b = mb.train_regressor(backend, binned, y, w, **params)
    assert [t.tobytes() for t in a.trees] == [t.tobytes() for t in b.trees]
    assert a.train_predictions.tobytes() == b.train_predictions.tobytes()
    ds = port.quantize_dense(x, 255)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert [t.tobytes() for t in a.trees] == [t.tobytes() for t in want.trees]


def test_logistic_against_replica(backend, port):
    x, y, w = _data(41, 6000, 8, 0.1, 2, "binary_logistic")
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=5, min_samples_leaf=4,
                  objective="binary_logistic")
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    model = mb.train_regressor(backend, binned, y, w, **params)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert _structure(model.trees) == _structure(want.trees)
    for got, exp in zip(model.trees, want.trees):
        np.testing.assert_allclose(got["leaf_value"], exp["leaf_value"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(model.train_predictions, want.predict(ds), rtol=1e-9, atol=1e-12)


COUNT_OBJECTIVES = {
    "poisson": dict(objective="poisson"),
    "tweedie": dict(objective="tweedie", tweedie_variance_power=1.3),
}


@pytest.mark.parametrize("name", sorted(COUNT_OBJECTIVES))
def test_count_objectives_against_replica(backend, port, name):
    """Poisson and Tweedie (log link, objective.cpp:383-429): the device's FP64 exp may
    differ from the host's by an ulp, so structures must match and leaf values and
    predictions agree to 1e-9 relative, as for the logistic objective."""
    x, y, w = _data(44, 6000, 8, 0.05, 2, name)
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=5, min_samples_leaf=4,
                  **COUNT_OBJECTIVES[name])
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    model = mb.train_regressor(backend, binned, y, w, **params)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert float(model.base_score).hex() == float(want.base_score).hex()
    assert _structure(model.trees) == _structure(want.trees)
    for got, exp in zip(model.trees, want.trees):
        np.testing.assert_allclose(got["leaf_value"], exp["leaf_value"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(model.train_predictions, want.predict(ds), rtol=1e-9, atol=1e-12)


def _loss(objective, margin, y, w, rho=1.5):
    """Weighted mean training loss on the link scale's margins."""
    if objective == "binary_logistic":
        per_row = np.where(y > 0.5, np.logaddexp(0.0, -margin), np.logaddexp(0.0, margin))
    elif objective == "poisson":
        per_row = np.exp(margin) - y * margin
    else:  # tweedie negative log-likelihood up to a label-only term
        per_row = -y * np.exp((1.0 - rho) * margin) / (1.0 - rho) + np.exp((2.0 - rho) * margin) / (2.0 - rho)
    return float(np.sum(w * per_row) / np.sum(w))


@pytest.mark.parametrize("name", ["binary_logistic", "poisson", "tweedie"])
def test_loss_against_fp64_reference(backend, port, name):
    """Fixed-point training against the FP64 reference restatement: the same trees on
    these inputs and the final training loss (logloss, Poisson or Tweedie deviance)
    within 1e-4."""
    x, y, w = _data(45, 20000, 10, 0.02, 2, name)
    extra = COUNT_OBJECTIVES.get(name, dict(objective=name))
    params = dict(n_estimators=5, learning_rate=0.2, max_depth=6, min_samples_leaf=5, **extra)
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    model = mb.train_regressor(backend, binned, y, w, **params)
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, **params)
    assert first_divergence(model.trees, want.trees) is None
    rho = params.get("tweedie_variance_power", 1.5)
    got_loss = _loss(name, model.train_predictions, y, w, rho)
    want_loss = _loss(name, want.predict(ds), y, w, rho)
    assert abs(got_loss - want_loss) <= 1e-4
    np.testing.assert_allclose(model.train_predictions, want.predict(ds), rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("max_bins", [64, 900])
def test_ovr_equals_independent_binary_fits(backend, port, max_bins):
    rng = np.random.default_rng(42)
    x = rng.normal(size=(4000, 6)).astype(np.float32)
    scores = x @ rng.normal(size=(6, 4)) + rng.gumbel(size=(4000, 4))
    labels = scores.argmax(axis=1).astype(np.float64)
    binned = mb.quantize_dense(x, max_bins)
    params = dict(n_estimators=2, learning_rate=0.3, max_depth=4, min_samples_leaf=3)
    models = mb.train_ovr(backend, binned, labels, 4, **params)
    assert len(models) == 4
    for k, m in enumerate(models):
        single = mb.train_regressor(backend, binned, (labels == k).astype(np.float64),
                                    objective="binary_logistic", **params)
        assert m.base_score == single.base_score
        for t1, t2 in zip(m.trees, single.trees):
            assert t1.tobytes() == t2.tobytes()


def test_training_errors(backend):
    x, y, w = _data(43, 300, 3)
    binned = mb.quantize_dense(x, 16)
    bad = y.copy()
    bad[5] = np.nan
    with pytest.raises(mb.TrainingError):
        mb.train_regressor(backend, binned, bad, n_estimators=1, max_depth=2)
    with pytest.raises(mb.TrainingError, match="weights"):
        mb.train_regressor(backend, binned, y, -w, n_estimators=1, max_depth=2)
    with pytest.raises(mb.TrainingError, match="learning_rate"):
        mb.train_regressor(backend, binned, y, learning_rate=0.0)
    with pytest.raises(mb.TrainingError, match="binary"):
        mb.train_regressor(backend, binned, y, objective="binary_logistic", n_estimators=1)
    # The reference's check order: every weight check before any label check, each at its
    # first failing row.
    big_w = w.copy()
    big_w[10:12] = 1.7e308
    with pytest.raises(mb.TrainingError, match="sample weight sum overflowed"):
        mb.train_regressor(backend, binned, y, big_w, n_estimators=1, max_depth=2)
    with pytest.raises(mb.TrainingError, match="finite non-negative"):
        mb.train_regressor(backend, binned, bad, -w, n_estimators=1, max_depth=2)
    big_y = y.copy()
    big_y[3:5] = 1.7e308
    with pytest.raises(mb.TrainingError, match="Label accumulation overflowed"):
        mb.train_regressor(backend, binned, big_y, n_estimators=1, max_depth=2)
    big_y[200] = np.nan
    with pytest.raises(mb.TrainingError, match="Label accumulation overflowed"):
        mb.train_regressor(backend, binned, big_y, n_estimators=1, max_depth=2)
    with pytest.raises(mb.TrainingError, match="poisson labels must be non-negative"):
        mb.train_regressor(backend, binned, -np.abs(y) - 1, objective="poisson", n_estimators=1, max_depth=2)


def test_scale_properties(backend):
    """Size-independent properties at 2M rows: count conservation, determinism of the
    fixed-point path, session == one-shot training."""
    n, f = 2_000_000, 32
    rng = np.random.default_rng(44)
    x = rng.normal(size=(n, f)).astype(np.float32)
    y = np.sin(x[:, 0]) + x[:, 1] * x[:, 2] + rng.normal(size=n) * 0.1
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=2, learning_rate=0.1, max_depth=8, min_samples_leaf=20)
    a = mb.train_regressor(backend, binned, y, **params)
    b = mb.train_regressor(backend, binned, y, **params)
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert a.train_predictions.tobytes() == b.train_predictions.tobytes()
    hist = backend.histograms_from_pairs(binned, np.column_stack([y, np.ones(n)]), np.arange(n))
    assert all(int(h["count"].sum()) == n for h in hist)
    t = mb.Trainer(backend, binned, y, **params)
    t.run(2)
    t.synchronize()
    m = t.export()
    for t1, t2 in zip(a.trees, m.trees):
        assert t1.tobytes() == t2.tobytes()
    stats = t.stats()
    assert stats["rounds"] == 2 and stats["kernel_launches"] > 0 and stats["hist_cells"] >= n * f
    # Every round partitions the root's n rows, and at most n rows at each of depths 0-6.
    assert 2 * n <= stats["part_rows"] <= 2 * 7 * n


def _random_bins(seed, rows, feats, nb=255):
    """A binned dataset of uniform random bins (no missing values) with an identity schema."""
    rng = np.random.default_rng(seed)
    bins = rng.integers(0, nb, size=(feats, rows), dtype=np.uint8)
    cnt = np.full(feats, nb - 1, np.uint32)
    bounds = np.tile(np.arange(nb - 1, dtype=np.float32) + 0.5, feats)
    return mb.BinnedDataset(rows, feats, nb, bins, np.zeros((feats, rows), bool), bounds,
                            (np.arange(feats, dtype=np.uint64) * (nb - 1)), cnt,
                            np.full(feats, nb, np.uint32), np.zeros(feats, np.uint64))


def test_full_size_properties(backend):
    """10M rows x 128 features, 255 bins, depth 8 (the benchmark's shape), through
    size-independent properties: two fits are bit-identical; the training predictions,
    applied from the final row segments, equal a traversal of every row through the trees
    bit for bit (so no row was misrouted by any partition); and in one layer launch over a
    root and its two children, every feature's parent histogram is exactly the sum of the
    children's (count, gradient and hessian), with the same gradient total in every
    feature."""
    n, f = 10_000_000, 128
    binned = _random_bins(46, n, f)
    rng = np.random.default_rng(47)
    b = binned.bins
    y = ((b[0].astype(np.float64) - 127.0) / 64.0) * ((b[1].astype(np.float64) - 127.0) / 64.0)
    y += np.sin(b[2] / 40.0) + 0.25 * (b[3] > 200) + rng.normal(size=n) * 0.1
    w = rng.uniform(0.5, 1.5, n)
    params = dict(n_estimators=2, learning_rate=0.1, max_depth=8, min_samples_leaf=20)
    a = mb.train_regressor(backend, binned, y, w, **params)
    a2 = mb.train_regressor(backend, binned, y, w, **params)
    assert [t.tobytes() for t in a.trees] == [t.tobytes() for t in a2.trees]
    assert a.train_predictions.tobytes() == a2.train_predictions.tobytes()
    assert a.predict(backend, binned).tobytes() == a.train_predictions.tobytes()
    assert sum(int(((t["flags"] & 1) == 1).sum()) for t in a.trees) > 2 * 100  # deep trees

    pairs = np.column_stack([y - y.mean(), w])
    rows = np.arange(n, dtype=np.uint64)
    go_left = b[5] <= 100
    parent, left, right = backend.layer_histograms(binned, pairs, [rows, rows[go_left], rows[~go_left]])
    totals = set()
    for feat in range(f):
        p_, l_, r_ = parent[feat], left[feat], right[feat]
        assert int(p_["count"].sum()) == n
        assert np.array_equal(p_["count"], l_["count"] + r_["count"])
        assert np.array_equal(p_["gradient_sum"], l_["gradient_sum"] + r_["gradient_sum"])
        assert np.array_equal(p_["hessian_sum"], l_["hessian_sum"] + r_["hessian_sum"])
        totals.add(math.fsum(p_["gradient_sum"]))
    assert len(totals) == 1


@pytest.mark.parametrize("max_bins", [64, 700])
def test_softmax_against_replica(backend, port, max_bins):
    """Native softmax: K trees per round in class order, each on the margins updated by
    the earlier classes. Base scores bit-exact; tree structures equal to the oracle's
    fixed-point replica; leaves and margins within 1e-9 (the device's FP64 exp and the
    host's may differ in the last bit). 700 bins: u16 storage, the wide kernels."""
    rng = np.random.default_rng(46)
    x = rng.normal(size=(6000, 7)).astype(np.float32)
    x[rng.random(x.shape) < 0.05] = np.nan
    y = (np.nan_to_num(x) @ rng.normal(size=(7, 4)) + rng.gumbel(size=(6000, 4))).argmax(1).astype(np.float64)
    w = rng.uniform(0.5, 1.5, 6000)
    params = dict(n_estimators=3, learning_rate=0.3, max_depth=5, min_samples_leaf=3, max_bins=max_bins)
    binned = mb.quantize_dense(x, max_bins)
    ds = port.quantize_dense(x, max_bins)
    model = mb.train_softmax(backend, binned, y, 4, w, **params)
    want = port.train_softmax(ds, y, 4, w, hist_mode=oracle.HIST_FIXED, **params)
    assert model.base_scores.tobytes() == want.base_scores.tobytes()
    assert len(model.trees) == 12
    assert _structure(model.trees) == _structure(want.trees)
    for got, exp in zip(model.trees, want.trees):
        np.testing.assert_allclose(got["leaf_value"], exp["leaf_value"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(model.train_margins, want.predict_margins(ds), rtol=1e-9, atol=1e-12)
    assert model.predict_margins(backend, binned).tobytes() == model.train_margins.tobytes()
    again = mb.train_softmax(backend, binned, y, 4, w, graph=False, **params)
    for t1, t2 in zip(model.trees, again.trees):
        assert t1.tobytes() == t2.tobytes()
    with pytest.raises(mb.TrainingError, match="class"):
        mb.train_softmax(backend, binned, y + 0.5, 4, **params)


LEAFWISE_CASES = {
    "max_leaves": dict(seed=61, rows=6000, feats=8, nan=0.05, ints=2, max_bins=128,
                       params=dict(n_estimators=3, learning_rate=0.2, max_depth=6, max_leaves=12)),
    "depth_bound": dict(seed=62, rows=4000, feats=6, nan=0.0, ints=0, max_bins=64,
                        params=dict(n_estimators=2, learning_rate=0.3, max_depth=4)),
    "deep": dict(seed=63, rows=20000, feats=20, nan=0.02, ints=3, max_bins=255,
                 params=dict(n_estimators=2, learning_rate=0.1, max_depth=10, max_leaves=40,
                             min_samples_leaf=5)),
    "monotone": dict(seed=64, rows=3000, feats=4, nan=0.0, ints=0, max_bins=64,
                     params=dict(n_estimators=2, learning_rate=0.3, max_depth=6, max_leaves=9,
                                 monotonic_constraints=[1, 0, -1, 0])),
    "interaction": dict(seed=65, rows=3000, feats=6, nan=0.0, ints=0, max_bins=64,
                        params=dict(n_estimators=2, learning_rate=0.3, max_depth=6, max_leaves=16,
                                    max_active_leaves=16, interaction_constraints=[[0, 1], [1, 2, 3], [4, 5]])),
    "regularized": dict(seed=66, rows=3000, feats=5, nan=0.1, ints=1, max_bins=64,
                        params=dict(n_estimators=2, learning_rate=0.3, max_depth=5, max_leaves=10,
                                    reg_lambda=2.0, reg_alpha=0.2, min_child_weight=0.5, gamma=0.001)),
    "wide_bins": dict(seed=68, rows=8000, feats=7, nan=0.05, ints=1, max_bins=1200,
                      params=dict(n_estimators=2, learning_rate=0.3, max_depth=6, max_leaves=14,
                                  min_samples_leaf=3)),
}


@pytest.mark.parametrize("name", sorted(LEAFWISE_CASES))
def test_leafwise_bit_exact_to_replica(backend, port, name):
    """Leaf-wise growth (tree_leafwise.cpp:56-142): every node, leaf value and training
    prediction equal the oracle's fixed-point replica."""
    c = LEAFWISE_CASES[name]
    x, y, w = _data(c["seed"], c["rows"], c["feats"], c["nan"], c["ints"])
    params = dict(c["params"], growth_strategy="leaf_wise")
    binned = mb.quantize_dense(x, c["max_bins"])
    model = mb.train_regressor(backend, binned, y, w, **params)
    ds = port.quantize_dense(x, c["max_bins"])
    want = port.train_regressor(ds, y, w, hist_mode=oracle.HIST_FIXED, **params)
    assert len(model.trees) == len(want.trees)
    for got, exp in zip(model.trees, want.trees):
        assert got.tobytes() == exp.tobytes()
    assert model.train_predictions.tobytes() == want.predict(ds).tobytes()


def test_leafwise_ovr_and_softmax(backend, port):
    rng = np.random.default_rng(67)
    x = rng.normal(size=(5000, 6)).astype(np.float32)
    x[rng.random(x.shape) < 0.03] = np.nan
    y = (np.nan_to_num(x) @ rng.normal(size=(6, 3)) + rng.gumbel(size=(5000, 3))).argmax(1).astype(np.float64)
    binned = mb.quantize_dense(x, 64)
    params = dict(n_estimators=2, learning_rate=0.3, max_depth=5, max_leaves=10, min_samples_leaf=3,
                  growth_strategy="leaf_wise")
    models = mb.train_ovr(backend, binned, y, 3, **params)
    for k, m in enumerate(models):
        single = mb.train_regressor(backend, binned, (y == k).astype(np.float64), objective="binary_logistic", **params)
        for t1, t2 in zip(m.trees, single.trees):
            assert t1.tobytes() == t2.tobytes()
    soft = mb.train_softmax(backend, binned, y, 3, **params)
    want = port.train_softmax(port.quantize_dense(x, 64), y, 3, hist_mode=oracle.HIST_FIXED, **params)
    assert _structure(soft.trees) == _structure(want.trees)


def test_leafwise_active_queue_limit(backend, port):
    """max_active_leaves below the leaves the growth needs fails as in the reference."""
    x, y, w = _data(68, 3000, 5)
    params = dict(n_estimators=1, max_depth=6, max_active_leaves=4, growth_strategy="leaf_wise")
    with pytest.raises(oracle.OracleError, match="max_active_leaves"):
        port.train_regressor(port.quantize_dense(x, 32), y, w, hist_mode=oracle.HIST_FIXED, **params)
    with pytest.raises(mb.TrainingError, match="max_active_leaves"):
        mb.train_regressor(backend, mb.quantize_dense(x, 32), y, w, **params)


@pytest.mark.parametrize("variant", ["weighted", "forest", "interaction"])
def test_fused_sibling_subtraction_equals_subtract_kernel(backend, monkeypatch, variant):
    """Siblings' histograms formed inside the split scan (the default for level-wise growth
    on u8 bins) and by subtract_kernel (MPSB_FUSED_SUB=0) give byte-identical fixed-point
    models, with forest feature masks and interaction constraints (features a node may not
    split on are skipped). The plain float path's fused subtraction is covered against the
    FP64 oracle by test_float_path_against_reference (its FP32 atomics do not repeat bit for
    bit between fits)."""
    x, y, w = _data(81, 20000, 24, 0.05, 3)
    binned = mb.quantize_dense(x, 255)
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=7, min_samples_leaf=3)
    if variant == "interaction":
        params["interaction_constraints"] = [[0, 1, 2, 3], [3, 4, 5, 6, 7], list(range(8, 24))]

    def fit():
        if variant == "forest":
            counts, subsets, seeds = mb.forest_samples(20000, 24, 6, random_state=3, max_features=0.5)
            return mb.train_forest(backend, binned, y, w, row_counts=counts, feature_subsets=subsets,
                                   seeds=seeds, max_depth=7, min_samples_leaf=3)
        return [mb.train_regressor(backend, binned, y, w, **params)]

    monkeypatch.setenv("MPSB_FUSED_SUB", "1")
    fused = fit()
    monkeypatch.setenv("MPSB_FUSED_SUB", "0")
    separate = fit()
    for a, b in zip(fused, separate):
        assert [t.tobytes() for t in a.trees] == [t.tobytes() for t in b.trees]
