"""GPU node-level entries against the CPU oracle through the C ABI.

Mirrors the reference's Metal tests (tests/metal/test_mps_histogram.py:17-77 and
tests/metal/test_mps_hot_path.py:17-140) with their tolerances: counts exact, G
rel/abs 2e-5, H 1e-6, gains 2e-5; partitions exact lists in row order. The fixed-point
histograms are additionally bit-exact to the oracle's fixed-point replica.
"""

from __future__ import annotations

import numpy as np
import pytest

import mpsboost_gb300 as mb
import oracle
from conftest import seeded_matrix

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("length", [1, 7, 257, 1025])
def test_gradients_match_oracle(backend, port, length):
    labels = np.linspace(-3.0, 4.0, length)
    preds = np.linspace(1.0, -2.0, length)
    got = backend.gradients(labels, preds)
    want = port.gradients("squared_error", labels, preds)
    np.testing.assert_allclose(got, want, rtol=2e-6, atol=2e-6)
    assert got.tobytes() == want.tobytes()  # pred - label in FP64 is exact on both


def _reference_matrix(rows=1025):
    return np.column_stack(
        (
            np.arange(rows, dtype=np.float32) % 13,
            np.where(np.arange(rows) < 1000, 0.0, 1.0).astype(np.float32),
            np.linspace(-1.0, 1.0, rows, dtype=np.float32),
        )
    )


@pytest.mark.parametrize("mode", ["fixed", "float"])
@pytest.mark.parametrize("max_bins", [16, 255, 257])
def test_histogram_matches_every_oracle_bin(backend, port, mode, max_bins):
    """tests/metal/test_mps_histogram.py:31-77: max_bins 16 and 255 (u8) and 257 (u16
    storage; the linspace column has 257 bins)."""
    x = _reference_matrix()
    labels = np.sin(np.arange(1025) / 17.0)
    selected = np.arange(3, 1025, 2)
    binned = mb.quantize_dense(x, max_bins)
    ds = port.quantize_dense(x, max_bins)
    pairs = port.gradients("squared_error", labels, np.zeros(1025))
    want = port.histograms(ds, pairs, selected)
    backend.set_hist_mode(mode)
    try:
        got = backend.histograms(binned, labels, np.zeros(1025), selected)["histograms"]
    finally:
        backend.set_hist_mode("fixed")
    for gf, wf in zip(got, want):
        assert np.array_equal(gf["count"], wf["count"])
        np.testing.assert_allclose(gf["gradient_sum"], wf["gradient_sum"], rtol=2e-5, atol=2e-5)
        np.testing.assert_allclose(gf["hessian_sum"], wf["hessian_sum"], rtol=1e-6, atol=1e-6)


def test_fixed_histograms_bit_exact_to_replica(backend, port):
    x = seeded_matrix(11, 20000, 40, 0.1, 4)
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    rng = np.random.default_rng(3)
    pairs = np.column_stack([rng.normal(size=20000) * 3, rng.uniform(0.2, 2.0, 20000)])
    rows = np.sort(rng.choice(20000, 12345, replace=False))
    got = backend.histograms_from_pairs(binned, pairs, rows)
    p32 = pairs.astype(np.float32)
    kg, kh = port.fixed_scales(p32)
    bins, miss = port.fixed_histograms(ds, p32, kg, kh, rows)
    for f, (gf, wf) in enumerate(zip(got, bins)):
        qg = wf["gradient_q"].copy()
        qh = wf["hessian_q"].copy()
        cnt = wf["count"].copy()
        qg[0] += miss[f]["gradient_q"]
        qh[0] += miss[f]["hessian_q"]
        cnt[0] += miss[f]["count"]
        assert np.array_equal(gf["count"], cnt)
        assert np.array_equal(gf["gradient_sum"], qg.astype(np.float64) * 2.0 ** -kg)
        assert np.array_equal(gf["hessian_sum"], qh.astype(np.float64) * 2.0 ** -kh)


def test_layer_histograms_equal_node_histograms(backend):
    x = seeded_matrix(12, 30000, 70, 0.05, 3)
    binned = mb.quantize_dense(x, 200)
    rng = np.random.default_rng(4)
    pairs = np.column_stack([rng.normal(size=30000), rng.uniform(0.5, 1.5, 30000)])
    perm = rng.permutation(30000)
    nodes = [np.sort(perm[:9000]), np.sort(perm[9000:9100]), np.sort(perm[9100:])]
    layer = backend.layer_histograms(binned, pairs, nodes)
    for rows, hist in zip(nodes, layer):
        single = backend.histograms_from_pairs(binned, pairs, rows)
        for a, b in zip(hist, single):
            assert a.tobytes() == b.tobytes()
    assert sum(int(h[0]["count"].sum()) for h in layer) == 30000


def test_split_scan_matches_oracle(backend, port):
    """tests/metal/test_mps_hot_path.py:17-112, full FindBestSplit semantics per feature."""
    rows = 257
    x = np.column_stack(
        (
            np.arange(rows, dtype=np.float32) % 17,
            np.linspace(-3.0, 3.0, rows, dtype=np.float32),
            np.where(np.arange(rows) < 180, 1.0, 9.0).astype(np.float32),
        )
    )
    labels = np.where(x[:, 0] < 8, -2.0, 3.0)
    selected = np.arange(1, rows, 3)
    binned = mb.quantize_dense(x, 32)
    ds = port.quantize_dense(x, 32)
    got = backend.split_candidates(binned, labels, np.zeros(rows), selected, min_samples_leaf=2,
                                   min_child_weight=0.0, reg_lambda=1.0, gamma=0.0)
    pairs = port.gradients("squared_error", labels, np.zeros(rows))
    want = port.scan_splits(ds, pairs, selected, min_samples_leaf=2, min_child_weight=0.0,
                            reg_lambda=1.0, gamma=0.0)
    for g, w in zip(got, want):
        assert g["valid"] == w["valid"]
        if not w["valid"]:
            continue
        assert (g["feature"], g["threshold_bin"], g["default_left"]) == (w["feature"], w["threshold_bin"], w["default_left"])
        assert (g["left_count"], g["right_count"]) == (w["left_count"], w["right_count"])
        assert g["gain"] == pytest.approx(w["gain"], rel=2e-5, abs=2e-5)


def test_split_scan_missing_and_constraints(backend, port):
    x = seeded_matrix(13, 3000, 6, 0.15, 2)
    binned = mb.quantize_dense(x, 64)
    ds = port.quantize_dense(x, 64)
    rng = np.random.default_rng(6)
    labels = np.nan_to_num(x[:, 2]) * 2 + np.isnan(x[:, 3]) * 3 + rng.normal(size=3000) * 0.1
    pairs = port.gradients("squared_error", labels, np.zeros(3000))
    rows = np.arange(3000)
    kw = dict(min_samples_leaf=5, min_child_weight=1.0, reg_lambda=0.7, reg_alpha=0.3,
              gamma=0.01, max_delta_step=2.0, monotonic_constraints=[1, -1, 0, 0, 1, -1])
    got = backend.split_candidates_from_pairs(binned, pairs, rows, **kw)
    want = port.scan_splits(ds, pairs, rows, **kw)
    for g, w in zip(got, want):
        assert g["valid"] == w["valid"]
        if w["valid"]:
            assert (g["threshold_bin"], g["default_left"], g["left_count"]) == (w["threshold_bin"], w["default_left"], w["left_count"])
            assert g["gain"] == pytest.approx(w["gain"], rel=2e-5, abs=2e-5)


def test_partition_matches_oracle(backend, port):
    """tests/metal/test_mps_hot_path.py:115-140 plus missing rows and many chunks."""
    rows = 513
    x = np.column_stack((np.arange(rows, dtype=np.float32) % 23, np.linspace(-1.0, 1.0, rows, dtype=np.float32)))
    binned = mb.quantize_dense(x, 32)
    selected = list(range(0, rows, 2))
    left, right = backend.partition_rows(binned, selected, 0, 10)
    assert left == [r for r in selected if binned.bins[0][r] <= 10]
    assert right == [r for r in selected if binned.bins[0][r] > 10]
    assert backend.partition_rows(binned, selected, 0, 10) == (left, right)
    x = seeded_matrix(14, 100000, 3, 0.2)
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    sel = np.sort(np.random.default_rng(1).choice(100000, 77777, replace=False))
    for dl in (True, False):
        gl, gr = backend.partition_rows(binned, sel, 1, 100, default_left=dl)
        wl, wr = port.partition_rows(ds, sel, 1, 100, default_left=dl)
        assert gl == wl.tolist() and gr == wr.tolist()


def test_node_entry_errors(backend):
    binned = mb.quantize_dense(seeded_matrix(15, 100, 2), 16)
    pairs = np.ones((100, 2))
    with pytest.raises(mb.TrainingError, match="empty"):
        backend.histograms_from_pairs(binned, pairs, [])
    with pytest.raises(mb.TrainingError, match="out of bounds"):
        backend.histograms_from_pairs(binned, pairs, [5, 100])
    with pytest.raises(mb.TrainingError, match="Gradient count"):
        backend.histograms_from_pairs(binned, pairs[:50], [1])
    with pytest.raises(mb.TrainingError, match="Hessian"):
        backend.histograms_from_pairs(binned, np.column_stack([np.ones(100), -np.ones(100)]), [1])
    with pytest.raises(mb.TrainingError, match="out of bounds"):
        backend.partition_rows(binned, [1, 2], 0, 99)
    with pytest.raises(mb.TrainingError, match="empty"):
        backend.partition_rows(binned, [], 0, 1)
    # 65536 bins and missing values leave no u16 value for the missing slot.
    col = np.arange(65537, dtype=np.float32)
    col[7] = np.nan
    full = mb.quantize_dense(col[:, None], 65536)
    assert int(full.bin_counts[0]) == 65536
    with pytest.raises(mb.UnsupportedError, match="65535"):
        backend.dataset(full)


def test_integer_pipe_conversions_match_hardware(tmp_path):
    """The integer-pipe int64->float and double->float conversions used by the gradient
    and split-scan kernels equal the hardware's correctly rounded conversions bit for bit
    (2^26 seeded inputs per family, ties, overflow and subnormal edges)."""
    import os
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = tmp_path / "conversions_check"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", os.path.join(root, "mpsboost_gb300", "csrc"), "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "native", "conversions_check.cu"), "-o", str(exe)],
                   check=True)
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr


def test_error_report_against_fp64_oracle(backend, port, record_property):
    """Max error of every histogram bin against the FP64 oracle's row-ordered sums, for the
    fixed-point path (exact int64 sums of values quantized to 2^-k) and the plain FP32
    path. Each bin's error stays within its a-priori bound: the FP64 -> FP32 rounding of
    the pair (2^-24 of each |value|) plus, fixed point, half a quantization unit per row,
    or, FP32 atomics, 2^-24 of the bin's absolute sum per added row. The figures are
    recorded as test properties."""
    x = seeded_matrix(13, 200_000, 24, 0.05, 3)
    binned = mb.quantize_dense(x, 255)
    ds = port.quantize_dense(x, 255)
    rng = np.random.default_rng(14)
    pairs = np.column_stack([rng.normal(size=200_000) * 2.0, rng.uniform(0.5, 1.5, 200_000)])
    rows = np.sort(rng.choice(200_000, 150_000, replace=False))
    want = port.histograms(ds, pairs, rows)
    absolute = port.histograms(ds, np.abs(pairs), rows)  # per-bin sums of |g|, |h|
    kg, kh = port.fixed_scales(pairs.astype(np.float32))
    report = {}
    for mode in ("fixed", "float"):
        backend.set_hist_mode(mode)
        try:
            got = backend.histograms_from_pairs(binned, pairs, rows)
        finally:
            backend.set_hist_mode("fixed")
        worst = {"g": 0.0, "h": 0.0, "g_rel_to_abs_sum": 0.0, "h_rel_to_abs_sum": 0.0}
        for gf, wf, af in zip(got, want, absolute):
            assert np.array_equal(gf["count"], wf["count"])
            n = wf["count"].astype(np.float64)
            for key, name, k in (("g", "gradient_sum", kg), ("h", "hessian_sum", kh)):
                err = np.abs(gf[name] - wf[name])
                s_abs = af[name]
                slack = n * 2.0 ** -52 * s_abs  # the oracle's own FP64 rounding
                if mode == "fixed":
                    bound = s_abs * 2.0 ** -24 + n * 2.0 ** -(k + 1) + slack
                else:
                    bound = s_abs * 2.0 ** -24 + n * s_abs * 2.0 ** -24 + slack
                assert np.all(err <= bound), (mode, key)
                worst[key] = max(worst[key], float(err.max()))
                nz = s_abs > 0
                if nz.any():
                    worst[key + "_rel_to_abs_sum"] = max(worst[key + "_rel_to_abs_sum"],
                                                         float((err[nz] / s_abs[nz]).max()))
        report[mode] = worst
        record_property(f"hist_max_error_{mode}", worst)
    print("histogram max errors vs FP64 oracle:", report)
    # Fixed point: the quantization error dominates and is far below FP32 accumulation's.
    assert report["fixed"]["g_rel_to_abs_sum"] < 1e-6


def test_leaf_error_report_against_fp64_oracle(backend, port, record_property):
    """Max relative error of the leaf values and training predictions against the FP64
    oracle's trees (same structures on these inputs), for both histogram paths."""
    x = seeded_matrix(15, 50_000, 16, 0.0, 0)
    rng = np.random.default_rng(16)
    y = np.sin(x[:, 0]) + 2.0 * x[:, 1] * (x[:, 2] > 0) + rng.normal(size=50_000) * 0.05
    params = dict(n_estimators=3, learning_rate=0.3, max_depth=5, min_samples_leaf=50)
    binned = mb.quantize_dense(x, 64)
    ds = port.quantize_dense(x, 64)
    want = port.train_regressor(ds, y, None, hist_mode=oracle.HIST_FP64, **params)
    ref_pred = want.predict(ds)
    report = {}
    for mode in ("fixed", "float"):
        model = mb.train_regressor(backend, binned, y, None, hist_mode=mode, **params)
        leaf_err = 0.0
        for got_t, exp_t in zip(model.trees, want.trees):
            assert [(int(a["feature_index"]), int(a["threshold_bin"])) for a in got_t] == \
                   [(int(b["feature_index"]), int(b["threshold_bin"])) for b in exp_t]
            leaf = (exp_t["flags"] & 1) == 1
            rel = np.abs(got_t["leaf_value"][leaf] - exp_t["leaf_value"][leaf]) / \
                np.maximum(np.abs(exp_t["leaf_value"][leaf]), 1e-12)
            leaf_err = max(leaf_err, float(rel.max()))
        pred_err = float(np.max(np.abs(model.train_predictions - ref_pred) / np.maximum(np.abs(ref_pred), 1e-12)))
        report[mode] = {"leaf_rel": leaf_err, "prediction_rel": pred_err}
        record_property(f"leaf_max_error_{mode}", report[mode])
        assert leaf_err <= 1e-5 and pred_err <= 1e-5
    print("leaf / prediction max relative errors vs FP64 oracle:", report)
