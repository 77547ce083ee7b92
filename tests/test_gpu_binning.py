"""Quantile binning on the device against the host restatement (QuantizeDense /
TransformDense, binned_dataset.cpp:95-238; the host path is pinned to the reference in
test_oracle_pin.py). Bins, missing flags, boundary counts and bin counts are identical;
boundaries are equal as floats (a boundary at zero may carry either sign). Up to 256 bins
the boundaries come from the radix selection, above 256 (u16 bins) from a per-feature
sort."""

from __future__ import annotations

import numpy as np
import pytest

import mpsboost_gb300 as mb

pytestmark = pytest.mark.gpu


def _same(dev: mb.DeviceBinnedDataset, host: mb.BinnedDataset):
    got = dev.to_host()
    assert np.array_equal(got.bins, host.bins)
    assert np.array_equal(got.missing, host.missing)
    assert np.array_equal(got.boundary_counts, host.boundary_counts)
    assert np.array_equal(got.boundary_offsets, host.boundary_offsets)
    assert np.array_equal(got.bin_counts, host.bin_counts)
    assert np.array_equal(got.missing_counts, host.missing_counts)
    assert np.array_equal(got.boundaries_flat, host.boundaries_flat)  # float equality


def _matrix(seed, rows, cols):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(rows, cols)).astype(np.float32)
    if cols > 1:
        x[:, 1] = rng.integers(0, 7, rows)                  # few distinct values
    if cols > 2:
        x[:, 2] = np.round(x[:, 2], 1)                      # many ties
    if cols > 3:
        x[:, 3] = np.where(rng.random(rows) < 0.5, -0.0, 0.0)  # signed zeros only
    x[rng.random((rows, cols)) < 0.07] = np.nan             # missing cells
    if cols > 5:
        x[:, 5] = 3.25                                      # constant
    if cols > 6:
        x[:, 6] = np.nan                                    # all missing
    if cols > 7:
        x[:, 7] = np.exp(rng.normal(size=rows) * 8).astype(np.float32)  # wide range
    return x


@pytest.mark.parametrize("rows,cols,max_bins", [(1, 3, 16), (7, 9, 4), (1000, 10, 255), (50_000, 12, 64),
                                                (123_457, 8, 256), (20_000, 40, 2), (3, 4, 300),
                                                (50_000, 9, 1000), (123_457, 8, 4096), (30_000, 5, 65536),
                                                (70_001, 3, 65535)])
def test_quantize_matches_host(backend, rows, cols, max_bins):
    """256 bins with missing values train on the wide layout; above 256 the bins are u16."""
    x = _matrix(rows + cols, rows, cols)
    _same(mb.quantize_device(backend, x, max_bins), mb.quantize_dense(x, max_bins))


def test_layouts_and_dtypes(backend):
    x = _matrix(3, 5000, 9)
    host = mb.quantize_dense(x, 128)
    _same(mb.quantize_device(backend, np.asfortranarray(x), 128), host)    # column-major
    _same(mb.quantize_device(backend, x.astype(np.float64), 128), host)    # float64 input
    wide = np.zeros((5000, 18), np.float32)
    wide[:, ::2] = x
    _same(mb.quantize_device(backend, wide[:, ::2], 128), host)              # strided view


@pytest.mark.parametrize("max_bins", [200, 3000])
def test_transform_matches_host(backend, max_bins):
    x = _matrix(11, 20_000, 10)
    y = _matrix(12, 7_000, 10)
    host = mb.quantize_dense(x, max_bins)
    dev = mb.quantize_device(backend, x, max_bins)
    _same(dev.transform(y), host.transform(y))


@pytest.mark.parametrize("max_bins", [255, 1024])
def test_training_on_device_bins_equals_host_bins(backend, max_bins):
    x = _matrix(13, 30_000, 10)
    rng = np.random.default_rng(14)
    y = np.nan_to_num(x[:, 0]) * 2 + rng.normal(size=x.shape[0])
    params = dict(n_estimators=3, learning_rate=0.2, max_depth=6, min_samples_leaf=3)
    a = mb.train_regressor(backend, mb.quantize_dense(x, max_bins), y, **params)
    dev = mb.quantize_device(backend, x, max_bins)
    b = mb.train_regressor(backend, dev, y, **params)
    for t1, t2 in zip(a.trees, b.trees):
        assert t1.tobytes() == t2.tobytes()
    assert np.array_equal(a.train_predictions, b.train_predictions)
    assert np.array_equal(b.predict(backend, dev), b.train_predictions)


def test_quantize_errors(backend):
    x = np.ones((10, 3), np.float32)
    bad = x.copy()
    bad[4, 1] = np.inf
    with pytest.raises(mb.DataError, match="Inf"):
        mb.quantize_device(backend, bad, 16)
    big = np.ones((10, 3), np.float64)
    big[2, 2] = 1e39
    with pytest.raises(mb.DataError, match="float32"):
        mb.quantize_device(backend, big, 16)
    full = np.arange(65537, dtype=np.float32)[:, None]  # 65536 bins and a missing value
    full[9] = np.nan
    with pytest.raises(mb.UnsupportedError, match="65535"):
        mb.quantize_device(backend, full, 65536)
    with pytest.raises(mb.DataError, match="max_bins"):
        mb.quantize_device(backend, x, 1)


def test_quantize_at_scale(backend):
    """2M x 64 with missing values: the device and host binnings agree cell for cell."""
    rng = np.random.default_rng(15)
    x = rng.normal(size=(2_000_000, 64)).astype(np.float32)
    x[:, 32:] = np.exp(x[:, 32:])
    x[rng.random(x.shape) < 0.02] = np.nan
    _same(mb.quantize_device(backend, x, 255), mb.quantize_dense(x, 255))


def test_model_files_of_gpu_models(backend, tmp_path):
    """GPU-trained models write the native model file with their training schema and
    read back to the same predictions (device-quantized data carries the schema)."""
    x = _matrix(16, 8_000, 9)
    rng = np.random.default_rng(17)
    y = np.nan_to_num(x[:, 0]) + rng.normal(size=x.shape[0]) * 0.1
    params = dict(n_estimators=2, learning_rate=0.3, max_depth=4)
    host = mb.quantize_dense(x, 64)
    dev = mb.quantize_device(backend, x, 64)
    a = mb.train_regressor(backend, host, y, **params)
    b = mb.train_regressor(backend, dev, y, **params)
    assert a.to_bytes() == b.to_bytes()  # same trees, same schema
    path = tmp_path / "gpu.mpsb"
    b.save(str(path))
    c = mb.RegressionModel.load(str(path))
    assert np.array_equal(c.predict(backend, host), a.train_predictions)
