"""The histogram entry that allocates nothing, checked against the regular entry.

mpsb_cuda_build_histogram_noalloc serves callers that may not call cudaMalloc (a plugin
whose host process owns all device memory through its own pool, or a serving loop that
cannot take cudaMalloc's implicit synchronisation): they pass device buffers they already
own and the library keeps its intermediates in a fixed array of its own. This file runs
last so that, if it fails, a stop-at-first-failure run has already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import mpsboost_gb300 as mb
from mpsboost_gb300 import _lib

pytestmark = pytest.mark.gpu


def _column_blocked(bins_feature_major: np.ndarray) -> np.ndarray:
    features, rows = bins_feature_major.shape
    nfb = (features + 31) // 32
    padded = np.zeros((nfb * 32, rows), np.uint8)
    padded[:features] = bins_feature_major
    return np.ascontiguousarray(padded.reshape(nfb, 32, rows).transpose(0, 2, 1))


def _noalloc(torch, blocked, rows, pairs32, features):
    dev = torch.device("cuda", 0)
    d_bins = torch.from_numpy(blocked).to(dev)
    d_rows = torch.from_numpy(rows.astype(np.int32)).to(dev)
    d_pairs = torch.from_numpy(pairs32).to(dev)
    d_out = torch.empty(features * 256 * _lib.HIST_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(_lib.load().mpsb_cuda_build_histogram_noalloc(
        C.c_void_p(d_bins.data_ptr()), blocked.shape[1], features, C.c_void_p(d_rows.data_ptr()),
        rows.size, C.c_void_p(d_pairs.data_ptr()), C.c_void_p(d_out.data_ptr()), C.c_void_p(stream)))
    torch.cuda.synchronize(dev)
    return d_out.cpu().numpy().view(_lib.HIST_DTYPE).reshape(features, 256)


def test_noalloc_matches_regular_entry_twice_in_a_row():
    torch = pytest.importorskip("torch")
    backend = mb.CudaBackend(0)
    rng = np.random.default_rng(20260719)
    for call, (n, features) in enumerate([(50_000, 70), (120_000, 33)]):
        x = rng.normal(size=(n, features)).astype(np.float32)
        binned = mb.quantize_dense(x, 255)
        pairs = np.column_stack([rng.normal(size=n) * 2.0, rng.uniform(0.5, 1.5, n)])
        rows = np.sort(rng.choice(n, n // 3, replace=False))
        want = backend.histograms_from_pairs(binned, pairs, rows)
        got = _noalloc(torch, _column_blocked(binned.bins), rows, pairs.astype(np.float32), features)
        for f in range(features):
            nb = int(binned.bin_counts[f])
            g, w = got[f, :nb], want[f]
            assert np.array_equal(g["count"], w["count"]), (call, f)
            np.testing.assert_allclose(g["gradient_sum"], w["gradient_sum"], rtol=2e-5, atol=2e-5)
            np.testing.assert_allclose(g["hessian_sum"], w["hessian_sum"], rtol=1e-6, atol=1e-6)
            assert int(got[f, nb:]["count"].sum()) == 0
        assert int(got["count"].sum()) == features * rows.size


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.mpsb_cuda_build_histogram_noalloc(dummy, 10, 257, dummy, 5, dummy, dummy, None)
    assert rc == _lib.MPSB_ERR_UNSUPPORTED
    assert b"256 features" in lib.mpsb_cuda_last_error()
