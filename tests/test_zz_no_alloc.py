"""The histogram entry that allocates nothing, checked against the oracle and the regular entry.

mpsb_cuda_build_histogram_noalloc serves callers that may not call cudaMalloc (a plugin
whose host process owns all device memory through its own pool, or a serving loop that
cannot take cudaMalloc's implicit synchronisation): they pass device buffers they already
own and the library keeps its intermediates in a fixed array of its own. Its sums are
exact int64 fixed point, so every bin must equal the oracle's fixed-point replica bit for
bit (and the regular entry's bytes). This file runs last so that, if it fails, a
stop-at-first-failure run has already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import mpsboost_gb300 as mb
from mpsboost_gb300 import _lib
from conftest import seeded_matrix

pytestmark = pytest.mark.gpu


def _column_blocked(bins_feature_major: np.ndarray) -> np.ndarray:
    features, rows = bins_feature_major.shape
    nfb = (features + 31) // 32
    padded = np.zeros((nfb * 32, rows), np.uint8)
    padded[:features] = bins_feature_major
    return np.ascontiguousarray(padded.reshape(nfb, 32, rows).transpose(0, 2, 1))


def _noalloc(torch, blocked, rows, pairs32, features, stream=None):
    dev = torch.device("cuda", 0)
    stream = stream or torch.cuda.current_stream(dev)
    with torch.cuda.stream(stream):
        d_bins = torch.from_numpy(blocked).to(dev)
        d_rows = torch.from_numpy(rows.astype(np.int32)).to(dev)
        d_pairs = torch.from_numpy(np.ascontiguousarray(pairs32)).to(dev)
        d_out = torch.empty(features * 256 * _lib.HIST_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    _lib.check(_lib.load().mpsb_cuda_build_histogram_noalloc(
        C.c_void_p(d_bins.data_ptr()), blocked.shape[1], features, C.c_void_p(d_rows.data_ptr()),
        rows.size, C.c_void_p(d_pairs.data_ptr()), C.c_void_p(d_out.data_ptr()),
        C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    return d_out.cpu().numpy().view(_lib.HIST_DTYPE).reshape(features, 256)


def _replica(port, binned, pairs32, rows):
    """The oracle's exact int64 sums as the entry reports them: missing rows in bin 0."""
    ds = port.dataset_from_bins(binned)
    kg, kh = port.fixed_scales(pairs32)
    bins, miss = port.fixed_histograms(ds, pairs32, kg, kh, rows)
    out = []
    for f, wf in enumerate(bins):
        cnt, qg, qh = wf["count"].copy(), wf["gradient_q"].copy(), wf["hessian_q"].copy()
        cnt[0] += miss[f]["count"]
        qg[0] += miss[f]["gradient_q"]
        qh[0] += miss[f]["hessian_q"]
        out.append((cnt, qg.astype(np.float64) * 2.0 ** -kg, qh.astype(np.float64) * 2.0 ** -kh))
    return out


# (rows, features, missing fraction, non-default stream): two calls in a row on the
# default stream, then the largest layout the fixed scratch holds (256 features = eight
# full feature blocks) on a stream of its own.
CASES = [(50_000, 70, 0.0, False), (120_000, 33, 0.05, False), (4_096, 256, 0.02, True)]


def test_noalloc_bit_exact_to_replica_on_consecutive_calls(port):
    torch = pytest.importorskip("torch")
    backend = mb.CudaBackend(0)
    rng = np.random.default_rng(20260719)
    side = torch.cuda.Stream(torch.device("cuda", 0))
    for call, (n, features, nan_fraction, own_stream) in enumerate(CASES):
        x = seeded_matrix(100 + call, n, features, nan_fraction, 3)
        binned = mb.quantize_dense(x, 255)
        pairs = np.column_stack([rng.normal(size=n) * 2.0, rng.uniform(0.5, 1.5, n)])
        p32 = pairs.astype(np.float32)
        rows = np.sort(rng.choice(n, n // 3, replace=False))
        got = _noalloc(torch, _column_blocked(binned.bins), rows, p32, features,
                       side if own_stream else None)
        want = _replica(port, binned, p32, rows)
        regular = backend.histograms_from_pairs(binned, p32.astype(np.float64), rows)
        for f in range(features):
            nb = int(binned.bin_counts[f])
            g = got[f, :nb]
            cnt, gs, hs = want[f]
            assert np.array_equal(g["count"], cnt), (call, f)
            assert np.array_equal(g["gradient_sum"], gs), (call, f)
            assert np.array_equal(g["hessian_sum"], hs), (call, f)
            assert g.tobytes() == regular[f].tobytes(), (call, f)
            assert int(got[f, nb:]["count"].sum()) == 0
        assert int(got["count"].sum()) == features * rows.size


def test_noalloc_reports_invalid_pairs_as_nan():
    """A NaN gradient cannot raise without a synchronisation: every bin comes back with
    count 0 and NaN sums, and the next valid call is unaffected."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    n, features = 8_192, 40
    binned = mb.quantize_dense(seeded_matrix(7, n, features), 255)
    blocked = _column_blocked(binned.bins)
    rows = np.arange(0, n, 2)
    p32 = np.column_stack([rng.normal(size=n), rng.uniform(0.5, 1.5, n)]).astype(np.float32)
    bad = p32.copy()
    bad[123, 0] = np.nan
    got = _noalloc(torch, blocked, rows, bad, features)
    assert int(got["count"].sum()) == 0
    assert np.isnan(got["gradient_sum"]).all() and np.isnan(got["hessian_sum"]).all()
    again = _noalloc(torch, blocked, rows, p32, features)
    assert int(again["count"].sum()) == features * rows.size
    assert np.isfinite(again["gradient_sum"]).all()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.mpsb_cuda_build_histogram_noalloc(dummy, 10, 257, dummy, 5, dummy, dummy, None)
    assert rc == _lib.MPSB_ERR_UNSUPPORTED
    assert b"256 features" in lib.mpsb_cuda_last_error()
