"""The C-ABI library without a GPU: it builds, loads, exports every declared symbol, its
struct layouts match the header, binning matches the oracle, and device entries fail
loudly (never silently on the CPU) when no GB300 is present."""

from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

import mpsboost_gb300 as mb
from mpsboost_gb300 import _lib
from conftest import seeded_matrix

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "mpsb_cuda.h")


def declared_functions() -> set[str]:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(mpsb_\w+)\s*\(", text))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name
    assert names == set(_lib.SIGNATURES), sorted(names ^ set(_lib.SIGNATURES))
    assert lib.mpsb_cuda_abi_version() == 2


def test_struct_layouts():
    assert C.sizeof(_lib.TrainParams) == 12 * 4 + 8 + 9 * 8 + 3 * 8
    assert _lib.NODE_DTYPE.itemsize == 40
    assert _lib.HIST_DTYPE.itemsize == 24
    assert _lib.SPLIT_DTYPE.itemsize == 72
    import oracle

    assert C.sizeof(oracle.Params) == C.sizeof(_lib.TrainParams)
    for (a, ta), (b, tb) in zip(oracle.Params._fields_, _lib.TrainParams._fields_):
        assert a == b and C.sizeof(ta) == C.sizeof(tb)
        assert getattr(oracle.Params, a).offset == getattr(_lib.TrainParams, b).offset


@pytest.mark.parametrize("max_bins,nan,ints", [(255, 0.0, 2), (16, 0.1, 1), (256, 0.2, 0), (300, 0.05, 3), (2, 0.0, 0)])
def test_product_binning_matches_oracle(port, max_bins, nan, ints):
    x = seeded_matrix(31 + max_bins, 2500, 6, nan, ints)
    got = mb.quantize_dense(x, max_bins)
    want = port.quantize_dense(x, max_bins)
    assert np.array_equal(got.bins.astype(np.uint16), want.bins)
    assert np.array_equal(got.missing, want.missing)
    assert got.boundaries_flat.tobytes() == want.boundaries_flat.tobytes()
    assert np.array_equal(got.bin_counts, want.bin_counts)
    assert np.array_equal(got.missing_counts, want.missing_counts)
    x2 = seeded_matrix(99, 400, 6, 0.1)
    t1, t2 = got.transform(x2), port.transform_dense(want, x2)
    assert np.array_equal(t1.bins.astype(np.uint16), t2.bins) and np.array_equal(t1.missing, t2.missing)


def test_binning_float64_and_strided(port):
    x = seeded_matrix(5, 800, 8, 0.1).astype(np.float64)[:, ::2]
    got = mb.quantize_dense(x, 64)
    want = port.quantize_dense(x, 64)
    assert np.array_equal(got.bins.astype(np.uint16), want.bins)


def test_binning_errors():
    with pytest.raises(mb.DataError, match="Inf"):
        mb.quantize_dense(np.array([[np.inf]], np.float32), 8)
    with pytest.raises(mb.DataError):
        mb.quantize_dense(np.zeros((0, 3), np.float32), 8)
    with pytest.raises(mb.DataError, match="max_bins"):
        mb.quantize_dense(np.zeros((3, 3), np.float32), 1)
    with pytest.raises(mb.DataError, match="float32 range"):
        mb.quantize_dense(np.array([[1e300]], np.float64), 8)


def test_params_validation():
    with pytest.raises(ValueError, match="unknown parameter"):
        mb.make_params(nonsense=1)
    with pytest.raises(ValueError, match="objective"):
        mb.make_params(objective="hinge")
    p, keep = mb.make_params(monotonic_constraints=[1, 0, -1], interaction_constraints=[[0, 1], [2]])
    assert p.n_monotonic == 3 and p.n_interaction_groups == 2


def test_device_entries_fail_loudly_without_gpu():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(mb.BackendError):
        mb.CudaBackend(0)


def test_c_errors_surface_messages():
    lib = _lib.load()
    out = C.c_void_p()
    rc = lib.mpsb_cuda_backend_create(-1, C.byref(out))
    assert rc == _lib.MPSB_ERR_BACKEND
    assert lib.mpsb_cuda_last_error()
