"""Python host mirror of the reference's native interface for the training hot path.

Names and argument meaning follow the reference's pybind11 module (``_native``) and its
C++ types:

* :func:`quantize_dense` / :meth:`BinnedDataset.transform` -- ``_quantize_dense``
  (src/python/binding_dataset.cpp), QuantizeDense / TransformDense
  (include/mpsboost/binned_dataset.hpp:137-144).
* :class:`CudaBackend` -- ``_MpsBackend`` (src/python/binding_backend.cpp:18-84):
  ``gradients``, ``histograms``, ``layer_histograms``, ``split_candidates``,
  ``partition_rows``, plus the device-resident :meth:`CudaBackend.dataset`.
* :func:`train_regressor` -- ``_train_regressor_mps`` (src/python/binding_model.cpp:34-45)
  over TrainRegressionModel (include/mpsboost/trainer.hpp:133-139).
* :func:`train_ovr` -- the one-vs-rest multiclass fit of
  src/mpsboost/estimators/multiclass.py:113-160, all K trees of a round in one launch.

Every device computation runs in ``libmpsb_cuda.so``; nothing here computes on the CPU
except binning (which the reference also does on the CPU) and the argument checks.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import HIST_DTYPE, NODE_DTYPE, SPLIT_DTYPE, TrainParams, check, ptr

OBJECTIVES = {"squared_error": 0, "binary_logistic": 1, "quantile": 2, "poisson": 3, "tweedie": 4}

# C++ defaults of TrainingParameters / TreeTrainingParameters (trainer.hpp:29-35,
# tree.hpp:57-71).
DEFAULT_PARAMS = dict(
    n_estimators=100,
    learning_rate=0.1,
    max_bins=256,
    objective="squared_error",
    max_depth=6,
    max_leaves=0,
    max_active_leaves=0,
    min_samples_leaf=1,
    min_child_weight=0.0,
    reg_lambda=1.0,
    reg_alpha=0.0,
    max_delta_step=0.0,
    gamma=0.0,
    min_gain_to_split=0.0,
    split_strategy="best_gain",
    growth_strategy="level_wise",
    random_seed=0,
    objective_alpha=0.5,
    tweedie_variance_power=1.5,
    monotonic_constraints=None,
    interaction_constraints=None,
)


def make_params(**overrides) -> tuple[TrainParams, list]:
    """``(TrainParams, keepalive)`` from keyword overrides of :data:`DEFAULT_PARAMS`."""

    unknown = set(overrides) - set(DEFAULT_PARAMS)
    if unknown:
        raise ValueError(f"unknown parameter(s): {sorted(unknown)}")
    v = dict(DEFAULT_PARAMS, **overrides)
    p = TrainParams()
    for name in (
        "n_estimators", "max_bins", "max_depth", "max_leaves", "max_active_leaves",
        "random_seed", "min_samples_leaf", "learning_rate", "objective_alpha",
        "tweedie_variance_power", "min_child_weight", "reg_lambda", "reg_alpha",
        "max_delta_step", "gamma", "min_gain_to_split",
    ):
        setattr(p, name, v[name])
    obj = v["objective"]
    if isinstance(obj, str):
        if obj not in OBJECTIVES:
            raise ValueError("unknown training objective")
        obj = OBJECTIVES[obj]
    p.objective = obj
    try:
        p.split_strategy = {"best_gain": 0, "random_threshold": 1}[v["split_strategy"]]
        p.growth_strategy = {"level_wise": 0, "leaf_wise": 1}[v["growth_strategy"]]
    except KeyError as exc:
        raise ValueError(f"unknown split or growth strategy: {exc}") from None
    keep: list = []
    if v["monotonic_constraints"] is not None:
        mono = np.ascontiguousarray(v["monotonic_constraints"], dtype=np.int8)
        keep.append(mono)
        p.n_monotonic = mono.size
        p.monotonic_constraints = mono.ctypes.data_as(C.POINTER(C.c_int8))
    if v["interaction_constraints"]:
        groups = [list(g) for g in v["interaction_constraints"]]
        offsets = np.cumsum([0] + [len(g) for g in groups]).astype(np.uint32)
        feats = np.asarray([f for g in groups for f in g] or [0], dtype=np.uint32)
        keep += [offsets, feats]
        p.n_interaction_groups = len(groups)
        p.interaction_offsets = offsets.ctypes.data_as(C.POINTER(C.c_uint32))
        p.interaction_features = feats.ctypes.data_as(C.POINTER(C.c_uint32))
    return p, keep


# --------------------------------------------------------------------------------------
# Binning (host, reference semantics)
# --------------------------------------------------------------------------------------
@dataclass
class BinnedDataset:
    """Feature-major bins + missing mask + frozen schema (binned_dataset.hpp:81-126)."""

    rows: int
    features: int
    max_bins: int
    bins: np.ndarray  # [features, rows] uint8 (max_bins <= 256) or uint16
    missing: np.ndarray  # [features, rows] bool
    boundaries_flat: np.ndarray
    boundary_offsets: np.ndarray
    boundary_counts: np.ndarray
    bin_counts: np.ndarray
    missing_counts: np.ndarray
    _device: dict = field(default_factory=dict, repr=False)

    @property
    def boundaries(self) -> list[list[float]]:
        return [
            self.boundaries_flat[o : o + c].tolist()
            for o, c in zip(self.boundary_offsets, self.boundary_counts)
        ]

    @property
    def bin_width(self) -> int:
        return 8 if self.max_bins <= 256 else 16

    def transform(self, matrix, n_threads: int = 0) -> "BinnedDataset":
        """Bin new data with this schema (TransformDense, binned_dataset.cpp:190-238)."""

        x, st, rs, cs = _as_matrix(matrix)
        if x.shape[1] != self.features:
            raise _lib.DataError("Prediction input feature count does not match the binned schema")
        rows, feats = x.shape
        wide = self.max_bins > 256
        bins = np.empty((feats, rows), np.uint16 if wide else np.uint8)
        missing = np.empty((feats, rows), np.uint8)
        lib = _lib.load()
        bnd = np.ascontiguousarray(self.boundaries_flat, np.float32)
        check(
            lib.mpsb_transform_dense(
                ptr(x), st, rows, feats, rs, cs, self.max_bins, ptr(bnd),
                ptr(self.boundary_offsets), ptr(self.boundary_counts), n_threads, ptr(bins), ptr(missing),
            )
        )
        return BinnedDataset(
            rows, feats, self.max_bins, bins, missing.astype(bool), self.boundaries_flat,
            self.boundary_offsets, self.boundary_counts, self.bin_counts,
            missing.sum(axis=1).astype(np.uint64),
        )


def _as_matrix(matrix) -> tuple[np.ndarray, int, int, int]:
    """``(array, scalar type, row stride, column stride)`` of a 2-D float view.

    Size-1 axes get their natural stride (numpy may report 0 for them); broadcast or
    reversed views are read from a dense copy."""

    x = np.asarray(matrix)
    if x.dtype not in (np.float32, np.float64):
        x = x.astype(np.float32)
    if x.ndim != 2:
        raise _lib.DataError("Input matrix must be two-dimensional")
    if x.shape[0] == 0 or x.shape[1] == 0:
        raise _lib.DataError("Input matrix must contain at least one row and one feature")

    def strides(a):
        rs = a.strides[0] if a.shape[0] > 1 else a.itemsize * a.shape[1]
        cs = a.strides[1] if a.shape[1] > 1 else a.itemsize
        return rs, cs

    rs, cs = strides(x)
    if rs < x.itemsize or cs < x.itemsize:
        x = np.array(x, order="C")
        rs, cs = strides(x)
    return x, 1 if x.dtype == np.float32 else 2, rs, cs


def quantize_dense(matrix, max_bins: int = 256, n_threads: int = 0) -> BinnedDataset:
    """Quantile-bin a float32/float64 matrix (QuantizeDense, binned_dataset.cpp:126-188)."""

    x, st, rs, cs = _as_matrix(matrix)
    rows, feats = x.shape
    if not 2 <= max_bins <= 65536:
        raise _lib.DataError("max_bins must be in [2, 65536]")
    wide = max_bins > 256
    bins = np.empty((feats, rows), np.uint16 if wide else np.uint8)
    missing = np.empty((feats, rows), np.uint8)
    bnd = np.empty(max(feats * (max_bins - 1), 1), np.float32)
    off = np.empty(feats, np.uint64)
    cnt = np.empty(feats, np.uint32)
    binc = np.empty(feats, np.uint32)
    miss = np.empty(feats, np.uint64)
    lib = _lib.load()
    check(
        lib.mpsb_quantize_dense(
            ptr(x), st, rows, feats, rs, cs, max_bins, n_threads, ptr(bins),
            ptr(missing), ptr(bnd), ptr(off), ptr(cnt), ptr(binc), ptr(miss),
        )
    )
    total = int(cnt.sum())
    return BinnedDataset(rows, feats, max_bins, bins, missing.astype(bool), bnd[:total].copy(), off, cnt, binc, miss)


# --------------------------------------------------------------------------------------
# Backend
# --------------------------------------------------------------------------------------
class DeviceDataset:
    """A binned dataset resident in HBM: column-blocked u8 bins with missing rows at slot
    255, or u16 bins for a wide dataset (a feature with more than 256 bins, or 256 bins and
    missing values) with missing rows at its last histogram slot."""

    @classmethod
    def _adopt(cls, backend: "CudaBackend", handle, rows: int, features: int) -> "DeviceDataset":
        self = cls.__new__(cls)
        self.backend = backend
        self.binned = None
        self.rows = rows
        self.features = features
        self.handle = handle
        return self

    def __init__(self, backend: "CudaBackend", binned: BinnedDataset):
        lib = _lib.load()
        self.backend = backend
        self.binned = binned
        self.rows = binned.rows
        self.features = binned.features
        bins = np.ascontiguousarray(binned.bins)
        missing = np.ascontiguousarray(binned.missing, dtype=np.uint8) if binned.missing.any() else None
        counts = np.ascontiguousarray(binned.bin_counts, dtype=np.uint32)
        handle = C.c_void_p()
        check(
            lib.mpsb_cuda_dataset_create(
                backend.handle, ptr(bins), bins.dtype.itemsize, ptr(missing), binned.rows,
                binned.features, ptr(counts), C.byref(handle),
            )
        )
        self.handle = handle

    @property
    def uses_tma(self) -> bool:
        """Row-major histogram levels stage gathered rows with TMA gather4 copies."""
        return bool(_lib.load().mpsb_cuda_dataset_uses_tma(self.handle))

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().mpsb_cuda_dataset_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceBinnedDataset:
    """A matrix quantile-binned on the GPU and kept there (QuantizeDense on the device).

    Usable wherever a ``BinnedDataset`` is (training, prediction) on the backend that
    binned it; ``to_host()`` returns the same bins and schema as ``quantize_dense``."""

    def __init__(self, backend: "CudaBackend", handle, rows: int, features: int, max_bins: int):
        self.backend = backend
        self.rows = rows
        self.features = features
        self.max_bins = max_bins
        self._dev = DeviceDataset._adopt(backend, handle, rows, features)
        lib = _lib.load()
        total = int(lib.mpsb_cuda_dataset_boundary_total(handle))
        self.boundaries_flat = np.empty(max(total, 1), np.float32)
        self.boundary_offsets = np.empty(features, np.uint64)
        self.boundary_counts = np.empty(features, np.uint32)
        self.bin_counts = np.empty(features, np.uint32)
        self.missing_counts = np.empty(features, np.uint64)
        check(lib.mpsb_cuda_dataset_schema(handle, ptr(self.boundaries_flat), ptr(self.boundary_offsets),
                                           ptr(self.boundary_counts), ptr(self.bin_counts),
                                           ptr(self.missing_counts)))
        self.boundaries_flat = self.boundaries_flat[:total]

    def to_host(self) -> BinnedDataset:
        lib = _lib.load()
        wide = self.max_bins > 256  # quantize_dense's storage: u16 above 256 bins
        bins = np.empty((self.features, self.rows), np.uint16 if wide else np.uint8)
        missing = np.empty((self.features, self.rows), np.uint8)
        export = lib.mpsb_cuda_dataset_export16 if wide else lib.mpsb_cuda_dataset_export
        check(export(self._dev.handle, ptr(bins), ptr(missing)))
        return BinnedDataset(self.rows, self.features, self.max_bins, bins, missing.astype(bool),
                             self.boundaries_flat.copy(), self.boundary_offsets.copy(),
                             self.boundary_counts.copy(), self.bin_counts.copy(), self.missing_counts.copy())

    def transform(self, matrix) -> "DeviceBinnedDataset":
        """Bin new data on the device with this schema (TransformDense)."""

        x, st, rs, cs = _as_matrix(matrix)
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.mpsb_cuda_dataset_transform(self.backend.handle, self._dev.handle, ptr(x), st,
                                              x.shape[0], x.shape[1], rs, cs, C.byref(h)))
        return DeviceBinnedDataset(self.backend, h, x.shape[0], x.shape[1], self.max_bins)

    def close(self) -> None:
        self._dev.close()


def quantize_device(backend: "CudaBackend", matrix, max_bins: int = 256) -> DeviceBinnedDataset:
    """Quantile-bin a float32/float64 matrix on the GPU (QuantizeDense,
    binned_dataset.cpp:126-188) and keep the bins resident for training."""

    x, st, rs, cs = _as_matrix(matrix)
    lib = _lib.load()
    h = C.c_void_p()
    check(lib.mpsb_cuda_dataset_quantize(backend.handle, ptr(x), st, x.shape[0], x.shape[1], rs, cs,
                                         max_bins, C.byref(h)))
    return DeviceBinnedDataset(backend, h, x.shape[0], x.shape[1], max_bins)


class CudaBackend:
    """One GB300 and one CUDA stream (MpsBackend, backend.hpp:140-195)."""

    def __init__(self, device: int = 0, hist_mode: str = "fixed"):
        lib = _lib.load()
        handle = C.c_void_p()
        check(lib.mpsb_cuda_backend_create(device, C.byref(handle)))
        self.handle = handle
        self.set_hist_mode(hist_mode)

    def set_hist_mode(self, mode: str) -> None:
        code = {"fixed": _lib.HIST_FIXED, "float": _lib.HIST_FLOAT}[mode]
        check(_lib.load().mpsb_cuda_backend_set_hist_mode(self.handle, code))
        self.hist_mode = mode

    @property
    def info(self) -> dict:
        inf = _lib.Info()
        check(_lib.load().mpsb_cuda_backend_info(self.handle, C.byref(inf)))
        return {
            "available": bool(inf.available),
            "device_name": inf.device_name.decode(),
            "sm_count": inf.sm_count,
            "compute_capability": (inf.cc_major, inf.cc_minor),
            "total_memory": inf.total_memory,
        }

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().mpsb_cuda_backend_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- datasets ------------------------------------------------------------------------
    def dataset(self, binned) -> DeviceDataset:
        if isinstance(binned, DeviceBinnedDataset):
            if binned.backend is not self:
                raise ValueError("a device-binned dataset trains on the backend that binned it")
            return binned._dev
        key = id(self)
        dev = binned._device.get(key)
        if dev is None:
            dev = DeviceDataset(self, binned)
            binned._device[key] = dev
        return dev

    # -- node-level entries (binding_backend.cpp:19-71) ----------------------------------
    def gradients(self, labels, predictions) -> np.ndarray:
        """Squared-error pairs ``[n, 2]`` (GradientComputer::ComputeSquaredError)."""

        y = np.ascontiguousarray(labels, dtype=np.float64)
        p = np.ascontiguousarray(predictions, dtype=np.float64)
        if y.size == 0:
            raise _lib.TrainingError("Labels must not be empty")
        if y.size != p.size:
            raise _lib.TrainingError("Label and prediction lengths do not match")
        out = np.empty((y.size, 2), np.float64)
        check(_lib.load().mpsb_cuda_squared_error(self.handle, ptr(y), ptr(p), y.size, ptr(out)))
        return out

    def autotune(self, dataset, labels, weights=None, *, rounds_per_trial: int = 3,
                 hist_mode: str = "fixed", **params) -> dict:
        """Times boosting rounds of this fit's shape under candidate launch shapes and keeps
        the fastest for every later fit of the same shape (mpsb_cuda_autotune)."""

        dev = self.dataset(dataset)
        y = np.ascontiguousarray(labels, dtype=np.float64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        p, keep = make_params(**params)
        out = _lib.Tuning()
        check(_lib.load().mpsb_cuda_autotune(self.handle, dev.handle, ptr(y), ptr(w), y.size, C.byref(p),
                                             _options(hist_mode, True, True), rounds_per_trial,
                                             C.byref(out)))
        del keep
        return {name: getattr(out, name) for name, _ in _lib.Tuning._fields_}

    @staticmethod
    def autotune_clear() -> None:
        _lib.load().mpsb_cuda_autotune_clear()

    def histograms_from_pairs(self, dataset: BinnedDataset, pairs, rows) -> list[np.ndarray]:
        """Per-feature HistogramBin arrays of one node (HistogramBuilder::BuildHistograms)."""

        return self.layer_histograms(dataset, pairs, [rows])[0]

    def layer_histograms(self, dataset: BinnedDataset, pairs, node_rows) -> list[list[np.ndarray]]:
        """All nodes of a layer in one launch (LayerHistogramBuilder::BuildLayerHistograms)."""

        dev = self.dataset(dataset)
        g = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 2)
        parts = [np.ascontiguousarray(r, dtype=np.uint64).ravel() for r in node_rows]
        if not parts:
            return []
        rows = np.concatenate(parts) if parts else np.empty(0, np.uint64)
        offsets = np.cumsum([0] + [p.size for p in parts]).astype(np.uint64)
        per_node = int(dataset.bin_counts.sum())
        out = np.empty(per_node * len(parts), HIST_DTYPE)
        check(
            _lib.load().mpsb_cuda_build_layer_histograms(
                self.handle, dev.handle, ptr(rows), ptr(offsets), len(parts), ptr(g), g.shape[0], ptr(out)
            )
        )
        splits = np.cumsum(dataset.bin_counts)[:-1]
        return [np.split(out[i * per_node : (i + 1) * per_node], splits) for i in range(len(parts))]

    def histograms(self, dataset: BinnedDataset, labels, predictions, rows) -> dict:
        """The reference hook's shape: squared-error pairs, then one node's histograms."""

        pairs = self.gradients(labels, predictions)
        return {"histograms": self.histograms_from_pairs(dataset, pairs, rows)}

    def split_candidates_from_pairs(self, dataset: BinnedDataset, pairs, rows, **params) -> np.ndarray:
        dev = self.dataset(dataset)
        g = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 2)
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        p, keep = make_params(**params)
        out = np.empty(dataset.features, SPLIT_DTYPE)
        check(
            _lib.load().mpsb_cuda_scan_splits(
                self.handle, dev.handle, ptr(r), r.size, ptr(g), g.shape[0], C.byref(p), ptr(out)
            )
        )
        del keep
        return out

    def split_candidates(self, dataset, labels, predictions, rows, *, min_samples_leaf=1,
                         min_child_weight=0.0, reg_lambda=1.0, gamma=0.0) -> np.ndarray:
        """Best split per feature of one node (ScanSplitsForTest, backend.hpp:173-180)."""

        pairs = self.gradients(labels, predictions)
        return self.split_candidates_from_pairs(
            dataset, pairs, rows, min_samples_leaf=min_samples_leaf,
            min_child_weight=min_child_weight, reg_lambda=reg_lambda, gamma=gamma,
        )

    def partition_rows(self, dataset: BinnedDataset, rows, feature: int, threshold: int,
                       default_left: bool = True) -> tuple[list[int], list[int]]:
        """Stable left/right split of node rows (PartitionRowsForTest, backend.hpp:181-185)."""

        dev = self.dataset(dataset)
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        left = np.empty(max(r.size, 1), np.uint64)
        right = np.empty(max(r.size, 1), np.uint64)
        nl = C.c_uint64()
        check(
            _lib.load().mpsb_cuda_partition_rows(
                self.handle, dev.handle, ptr(r), r.size, feature, threshold, int(bool(default_left)),
                ptr(left), ptr(right), C.byref(nl),
            )
        )
        return left[: nl.value].tolist(), right[: r.size - nl.value].tolist()

    # -- timing ----------------------------------------------------------------------------
    def timer_begin(self) -> None:
        check(_lib.load().mpsb_cuda_timer_begin(self.handle))

    def timer_end(self) -> float:
        ms = C.c_float()
        check(_lib.load().mpsb_cuda_timer_end(self.handle, C.byref(ms)))
        return float(ms.value)

    def synchronize(self) -> None:
        check(_lib.load().mpsb_cuda_synchronize(self.handle))


# --------------------------------------------------------------------------------------
# Models and training
# --------------------------------------------------------------------------------------
_OBJECTIVE_CODES = {"squared_error": 0, "binary_logistic": 1, "quantile": 2, "poisson": 3, "tweedie": 4}


def _schema_of(dataset) -> dict:
    """The quantization schema a model file stores (QuantizationSchema)."""

    return dict(features=int(dataset.features), max_bins=int(dataset.max_bins),
                boundaries=np.ascontiguousarray(dataset.boundaries_flat, np.float32),
                boundary_offsets=np.ascontiguousarray(dataset.boundary_offsets, np.uint64),
                boundary_counts=np.ascontiguousarray(dataset.boundary_counts, np.uint32),
                bin_counts=np.ascontiguousarray(dataset.bin_counts, np.uint32),
                missing_counts=np.ascontiguousarray(dataset.missing_counts, np.uint64))


@dataclass
class RegressionModel:
    """base_score + learning_rate * sum of flat trees (RegressionModel, trainer.hpp:37-76)."""

    base_score: float
    learning_rate: float
    trees: list
    train_predictions: np.ndarray | None = None
    objective: int = 0
    objective_alpha: float = 0.5
    tweedie_variance_power: float = 1.5
    schema: dict | None = None

    @classmethod
    def _from_handle(cls, handle) -> "RegressionModel":
        lib = _lib.load()
        trees = []
        for t in range(lib.mpsb_cuda_model_tree_count(handle)):
            nodes = np.empty(lib.mpsb_cuda_model_tree_node_count(handle, t), NODE_DTYPE)
            check(lib.mpsb_cuda_model_tree_nodes(handle, t, ptr(nodes)))
            trees.append(nodes)
        model = cls(lib.mpsb_cuda_model_base_score(handle), lib.mpsb_cuda_model_learning_rate(handle), trees)
        obj, alpha, power = C.c_uint32(), C.c_double(), C.c_double()
        check(lib.mpsb_cuda_model_get_objective(handle, C.byref(obj), C.byref(alpha), C.byref(power)))
        model.objective, model.objective_alpha, model.tweedie_variance_power = obj.value, alpha.value, power.value
        feats, bins, nb = C.c_uint32(), C.c_uint32(), C.c_uint64()
        if lib.mpsb_cuda_model_get_schema(handle, C.byref(feats), C.byref(bins), C.byref(nb),
                                          None, None, None, None, None) == 0:
            f = feats.value
            sc = dict(features=f, max_bins=bins.value, boundaries=np.empty(nb.value, np.float32),
                      boundary_offsets=np.empty(f, np.uint64), boundary_counts=np.empty(f, np.uint32),
                      bin_counts=np.empty(f, np.uint32), missing_counts=np.empty(f, np.uint64))
            check(lib.mpsb_cuda_model_get_schema(handle, None, None, None, ptr(sc["boundaries"]),
                                                 ptr(sc["boundary_offsets"]), ptr(sc["boundary_counts"]),
                                                 ptr(sc["bin_counts"]), ptr(sc["missing_counts"])))
            model.schema = sc
        return model

    # -- the native model file (SerializeModel / DeserializeModel, trainer.hpp:152-160) --
    def to_bytes(self, dataset=None) -> bytes:
        """Model file bytes (format 1.4). ``dataset``: the training data whose schema the
        file stores, when the model does not carry one."""

        lib = _lib.load()
        h = self._handle(lib, dataset)
        try:
            size = C.c_uint64()
            check(lib.mpsb_cuda_model_serialize(h, None, 0, C.byref(size)))
            out = np.empty(size.value, np.uint8)
            check(lib.mpsb_cuda_model_serialize(h, ptr(out), out.size, C.byref(size)))
        finally:
            lib.mpsb_cuda_model_destroy(h)
        return out.tobytes()

    @classmethod
    def from_bytes(cls, data: bytes) -> "RegressionModel":
        lib = _lib.load()
        buf = np.frombuffer(bytes(data), np.uint8)
        h = C.c_void_p()
        check(lib.mpsb_cuda_model_deserialize(ptr(buf) if buf.size else None, buf.size, 0, C.byref(h)))
        try:
            return cls._from_handle(h)
        finally:
            lib.mpsb_cuda_model_destroy(h)

    def save(self, path: str, dataset=None) -> None:
        """Atomic save (SaveModelFile): temporary file, fsync, rename."""

        lib = _lib.load()
        h = self._handle(lib, dataset)
        try:
            check(lib.mpsb_cuda_model_save(h, os.fsencode(path)))
        finally:
            lib.mpsb_cuda_model_destroy(h)

    @classmethod
    def load(cls, path: str) -> "RegressionModel":
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.mpsb_cuda_model_load(os.fsencode(path), 0, C.byref(h)))
        try:
            return cls._from_handle(h)
        finally:
            lib.mpsb_cuda_model_destroy(h)

    def predict(self, backend: CudaBackend, dataset: BinnedDataset) -> np.ndarray:
        """Device batch prediction over a binned dataset with the training schema."""

        lib = _lib.load()
        dev = backend.dataset(dataset)
        handle = self._handle(lib)
        out = np.empty(dataset.rows, np.float64)
        try:
            check(lib.mpsb_cuda_model_predict(backend.handle, handle, dev.handle, ptr(out)))
        finally:
            lib.mpsb_cuda_model_destroy(handle)
        return out

    def _handle(self, lib, dataset=None):
        counts = np.asarray([len(t) for t in self.trees], np.uint32)
        nodes = np.concatenate(self.trees) if self.trees else np.empty(0, NODE_DTYPE)
        nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        h = C.c_void_p()
        check(lib.mpsb_cuda_model_create(self.base_score, self.learning_rate, len(self.trees),
                                         ptr(counts), ptr(nodes), C.byref(h)))
        try:
            check(lib.mpsb_cuda_model_set_objective(h, int(self.objective), float(self.objective_alpha),
                                                    float(self.tweedie_variance_power)))
            sc = _schema_of(dataset) if dataset is not None else self.schema
            if sc is not None:
                check(lib.mpsb_cuda_model_set_schema(
                    h, sc["features"], sc["max_bins"], ptr(sc["boundaries"]), sc["boundaries"].size,
                    ptr(sc["boundary_offsets"]), ptr(sc["boundary_counts"]), ptr(sc["bin_counts"]),
                    ptr(sc["missing_counts"])))
        except Exception:
            lib.mpsb_cuda_model_destroy(h)
            raise
        return h


@dataclass
class MulticlassModel:
    """Native softmax model (MulticlassModel, trainer.hpp:87-131): per-class base scores
    and trees ordered (round, class); margins[row, k] = base_k + lr * sum of class k's
    trees."""

    base_scores: np.ndarray
    learning_rate: float
    trees: list
    train_margins: np.ndarray | None = None
    schema: dict | None = None
    class_labels: np.ndarray | None = None  # None: 0..K-1

    @property
    def class_count(self) -> int:
        return int(self.base_scores.size)

    @classmethod
    def _from_handle(cls, handle) -> "MulticlassModel":
        lib = _lib.load()
        reg = RegressionModel._from_handle(handle)
        base = np.empty(lib.mpsb_cuda_model_class_count(handle), np.float64)
        check(lib.mpsb_cuda_model_class_base_scores(handle, ptr(base)))
        labels = np.empty(base.size, np.float64)
        check(lib.mpsb_cuda_model_class_labels(handle, ptr(labels)))
        return cls(base, reg.learning_rate, reg.trees, schema=reg.schema, class_labels=labels)

    def _handle(self, lib, dataset=None):
        counts = np.asarray([len(t) for t in self.trees], np.uint32)
        nodes = np.ascontiguousarray(np.concatenate(self.trees), dtype=NODE_DTYPE)
        base = np.ascontiguousarray(self.base_scores, np.float64)
        labels = None if self.class_labels is None else np.ascontiguousarray(self.class_labels, np.float64)
        h = C.c_void_p()
        check(lib.mpsb_cuda_model_create_softmax(base.size, self.learning_rate, ptr(base), ptr(labels),
                                                 len(self.trees), ptr(counts), ptr(nodes), C.byref(h)))
        try:
            sc = _schema_of(dataset) if dataset is not None else self.schema
            if sc is not None:
                check(lib.mpsb_cuda_model_set_schema(
                    h, sc["features"], sc["max_bins"], ptr(sc["boundaries"]), sc["boundaries"].size,
                    ptr(sc["boundary_offsets"]), ptr(sc["boundary_counts"]), ptr(sc["bin_counts"]),
                    ptr(sc["missing_counts"])))
        except Exception:
            lib.mpsb_cuda_model_destroy(h)
            raise
        return h

    def predict_margins(self, backend: CudaBackend, dataset) -> np.ndarray:
        """[rows, classes] margins on the device (MulticlassModel::PredictMargins)."""

        lib = _lib.load()
        dev = backend.dataset(dataset)
        h = self._handle(lib)
        out = np.empty((dataset.rows, self.class_count), np.float64)
        try:
            check(lib.mpsb_cuda_model_predict_margins(backend.handle, h, dev.handle, ptr(out)))
        finally:
            lib.mpsb_cuda_model_destroy(h)
        return out

    def predict_proba(self, backend: CudaBackend, dataset) -> np.ndarray:
        m = self.predict_margins(backend, dataset)
        e = np.exp(m - m.max(axis=1, keepdims=True))
        return e / e.sum(axis=1, keepdims=True)

    def to_bytes(self, dataset=None) -> bytes:
        lib = _lib.load()
        h = self._handle(lib, dataset)
        try:
            size = C.c_uint64()
            check(lib.mpsb_cuda_model_serialize(h, None, 0, C.byref(size)))
            out = np.empty(size.value, np.uint8)
            check(lib.mpsb_cuda_model_serialize(h, ptr(out), out.size, C.byref(size)))
        finally:
            lib.mpsb_cuda_model_destroy(h)
        return out.tobytes()

    @classmethod
    def from_bytes(cls, data: bytes) -> "MulticlassModel":
        lib = _lib.load()
        buf = np.frombuffer(bytes(data), np.uint8)
        h = C.c_void_p()
        check(lib.mpsb_cuda_model_deserialize(ptr(buf) if buf.size else None, buf.size, 1, C.byref(h)))
        try:
            return cls._from_handle(h)
        finally:
            lib.mpsb_cuda_model_destroy(h)


def train_softmax(backend: CudaBackend, dataset, labels, n_classes: int, weights=None, *,
                  hist_mode: str = "fixed", graph: bool = True, **params) -> MulticlassModel:
    """Native softmax boosting (TrainMulticlassSoftmaxModel, multiclass_trainer.cpp:104-149):
    each round fits one tree per class in class order on the device."""

    dev = backend.dataset(dataset)
    y = np.ascontiguousarray(labels, dtype=np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    params.setdefault("max_bins", dataset.max_bins)
    p, keep = make_params(**params)
    lib = _lib.load()
    h = C.c_void_p()
    check(lib.mpsb_cuda_train_softmax(backend.handle, dev.handle, ptr(y), ptr(w), y.size, C.byref(p),
                                      int(n_classes), _options(hist_mode, True, graph), C.byref(h)))
    del keep
    try:
        m = MulticlassModel._from_handle(h)
        m.train_margins = np.empty((y.size, int(n_classes)), np.float64)
        check(lib.mpsb_cuda_model_train_predictions(h, ptr(m.train_margins)))
    finally:
        lib.mpsb_cuda_model_destroy(h)
    if m.schema is None:
        m.schema = _schema_of(dataset)
    return m


def _train(backend, dataset, labels, weights, options, n_classes, **params):
    dev = backend.dataset(dataset)
    y = np.ascontiguousarray(labels, dtype=np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    params.setdefault("max_bins", dataset.max_bins)
    p, keep = make_params(**params)
    lib = _lib.load()
    if n_classes:
        handles = (C.c_void_p * n_classes)()
        check(lib.mpsb_cuda_train_ovr(backend.handle, dev.handle, ptr(y), ptr(w), y.size, n_classes,
                                      C.byref(p), options, handles))
        raw = list(handles)
    else:
        h = C.c_void_p()
        check(lib.mpsb_cuda_train_regressor(backend.handle, dev.handle, ptr(y), ptr(w), y.size,
                                            C.byref(p), options, C.byref(h)))
        raw = [h.value]
    del keep
    models = []
    for h in raw:
        m = RegressionModel._from_handle(h)
        m.train_predictions = np.empty(dataset.rows, np.float64)
        check(lib.mpsb_cuda_model_train_predictions(h, ptr(m.train_predictions)))
        lib.mpsb_cuda_model_destroy(h)
        if m.schema is None:
            m.schema = _schema_of(dataset)
        models.append(m)
    return models


def train_regressor(backend: CudaBackend, dataset: BinnedDataset, labels, weights=None, *,
                    hist_mode: str = "fixed", batched: bool = True, graph: bool = True,
                    **params) -> RegressionModel:
    """Boosted regression trees on the GPU (TrainRegressionModel, trainer.cpp:226-266)."""

    options = _options(hist_mode, batched, graph)
    return _train(backend, dataset, labels, weights, options, 0, **params)[0]


def train_ovr(backend: CudaBackend, dataset: BinnedDataset, labels, n_classes: int, weights=None, *,
              hist_mode: str = "fixed", graph: bool = True, **params) -> list[RegressionModel]:
    """K binary-logistic models, one per class, built side by side in the same launches."""

    params.setdefault("objective", "binary_logistic")
    options = _options(hist_mode, True, graph)
    return _train(backend, dataset, labels, weights, options, int(n_classes), **params)


def forest_samples(n_rows: int, n_features: int, n_trees: int, *, random_state=None,
                   bootstrap: bool = True, sample_fraction: float = 1.0,
                   max_features: float = 1.0):
    """Per-tree row multiplicities, feature subsets and seeds drawn as the reference's
    forest draws them (forest.py:120-127, forest_sampling.py:94-116, randomization.py:43-84):
    a generator seeded with random_state gives each tree a row seed and a feature seed;
    rows are ceil(n * sample_fraction) draws with replacement (bootstrap) or without, the
    features ceil(F * max_features) distinct draws; the feature seed also seeds the tree's
    random thresholds. Returns (row_counts uint8 [n_trees, n_rows], subsets, seeds)."""

    from math import ceil

    gen = np.random.default_rng(random_state)
    jobs = [(int(gen.integers(0, np.iinfo(np.int32).max)), int(gen.integers(0, np.iinfo(np.int32).max)))
            for _ in range(n_trees)]
    counts = np.zeros((n_trees, n_rows), np.uint8)
    subsets, seeds = [], []
    n_draw = max(1, int(ceil(n_rows * float(sample_fraction))))
    n_feat = max(1, int(ceil(n_features * float(max_features))))
    for t, (row_seed, feature_seed) in enumerate(jobs):
        if bootstrap:
            rows = np.random.default_rng(row_seed).integers(0, n_rows, size=n_draw, dtype=np.int64)
        else:
            rows = np.random.default_rng(row_seed).choice(n_rows, size=n_draw, replace=False)
        c = np.bincount(rows, minlength=n_rows)
        if c.max() > 255:
            raise ValueError("a row is drawn more than 255 times")
        counts[t] = c.astype(np.uint8)
        subsets.append(np.random.default_rng(feature_seed).choice(n_features, size=n_feat, replace=False))
        seeds.append(feature_seed)
    return counts, subsets, np.asarray(seeds, np.uint32)


def train_forest(backend: CudaBackend, dataset: BinnedDataset, labels, weights=None, *,
                 row_counts, feature_subsets, seeds=None, hist_mode: str = "fixed",
                 **params) -> list[RegressionModel]:
    """Independent single-round trees, one per (row multiset, feature subset), every tree's
    frontier of a batch built in the same launches (the fits of _ForestMixin.fit,
    forest.py:101-183). Returns one single-tree model per tree; a forest predicts the mean
    of their predictions."""

    dev = backend.dataset(dataset)
    y = np.ascontiguousarray(labels, dtype=np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    counts = np.ascontiguousarray(row_counts, dtype=np.uint8)
    n_trees = counts.shape[0]
    if counts.shape != (n_trees, y.size) or len(feature_subsets) != n_trees:
        raise ValueError("row_counts must be [n_trees, n_rows] with one feature subset per tree")
    offsets = np.zeros(n_trees + 1, np.uint32)
    offsets[1:] = np.cumsum([len(f) for f in feature_subsets])
    feats = np.ascontiguousarray(np.concatenate([np.asarray(f, np.uint32) for f in feature_subsets]))
    sd = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.uint32)
    params.setdefault("max_bins", dataset.max_bins)
    params.setdefault("learning_rate", 1.0)
    params["n_estimators"] = 1
    p, keep = make_params(**params)
    lib = _lib.load()
    handles = (C.c_void_p * n_trees)()
    check(lib.mpsb_cuda_train_forest(backend.handle, dev.handle, ptr(y), ptr(w), y.size, C.byref(p),
                                     n_trees, ptr(counts), ptr(offsets), ptr(feats), ptr(sd),
                                     _options(hist_mode, True, False), handles))
    del keep
    models = []
    for h in list(handles):
        m = RegressionModel._from_handle(h)
        lib.mpsb_cuda_model_destroy(h)
        if m.schema is None:
            m.schema = _schema_of(dataset)
        models.append(m)
    return models


def _options(hist_mode: str, batched: bool, graph: bool) -> int:
    opts = 0
    if hist_mode == "float":
        opts |= _lib.OPT_FLOAT_HIST
    elif hist_mode != "fixed":
        raise ValueError("hist_mode must be 'fixed' or 'float'")
    if not batched:
        opts |= _lib.OPT_PER_NODE
    if not graph:
        opts |= _lib.OPT_NO_GRAPH
    return opts


class Trainer:
    """A training session with device-resident inputs (benchmarks and timing)."""

    def __init__(self, backend: CudaBackend, dataset: BinnedDataset, labels, weights=None, *,
                 options: int = 0, **params):
        self.backend = backend
        self._dev = backend.dataset(dataset)
        y = np.ascontiguousarray(labels, dtype=np.float64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        params.setdefault("max_bins", dataset.max_bins)
        p, keep = make_params(**params)
        h = C.c_void_p()
        check(_lib.load().mpsb_cuda_trainer_create(backend.handle, self._dev.handle, ptr(y), ptr(w), y.size,
                                                   C.byref(p), options, C.byref(h)))
        del keep
        self.handle = h

    def run(self, rounds: int) -> None:
        check(_lib.load().mpsb_cuda_trainer_run(self.handle, rounds))

    def synchronize(self) -> None:
        check(_lib.load().mpsb_cuda_trainer_synchronize(self.handle))

    def stats(self) -> dict:
        s = _lib.Stats()
        check(_lib.load().mpsb_cuda_trainer_stats(self.handle, C.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def reset_stats(self) -> None:
        check(_lib.load().mpsb_cuda_trainer_reset_stats(self.handle))

    def level_stats(self, n_levels: int = 32) -> list[tuple[float, int]]:
        """Per depth level: (histogram-build ms, cells) since the last reset (timing mode)."""
        ms = np.zeros(n_levels, np.float64)
        cells = np.zeros(n_levels, np.uint64)
        check(_lib.load().mpsb_cuda_trainer_level_stats(self.handle, n_levels, ptr(ms), ptr(cells)))
        return [(float(a), int(c)) for a, c in zip(ms, cells) if c or a]

    def export(self) -> RegressionModel:
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.mpsb_cuda_trainer_export(self.handle, C.byref(h)))
        m = RegressionModel._from_handle(h)
        m.train_predictions = np.empty(self._dev.rows, np.float64)
        check(lib.mpsb_cuda_model_train_predictions(h, ptr(m.train_predictions)))
        lib.mpsb_cuda_model_destroy(h)
        return m

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().mpsb_cuda_trainer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
