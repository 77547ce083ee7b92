"""CPU oracle of the MPSBoost training hot path -- TEST INFRASTRUCTURE ONLY.

Loads one of two shared libraries with the same C API (``oracle/oracle.h``):

* ``kind="port"``: ``_build/liborc.so``, the plain-C restatement in ``oracle.c``
  (built from this directory with ``make``; it travels and builds anywhere).
* ``kind="reference"``: ``_ref/libmpsb_ref.so``, the reference's own C++ core compiled
  in place from its sources with ``make ref`` (only where those sources exist).

Only tests, ``__graft_entry__.smoke`` and the benchmark's CPU-baseline leg may import
this package; the product never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liborc.so")
REF_LIB = os.path.join(HERE, "_ref", "libmpsb_ref.so")
# The reference project's checkout: MPSB_REFERENCE_ROOT, else a directory named
# ``reference`` beside this repository.
REFERENCE_ROOT = os.environ.get(
    "MPSB_REFERENCE_ROOT", os.path.normpath(os.path.join(HERE, "..", "..", "reference")))

SQUARED_ERROR, BINARY_LOGISTIC, QUANTILE, POISSON, TWEEDIE = range(5)
HIST_FP64, HIST_FIXED = 0, 1
OBJECTIVES = {
    "squared_error": SQUARED_ERROR,
    "binary_logistic": BINARY_LOGISTIC,
    "quantile": QUANTILE,
    "poisson": POISSON,
    "tweedie": TWEEDIE,
}

NODE_DTYPE = np.dtype(
    [
        ("feature_index", "<u4"),
        ("threshold_bin", "<u4"),
        ("left_child", "<u4"),
        ("right_child", "<u4"),
        ("leaf_value", "<f8"),
        ("gain", "<f8"),
        ("default_left", "u1"),
        ("flags", "u1"),
        ("reserved", "u1", (6,)),
    ]
)
HIST_DTYPE = np.dtype([("count", "<u8"), ("gradient_sum", "<f8"), ("hessian_sum", "<f8")])
FIXED_DTYPE = np.dtype([("count", "<u8"), ("gradient_q", "<i8"), ("hessian_q", "<i8")])
SPLIT_DTYPE = np.dtype(
    [
        ("valid", "<u4"),
        ("feature", "<u4"),
        ("threshold_bin", "<u4"),
        ("default_left", "<u4"),
        ("left_count", "<u8"),
        ("right_count", "<u8"),
        ("left_gradient_sum", "<f8"),
        ("left_hessian_sum", "<f8"),
        ("right_gradient_sum", "<f8"),
        ("right_hessian_sum", "<f8"),
        ("gain", "<f8"),
    ]
)


class Params(C.Structure):
    """``orc_params`` (oracle.h); field meaning follows trainer.hpp:20-36 / tree.hpp:47-72."""

    _fields_ = [
        ("n_estimators", C.c_uint32),
        ("max_bins", C.c_uint32),
        ("objective", C.c_uint32),
        ("max_depth", C.c_uint32),
        ("max_leaves", C.c_uint32),
        ("max_active_leaves", C.c_uint32),
        ("split_strategy", C.c_uint32),
        ("growth_strategy", C.c_uint32),
        ("random_seed", C.c_uint32),
        ("n_monotonic", C.c_uint32),
        ("n_interaction_groups", C.c_uint32),
        ("reserved", C.c_uint32),
        ("min_samples_leaf", C.c_uint64),
        ("learning_rate", C.c_double),
        ("objective_alpha", C.c_double),
        ("tweedie_variance_power", C.c_double),
        ("min_child_weight", C.c_double),
        ("reg_lambda", C.c_double),
        ("reg_alpha", C.c_double),
        ("max_delta_step", C.c_double),
        ("gamma", C.c_double),
        ("min_gain_to_split", C.c_double),
        ("monotonic_constraints", C.POINTER(C.c_int8)),
        ("interaction_offsets", C.POINTER(C.c_uint32)),
        ("interaction_features", C.POINTER(C.c_uint32)),
    ]


# C++ defaults of TrainingParameters / TreeTrainingParameters (trainer.hpp:29-35,
# tree.hpp:57-71).
DEFAULTS = dict(
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


def make_params(**overrides):
    """Return ``(Params, keepalive)`` from keyword overrides of ``DEFAULTS``."""

    unknown = set(overrides) - set(DEFAULTS)
    if unknown:
        raise ValueError(f"unknown parameter(s): {sorted(unknown)}")
    v = dict(DEFAULTS, **overrides)
    p = Params()
    for name in (
        "n_estimators", "max_bins", "max_depth", "max_leaves", "max_active_leaves",
        "random_seed", "min_samples_leaf", "learning_rate", "objective_alpha",
        "tweedie_variance_power", "min_child_weight", "reg_lambda", "reg_alpha",
        "max_delta_step", "gamma", "min_gain_to_split",
    ):
        setattr(p, name, v[name])
    p.objective = OBJECTIVES[v["objective"]] if isinstance(v["objective"], str) else v["objective"]
    p.split_strategy = {"best_gain": 0, "random_threshold": 1}[v["split_strategy"]]
    p.growth_strategy = {"level_wise": 0, "leaf_wise": 1}[v["growth_strategy"]]
    keep = []
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


class OracleError(RuntimeError):
    """Raised with the oracle's message; ``code`` is the oracle.h error code."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def build(reference: bool | None = None, quiet: bool = True) -> None:
    """Build the port (always) and the reference library (when its sources exist)."""

    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=out)
    if reference is None:
        reference = os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "core"))
    if reference:
        subprocess.run(["make", "-C", HERE, "ref", f"REF={REFERENCE_ROOT}"], check=True, stdout=out)


def reference_available() -> bool:
    return os.path.exists(REF_LIB)


@dataclass
class Dataset:
    oracle: "Oracle"
    handle: int
    rows: int
    features: int
    max_bins: int
    bin_counts: np.ndarray
    missing_counts: np.ndarray
    boundary_offsets: np.ndarray
    boundary_counts: np.ndarray
    boundaries_flat: np.ndarray
    _bins: np.ndarray | None = field(default=None, repr=False)
    _missing: np.ndarray | None = field(default=None, repr=False)

    @property
    def boundaries(self):
        return [
            self.boundaries_flat[o : o + c].tolist()
            for o, c in zip(self.boundary_offsets, self.boundary_counts)
        ]

    @property
    def bins(self) -> np.ndarray:
        """Feature-major ``[features, rows]`` bins (missing rows hold bin 0)."""
        if self._bins is None:
            out = np.empty((self.features, self.rows), dtype=np.uint16)
            self.oracle._check(self.oracle._fn("dataset_bins")(C.c_void_p(self.handle), _ptr(out)))
            self._bins = out
        return self._bins

    @property
    def missing(self) -> np.ndarray:
        if self._missing is None:
            out = np.empty((self.features, self.rows), dtype=np.uint8)
            self.oracle._check(self.oracle._fn("dataset_missing")(C.c_void_p(self.handle), _ptr(out)))
            self._missing = out.astype(bool)
        return self._missing

    def __del__(self):
        try:
            self.oracle._fn("dataset_free")(C.c_void_p(self.handle))
        except Exception:
            pass


@dataclass
class Model:
    base_score: float
    trees: list
    handle: int
    oracle: "Oracle"

    def predict(self, dataset: Dataset) -> np.ndarray:
        out = np.empty(dataset.rows, dtype=np.float64)
        self.oracle._check(
            self.oracle._fn("model_predict")(C.c_void_p(self.handle), C.c_void_p(dataset.handle), _ptr(out))
        )
        return out

    def __del__(self):
        try:
            self.oracle._fn("model_free")(C.c_void_p(self.handle))
        except Exception:
            pass


@dataclass
class SoftmaxModel:
    base_scores: np.ndarray
    trees: list
    handle: int
    oracle: "Oracle"

    def predict_margins(self, dataset: Dataset) -> np.ndarray:
        out = np.empty((dataset.rows, self.base_scores.size), dtype=np.float64)
        self.oracle._check(self.oracle._fn("softmax_predict_margins")(C.c_void_p(self.handle),
                                                                      C.c_void_p(dataset.handle), _ptr(out)))
        return out

    def __del__(self):
        try:
            self.oracle._fn("softmax_free")(C.c_void_p(self.handle))
        except Exception:
            pass


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """ctypes front end over ``orc_*`` (port) or ``ref_*`` (compiled reference)."""

    def __init__(self, kind: str = "port"):
        if kind == "port":
            path, self.prefix = PORT_LIB, "orc_"
            if not os.path.exists(path):
                build(reference=False)
        elif kind == "reference":
            path, self.prefix = REF_LIB, "ref_"
            if not os.path.exists(path):
                raise FileNotFoundError(f"reference oracle not built: {path}")
        else:
            raise ValueError(kind)
        self.kind = kind
        self.lib = C.CDLL(path)
        getattr(self.lib, self.prefix + "last_error").restype = C.c_char_p
        for name in ("tree_node_count", "model_tree_count", "model_tree_node_count", "softmax_tree_count",
                     "softmax_class_count", "softmax_tree_node_count"):
            self._fn(name).restype = C.c_uint32
        self._fn("model_base_score").restype = C.c_double

    def _fn(self, name: str):
        return getattr(self.lib, self.prefix + name)

    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = getattr(self.lib, self.prefix + "last_error")().decode()
            raise OracleError(rc, msg)

    # -- datasets -------------------------------------------------------------------
    def _wrap_dataset(self, handle: int) -> Dataset:
        rows, feats, max_bins, nb = C.c_uint64(), C.c_uint32(), C.c_uint32(), C.c_uint64()
        h = C.c_void_p(handle)
        self._check(self._fn("dataset_info")(h, C.byref(rows), C.byref(feats), C.byref(max_bins), C.byref(nb)))
        f = feats.value
        off = np.empty(f, np.uint64)
        cnt = np.empty(f, np.uint32)
        bins = np.empty(f, np.uint32)
        miss = np.empty(f, np.uint64)
        self._check(self._fn("dataset_metadata")(h, _ptr(off), _ptr(cnt), _ptr(bins), _ptr(miss)))
        bnd = np.empty(max(nb.value, 1), np.float32)
        self._check(self._fn("dataset_boundaries")(h, _ptr(bnd)))
        return Dataset(self, handle, rows.value, f, max_bins.value, bins, miss, off, cnt, bnd[: nb.value])

    def quantize_dense(self, matrix, max_bins: int) -> Dataset:
        x = np.asarray(matrix)
        if x.dtype not in (np.float32, np.float64):
            x = x.astype(np.float32)
        if x.ndim != 2:
            raise ValueError("matrix must be 2-D")
        st = 1 if x.dtype == np.float32 else 2
        out = C.c_void_p()
        self._check(
            self._fn("quantize_dense")(
                _ptr(x), C.c_int(st), C.c_uint64(x.shape[0]), C.c_uint32(x.shape[1]),
                C.c_uint64(x.strides[0]), C.c_uint64(x.strides[1]), C.c_uint32(max_bins), C.byref(out),
            )
        )
        return self._wrap_dataset(out.value)

    def transform_dense(self, schema: Dataset, matrix) -> Dataset:
        x = np.asarray(matrix)
        if x.dtype not in (np.float32, np.float64):
            x = x.astype(np.float32)
        st = 1 if x.dtype == np.float32 else 2
        out = C.c_void_p()
        self._check(
            self._fn("transform_dense")(
                C.c_void_p(schema.handle), _ptr(x), C.c_int(st), C.c_uint64(x.shape[0]),
                C.c_uint32(x.shape[1]), C.c_uint64(x.strides[0]), C.c_uint64(x.strides[1]), C.byref(out),
            )
        )
        return self._wrap_dataset(out.value)

    def dataset_subset(self, dataset: Dataset, rows, features) -> Dataset:
        """matrix[rows][:, features] with the source's bins (a forest tree's sample)."""

        self._port_only()
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        f = np.ascontiguousarray(features, dtype=np.uint32)
        out = C.c_void_p()
        self._check(self.lib.orc_dataset_subset(C.c_void_p(dataset.handle), _ptr(r), C.c_uint64(r.size),
                                                _ptr(f), C.c_uint32(f.size), C.byref(out)))
        return self._wrap_dataset(out.value)

    def dataset_from_bins(self, binned) -> Dataset:
        """The oracle's dataset over bins computed elsewhere (fields of a binned dataset:
        feature-major ``bins``, ``missing``, ``max_bins``, the packed schema)."""

        self._port_only()
        b = np.ascontiguousarray(binned.bins)
        m = np.ascontiguousarray(binned.missing, dtype=np.uint8)
        bnd = np.ascontiguousarray(binned.boundaries_flat, dtype=np.float32)
        off = np.ascontiguousarray(binned.boundary_offsets, dtype=np.uint64)
        cnt = np.ascontiguousarray(binned.boundary_counts, dtype=np.uint32)
        nb = np.ascontiguousarray(binned.bin_counts, dtype=np.uint32)
        out = C.c_void_p()
        self._check(self.lib.orc_dataset_from_bins(
            _ptr(b), C.c_uint32(b.itemsize), _ptr(m), C.c_uint64(b.shape[1]), C.c_uint32(b.shape[0]),
            C.c_uint32(binned.max_bins), _ptr(bnd), _ptr(off), _ptr(cnt), _ptr(nb), C.byref(out)))
        return self._wrap_dataset(out.value)

    # -- objectives / histograms -------------------------------------------------------
    def gradients(self, objective, labels, predictions, alpha=0.5, variance_power=1.5) -> np.ndarray:
        y = np.ascontiguousarray(labels, dtype=np.float64)
        p = np.ascontiguousarray(predictions, dtype=np.float64)
        out = np.empty((y.size, 2), np.float64)
        obj = OBJECTIVES[objective] if isinstance(objective, str) else objective
        self._check(
            self._fn("gradients")(
                C.c_uint32(obj), C.c_double(alpha), C.c_double(variance_power), _ptr(y), _ptr(p),
                C.c_uint64(y.size), _ptr(out),
            )
        )
        return out

    def histograms(self, dataset: Dataset, pairs, rows) -> list[np.ndarray]:
        g = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 2)
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        out = np.empty(int(dataset.bin_counts.sum()), HIST_DTYPE)
        self._check(
            self._fn("histograms")(
                C.c_void_p(dataset.handle), _ptr(g), C.c_uint64(g.shape[0]), _ptr(r), C.c_uint64(r.size), _ptr(out)
            )
        )
        return np.split(out, np.cumsum(dataset.bin_counts)[:-1])

    # -- trees / models ----------------------------------------------------------------
    def _tree_nodes(self, handle) -> np.ndarray:
        n = self._fn("tree_node_count")(C.c_void_p(handle))
        out = np.empty(n, NODE_DTYPE)
        self._check(self._fn("tree_nodes")(C.c_void_p(handle), _ptr(out)))
        return out

    def train_single_tree(self, dataset: Dataset, pairs, **params):
        g = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 2)
        p, keep = make_params(**params)
        out = C.c_void_p()
        self._check(
            self._fn("train_single_tree")(
                C.c_void_p(dataset.handle), _ptr(g), C.c_uint64(g.shape[0]), C.byref(p), C.byref(out)
            )
        )
        del keep
        nodes = self._tree_nodes(out.value)
        pred = np.empty(dataset.rows, np.float64)
        self._check(self._fn("tree_predict")(out, C.c_void_p(dataset.handle), _ptr(pred)))
        self._fn("tree_free")(out)
        return nodes, pred

    def train_regressor(self, dataset: Dataset, labels, weights=None, hist_mode: int | None = None, **params) -> Model:
        y = np.ascontiguousarray(labels, dtype=np.float64)
        w = np.ones_like(y) if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        params.setdefault("max_bins", dataset.max_bins)
        p, keep = make_params(**params)
        out = C.c_void_p()
        if hist_mode is None or hist_mode == HIST_FP64 and self.kind == "reference":
            rc = self._fn("train_regressor")(
                C.c_void_p(dataset.handle), _ptr(y), _ptr(w), C.c_uint64(y.size), C.byref(p), C.byref(out)
            )
        else:
            if self.kind != "port":
                raise ValueError("hist_mode is only available in the port")
            rc = self.lib.orc_train_regressor_mode(
                C.c_void_p(dataset.handle), _ptr(y), _ptr(w), C.c_uint64(y.size), C.byref(p),
                C.c_int(hist_mode), C.byref(out),
            )
        self._check(rc)
        del keep
        count = self._fn("model_tree_count")(out)
        trees = []
        for t in range(count):
            n = self._fn("model_tree_node_count")(out, C.c_uint32(t))
            nodes = np.empty(n, NODE_DTYPE)
            self._check(self._fn("model_tree_nodes")(out, C.c_uint32(t), _ptr(nodes)))
            trees.append(nodes)
        return Model(self._fn("model_base_score")(out), trees, out.value, self)

    def train_softmax(self, dataset: Dataset, labels, n_classes: int, weights=None,
                      hist_mode: int | None = None, **params) -> "SoftmaxModel":
        """TrainMulticlassSoftmaxModel (multiclass_trainer.cpp:104-149)."""

        y = np.ascontiguousarray(labels, dtype=np.float64)
        w = np.ones_like(y) if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        params.setdefault("max_bins", dataset.max_bins)
        p, keep = make_params(**params)
        out = C.c_void_p()
        if hist_mode is None or hist_mode == HIST_FP64 and self.kind == "reference":
            rc = self._fn("train_softmax")(C.c_void_p(dataset.handle), _ptr(y), _ptr(w), C.c_uint64(y.size),
                                           C.byref(p), C.c_uint32(n_classes), C.byref(out))
        else:
            self._port_only()
            rc = self.lib.orc_train_softmax_mode(C.c_void_p(dataset.handle), _ptr(y), _ptr(w), C.c_uint64(y.size),
                                                 C.byref(p), C.c_uint32(n_classes), C.c_int(hist_mode),
                                                 C.byref(out))
        self._check(rc)
        del keep
        k = self._fn("softmax_class_count")(out)
        base = np.empty(k, np.float64)
        self._check(self._fn("softmax_base_scores")(out, _ptr(base)))
        trees = []
        for t in range(self._fn("softmax_tree_count")(out)):
            nodes = np.empty(self._fn("softmax_tree_node_count")(out, C.c_uint32(t)), NODE_DTYPE)
            self._check(self._fn("softmax_tree_nodes")(out, C.c_uint32(t), _ptr(nodes)))
            trees.append(nodes)
        return SoftmaxModel(base, trees, out.value, self)

    # -- the reference's model file codec (reference only) --------------------------------
    def model_to_bytes(self, model: Model) -> bytes:
        """SerializeModel of a model trained by the compiled reference."""

        if self.kind != "reference":
            raise ValueError("only available with the compiled reference")
        size = C.c_uint64()
        self._check(self.lib.ref_model_serialize(C.c_void_p(model.handle), None, C.c_uint64(0), C.byref(size)))
        out = np.empty(size.value, np.uint8)
        self._check(self.lib.ref_model_serialize(C.c_void_p(model.handle), _ptr(out), C.c_uint64(out.size),
                                                 C.byref(size)))
        return out.tobytes()

    def softmax_to_bytes(self, model: "SoftmaxModel") -> bytes:
        """SerializeModel of a softmax model trained by the compiled reference."""

        if self.kind != "reference":
            raise ValueError("only available with the compiled reference")
        size = C.c_uint64()
        self._check(self.lib.ref_softmax_serialize(C.c_void_p(model.handle), None, C.c_uint64(0), C.byref(size)))
        out = np.empty(size.value, np.uint8)
        self._check(self.lib.ref_softmax_serialize(C.c_void_p(model.handle), _ptr(out), C.c_uint64(out.size),
                                                   C.byref(size)))
        return out.tobytes()

    def softmax_from_bytes(self, data: bytes) -> "SoftmaxModel":
        """DeserializeMulticlassModel of the reference."""

        if self.kind != "reference":
            raise ValueError("only available with the compiled reference")
        buf = np.frombuffer(bytes(data), np.uint8).copy()
        out = C.c_void_p()
        self._check(self.lib.ref_softmax_deserialize(_ptr(buf), C.c_uint64(buf.size), C.byref(out)))
        k = self._fn("softmax_class_count")(out)
        base = np.empty(k, np.float64)
        self._check(self._fn("softmax_base_scores")(out, _ptr(base)))
        trees = []
        for t in range(self._fn("softmax_tree_count")(out)):
            nodes = np.empty(self._fn("softmax_tree_node_count")(out, C.c_uint32(t)), NODE_DTYPE)
            self._check(self._fn("softmax_tree_nodes")(out, C.c_uint32(t), _ptr(nodes)))
            trees.append(nodes)
        return SoftmaxModel(base, trees, out.value, self)

    def model_from_bytes(self, data: bytes) -> Model:
        """DeserializeModel of the reference."""

        if self.kind != "reference":
            raise ValueError("only available with the compiled reference")
        buf = np.frombuffer(bytes(data), np.uint8).copy()
        out = C.c_void_p()
        self._check(self.lib.ref_model_deserialize(_ptr(buf), C.c_uint64(buf.size), C.byref(out)))
        count = self._fn("model_tree_count")(out)
        trees = []
        for t in range(count):
            nodes = np.empty(self._fn("model_tree_node_count")(out, C.c_uint32(t)), NODE_DTYPE)
            self._check(self._fn("model_tree_nodes")(out, C.c_uint32(t), _ptr(nodes)))
            trees.append(nodes)
        return Model(self._fn("model_base_score")(out), trees, out.value, self)

    # -- port-only hooks ---------------------------------------------------------------
    def _port_only(self):
        if self.kind != "port":
            raise ValueError("only available in the port")

    def set_threads(self, threads: int) -> None:
        """Threads of the port's feature-parallel loops (0 = all cores; 1 = the
        reference's single-threaded timing). Results do not depend on it."""
        self._port_only()
        self.lib.orc_set_threads(C.c_int(threads))

    def fixed_scales(self, pairs32) -> tuple[int, int]:
        self._port_only()
        g = np.ascontiguousarray(pairs32, dtype=np.float32).reshape(-1, 2)
        kg, kh = C.c_int32(), C.c_int32()
        self._check(self.lib.orc_fixed_scales(_ptr(g), C.c_uint64(g.shape[0]), C.byref(kg), C.byref(kh)))
        return kg.value, kh.value

    def fixed_histograms(self, dataset: Dataset, pairs32, kg: int, kh: int, rows):
        """Return ``(per-feature bins, missing bins)`` of exact int64 sums."""
        self._port_only()
        g = np.ascontiguousarray(pairs32, dtype=np.float32).reshape(-1, 2)
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        bins = np.empty(int(dataset.bin_counts.sum()), FIXED_DTYPE)
        miss = np.empty(dataset.features, FIXED_DTYPE)
        self._check(
            self.lib.orc_fixed_histograms(
                C.c_void_p(dataset.handle), _ptr(g), C.c_int32(kg), C.c_int32(kh), _ptr(r),
                C.c_uint64(r.size), _ptr(bins), _ptr(miss),
            )
        )
        return np.split(bins, np.cumsum(dataset.bin_counts)[:-1]), miss

    def train_single_tree_fixed(self, dataset: Dataset, pairs32, kg: int, kh: int, **params):
        self._port_only()
        g = np.ascontiguousarray(pairs32, dtype=np.float32).reshape(-1, 2)
        p, keep = make_params(**params)
        out = C.c_void_p()
        self._check(
            self.lib.orc_train_single_tree_fixed(
                C.c_void_p(dataset.handle), _ptr(g), C.c_uint64(g.shape[0]), C.c_int32(kg), C.c_int32(kh),
                C.byref(p), C.byref(out),
            )
        )
        del keep
        nodes = self._tree_nodes(out.value)
        pred = np.empty(dataset.rows, np.float64)
        self._check(self._fn("tree_predict")(out, C.c_void_p(dataset.handle), _ptr(pred)))
        self._fn("tree_free")(out)
        return nodes, pred

    def weighted_pairs32(self, objective, labels, predictions, weights, alpha=0.5, variance_power=1.5):
        self._port_only()
        y = np.ascontiguousarray(labels, dtype=np.float64)
        p = np.ascontiguousarray(predictions, dtype=np.float64)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        out = np.empty((y.size, 2), np.float32)
        obj = OBJECTIVES[objective] if isinstance(objective, str) else objective
        self._check(
            self.lib.orc_weighted_pairs32(
                C.c_uint32(obj), C.c_double(alpha), C.c_double(variance_power), _ptr(y), _ptr(p), _ptr(w),
                C.c_uint64(y.size), _ptr(out),
            )
        )
        return out

    def scan_splits(self, dataset: Dataset, pairs, rows, **params) -> np.ndarray:
        self._port_only()
        g = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 2)
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        p, keep = make_params(**params)
        out = np.empty(dataset.features, SPLIT_DTYPE)
        self._check(
            self.lib.orc_scan_splits(
                C.c_void_p(dataset.handle), _ptr(g), C.c_uint64(g.shape[0]), _ptr(r), C.c_uint64(r.size),
                C.byref(p), _ptr(out),
            )
        )
        del keep
        return out

    def partition_rows(self, dataset: Dataset, rows, feature: int, threshold_bin: int, default_left: bool = True):
        self._port_only()
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        left = np.empty(max(r.size, 1), np.uint64)
        right = np.empty(max(r.size, 1), np.uint64)
        nl = C.c_uint64()
        self._check(
            self.lib.orc_partition_rows(
                C.c_void_p(dataset.handle), _ptr(r), C.c_uint64(r.size), C.c_uint32(feature),
                C.c_uint32(threshold_bin), C.c_int(int(default_left)), _ptr(left), _ptr(right), C.byref(nl),
            )
        )
        return left[: nl.value].copy(), right[: r.size - nl.value].copy()
