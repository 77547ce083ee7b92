"""Sklearn-style estimators that train on the CUDA backend (``device="cuda"``).

The reference's estimators pick a backend per fit and call one native entry per model
(``src/mpsboost/estimators/base.py:167-212`` calls ``_native._train_regressor_mps``, which
is ``src/python/binding_model.cpp:34-45``: QuantizeDense then TrainRegressionModel on a
fresh backend). This module is that route for CUDA:

* :func:`_train_regressor_cuda` has the binding's arguments (matrix, labels, sample
  weights, :class:`TrainingParameters`) and returns a model with ``tree_count`` and
  ``predict(matrix)``; the matrix is quantile-binned on the GPU (the same bins as the
  host's QuantizeDense) and training runs on the device-resident trainer.
* :class:`MPSBoostRegressor`, :class:`MPSBoostClassifier` (binary logistic; one-vs-rest
  with all K trees of a round in the same launches, or native softmax, for more classes)
  and :class:`RandomForestRegressor` keep the reference's constructor parameters, their
  defaults (except ``device``), validation messages, fitted attributes and prediction
  semantics. ``device`` is ``"cuda"`` or ``"auto"``; either fails with ``BackendError``
  when no usable GPU is present, since this package has no CPU trainer.

Not provided: categorical features (outside the training hot path) and model
persistence beyond the native model bytes (``model_.to_bytes()``).
"""

from __future__ import annotations

import math
import threading
from time import perf_counter
from typing import Any

import numpy as np

from . import backend as _be
from ._lib import BackendError, UnsupportedError
from .device_policy import choose_device, cuda_device_count, decision_to_dict

_local = threading.local()


def _backend(device: int = 0) -> _be.CudaBackend:
    """One backend per host thread and device (the reference's one-backend-per-thread rule)."""

    cache = getattr(_local, "backends", None)
    if cache is None:
        cache = _local.backends = {}
    b = cache.get(device)
    if b is None:
        b = cache[device] = _be.CudaBackend(device)
    return b


class TrainingParameters:
    """The named training-parameter object of ``_native._TrainingParameters``
    (``src/python/binding_dataset.cpp:133-155``): same argument order, names and defaults."""

    def __init__(self, n_estimators, learning_rate, max_bins, max_depth, min_samples_leaf,
                 min_child_weight, reg_lambda, reg_alpha=0.0, max_delta_step=0.0, gamma=0.0,
                 min_gain_to_split=0.0, objective="squared_error", split_strategy="best_gain",
                 growth_strategy="level_wise", max_leaves=0, max_active_leaves=0, random_seed=0,
                 monotonic_constraints=(), interaction_constraints=(), objective_alpha=0.5,
                 tweedie_variance_power=1.5):
        self.n_estimators = n_estimators
        self.learning_rate = learning_rate
        self.max_bins = max_bins
        self.max_depth = max_depth
        self.min_samples_leaf = min_samples_leaf
        self.min_child_weight = min_child_weight
        self.reg_lambda = reg_lambda
        self.reg_alpha = reg_alpha
        self.max_delta_step = max_delta_step
        self.gamma = gamma
        self.min_gain_to_split = min_gain_to_split
        self.objective = objective
        self.split_strategy = split_strategy
        self.growth_strategy = growth_strategy
        self.max_leaves = max_leaves
        self.max_active_leaves = max_active_leaves
        self.random_seed = random_seed
        self.monotonic_constraints = list(monotonic_constraints)
        self.interaction_constraints = [list(g) for g in interaction_constraints]
        self.objective_alpha = objective_alpha
        self.tweedie_variance_power = tweedie_variance_power

    def as_kwargs(self) -> dict:
        """Keyword arguments of :func:`mpsboost_gb300.backend.make_params`."""

        kw = {name: getattr(self, name) for name in (
            "n_estimators", "learning_rate", "max_bins", "max_depth", "min_samples_leaf",
            "min_child_weight", "reg_lambda", "reg_alpha", "max_delta_step", "gamma",
            "min_gain_to_split", "objective", "split_strategy", "growth_strategy", "max_leaves",
            "max_active_leaves", "random_seed", "objective_alpha", "tweedie_variance_power")}
        kw["monotonic_constraints"] = self.monotonic_constraints or None
        kw["interaction_constraints"] = self.interaction_constraints or None
        return kw


def _as_matrix(X) -> np.ndarray:
    """Dense 2-D float32/float64 input (as_dense_matrix, src/mpsboost/matrix.py)."""

    x = np.asarray(X)
    if x.ndim != 2:
        raise ValueError("X must be a two-dimensional array")
    if x.shape[0] == 0 or x.shape[1] == 0:
        raise ValueError("X must contain at least one row and one feature")
    if x.dtype not in (np.float32, np.float64):
        x = x.astype(np.float32)
    return x


def _as_labels(y, n: int) -> np.ndarray:
    labels = np.asarray(y, dtype=np.float64).reshape(-1)
    if labels.shape[0] != n:
        raise ValueError("label count must match the number of rows")
    if not np.all(np.isfinite(labels)):
        raise ValueError("labels must be finite")
    return labels


def _as_weights(w, n: int) -> np.ndarray | None:
    if w is None:
        return None
    weights = np.asarray(w, dtype=np.float64).reshape(-1)
    if weights.shape[0] != n:
        raise ValueError("sample_weight length must match the number of rows")
    if not np.all(np.isfinite(weights)) or np.any(weights < 0.0):
        raise ValueError("sample_weight must be finite and non-negative")
    if not np.any(weights > 0.0):
        raise ValueError("sample_weight must contain a positive value")
    return weights


def _host_schema(schema: dict) -> _be.BinnedDataset:
    """A zero-row binned dataset carrying a trained model's quantization schema."""

    f = int(schema["features"])
    return _be.BinnedDataset(0, f, int(schema["max_bins"]), np.empty((f, 0), np.uint8),
                             np.empty((f, 0), bool), schema["boundaries"], schema["boundary_offsets"],
                             schema["boundary_counts"], schema["bin_counts"], schema["missing_counts"])


class CudaRegressionModel:
    """A trained native model (the binding's RegressionModel): ``tree_count``, raw-margin
    ``predict(matrix)`` in float32 (RegressionModel::Predict, trainer.cpp:268-282), and the
    native model-file bytes."""

    def __init__(self, model: _be.RegressionModel, device: int = 0):
        self.model = model
        self.device = device

    @property
    def tree_count(self) -> int:
        return len(self.model.trees)

    def predict(self, matrix) -> np.ndarray:
        x = _as_matrix(matrix)
        binned = _host_schema(self.model.schema).transform(x)
        return self.model.predict(_backend(self.device), binned).astype(np.float32)

    def to_bytes(self) -> bytes:
        return self.model.to_bytes()


def _train_regressor_cuda(matrix, labels, sample_weights, parameters: TrainingParameters,
                          device: int = 0) -> CudaRegressionModel:
    """``_train_regressor_mps`` (binding_model.cpp:34-45) on the CUDA backend: bin the
    matrix with ``parameters.max_bins`` and train ``parameters.n_estimators`` trees."""

    x = _as_matrix(matrix)
    y = _as_labels(labels, x.shape[0])
    w = _as_weights(sample_weights, x.shape[0])
    b = _backend(device)
    dset = _be.quantize_device(b, x, int(parameters.max_bins))
    try:
        model = _be.train_regressor(b, dset, y, w, **parameters.as_kwargs())
    finally:
        dset.close()
    return CudaRegressionModel(model, device)


def _select_cuda(requested: str, n_samples: int, n_features: int, n_estimators: int,
                 max_bins: int) -> dict:
    """The device decision of one fit; a GPU is required (there is no CPU trainer here)."""

    count = cuda_device_count()
    decision = choose_device(requested="cuda" if requested == "cuda" else "auto", n_samples=n_samples,
                             n_features=n_features, n_estimators=n_estimators, max_bins=max_bins,
                             cuda_available=count > 0, cuda_work_threshold=1)
    if count == 0:
        raise BackendError("no GPU of compute capability 10.3 (GB300) is available to the CUDA backend")
    if decision.selected != "cuda":
        raise BackendError(f"device decision selected {decision.selected!r}; this package trains on CUDA only")
    return decision_to_dict(decision)


class MPSBoostRegressor:
    """Squared-error (or quantile / Poisson / Tweedie) histogram GBDT regressor on the GPU.

    The constructor only stores parameters (``base.py:24-112``); ``fit`` replaces fitted
    state only after a complete success."""

    _estimator_type = "regressor"
    _native_objective = "squared_error"
    _split_strategy = "best_gain"
    _fitted_error_message = "MPSBoostRegressor is not fitted or loaded"
    _PARAMETER_NAMES = (
        "n_estimators", "learning_rate", "max_depth", "max_bins", "growth_strategy", "max_leaves",
        "max_active_leaves", "min_gain_to_split", "loss", "quantile_alpha", "tweedie_variance_power",
        "min_child_weight", "min_samples_leaf", "reg_lambda", "reg_alpha", "max_delta_step",
        "monotonic_constraints", "interaction_constraints", "categorical_features", "random_state",
        "n_jobs", "device", "verbosity",
    )

    def __init__(self, n_estimators: int = 100, learning_rate: float = 0.1, max_depth: int = 6,
                 max_bins: int = 256, growth_strategy: str = "level_wise", max_leaves: int | None = None,
                 max_active_leaves: int | None = None, min_gain_to_split: float = 0.0,
                 loss: str = "squared_error", quantile_alpha: float = 0.5,
                 tweedie_variance_power: float = 1.5, min_child_weight: float = 1.0,
                 min_samples_leaf: int = 20, reg_lambda: float = 1.0, reg_alpha: float = 0.0,
                 max_delta_step: float = 0.0, monotonic_constraints: Any = None,
                 interaction_constraints: Any = None, categorical_features: Any = None,
                 random_state: int | None = None, n_jobs: int | None = None, device: str = "cuda",
                 verbosity: int = 1) -> None:
        self.n_estimators = n_estimators
        self.learning_rate = learning_rate
        self.max_depth = max_depth
        self.max_bins = max_bins
        self.growth_strategy = growth_strategy
        self.max_leaves = max_leaves
        self.max_active_leaves = max_active_leaves
        self.min_gain_to_split = min_gain_to_split
        self.loss = loss
        self.quantile_alpha = quantile_alpha
        self.tweedie_variance_power = tweedie_variance_power
        self.min_child_weight = min_child_weight
        self.min_samples_leaf = min_samples_leaf
        self.reg_lambda = reg_lambda
        self.reg_alpha = reg_alpha
        self.max_delta_step = max_delta_step
        self.monotonic_constraints = monotonic_constraints
        self.interaction_constraints = interaction_constraints
        self.categorical_features = categorical_features
        self.random_state = random_state
        self.n_jobs = n_jobs
        self.device = device
        self.verbosity = verbosity
        self._fit_lock = threading.Lock()

    # -- sklearn protocol -------------------------------------------------------------
    def get_params(self, deep: bool = True) -> dict[str, Any]:
        del deep
        return {name: getattr(self, name) for name in self._PARAMETER_NAMES}

    def set_params(self, **parameters: Any):
        unknown = sorted(set(parameters) - set(self._PARAMETER_NAMES))
        if unknown:
            raise ValueError(f"Unknown parameter(s): {', '.join(unknown)}")
        for name, value in parameters.items():
            setattr(self, name, value)
        if parameters:
            self._clear_fitted_state()
        return self

    # -- validation (model_state.py:148-275) ------------------------------------------
    def _validate_parameters(self) -> None:
        integer_ranges = {
            "n_estimators": (self.n_estimators, 1, 2**32 - 1),
            "max_depth": (self.max_depth, 0, 31),
            "max_bins": (self.max_bins, 2, 65536),
            "min_samples_leaf": (self.min_samples_leaf, 1, 2**63 - 1),
            "verbosity": (self.verbosity, 0, 3),
        }
        for optional_name in ("max_leaves", "max_active_leaves"):
            value = getattr(self, optional_name)
            if value is not None:
                integer_ranges[optional_name] = (value, 2, 2**32 - 1)
        if self.n_jobs is not None:
            integer_ranges["n_jobs"] = (self.n_jobs, -1, 2**31 - 1)
        for name, (value, minimum, maximum) in integer_ranges.items():
            if isinstance(value, bool) or not isinstance(value, int):
                raise TypeError(f"{name} must be an integer")
            if not minimum <= value <= maximum:
                raise ValueError(f"{name} must be in [{minimum}, {maximum}]")
        if self.n_jobs == 0:
            raise ValueError("n_jobs must be None, -1, or a non-zero integer")
        for name, value, lower, upper, lower_inclusive in (
            ("learning_rate", self.learning_rate, 0.0, 1.0, False),
            ("min_child_weight", self.min_child_weight, 0.0, np.inf, True),
            ("min_gain_to_split", self.min_gain_to_split, 0.0, np.inf, True),
            ("reg_lambda", self.reg_lambda, 0.0, np.inf, True),
            ("reg_alpha", self.reg_alpha, 0.0, np.inf, True),
            ("max_delta_step", self.max_delta_step, 0.0, np.inf, True),
        ):
            if isinstance(value, bool) or not isinstance(value, (int, float)):
                raise TypeError(f"{name} must be a real number")
            numeric = float(value)
            valid_lower = numeric >= lower if lower_inclusive else numeric > lower
            if not np.isfinite(numeric) or not valid_lower or numeric > upper:
                bracket = "[" if lower_inclusive else "("
                raise ValueError(f"{name} must be in {bracket}{lower}, {upper}]")
        if self.growth_strategy not in {"level_wise", "leaf_wise"}:
            raise ValueError("growth_strategy must be 'level_wise' or 'leaf_wise'")
        if (self.max_active_leaves is not None and self.max_leaves is not None
                and self.max_active_leaves > self.max_leaves):
            raise ValueError("max_active_leaves must not exceed max_leaves")
        if self.device not in {"cuda", "auto"}:
            raise ValueError("device must be 'cuda' or 'auto'")
        if self.random_state is not None and (isinstance(self.random_state, bool)
                                              or not isinstance(self.random_state, int)):
            raise TypeError("random_state must be an integer or None")
        if self.categorical_features is not None:
            raise UnsupportedError("categorical_features are not supported on the CUDA backend")
        self._validate_objective_parameters()

    def _validate_objective_parameters(self) -> None:
        if self._native_objective == "squared_error":
            if self.loss not in {"squared_error", "quantile", "poisson", "tweedie"}:
                raise ValueError("loss must be 'squared_error', 'quantile', 'poisson', or 'tweedie'")
        elif getattr(self, "loss", "squared_error") != "squared_error":
            raise ValueError("loss is only supported by regression estimators")
        for name, lower, upper in (("quantile_alpha", 0.0, 1.0), ("tweedie_variance_power", 1.0, 2.0)):
            value = getattr(self, name)
            if isinstance(value, bool) or not isinstance(value, (int, float)):
                raise TypeError(f"{name} must be numeric")
            numeric = float(value)
            if not np.isfinite(numeric) or not lower < numeric < upper:
                raise ValueError(f"{name} must be in ({lower}, {upper})")

    def _resolved_native_objective(self) -> str:
        return self._native_objective if self._native_objective != "squared_error" else self.loss

    def _normalized_monotonic_constraints(self, n_features: int) -> list[int]:
        if self.monotonic_constraints is None:
            return []
        values = list(self.monotonic_constraints)
        if len(values) != n_features:
            raise ValueError("monotonic_constraints length must match feature count")
        out = []
        for v in values:
            if isinstance(v, bool) or not isinstance(v, (int, np.integer)):
                raise TypeError("monotonic_constraints values must be integers")
            if int(v) not in {-1, 0, 1}:
                raise ValueError("monotonic_constraints values must be -1, 0, or 1")
            out.append(int(v))
        return out

    def _normalized_interaction_constraints(self, n_features: int) -> list[list[int]]:
        if self.interaction_constraints is None:
            return []
        groups = []
        for group in self.interaction_constraints:
            g = []
            for v in group:
                if isinstance(v, bool) or not isinstance(v, (int, np.integer)):
                    raise TypeError("interaction_constraints values must be integers")
                i = int(v) + (n_features if int(v) < 0 else 0)
                if not 0 <= i < n_features:
                    raise ValueError("interaction constraint feature index is out of range")
                g.append(i)
            if not g:
                raise ValueError("interaction constraint groups must be non-empty")
            if len(set(g)) != len(g):
                raise ValueError("interaction constraint groups must not contain duplicates")
            groups.append(sorted(g))
        return groups

    def _parameters(self, n_features: int) -> TrainingParameters:
        return TrainingParameters(
            self.n_estimators, self.learning_rate, self.max_bins, self.max_depth, self.min_samples_leaf,
            self.min_child_weight, self.reg_lambda, reg_alpha=self.reg_alpha,
            max_delta_step=self.max_delta_step, min_gain_to_split=self.min_gain_to_split,
            objective=self._resolved_native_objective(), split_strategy=self._split_strategy,
            growth_strategy=self.growth_strategy, max_leaves=self.max_leaves or 0,
            max_active_leaves=self.max_active_leaves or 0,
            random_seed=0 if self.random_state is None else self.random_state,
            monotonic_constraints=self._normalized_monotonic_constraints(n_features),
            interaction_constraints=self._normalized_interaction_constraints(n_features),
            objective_alpha=self.quantile_alpha, tweedie_variance_power=self.tweedie_variance_power)

    # -- fitted state -----------------------------------------------------------------
    _FITTED = ("model_", "n_features_in_", "device_", "device_decision_", "n_estimators_",
               "training_summary_", "classes_", "estimators_", "feature_subsets_")

    def _clear_fitted_state(self) -> None:
        for name in self._FITTED:
            if hasattr(self, name):
                delattr(self, name)

    def _require_model(self):
        if not hasattr(self, "model_") and not hasattr(self, "estimators_"):
            raise RuntimeError(self._fitted_error_message)

    def _training_labels(self, y, n: int) -> np.ndarray:
        return _as_labels(y, n)

    def fit(self, X: Any, y: Any, sample_weight: Any = None):
        if not self._fit_lock.acquire(blocking=False):
            raise RuntimeError("Concurrent fit calls on the same estimator are not supported")
        try:
            self._validate_parameters()
            matrix = _as_matrix(X)
            labels = self._training_labels(y, matrix.shape[0])
            weights = _as_weights(sample_weight, matrix.shape[0])
            decision = _select_cuda(self.device, matrix.shape[0], matrix.shape[1], self.n_estimators,
                                    self.max_bins)
            started = perf_counter()
            candidate = _train_regressor_cuda(matrix, labels, weights, self._parameters(matrix.shape[1]))
            elapsed = perf_counter() - started
            self._clear_fitted_state()
            self.model_ = candidate
            self.n_features_in_ = matrix.shape[1]
            self.device_ = "cuda"
            self.device_decision_ = decision
            self.n_estimators_ = candidate.tree_count
            self.training_summary_ = {"fit_seconds": elapsed, "device": "cuda", "device_decision": decision,
                                      "n_estimators": candidate.tree_count,
                                      "native_objective": self._resolved_native_objective(),
                                      "weighted": sample_weight is not None}
            return self
        except Exception:
            self._clear_fitted_state()
            raise
        finally:
            self._fit_lock.release()

    def _predict_raw(self, X) -> np.ndarray:
        self._require_model()
        x = _as_matrix(X)
        if x.shape[1] != self.n_features_in_:
            raise ValueError("prediction feature count does not match training data")
        return self.model_.predict(x)

    def predict(self, X: Any) -> np.ndarray:
        """One-dimensional float32 predictions (exp of the margin for Poisson / Tweedie)."""

        raw = self._predict_raw(X)
        if self._resolved_native_objective() in {"poisson", "tweedie"}:
            return np.exp(raw.astype(np.float64)).astype(np.float32)
        return raw

    def score(self, X: Any, y: Any, sample_weight: Any = None) -> float:
        """Weighted R^2 (base.py:268-286)."""

        predictions = self.predict(X).astype(np.float64)
        labels = _as_labels(y, predictions.shape[0])
        weights = np.ones_like(labels) if sample_weight is None else _as_weights(sample_weight, labels.size)
        residual = float(np.sum(weights * (labels - predictions) ** 2))
        centered = labels - float(np.average(labels, weights=weights))
        total = float(np.sum(weights * centered ** 2))
        if total == 0.0:
            return 1.0 if residual == 0.0 else 0.0
        return float(1.0 - residual / total)


def _sigmoid(m: np.ndarray) -> np.ndarray:
    p = np.empty_like(m, dtype=np.float64)
    pos = m >= 0.0
    p[pos] = 1.0 / (1.0 + np.exp(-m[pos]))
    e = np.exp(m[~pos])
    p[~pos] = e / (1.0 + e)
    return p


class MPSBoostClassifier(MPSBoostRegressor):
    """Binary-logistic histogram GBDT classifier on the GPU; for more than two classes
    one-vs-rest (``multi_strategy`` "auto" or "ovr": the K binary fits of a round built in
    the same launches) or native softmax ("softmax"). ``multiclass.py:28-200``."""

    _estimator_type = "classifier"
    _native_objective = "binary_logistic"
    _fitted_error_message = "MPSBoostClassifier is not fitted or loaded"
    _PARAMETER_NAMES = MPSBoostRegressor._PARAMETER_NAMES + ("multi_strategy",)

    def __init__(self, *args, multi_strategy: str = "auto", **kwargs):
        super().__init__(*args, **kwargs)
        self.multi_strategy = multi_strategy

    def fit(self, X: Any, y: Any, sample_weight: Any = None):
        matrix = _as_matrix(X)
        labels = _as_labels(y, matrix.shape[0])
        classes = np.unique(labels)
        if classes.size < 2:
            raise ValueError("classification requires at least two classes")
        if self.multi_strategy not in {"auto", "softmax", "ovr"}:
            raise ValueError("multi_strategy must be 'auto', 'softmax', or 'ovr'")
        encoded = np.searchsorted(classes, labels).astype(np.float64)
        if classes.size == 2:
            fitted = super().fit(matrix, encoded, sample_weight=sample_weight)
            fitted.classes_ = classes
            fitted._strategy_ = "binary_logistic"
            return fitted
        if not self._fit_lock.acquire(blocking=False):
            raise RuntimeError("Concurrent fit calls on the same estimator are not supported")
        try:
            self._validate_parameters()
            weights = _as_weights(sample_weight, matrix.shape[0])
            decision = _select_cuda(self.device, matrix.shape[0], matrix.shape[1],
                                    self.n_estimators * int(classes.size), self.max_bins)
            b = _backend(0)
            kw = self._parameters(matrix.shape[1]).as_kwargs()
            started = perf_counter()
            dset = _be.quantize_device(b, matrix, int(self.max_bins))
            try:
                if self.multi_strategy == "softmax":
                    kw.pop("objective")
                    model = _be.train_softmax(b, dset, encoded, int(classes.size), weights, **kw)
                    strategy = "native_softmax"
                else:
                    model = _be.train_ovr(b, dset, encoded, int(classes.size), weights, **kw)
                    strategy = "one_vs_rest"
            finally:
                dset.close()
            elapsed = perf_counter() - started
            self._clear_fitted_state()
            if strategy == "native_softmax":
                self.model_ = model
                self.n_estimators_ = len(model.trees)
            else:
                self.estimators_ = tuple(CudaRegressionModel(m) for m in model)
                self.n_estimators_ = sum(len(m.trees) for m in model)
            self._strategy_ = strategy
            self.classes_ = classes.copy()
            self.n_features_in_ = matrix.shape[1]
            self.device_ = "cuda"
            self.device_decision_ = decision
            self.training_summary_ = {"fit_seconds": elapsed, "strategy": strategy,
                                      "requested_strategy": self.multi_strategy, "device": "cuda",
                                      "classes": self.classes_.tolist(), "n_classes": int(classes.size),
                                      "n_estimators": self.n_estimators_,
                                      "weighted": sample_weight is not None}
            return self
        except Exception:
            self._clear_fitted_state()
            raise
        finally:
            self._fit_lock.release()

    def decision_function(self, X: Any) -> np.ndarray:
        """Raw margins: one column for binary models, one per class otherwise."""

        self._require_model()
        x = _as_matrix(X)
        if x.shape[1] != self.n_features_in_:
            raise ValueError("prediction feature count does not match training data")
        strategy = getattr(self, "_strategy_", "binary_logistic")
        if strategy == "one_vs_rest":
            return np.column_stack([e.predict(x).astype(np.float64) for e in self.estimators_])
        if strategy == "native_softmax":
            binned = _host_schema(self.model_.schema).transform(x)
            return self.model_.predict_margins(_backend(0), binned)
        return self.model_.predict(x).astype(np.float64)

    def predict_proba(self, X: Any) -> np.ndarray:
        strategy = getattr(self, "_strategy_", "binary_logistic")
        margins = self.decision_function(X)
        if strategy == "native_softmax":
            e = np.exp(margins - margins.max(axis=1, keepdims=True))
            return (e / e.sum(axis=1, keepdims=True)).astype(np.float32)
        if strategy == "one_vs_rest":  # normalized one-vs-rest probabilities (multiclass.py:162-181)
            scores = 1.0 / (1.0 + np.exp(-np.clip(margins, -709.0, 709.0)))
            sums = scores.sum(axis=1, keepdims=True)
            zero = sums[:, 0] <= 0.0
            if np.any(zero):
                scores[zero, :] = 1.0 / float(scores.shape[1])
                sums = scores.sum(axis=1, keepdims=True)
            return (scores / sums).astype(np.float32)
        p = _sigmoid(margins)
        return np.column_stack((1.0 - p, p)).astype(np.float32)

    def predict(self, X: Any) -> np.ndarray:
        return self.classes_[np.argmax(self.predict_proba(X), axis=1)]

    def score(self, X: Any, y: Any, sample_weight: Any = None) -> float:
        """Weighted accuracy."""

        predictions = self.predict(X)
        labels = np.asarray(y).reshape(-1)
        weights = None if sample_weight is None else _as_weights(sample_weight, labels.size)
        return float(np.average((predictions == labels).astype(np.float64), weights=weights))


class RandomForestRegressor(MPSBoostRegressor):
    """Random forest of independent single-round trees on the GPU (``forest.py:30-183``,
    ``forest_public.py:27-41``): each tree fits a row sample (bootstrap or without
    replacement, ``sample_fraction`` of the rows) and ``ceil(max_features * F)`` features
    drawn as the reference draws them, and every tree of a batch is built in the same
    launches. The trees use the whole matrix's bins, where the reference re-bins each
    sample. Predictions are the mean of the trees'."""

    _fitted_error_message = "RandomForestRegressor is not fitted"
    _PARAMETER_NAMES = (
        "n_estimators", "max_depth", "max_bins", "min_child_weight", "min_samples_leaf", "reg_lambda",
        "reg_alpha", "max_delta_step", "monotonic_constraints", "interaction_constraints",
        "categorical_features", "max_features", "sample_fraction", "bootstrap", "n_jobs",
        "random_state", "device", "verbosity",
    )

    def __init__(self, n_estimators: int = 100, max_depth: int = 6, max_bins: int = 256,
                 min_child_weight: float = 1.0, min_samples_leaf: int = 20, reg_lambda: float = 1.0,
                 reg_alpha: float = 0.0, max_delta_step: float = 0.0, monotonic_constraints: Any = None,
                 interaction_constraints: Any = None, categorical_features: Any = None,
                 max_features: float = 1.0, sample_fraction: float = 1.0, bootstrap: bool = True,
                 n_jobs: int = 1, random_state: int | None = None, device: str = "cuda",
                 verbosity: int = 1) -> None:
        super().__init__(n_estimators=n_estimators, learning_rate=1.0, max_depth=max_depth,
                         max_bins=max_bins, min_child_weight=min_child_weight,
                         min_samples_leaf=min_samples_leaf, reg_lambda=reg_lambda, reg_alpha=reg_alpha,
                         max_delta_step=max_delta_step, monotonic_constraints=monotonic_constraints,
                         interaction_constraints=interaction_constraints,
                         categorical_features=categorical_features, random_state=random_state,
                         n_jobs=n_jobs, device=device, verbosity=verbosity)
        self.max_features = max_features
        self.sample_fraction = sample_fraction
        self.bootstrap = bootstrap

    def _validate_forest_parameters(self) -> None:
        self._validate_parameters()
        for name in ("max_features", "sample_fraction"):
            value = getattr(self, name)
            if isinstance(value, bool) or not isinstance(value, (int, float)):
                raise TypeError(f"{name} must be a real number")
            if not math.isfinite(float(value)) or not 0.0 < float(value) <= 1.0:
                raise ValueError(f"{name} must be in (0, 1]")
        if not isinstance(self.bootstrap, bool):
            raise TypeError("bootstrap must be a bool")

    def fit(self, X: Any, y: Any, sample_weight: Any = None):
        if not self._fit_lock.acquire(blocking=False):
            raise RuntimeError("concurrent fit is not supported for one estimator")
        try:
            self._validate_forest_parameters()
            matrix = _as_matrix(X)
            labels = _as_labels(y, matrix.shape[0])
            weights = _as_weights(sample_weight, matrix.shape[0])
            decision = _select_cuda(self.device, matrix.shape[0], matrix.shape[1], self.n_estimators,
                                    self.max_bins)
            counts, subsets, seeds = _be.forest_samples(
                matrix.shape[0], matrix.shape[1], self.n_estimators, random_state=self.random_state,
                bootstrap=self.bootstrap, sample_fraction=self.sample_fraction, max_features=self.max_features)
            subsets = [np.sort(s) for s in subsets]
            kw = self._parameters(matrix.shape[1]).as_kwargs()
            for name in ("n_estimators", "learning_rate", "objective"):
                kw.pop(name)
            b = _backend(0)
            started = perf_counter()
            dset = _be.quantize_device(b, matrix, int(self.max_bins))
            try:
                trees = _be.train_forest(b, dset, labels, weights, row_counts=counts, feature_subsets=subsets,
                                         seeds=seeds, **kw)
            finally:
                dset.close()
            elapsed = perf_counter() - started
            self._clear_fitted_state()
            # One model whose prediction is the trees' mean: base = mean base score,
            # learning rate 1 / n_trees over every tree's leaves.
            combined = _be.RegressionModel(float(np.mean([t.base_score for t in trees])), 1.0 / len(trees),
                                           [t.trees[0] for t in trees])
            combined.schema = trees[0].schema
            self.model_ = CudaRegressionModel(combined)
            self.feature_subsets_ = tuple(subsets)
            self.n_features_in_ = matrix.shape[1]
            self.n_estimators_ = len(trees)
            self.device_ = "cuda"
            self.device_decision_ = decision
            self.training_summary_ = {"fit_seconds": elapsed, "device": "cuda", "n_estimators": len(trees),
                                      "bootstrap": self.bootstrap, "max_features": self.max_features,
                                      "sample_fraction": self.sample_fraction}
            return self
        except Exception:
            self._clear_fitted_state()
            raise
        finally:
            self._fit_lock.release()


GradientBoostingRegressor = MPSBoostRegressor
GradientBoostingClassifier = MPSBoostClassifier
