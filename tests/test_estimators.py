"""The Python device="cuda" route on the CPU machine: device policy, parameters, validation.

The policy restates the reference's (src/mpsboost/device_policy.py) with CUDA added, so
the reference's own cases (tests/unit/test_device_policy.py) must hold unchanged when no
GPU is reported, and explicit "cuda" requests must be honored. Estimator fits need a GPU:
here they must fail loudly with BackendError, never fall back to a CPU path.
"""

from __future__ import annotations

import numpy as np
import pytest

import mpsboost_gb300 as mb
from mpsboost_gb300 import estimators as est


def _decide(**kw):
    base = dict(requested="auto", n_samples=10, n_features=2, n_estimators=1, max_bins=16)
    base.update(kw)
    return mb.choose_device(**base)


def test_reference_policy_cases_hold_without_cuda():
    assert _decide(requested="cpu", mps_available=True).reason == "explicit cpu request"
    mps = _decide(requested="mps", mps_available=False)
    assert (mps.selected, mps.reason) == ("mps", "explicit mps request")
    unavailable = _decide(n_samples=10_000, n_features=100, n_estimators=100, max_bins=256)
    assert (unavailable.selected, unavailable.reason) == ("cpu", "mps unavailable")
    small = _decide(n_samples=100, n_features=8, n_estimators=20, max_bins=64, mps_available=True)
    assert (small.selected, small.reason) == ("cpu", "estimated work below mps threshold")
    big = _decide(n_samples=50_000, n_features=100, n_estimators=200, max_bins=256, mps_available=True)
    assert (big.selected, big.reason, big.estimated_work) == ("mps", "estimated work meets mps threshold",
                                                              256_000_000_000)


def test_cuda_requests_and_auto_choice():
    explicit = _decide(requested="cuda")
    assert (explicit.selected, explicit.reason) == ("cuda", "explicit cuda request")
    big = dict(n_samples=50_000, n_features=100, n_estimators=200, max_bins=256)
    assert _decide(**big, cuda_available=True, mps_available=True).selected == "cuda"
    small = _decide(cuda_available=True)
    assert (small.selected, small.reason) == ("cpu", "estimated work below cuda threshold")
    assert _decide(cuda_available=True, cuda_work_threshold=1).selected == "cuda"
    d = mb.device_policy.decision_to_dict(explicit)
    assert d["selected"] == "cuda" and d["cuda_available"] is False


@pytest.mark.parametrize("kwargs, message", [
    ({"requested": "gpu"}, "requested device"),
    ({"n_samples": 0}, "positive"),
    ({"max_bins": 0}, "positive"),
    ({"mps_available": 1}, "bool"),
    ({"cuda_available": 1}, "bool"),
    ({"cuda_work_threshold": 0}, "positive"),
])
def test_invalid_policy_inputs_fail_early(kwargs, message):
    with pytest.raises((TypeError, ValueError), match=message):
        _decide(**kwargs)


def test_training_parameters_mirror_the_binding_object():
    p = est.TrainingParameters(50, 0.1, 255, 6, 20, 1.0, 1.0, objective="binary_logistic",
                               monotonic_constraints=[1, 0], interaction_constraints=[[0, 1]])
    kw = p.as_kwargs()
    assert kw["objective"] == "binary_logistic" and kw["max_bins"] == 255
    params, keep = mb.make_params(**kw)
    assert params.n_estimators == 50 and params.objective == 1 and params.n_monotonic == 2
    assert params.n_interaction_groups == 1
    assert est.TrainingParameters(1, 0.1, 16, 3, 1, 0.0, 1.0).as_kwargs()["monotonic_constraints"] is None


def test_estimator_parameters_and_validation():
    reg = mb.GradientBoostingRegressor(n_estimators=5, max_depth=3)
    assert reg.get_params()["device"] == "cuda" and reg.get_params()["min_samples_leaf"] == 20
    assert reg.set_params(learning_rate=0.2) is reg and reg.learning_rate == 0.2
    with pytest.raises(ValueError, match="Unknown parameter"):
        reg.set_params(colour=1)
    x = np.zeros((10, 2), np.float32)
    y = np.arange(10.0)
    for bad, exc, msg in [
        (dict(device="mps"), ValueError, "device must be"),
        (dict(n_estimators=0), ValueError, r"n_estimators must be in"),
        (dict(learning_rate=0.0), ValueError, "learning_rate"),
        (dict(loss="huber"), ValueError, "loss must be"),
        (dict(categorical_features=[0]), mb.UnsupportedError, "categorical"),
        (dict(max_depth=True), TypeError, "max_depth must be an integer"),
    ]:
        with pytest.raises(exc, match=msg):
            mb.GradientBoostingRegressor(**bad).fit(x, y)
    with pytest.raises(ValueError, match="multi_strategy"):
        mb.GradientBoostingClassifier(multi_strategy="tree").fit(x, (y > 4).astype(float))
    with pytest.raises(ValueError, match="max_features"):
        mb.RandomForestRegressor(max_features=1.5).fit(x, y)
    with pytest.raises(RuntimeError, match="not fitted"):
        reg.predict(x)


@pytest.mark.skipif(mb.cuda_available(), reason="checks the no-GPU behaviour")
def test_fit_without_gpu_fails_loudly():
    x = np.random.default_rng(0).normal(size=(50, 3)).astype(np.float32)
    y = x[:, 0].astype(np.float64)
    for model in (mb.GradientBoostingRegressor(n_estimators=2), mb.RandomForestRegressor(n_estimators=2),
                  mb.GradientBoostingClassifier(n_estimators=2, device="auto")):
        with pytest.raises(mb.BackendError, match="no GPU"):
            model.fit(x, (y > 0).astype(float) if isinstance(model, mb.MPSBoostClassifier) else y)
        assert not hasattr(model, "model_")
