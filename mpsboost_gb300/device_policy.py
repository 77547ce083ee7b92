"""Device selection with CUDA beside the reference's CPU and MPS choices.

Restates the reference's policy (``src/mpsboost/device_policy.py:15-99``) with one more
device: explicit requests are honored, ``auto`` picks CUDA when a usable GPU is present
and the estimated histogram work reaches ``cuda_work_threshold``, then MPS under the
reference's own rule, then CPU. The messages and the work estimate are the reference's.
This package trains on CUDA only: its estimators accept ``device="cuda"`` or ``"auto"``
and raise ``BackendError`` when no GPU is usable, never falling back to a CPU path.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Literal

RequestedDevice = Literal["cpu", "mps", "cuda", "auto"]
ResolvedDevice = Literal["cpu", "mps", "cuda"]


@dataclass(frozen=True)
class DeviceDecision:
    """Immutable record explaining one backend-selection decision."""

    requested: RequestedDevice
    selected: ResolvedDevice
    reason: str
    estimated_work: int
    mps_available: bool
    cuda_available: bool = False


def cuda_device_count() -> int:
    """GPUs the CUDA backend can train on (compute capability 10.3); 0 without a driver."""

    from . import _lib

    n = C.c_int32(0)
    _lib.check(_lib.load().mpsb_cuda_device_count(C.byref(n)))
    return int(n.value)


def cuda_available() -> bool:
    return cuda_device_count() > 0


def _estimated_histogram_work(*, n_samples: int, n_features: int, n_estimators: int, max_bins: int) -> int:
    """Estimated tree histogram work with overflow-safe Python integers."""

    for name, value in (("n_samples", n_samples), ("n_features", n_features),
                        ("n_estimators", n_estimators), ("max_bins", max_bins)):
        if isinstance(value, bool) or not isinstance(value, int):
            raise TypeError(f"{name} must be an integer")
        if value <= 0:
            raise ValueError(f"{name} must be positive")
    return n_samples * n_features * n_estimators * max_bins


def _check_threshold(name: str, value: int) -> None:
    if isinstance(value, bool) or not isinstance(value, int):
        raise TypeError(f"{name} must be an integer")
    if value <= 0:
        raise ValueError(f"{name} must be positive")


def choose_device(*, requested: RequestedDevice, n_samples: int, n_features: int, n_estimators: int,
                  max_bins: int, mps_available: bool = False, cuda_available: bool = False,
                  mps_work_threshold: int = 134_217_728,
                  cuda_work_threshold: int = 134_217_728) -> DeviceDecision:
    """Choose the backend for one fit call and explain the decision."""

    if requested not in {"cpu", "mps", "cuda", "auto"}:
        raise ValueError("requested device must be 'cpu', 'mps', 'cuda', or 'auto'")
    for name, flag in (("mps_available", mps_available), ("cuda_available", cuda_available)):
        if not isinstance(flag, bool):
            raise TypeError(f"{name} must be a bool")
    _check_threshold("mps_work_threshold", mps_work_threshold)
    _check_threshold("cuda_work_threshold", cuda_work_threshold)
    work = _estimated_histogram_work(n_samples=n_samples, n_features=n_features,
                                     n_estimators=n_estimators, max_bins=max_bins)

    def decide(selected: ResolvedDevice, reason: str) -> DeviceDecision:
        return DeviceDecision(requested, selected, reason, work, mps_available, cuda_available)

    if requested != "auto":
        return decide(requested, f"explicit {requested} request")
    if cuda_available and work >= cuda_work_threshold:
        return decide("cuda", "estimated work meets cuda threshold")
    if not mps_available:
        if cuda_available:
            return decide("cpu", "estimated work below cuda threshold")
        return decide("cpu", "mps unavailable")
    if work < mps_work_threshold:
        return decide("cpu", "estimated work below mps threshold")
    return decide("mps", "estimated work meets mps threshold")


def decision_to_dict(decision: DeviceDecision) -> dict[str, object]:
    """Convert a decision to a stable serializable diagnostic mapping."""

    return {
        "requested": decision.requested,
        "selected": decision.selected,
        "reason": decision.reason,
        "estimated_work": int(decision.estimated_work),
        "mps_available": bool(decision.mps_available),
        "cuda_available": bool(decision.cuda_available),
    }
