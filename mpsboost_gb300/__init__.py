"""GB300 (sm_103a) CUDA backend for the MPSBoost GBDT training hot path.

gradient/hessian -> histogram build (+ sibling subtraction) -> split-gain scan -> row
partition, behind the reference's backend contract (include/mpsboost/backend.hpp) and
exposed through the C ABI in ``include/mpsb_cuda.h``. See ``backend`` for the Python
mirror of the reference's native interface, ``estimators`` for the sklearn-style
estimators with ``device="cuda"`` and ``device_policy`` for the device decision.
"""

from ._lib import BackendError, DataError, TrainingError, UnsupportedError
from .backend import (
    DEFAULT_PARAMS,
    BinnedDataset,
    CudaBackend,
    DeviceBinnedDataset,
    MulticlassModel,
    RegressionModel,
    Trainer,
    forest_samples,
    make_params,
    quantize_dense,
    quantize_device,
    train_forest,
    train_ovr,
    train_regressor,
    train_softmax,
)

from .device_policy import DeviceDecision, choose_device, cuda_available, cuda_device_count
from .estimators import (
    GradientBoostingClassifier,
    GradientBoostingRegressor,
    MPSBoostClassifier,
    MPSBoostRegressor,
    RandomForestRegressor,
)

__all__ = [
    "DeviceDecision",
    "GradientBoostingClassifier",
    "GradientBoostingRegressor",
    "MPSBoostClassifier",
    "MPSBoostRegressor",
    "RandomForestRegressor",
    "choose_device",
    "cuda_available",
    "cuda_device_count",
    "BackendError",
    "BinnedDataset",
    "CudaBackend",
    "DataError",
    "DEFAULT_PARAMS",
    "DeviceBinnedDataset",
    "MulticlassModel",
    "RegressionModel",
    "Trainer",
    "TrainingError",
    "forest_samples",
    "train_forest",
    "UnsupportedError",
    "make_params",
    "quantize_dense",
    "quantize_device",
    "train_ovr",
    "train_regressor",
    "train_softmax",
]
