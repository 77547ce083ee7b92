"""ctypes binding of ``libmpsb_cuda.so`` (the C ABI declared in ``include/mpsb_cuda.h``).

The library is built in-tree by :func:`mpsboost_gb300.build.build`; loading fails loudly
when it cannot be built or loaded -- there is no CPU fallback for any device entry.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

MPSB_OK = 0
MPSB_ERR_TRAINING = 1
MPSB_ERR_DATA = 2
MPSB_ERR_BACKEND = 3
MPSB_ERR_UNSUPPORTED = 4

HIST_FIXED = 0
HIST_FLOAT = 1

OPT_FLOAT_HIST = 1 << 0
OPT_NO_GRAPH = 1 << 1
OPT_PER_NODE = 1 << 2
OPT_TIMING = 1 << 3


class TrainParams(C.Structure):
    """``mpsb_train_params`` (TrainingParameters + TreeTrainingParameters)."""

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


class Info(C.Structure):
    _fields_ = [
        ("available", C.c_uint32),
        ("sm_count", C.c_uint32),
        ("cc_major", C.c_uint32),
        ("cc_minor", C.c_uint32),
        ("total_memory", C.c_uint64),
        ("device_name", C.c_char * 96),
    ]


ABI_VERSION = 2  # MPSB_CUDA_ABI_VERSION of the structs below


class Stats(C.Structure):
    _fields_ = [
        ("rounds", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("hist_launches", C.c_uint64),
        ("hist_cells", C.c_uint64),
        ("hist_rows", C.c_uint64),
        ("hist_ms", C.c_double),
        ("hist_timed_launches", C.c_uint64),
        ("part_rows", C.c_uint64),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("hist_threads", C.c_uint32),
        ("hist_stages", C.c_uint32),
        ("root_threads", C.c_uint32),
        ("items_per_sm", C.c_uint32),
        ("blocked_levels", C.c_uint32),
        ("scan_threads", C.c_uint32),
        ("ms_per_round", C.c_double),
        ("default_ms_per_round", C.c_double),
        ("trials", C.c_uint32),
    ]


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

# Every symbol include/mpsb_cuda.h declares, with its ctypes signature.
_VP = C.c_void_p
_U32, _U64, _I32, _F64 = C.c_uint32, C.c_uint64, C.c_int, C.c_double
SIGNATURES = {
    "mpsb_cuda_last_error": (C.c_char_p, []),
    "mpsb_cuda_abi_version": (_I32, []),
    "mpsb_cuda_device_count": (_I32, [C.POINTER(_I32)]),
    "mpsb_cuda_backend_create": (_I32, [_I32, C.POINTER(_VP)]),
    "mpsb_cuda_backend_destroy": (None, [_VP]),
    "mpsb_cuda_backend_info": (_I32, [_VP, C.POINTER(Info)]),
    "mpsb_cuda_backend_set_hist_mode": (_I32, [_VP, _I32]),
    "mpsb_cuda_timer_begin": (_I32, [_VP]),
    "mpsb_cuda_timer_end": (_I32, [_VP, C.POINTER(C.c_float)]),
    "mpsb_cuda_synchronize": (_I32, [_VP]),
    "mpsb_cuda_host_register": (_I32, [_VP, _U64]),
    "mpsb_cuda_host_unregister": (_I32, [_VP]),
    "mpsb_quantize_dense": (_I32, [_VP, _I32, _U64, _U32, _U64, _U64, _U32, _U32, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "mpsb_transform_dense": (_I32, [_VP, _I32, _U64, _U32, _U64, _U64, _U32, _VP, _VP, _VP, _U32, _VP, _VP]),
    "mpsb_cuda_dataset_create": (_I32, [_VP, _VP, _U32, _VP, _U64, _U32, _VP, C.POINTER(_VP)]),
    "mpsb_cuda_dataset_create_async": (_I32, [_VP, _VP, _U32, _VP, _U64, _U32, _VP, C.POINTER(_VP)]),
    "mpsb_cuda_dataset_wait": (_I32, [_VP]),
    "mpsb_cuda_dataset_destroy": (None, [_VP]),
    "mpsb_cuda_dataset_uses_tma": (_I32, [_VP]),
    "mpsb_cuda_squared_error": (_I32, [_VP, _VP, _VP, _U64, _VP]),
    "mpsb_cuda_build_histograms": (_I32, [_VP, _VP, _VP, _U64, _VP, _U64, _VP]),
    "mpsb_cuda_build_layer_histograms": (_I32, [_VP, _VP, _VP, _VP, _U32, _VP, _U64, _VP]),
    "mpsb_cuda_scan_splits": (_I32, [_VP, _VP, _VP, _U64, _VP, _U64, C.POINTER(TrainParams), _VP]),
    "mpsb_cuda_partition_rows": (_I32, [_VP, _VP, _VP, _U64, _U32, _U32, _I32, _VP, _VP, C.POINTER(_U64)]),
    "mpsb_cuda_build_histogram_noalloc": (_I32, [_VP, _U32, _U32, _VP, _U32, _VP, _VP, _VP]),
    "mpsb_cuda_train_regressor": (_I32, [_VP, _VP, _VP, _VP, _U64, C.POINTER(TrainParams), _U32, C.POINTER(_VP)]),
    "mpsb_cuda_dataset_quantize": (_I32, [_VP, _VP, C.c_int, _U64, _U32, _U64, _U64, _U32, C.POINTER(_VP)]),
    "mpsb_cuda_dataset_transform": (_I32, [_VP, _VP, _VP, C.c_int, _U64, _U32, _U64, _U64, C.POINTER(_VP)]),
    "mpsb_cuda_dataset_boundary_total": (_U64, [_VP]),
    "mpsb_cuda_dataset_schema": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "mpsb_cuda_dataset_export": (_I32, [_VP, _VP, _VP]),
    "mpsb_cuda_dataset_export16": (_I32, [_VP, _VP, _VP]),
    "mpsb_cuda_model_set_schema": (_I32, [_VP, _U32, _U32, _VP, _U64, _VP, _VP, _VP, _VP]),
    "mpsb_cuda_model_set_objective": (_I32, [_VP, _U32, _F64, _F64]),
    "mpsb_cuda_model_get_objective": (_I32, [_VP, _VP, _VP, _VP]),
    "mpsb_cuda_model_get_schema": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "mpsb_cuda_model_serialize": (_I32, [_VP, _VP, _U64, _VP]),
    "mpsb_cuda_model_deserialize": (_I32, [_VP, _U64, C.c_int, C.POINTER(_VP)]),
    "mpsb_cuda_model_save": (_I32, [_VP, C.c_char_p]),
    "mpsb_cuda_model_load": (_I32, [C.c_char_p, C.c_int, C.POINTER(_VP)]),
    "mpsb_cuda_train_softmax": (_I32, [_VP, _VP, _VP, _VP, _U64, C.POINTER(TrainParams), _U32, _U32, C.POINTER(_VP)]),
    "mpsb_cuda_model_class_count": (_U32, [_VP]),
    "mpsb_cuda_model_class_base_scores": (_I32, [_VP, _VP]),
    "mpsb_cuda_model_predict_margins": (_I32, [_VP, _VP, _VP, _VP]),
    "mpsb_cuda_model_class_labels": (_I32, [_VP, _VP]),
    "mpsb_cuda_model_create_softmax": (_I32, [_U32, _F64, _VP, _VP, _U32, _VP, _VP, C.POINTER(_VP)]),
    "mpsb_cuda_train_ovr": (_I32, [_VP, _VP, _VP, _VP, _U64, _U32, C.POINTER(TrainParams), _U32, _VP]),
    "mpsb_cuda_train_forest": (_I32, [_VP, _VP, _VP, _VP, _U64, C.POINTER(TrainParams), _U32, _VP, _VP,
                                      _VP, _VP, _U32, _VP]),
    "mpsb_cuda_model_create": (_I32, [_F64, _F64, _U32, _VP, _VP, C.POINTER(_VP)]),
    "mpsb_cuda_model_tree_count": (_U32, [_VP]),
    "mpsb_cuda_model_base_score": (_F64, [_VP]),
    "mpsb_cuda_model_learning_rate": (_F64, [_VP]),
    "mpsb_cuda_model_tree_node_count": (_U32, [_VP, _U32]),
    "mpsb_cuda_model_tree_nodes": (_I32, [_VP, _U32, _VP]),
    "mpsb_cuda_model_train_predictions": (_I32, [_VP, _VP]),
    "mpsb_cuda_model_predict": (_I32, [_VP, _VP, _VP, _VP]),
    "mpsb_cuda_model_destroy": (None, [_VP]),
    "mpsb_cuda_trainer_create": (_I32, [_VP, _VP, _VP, _VP, _U64, C.POINTER(TrainParams), _U32, C.POINTER(_VP)]),
    "mpsb_cuda_trainer_run": (_I32, [_VP, _U32]),
    "mpsb_cuda_trainer_synchronize": (_I32, [_VP]),
    "mpsb_cuda_trainer_stats": (_I32, [_VP, C.POINTER(Stats)]),
    "mpsb_cuda_trainer_reset_stats": (_I32, [_VP]),
    "mpsb_cuda_trainer_level_stats": (_I32, [_VP, _U32, _VP, _VP]),
    "mpsb_cuda_trainer_export": (_I32, [_VP, C.POINTER(_VP)]),
    "mpsb_cuda_autotune": (_I32, [_VP, _VP, _VP, _VP, _U64, _VP, _U32, _U32, C.POINTER(Tuning)]),
    "mpsb_cuda_autotune_clear": (None, []),
    "mpsb_cuda_trainer_destroy": (None, [_VP]),
}


class BackendError(RuntimeError):
    """CUDA runtime / device failure (the reference's BackendError)."""


class TrainingError(ValueError):
    """Contract or math violation (the reference's TrainingError)."""


class DataError(ValueError):
    """Input data violation (the reference's DataError)."""


class UnsupportedError(NotImplementedError):
    """A configuration the CUDA backend does not provide."""


_ERRORS = {
    MPSB_ERR_TRAINING: TrainingError,
    MPSB_ERR_DATA: DataError,
    MPSB_ERR_BACKEND: BackendError,
    MPSB_ERR_UNSUPPORTED: UnsupportedError,
}

_lock = threading.Lock()
_lib = None


def load() -> C.CDLL:
    """Build (when stale) and load the CUDA backend library; raise if impossible."""

    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            if not os.path.exists(path):
                raise BackendError(f"CUDA backend library missing: {path}")
            lib = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            if lib.mpsb_cuda_abi_version() != ABI_VERSION:
                raise BackendError(f"CUDA backend library {path} has ABI version "
                                   f"{lib.mpsb_cuda_abi_version()}, these bindings need {ABI_VERSION}")
            _lib = lib
    return _lib


def check(rc: int) -> None:
    if rc != MPSB_OK:
        msg = load().mpsb_cuda_last_error().decode(errors="replace")
        raise _ERRORS.get(rc, BackendError)(msg)


def ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)
