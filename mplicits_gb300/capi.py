"""ctypes binding of libmplicits.so (the C ABI declared in include/mplicits.h).

The library is built in-tree (``mplicits_gb300/libmplicits.so``) by
``mplicits_gb300.build``.  There is no fallback: if the library is missing or
cannot be loaded, every GPU entry point raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmplicits.so")

MPL_MAX_LAYERS = 8
MPL_OK = 0
MPL_ERR_INVALID_ARG = 1
MPL_ERR_UNSUPPORTED = 2
MPL_ERR_CAPACITY = 3
MPL_ERR_DEVICE_TIMEOUT = 4
MPL_ERR_CUDA = 5
MPL_ERR_NO_DEVICE = 6

MPL_FP32 = 0
MPL_BF16 = 1
MPL_F16 = 2
MPL_STORE = 0
MPL_ACCUMULATE = 1
MPL_POINTS_XYZ = 0
MPL_POINTS_GRID = 1

PRECISIONS = {"fp32": MPL_FP32, "bf16": MPL_BF16, "fp16": MPL_F16}
MPL_OPT_BF16_EPILOGUE_UNIT = 1
MPL_OPT_TC_TILES_IN_FLIGHT = 2
MPL_OPT_TC_GRAD_REVERSE = 3
MPL_OPT_TC_LAYER0_WARPS = 4
MPL_BATCH_NEIGH_DELTA = 1
MPL_BATCH_DITHER = 2


class MplNet(ctypes.Structure):
    _fields_ = [("n_layers", ctypes.c_int32),
                ("dims", ctypes.c_int32 * (MPL_MAX_LAYERS + 1)),
                ("omega", ctypes.c_float * MPL_MAX_LAYERS)]


class MplPoints(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32),
                ("grid_n", ctypes.c_int32),
                ("voxel_size", ctypes.c_float),
                ("offset", ctypes.c_float * 3),
                ("xyz", ctypes.c_void_p)]


class MplBand(ctypes.Structure):
    _fields_ = [("delta", ctypes.c_float),
                ("out_index", ctypes.c_void_p),
                ("count_dev", ctypes.c_void_p),
                ("capacity", ctypes.c_int64),
                ("lower", ctypes.c_float)]


class MplCamera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3),
                ("target", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3),
                ("fov_y_deg", ctypes.c_float),
                ("width", ctypes.c_int32),
                ("height", ctypes.c_int32)]


class MplLoss(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32),
                ("weight", ctypes.c_float * 4)]


MPL_LOSS_RESIDUAL = 0
MPL_LOSS_TRUE_SDF = 1


class MplBatchEntry(ctypes.Structure):
    _fields_ = [("net", MplNet),
                ("packed_dev", ctypes.c_void_p),
                ("points", MplPoints),
                ("index_dev", ctypes.c_void_p),
                ("n_dev", ctypes.c_void_p),
                ("n", ctypes.c_int64),
                ("S_dev", ctypes.c_void_p),
                ("store_mode", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class MplBatchPlan(ctypes.Structure):
    _fields_ = [("workspace_dev", ctypes.c_void_p),
                ("count", ctypes.c_int32),
                ("precision", ctypes.c_int32),
                ("width_count", ctypes.c_int32 * 3),
                ("reserved", ctypes.c_int32)]


class MplBatchConfig(ctypes.Structure):
    _fields_ = [("epilogue_unit", ctypes.c_int32),
                ("stages", ctypes.c_int32),
                ("ctas", ctypes.c_int32),
                ("tiles_in_flight", ctypes.c_int32)]


MPL_BATCH_MAX_ENTRIES = 1024


# (name, restype, argtypes) of every exported symbol; tests check that the
# library exports exactly what include/mplicits.h declares.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_F = ctypes.c_float
SIGNATURES = {
    "mpl_net_packed_bytes": (ctypes.c_int, [ctypes.POINTER(MplNet), ctypes.POINTER(_I64)]),
    "mpl_net_pack": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, _P, _P, _P]),
    "mpl_level_forward": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, ctypes.POINTER(MplPoints),
                                         _P, _P, _I64, _P, _I32, ctypes.POINTER(MplBand), _I32,
                                         _P]),
    "mpl_level_gradient": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, ctypes.POINTER(MplPoints),
                                          _P, _P, _I64, _P, _P, _I32, ctypes.POINTER(MplBand),
                                          _I32, _P]),
    "mpl_grid_points": (ctypes.c_int, [ctypes.POINTER(MplPoints), _P, _I64, _P, _P]),
    "mpl_band_compact": (ctypes.c_int, [_P, _P, _P, _I64, ctypes.POINTER(MplBand), _P]),
    "mpl_abs_max": (ctypes.c_int, [_P, _I64, _P, _P]),
    "mpl_mc_workspace_bytes": (ctypes.c_int, [_I64, ctypes.POINTER(_I64)]),
    "mpl_mc_count": (ctypes.c_int, [_P, _I64, _F, _P, _P, _P]),
    "mpl_mc_emit": (ctypes.c_int, [_P, _I64, _F, _F, _P, _P, _P, _P, _P, _P, _I64, _I64, _P]),
    "mpl_mc_noalloc": (ctypes.c_int, [_P, _I64, _F, _F, _P, _P, _P, _P, _P, _I64, _I64, _P, _P]),
    "mpl_trace_init": (ctypes.c_int, [ctypes.POINTER(MplCamera), _F, _P, _P, _P, _P, _P, _P]),
    "mpl_trace_step": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _P, _F, _F, _I32, _P, _P, _P, _P,
                                      _I64, _P]),
    "mpl_trace_march": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, _I32, _P, _P, _P, _I64, _P,
                                       _P, _P, _P, _F, _F, _I32, _I32, _P, _P, _I64, _I32, _P]),
    "mpl_trace_shade": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I32, _P, _P]),
    "mpl_train_scratch_floats": (ctypes.c_int, [ctypes.POINTER(MplNet), _I64,
                                                ctypes.POINTER(_I64)]),
    "mpl_train_forward": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, _P, _I64, _P, _P, _P, _P]),
    "mpl_train_loss": (ctypes.c_int, [_I64, _P, _P, _P, _P, _P, _P, ctypes.POINTER(MplLoss), _P,
                                      _P, _P]),
    "mpl_train_backward": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, _P, _I64, _P, _P, _P, _P,
                                          _P, _P]),
    "mpl_train_tc_scratch_bytes": (ctypes.c_int, [ctypes.POINTER(MplNet), _I64,
                                                  ctypes.POINTER(_I64)]),
    "mpl_train_tc_step": (ctypes.c_int, [ctypes.POINTER(MplNet), _P, _P, _I64, _P, _P, _P, _P,
                                         ctypes.POINTER(MplLoss), _P, _I64, _P, _P, _P, _P, _P]),
    "mpl_train_batch": (ctypes.c_int, [_P, _I64, _I32, _P, _P, _I64, _F, _F, _I32,
                                       ctypes.c_uint64, _P, _P, _P, _P]),
    "mpl_adam_step": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P, _F, _F, _F, _F, _I64, _P]),
    "mpl_scene_create": (ctypes.c_int, [_P, _I64, _P, _I64, _F, ctypes.POINTER(_P), _P]),
    "mpl_scene_destroy": (ctypes.c_int, [_P]),
    "mpl_scene_info": (ctypes.c_int, [_P, ctypes.POINTER(_F), ctypes.POINTER(_F),
                                      ctypes.POINTER(_I32), ctypes.POINTER(_I64)]),
    "mpl_scene_compute_distance": (ctypes.c_int, [_P, _P, _I64, _P, _P]),
    "mpl_calc_deltas_scratch_bytes": (ctypes.c_int, [_I64, _I32, ctypes.POINTER(_I64)]),
    "mpl_calc_deltas": (ctypes.c_int, [_P, _P, _I64, _I32, _F, _F, _I32, _F, _P, _P, _P, _P]),
    "mpl_batch_workspace_bytes": (ctypes.c_int, [_I32, ctypes.POINTER(_I64)]),
    "mpl_batch_prepare": (ctypes.c_int, [ctypes.POINTER(MplBatchEntry), _I32, _I32, _P, _I64,
                                         ctypes.POINTER(MplBatchPlan), _P]),
    "mpl_batch_run": (ctypes.c_int, [ctypes.POINTER(MplBatchPlan),
                                     ctypes.POINTER(MplBatchConfig), _P]),
    "mpl_batch_autotune": (ctypes.c_int, [ctypes.POINTER(MplBatchPlan), _I32,
                                          ctypes.POINTER(MplBatchConfig),
                                          ctypes.POINTER(ctypes.c_float), _P]),
    "mpl_set_option": (ctypes.c_int, [_I32, _I64]),
    "mpl_get_option": (ctypes.c_int, [_I32, ctypes.POINTER(_I64)]),
    "mpl_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "mpl_device_status": (ctypes.c_int, [ctypes.POINTER(_I32)]),
    "mpl_wait_selftest": (ctypes.c_int, [_I64, _P, _P]),
    "mpl_last_cuda_error": (ctypes.c_int, []),
    "mpl_abi_version": (ctypes.c_int, []),
}

_lib = None
_lock = threading.Lock()


class MplError(RuntimeError):
    """A libmplicits call returned a non-zero status."""

    def __init__(self, status, where, cuda_error=0):
        self.status = status
        msg = f"{where}: {status_string(status)} (status {status})"
        if status == MPL_ERR_CUDA:
            msg += f", cudaError {cuda_error}"
        super().__init__(msg)


def load(path=LIB_PATH):
    """Load libmplicits.so (raises if it is missing: there is no fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(
                    f"libmplicits.so not found at {path}; build it with "
                    "`python -m mplicits_gb300.build` (the GPU path has no fallback)")
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def status_string(status):
    try:
        return load().mpl_status_string(status).decode()
    except Exception:  # library unavailable: keep the numeric code meaningful
        return f"status {status}"


def check(status, where):
    if status != MPL_OK:
        raise MplError(status, where, load().mpl_last_cuda_error())


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t):
    """Device pointer of a tensor (or None)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def device_status():
    """Synchronise and read/clear the device status word (MPL_OK if clean)."""
    v = _I32(0)
    check(load().mpl_device_status(ctypes.byref(v)), "mpl_device_status")
    return v.value


def set_option(option, value):
    check(load().mpl_set_option(option, value), "mpl_set_option")


def get_option(option):
    v = _I64(0)
    check(load().mpl_get_option(option, ctypes.byref(v)), "mpl_get_option")
    return v.value
