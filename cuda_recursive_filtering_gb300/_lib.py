"""ctypes binding of libiir_gb300.so (declarations in include/iir_gb300.h).

Loading fails loudly when the shared library has not been built: there is no CPU or
PyTorch fallback for the filtering path.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libiir_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "iir_gb300.h")

IIR_OK = 0
IIR_ERR_INVALID_ARGUMENT = -1
IIR_ERR_UNSUPPORTED = -2
IIR_ERR_CUDA = -3
IIR_ERR_LOOKBACK_TIMEOUT = -4
IIR_ERR_OUT_OF_MEMORY = -5
IIR_ERR_TOO_LARGE = -6
IIR_NOALLOC_MAX_SAMPLES = 1 << 26

KERNELS = {"AUTO": 0, "PH": 1, "STCR": 2, "STCR_UNROLL": 3, "DTCR": 4, "DTCR_UNROLL": 5, "PLR": 6, "TC": 7}
KERNEL_NAMES = {v: k for k, v in KERNELS.items()}


class IirSegment(ctypes.Structure):
    """iir_segment (include/iir_gb300.h)."""
    _fields_ = [("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("n", ctypes.c_size_t), ("filter", ctypes.c_int),
                ("zi", ctypes.c_void_p), ("zf", ctypes.c_void_p)]


class IirError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


_lib = None


def load(path: str | None = None):
    """Loads the library (once). Raises ImportError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m cuda_recursive_filtering_gb300.build` "
            "(nvcc, sm_103a). There is no CPU fallback.")
    L = ctypes.CDLL(path)
    vp, sz, i, ll = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_longlong
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    pp = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "iir_sos_filter": ([vp, vp, sz, fp, i, i, vp], i),
        "iir_sos_filter_geom": ([vp, vp, sz, fp, i, i, i, i, vp], i),
        "iir_sos_filter_noalloc": ([vp, vp, sz, fp, i, vp], i),
        "iir_plan_create": ([pp, fp, i, i, i, i, sz], i),
        "iir_plan_create_plr_ba": ([pp, dp, dp, i, ctypes.c_double, i, i, sz], i),
        "iir_plan_execute": ([vp, vp, vp, sz, vp], i),
        "iir_plan_execute_host": ([vp, vp, vp, sz, sz, vp], i),
        "iir_plan_check": ([vp, vp], i),
        "iir_plan_set_timeout_ns": ([vp, ll], i),
        "iir_plan_debug_withhold": ([vp, ll], i),
        "iir_plan_info": ([vp, ip, ip, ip, ip, ip], i),
        "iir_plan_launches_per_execute": ([vp], i),
        "iir_plan_destroy": ([vp], i),
        "iir_status_string": ([i], ctypes.c_char_p),
        "iir_version": ([], i),
        "iir_cache_clear": ([], i),
        "iir_sos_filter_debug_withhold": ([ll, ll], i),
        "iir_batch_create": ([pp, fp, ip, i, sz, sz], i),
        "iir_batch_execute": ([vp, ctypes.POINTER(IirSegment), i, vp], i),
        "iir_batch_check": ([vp, vp], i),
        "iir_batch_set_timeout_ns": ([vp, ll], i),
        "iir_batch_debug_withhold": ([vp, ll], i),
        "iir_batch_filter_sections": ([vp, i], i),
        "iir_batch_set_shape": ([vp, i, i], i),
        "iir_batch_get_shape": ([vp, ip, ip, ip, ip, ip, ip], i),
        "iir_batch_destroy": ([vp], i),
        "iir_batch_bind": ([vp, ctypes.POINTER(IirSegment), i, pp], i),
        "iir_batch_launch_bound": ([vp, vp], i),
        "iir_batch_unbind": ([vp], i),
    }
    for name, (args, res) in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def status_string(status: int) -> str:
    return load().iir_status_string(status).decode()


def check(status: int, what: str = "") -> None:
    if status != IIR_OK:
        raise IirError(status, what)


def declared_functions(header: str = HEADER) -> list[str]:
    """Names of every function declared in include/iir_gb300.h."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(iir_[a-z0-9_]+)\s*\(", text)))
