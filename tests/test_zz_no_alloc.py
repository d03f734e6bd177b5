"""iir_sos_filter_noalloc (static scratch, no allocation) against iir_sos_filter.

Collected last on purpose: it must pass both in a fresh process (the first call sets the
static array up) and after every other test has run on the device. Two calls in a row with
different filters and sizes check that the shared array carries nothing wrong from one call
to the next (launch-versioned carry slots, rewritten tables).
Tolerance: max|err| <= 1e-4 * max|ref| against the FP64 oracle (the reference's accuracy gate,
src/test_accuracy.cu:178-188) and max|noalloc - iir_sos_filter| <= 1e-6 * max|ref| (both run
the PH realization with the same geometry and tables, so they normally agree exactly).
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import _lib

pytestmark = pytest.mark.gpu


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _sos(order, cutoff):
    from scipy import signal
    return np.ascontiguousarray(signal.butter(order, cutoff, output="sos"), np.float32)


def test_noalloc_matches_sos_filter(cuda_device):
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = [(4, 0.1, 3 * 8192 * 37 + 5), (8, 0.05, 1 << 20)]
    for order, cutoff, n in cases:  # two calls in a row on the shared array
        sos = _sos(order, cutoff)
        x_np = np.random.default_rng(order).uniform(-1, 1, n).astype(np.float32)
        x = torch.from_numpy(x_np).cuda()
        y_na = torch.empty_like(x)
        y_ref = torch.empty_like(x)
        st = L.iir_sos_filter_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_na.data_ptr()), n, _fp(sos),
                                      sos.shape[0], stream)
        assert st == _lib.IIR_OK, _lib.status_string(st)
        st = L.iir_sos_filter(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_ref.data_ptr()), n, _fp(sos),
                              sos.shape[0], _lib.KERNELS["PH"], stream)
        assert st == _lib.IIR_OK, _lib.status_string(st)
        torch.cuda.synchronize()
        a, b = y_na.cpu().numpy(), y_ref.cpu().numpy()
        _, gold = oracle.reference_golden(sos, x_np)
        scale = float(np.max(np.abs(gold)))
        assert np.all(np.isfinite(a))
        assert np.max(np.abs(a - b)) <= 1e-6 * scale
        assert np.max(np.abs(a - gold)) <= 1e-4 * scale


def test_noalloc_rejects_sizes(cuda_device):
    L = _lib.load()
    sos = _sos(2, 0.1)
    x = torch.zeros(16, device="cuda")
    y = torch.zeros(16, device="cuda")
    xp, yp = ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr())
    assert L.iir_sos_filter_noalloc(xp, yp, _lib.IIR_NOALLOC_MAX_SAMPLES + 1, _fp(sos), 1, None) == \
        _lib.IIR_ERR_TOO_LARGE
    nine = np.ascontiguousarray(np.tile(sos, (9, 1)), np.float32)
    assert L.iir_sos_filter_noalloc(xp, yp, 16, _fp(nine), 9, None) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_sos_filter_noalloc(xp, xp, 16, _fp(sos), 1, None) == _lib.IIR_ERR_INVALID_ARGUMENT
