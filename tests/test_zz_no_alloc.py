"""iir_sos_filter_noalloc (static scratch, no allocation) against iir_sos_filter.

The entry point exists for callers that cannot allocate device memory while they filter — a
real-time callback with a deadline, or a host whose device memory belongs to another allocator
— since cudaMalloc / cudaFree can synchronise the device and can fail under memory pressure.

Collected last on purpose: it must pass both in a fresh process (the first call sets the
static array up) and after every other test has run on the device. Consecutive calls with
different filters and sizes check that the shared array carries nothing wrong from one call
to the next (launch-versioned carry slots, rewritten tables).
Tolerances (the ones the parity tests use): against the FP64 oracle, max|err| <= 1e-4 *
max|ref| (the reference's gate, src/test_accuracy.cu:178-188) and max|err| / RMS(ref) <= 1e-5
(2e-5 at order 16). Against iir_sos_filter: max|noalloc - iir_sos_filter| <= 1e-5 * max|ref|,
the bound the parity tests put on two schedules of one realization (this entry point runs the
PH kernel with one lookback per section; iir_sos_filter may pick another schedule of PH for the
same filter, so the two agree to rounding, not bit for bit).
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


def _call_noalloc(L, x, y, n, sos, stream):
    return L.iir_sos_filter_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), n, _fp(sos),
                                    sos.shape[0], stream)


def test_noalloc_matches_sos_filter(cuda_device):
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    max_n = _lib.IIR_NOALLOC_MAX_SAMPLES
    cases = [(4, 0.1, 3 * 8192 * 37 + 5), (8, 0.05, 1 << 20), (2, 0.1, (1 << 20) + 3),
             (16, 0.1, max_n), (16, 0.1, max_n - 1), (2, 0.1, max_n)]
    for order, cutoff, n in cases:  # consecutive calls on the shared array
        sos = _sos(order, cutoff)
        x_np = np.random.default_rng(order + n % 7).uniform(-1, 1, n).astype(np.float32)
        x = torch.from_numpy(x_np).cuda()
        y_na = torch.empty_like(x)
        y_ref = torch.empty_like(x)
        st = _call_noalloc(L, x, y_na, n, sos, stream)
        assert st == _lib.IIR_OK, _lib.status_string(st)
        st = L.iir_sos_filter(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_ref.data_ptr()), n, _fp(sos),
                              sos.shape[0], _lib.KERNELS["PH"], stream)
        assert st == _lib.IIR_OK, _lib.status_string(st)
        torch.cuda.synchronize()
        a, b = y_na.cpu().numpy(), y_ref.cpu().numpy()
        _, gold = oracle.reference_golden(sos, x_np)
        e = oracle.errors(a, gold)
        scale = float(np.max(np.abs(gold)))
        assert e["finite"], (order, n)
        assert e["rel_max"] <= 1e-4, (order, n, e)
        assert e["rel_rms"] <= (2e-5 if order == 16 else 1e-5), (order, n, e)
        assert np.max(np.abs(a - b)) <= 1e-5 * scale, (order, n)
        del x, y_na, y_ref


def test_noalloc_allocates_nothing(cuda_device):
    """After one call (which sets the array up on a fresh process), a hundred more leave the
    device's free memory exactly where it was."""
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = (1 << 20) + 17
    x = torch.rand(n, device="cuda") * 2 - 1
    y = torch.empty_like(x)
    sos8, sos2 = _sos(8, 0.1), _sos(2, 0.2)
    assert _call_noalloc(L, x, y, n, sos8, stream) == _lib.IIR_OK
    assert _call_noalloc(L, x, y, n, sos2, stream) == _lib.IIR_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for i in range(100):
        assert _call_noalloc(L, x, y, n, sos8 if i % 2 else sos2, stream) == _lib.IIR_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


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
