"""Failure detection without a GPU fault: a chunk withholds its carries (host-side fault
injection through iir_plan_debug_withhold), its successors' bounded waits run out, the launch
records IIR_ERR_LOOKBACK_TIMEOUT, every block returns, and the plan keeps working. The
reference's lookback spin has no bound (include/ph_kernels.cuh:397-404)."""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import IirError, Plan
from cuda_recursive_filtering_gb300._lib import IIR_ERR_LOOKBACK_TIMEOUT

pytestmark = pytest.mark.gpu


def butter(order, cutoff=0.1):
    from scipy import signal
    return signal.butter(order, cutoff, output="sos")


@pytest.mark.parametrize("kernel,order", [("PH", 4), ("PH", 2), ("DTCR_UNROLL", 4), ("DTCR_UNROLL", 2), ("STCR", 4), ("STCR", 2),
                                          ("PLR", 4), ("TC", 8), ("TC", 16)])
def test_withheld_carry_times_out_and_plan_recovers(kernel, order, cuda_device):
    """Order 2 runs the single-section persistent pipeline, order 4 the per-chunk blocks, TC the
    precision form's tile pipeline (chunk 7 = tile 7)."""
    sos = butter(order)
    n = 1 << 20
    x = np.random.default_rng(0).uniform(-1, 1, n).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    plan = Plan(sos, kernel, max_n=n)
    plan.set_timeout_ns(20_000_000)  # 20 ms
    plan.debug_withhold(7)
    plan(xt)
    with pytest.raises(IirError) as ei:
        plan.check()
    assert ei.value.status == IIR_ERR_LOOKBACK_TIMEOUT
    # the next launch on the same plan is unaffected
    y = plan(xt)
    plan.check()
    _, ref = oracle.reference_golden(sos, x)
    assert oracle.errors(y.cpu().numpy(), ref)["rel_max"] <= 1e-4


@pytest.mark.parametrize("order", [2, 4])
def test_one_shot_reports_device_failure_on_a_later_call(order, cuda_device):
    """iir_sos_filter returns before its launch runs, so a lookback timeout of that launch is
    reported by the next call on the same cached plan (which launches nothing), or by
    iir_cache_clear; the calls after it filter correctly again."""
    import ctypes

    from cuda_recursive_filtering_gb300 import _lib
    L = _lib.load()
    sos = np.ascontiguousarray(butter(order), np.float32)
    n = 1 << 20
    x = np.random.default_rng(1).uniform(-1, 1, n).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    yt = torch.zeros_like(xt)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    fp = sos.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def call():
        return L.iir_sos_filter(ctypes.c_void_p(xt.data_ptr()), ctypes.c_void_p(yt.data_ptr()), n, fp,
                                sos.shape[0], _lib.KERNELS["PH"], stream)

    assert L.iir_cache_clear() == _lib.IIR_OK
    assert call() == _lib.IIR_OK
    assert L.iir_sos_filter_debug_withhold(7, 20_000_000) == _lib.IIR_OK
    assert call() == _lib.IIR_OK  # the failure happens on the device, after the call returned
    torch.cuda.synchronize()
    yt.zero_()
    assert call() == IIR_ERR_LOOKBACK_TIMEOUT
    torch.cuda.synchronize()
    assert float(yt.abs().max()) == 0.0  # the reporting call launched nothing
    assert call() == _lib.IIR_OK
    torch.cuda.synchronize()
    _, ref = oracle.reference_golden(sos, x)
    assert oracle.errors(yt.cpu().numpy(), ref)["rel_max"] <= 1e-4
    # reported by iir_cache_clear when no call follows
    assert L.iir_sos_filter_debug_withhold(3, 20_000_000) == _lib.IIR_OK
    assert call() == _lib.IIR_OK
    assert L.iir_cache_clear() == IIR_ERR_LOOKBACK_TIMEOUT
    assert L.iir_cache_clear() == _lib.IIR_OK


def test_one_shot_cache_is_bounded(cuda_device):
    """More distinct filters than the one-shot cache holds: the least recently used plans are
    freed (device memory comes back) and every call still filters correctly."""
    import ctypes

    from cuda_recursive_filtering_gb300 import _lib
    L = _lib.load()
    n = 1 << 16
    x = np.random.default_rng(2).uniform(-1, 1, n).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.iir_cache_clear() == _lib.IIR_OK
    free_full = None
    for i in range(80):
        sos = np.ascontiguousarray(butter(4, 0.05 + 0.004 * i), np.float32)
        st = L.iir_sos_filter(ctypes.c_void_p(xt.data_ptr()), ctypes.c_void_p(yt.data_ptr()), n,
                              sos.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 2, _lib.KERNELS["PH"], stream)
        assert st == _lib.IIR_OK
        if i % 20 == 19:
            torch.cuda.synchronize()
            _, ref = oracle.reference_golden(sos, x)
            assert oracle.errors(yt.cpu().numpy(), ref)["rel_max"] <= 1e-4
        if i == 31:  # the cache is full from here on
            torch.cuda.synchronize()
            free_full = torch.cuda.mem_get_info()[0]
    torch.cuda.synchronize()
    grown = free_full - torch.cuda.mem_get_info()[0]
    assert L.iir_cache_clear() == _lib.IIR_OK
    # 48 more filters replaced cached plans instead of adding to them
    assert grown < 16 * (1 << 20), grown
