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
