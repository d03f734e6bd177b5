"""CUDA-graph capture of plain plans: a plan's launch keeps its launch epoch on the device (the
reference's status contract, ph_kernels.cuh:16-29, with the index advanced by the last block),
so a captured launch replays correctly any number of times."""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import Plan

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel,order", [("DTCR_UNROLL", 2), ("PH", 2), ("PH", 8), ("STCR_UNROLL", 4), ("TC", 16)])
def test_plan_replays_in_a_cuda_graph(kernel, order, cuda_device):
    from scipy import signal
    sos = signal.butter(order, 0.1, output="sos")
    n = (1 << 22) + 17
    plan = Plan(sos, kernel, max_n=n)
    x = torch.empty(n, device="cuda")
    y = torch.empty(n, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        x.uniform_(-1, 1)
        plan(x, y, stream=s)  # first launch outside the capture
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan(x, y, stream=s)
    for seed in range(3):
        xn = np.random.default_rng(seed).uniform(-1, 1, n).astype(np.float32)
        x.copy_(torch.from_numpy(xn))
        y.zero_()
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        plan.check()
        _, ref = oracle.reference_golden(sos, xn)
        e = oracle.errors(y.cpu().numpy(), ref)
        assert e["rel_max"] <= 1e-4, (seed, e)
