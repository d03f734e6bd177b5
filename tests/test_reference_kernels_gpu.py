"""The reference's own GPU kernels against this library on the same inputs: PH_32, STCR_32_LOOP,
STCR_32_UNROLL_64, DTCR_32_LOOP and DTCR_32_UNROLL_64 (include/{ph,stcr,dtcr}_kernels.cuh at
BLOCK_SIZE 32, N_BLOCKS 64),
compiled from the reference's sources into device code and launched under its own contract
(oracle/refgpu.py). Both meet the reference's gate against the FP64 oracle (max|err| <= 1e-4
max|ref|, src/test_accuracy.cu:178-188), and this library's output of the same realization and
geometry agrees with the reference kernel's within 1e-5 of the output's peak (both are float32; each is within about 1e-6 of
FP64 here). Skipped where the cubins were not built (they need the reference's sources)."""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import Plan, workloads
from oracle import refgpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refgpu.available(), reason="reference kernels not built (oracle/_ref)")]


@pytest.mark.parametrize("kernel", tuple(refgpu.KERNELS))
@pytest.mark.parametrize("order", (2, 4, 8, 16))
def test_reference_kernel_agrees_with_library(kernel, order, cuda_device):
    from scipy import signal
    sos = signal.butter(order, 0.1, output="sos")
    n = 300 * refgpu.CHUNK  # whole chunks: the reference's kernels take no ragged tail
    x = workloads.uniform_signal(n, order, device="cuda")
    _, gold = oracle.reference_golden(sos, x.cpu().numpy())
    scale = float(np.max(np.abs(gold)))
    sn, g = oracle.normalise_sos(sos)
    rk = refgpu.RefKernel(kernel, sn, n)
    y_ref = torch.empty_like(x)
    xs = (x * np.float32(g)).contiguous()
    for _ in range(3):  # launch indices 0, 1, 2 on one status buffer
        y_ref.fill_(float("nan"))
        rk(xs, y_ref)
        torch.cuda.synchronize()
        e_ref = oracle.errors(y_ref.cpu().numpy(), gold)
        assert e_ref["finite"] and e_ref["rel_max"] <= 1e-4, e_ref
    rk.close()
    plan = Plan(sos, kernel, 32, 64, max_n=n)
    y = plan(x)
    plan.check()
    e = oracle.errors(y.cpu().numpy(), gold)
    assert e["rel_max"] <= 1e-4, e
    assert float((y - y_ref).abs().max()) <= 1e-5 * scale
