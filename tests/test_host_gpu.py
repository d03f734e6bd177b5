"""GPU parity of iir_plan_execute_host: host buffers in, host buffers out, through the C ABI.

Single-section plans on the two-pass schedule run the signal in pieces whose copies overlap
the filtering, and each piece starts from the state the previous one left (its last two
inputs and outputs). Tolerances as the other parity tests: the reference's gate
max|err| <= 1e-4 * max|ref| (src/test_accuracy.cu:178-188) and max|err| / RMS(ref) <= 1e-5 at
order 2 (2e-5 at order 16); the piecewise output agrees with the one-launch device output to
1e-6 * max|ref| (3e-5 for poles at radius 0.96, where the float32 round-off of either path is
about 1e-5 of max|ref|).
"""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import Plan, PlrPlan  # noqa: F401

pytestmark = pytest.mark.gpu


def butter(order, cutoff=0.1):
    from scipy import signal
    return signal.butter(order, cutoff, output="sos")


def golden(sos, x):
    return oracle.reference_golden(sos, x)[1]


def host(x, pinned=True):
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32))
    return t.pin_memory() if pinned else t


def device_run(plan, x):
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    y = plan(xd)
    plan.check()
    return y.cpu().numpy()


@pytest.mark.parametrize("kernel", ["DTCR_UNROLL", "PH", "STCR_UNROLL", "DTCR", "STCR"])
@pytest.mark.parametrize("cutoff", [0.1, 0.01])
def test_pieces_carry_state(kernel, cutoff, cuda_device):
    sos = butter(2, cutoff)
    piece = 50000
    n = 5 * piece + 777
    x = np.random.default_rng(11).uniform(-1, 1, n).astype(np.float32)
    ref = golden(sos, x)
    plan = Plan(sos, kernel, 32, 64, max_n=n)
    y = plan.filter_host(host(x), piece=piece)
    plan.check()
    y = y.numpy()
    e = oracle.errors(y, ref)
    yd = device_run(plan, x)
    ed = oracle.errors(yd, ref)
    # cutoff 0.01 (poles at radius 0.96): float32 round-off of the one-launch path itself is
    # above 1e-5 of the output RMS there, so the pieces are held to the one-launch error
    assert e["finite"] and e["rel_max"] <= 1e-4 and e["rel_rms"] <= max(1e-5, 1.5 * ed["rel_rms"]), (e, ed)
    d = np.max(np.abs(y.astype(np.float64) - yd)) / np.max(np.abs(ref))
    assert d <= (1e-6 if cutoff >= 0.1 else 3e-5), d


@pytest.mark.parametrize("n,piece", [(3 * 4096 + 1, 4096), (4 * 8192, 8192), (1000, 0), (2, 1024),
                                     ((1 << 22) + 5, 1 << 20)])
def test_piece_edges(n, piece, cuda_device):
    """Last piece of one sample, pieces that divide n, a signal shorter than one chunk."""
    sos = butter(2, 0.05)
    x = np.random.default_rng(n).uniform(-1, 1, n).astype(np.float32)
    plan = Plan(sos, "DTCR_UNROLL", 32, 64, max_n=1024)
    y = plan.filter_host(host(x), piece=piece)
    plan.check()
    e = oracle.errors(y.numpy(), golden(sos, x))
    assert e["rel_max"] <= 1e-4, e


def test_pageable_buffers_and_repeated_calls(cuda_device):
    """Pageable host memory works (copies are not overlapped); the staging buffers grow and
    are reused, and device launches of the same plan still follow."""
    sos = butter(2)
    plan = Plan(sos, "PH", 32, 64, max_n=1 << 16)
    for i, (n, piece, pinned) in enumerate([(100000, 30000, False), (300000, 70000, True), (5000, 0, True)]):
        x = np.random.default_rng(i).uniform(-1, 1, n).astype(np.float32)
        y = plan.filter_host(host(x, pinned), piece=piece)
        plan.check()
        assert oracle.errors(y.numpy(), golden(sos, x))["rel_max"] <= 1e-4, (n, piece)
        assert oracle.errors(device_run(plan, x), golden(sos, x))["rel_max"] <= 1e-4


@pytest.mark.parametrize("kernel,order", [("PH", 8), ("STCR_UNROLL", 4), ("TC", 16), ("PLR", 4)])
def test_other_plans_stage_whole_signal(kernel, order, cuda_device):
    sos = butter(order)
    n = 200000 + 3
    x = np.random.default_rng(order).uniform(-1, 1, n).astype(np.float32)
    plan = Plan(sos, kernel, max_n=n)
    y = plan.filter_host(host(x), piece=10000)
    plan.check()
    e = oracle.errors(y.numpy(), golden(sos, x))
    assert e["finite"] and e["rel_max"] <= 1e-4, e


def test_rejects_device_tensors(cuda_device):
    plan = Plan(butter(2), "PH", max_n=1024)
    with pytest.raises(ValueError):
        plan.filter_host(torch.zeros(1024, device="cuda"))
