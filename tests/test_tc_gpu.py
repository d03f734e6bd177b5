"""Precision form (IIR_KERNEL_TC): the cascade's chunk solve as tcgen05 TF32 GEMMs with split
(3-term) products (and GEMM 1 with BF16 split operands), chunk states joined by a D-dimensional
scan and decoupled lookback. Against
the FP64 oracle: max|err| <= 1e-4 * max|ref| (the reference's gate, src/test_accuracy.cu:178-188)
and max|err| / RMS(ref) <= 1e-5 at every order (the precision form's target)."""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import Plan, workloads

pytestmark = pytest.mark.gpu


def _check(y, x, sos, rms_tol=1e-5):
    _, ref = oracle.reference_golden(sos, x)
    e = oracle.errors(y, ref)
    assert e["finite"], e
    assert e["rel_max"] <= 1e-4, e
    assert e["rel_rms"] <= rms_tol, e
    return e


@pytest.mark.parametrize("order", (2, 4, 8, 16))
def test_tc_sizes(order, cuda_device):
    from scipy import signal
    sos = signal.butter(order, 0.1, output="sos")
    sizes = [1, 63, 64, 65, 8191, 8192, 8193, 3 * 8192 + 5, 160 * 8192 + 1234, (1 << 22) + 7]
    plan = Plan(sos, "TC", max_n=max(sizes))
    rng = np.random.default_rng(order)
    for n in sizes:
        x = rng.uniform(-1, 1, n).astype(np.float32)
        y = plan(torch.from_numpy(x).cuda())
        plan.check()
        if n >= 64:
            _check(y.cpu().numpy(), x, sos)


@pytest.mark.parametrize("order", (8, 16))
def test_tc_noise_plus_tones(order, cuda_device):
    """butter(order, 0.05) on N(0,1) noise plus 8 sinusoids spanning 60 dB (seed 2)."""
    from scipy import signal
    sos = signal.butter(order, 0.05, output="sos")
    xt = workloads.noise_plus_tones(1 << 21, 2)
    plan = Plan(sos, "TC", max_n=xt.numel())
    y = plan(xt)
    plan.check()
    _check(y.cpu().numpy(), xt.cpu().numpy(), sos)


def test_tc_unaligned_and_repeated(cuda_device):
    from scipy import signal
    sos = signal.butter(8, 0.1, output="sos")
    n = 50 * 8192 + 3
    x = np.random.default_rng(3).uniform(-1, 1, n).astype(np.float32)
    base = torch.zeros(n + 1, device="cuda")
    base[1:] = torch.from_numpy(x).cuda()
    plan = Plan(sos, "TC", max_n=n)
    out = torch.empty(n + 1, device="cuda")[1:]
    for _ in range(3):
        plan(base[1:], out)  # element-wise staging (unaligned)
    plan.check()
    _check(out.cpu().numpy(), x, sos)
    xt = torch.from_numpy(x).cuda()
    for _ in range(20):
        y = plan(xt)
    plan.check()
    _check(y.cpu().numpy(), x, sos)


def test_tc_slow_decay_full_lookback(cuda_device):
    """A resonance with pole radius 0.99995: the tile transition Phi^128 keeps 66% of the state
    over a tile, so the truncated lookback does not apply and tiles are joined by the full
    two-level decoupled lookback."""
    r, th = 0.99995, 0.01
    sos = np.array([[1e-4, 0.0, 0.0, 1.0, -2 * r * np.cos(th), r * r],
                    [1.0, 0.0, 0.0, 1.0, -1.6, 0.64]])
    n = 300 * 8192 + 11
    x = np.random.default_rng(5).uniform(-1, 1, n).astype(np.float32)
    plan = Plan(sos, "TC", max_n=n)
    y = plan(torch.from_numpy(x).cuda())
    plan.check()
    _check(y.cpu().numpy(), x, sos, rms_tol=1e-4)


@pytest.mark.parametrize("order", (2, 8, 16))
def test_tc_long_signal(order, cuda_device):
    """2^26 + 12345 samples: about 54 tiles per block, so every hand-off slot, x buffer and
    accumulator of the tile pipeline is reused many times within one launch (order 8: the
    tile split shared by both compute groups, the BF16 form of GEMM 1)."""
    from scipy import signal
    sos = signal.butter(order, 0.05, output="sos")
    n = (1 << 26) + 12345
    xt = workloads.uniform_signal(n, 7)
    plan = Plan(sos, "TC", max_n=n)
    for _ in range(2):
        y = plan(xt)
    plan.check()
    _check(y.cpu().numpy(), xt.cpu().numpy(), sos)


@pytest.mark.parametrize("order,cutoff", [(8, 0.02), (16, 0.05), (16, 0.3)])
def test_tc_cheby1(order, cutoff, cuda_device):
    """Chebyshev type I (1 dB ripple): poles closer to the unit circle than Butterworth's of the
    same order, the harder case for the state basis."""
    from scipy import signal
    sos = signal.cheby1(order, 1.0, cutoff, output="sos")
    n = (1 << 21) + 5
    x = np.random.default_rng(order).uniform(-1, 1, n).astype(np.float32)
    plan = Plan(sos, "TC", max_n=n)
    y = plan(torch.from_numpy(x).cuda())
    plan.check()
    _check(y.cpu().numpy(), x, sos, rms_tol=2e-5)


@pytest.mark.parametrize("order", (8, 16))
@pytest.mark.parametrize("form", ("6", "3", "0"))
def test_tc_bf16_split_forms(order, form, monkeypatch, cuda_device):
    """GEMM 1's operand form forced by IIR_GB300_TC_BF16 (read when the plan is created) on the
    precision workload, including ragged sizes: BF16 split operands with three parts and six
    products (the default up to 8 states) keep the float32 bar (max|err| / RMS <= 1e-5), as
    TF32 hi / lo operands ("0", the default with 16 states) do; two parts and three products keep
    the reference's gate (max|err| <= 1e-4 max|ref|) at about 4e-5 RMS, so their RMS bound here
    is 1e-4."""
    from scipy import signal
    sos = signal.butter(order, 0.05, output="sos")
    monkeypatch.setenv("IIR_GB300_TC_BF16", form)
    xt = workloads.noise_plus_tones(1 << 21, 2)
    plan = Plan(sos, "TC", max_n=xt.numel())
    monkeypatch.delenv("IIR_GB300_TC_BF16")
    for n in (xt.numel(), 8192 * 37 + 11, 100):
        y = plan(xt[:n])
        plan.check()
        _check(y.cpu().numpy(), xt[:n].cpu().numpy(), sos, rms_tol=1e-5 if form == "6" else 1e-4)
