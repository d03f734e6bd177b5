"""Long signals: the steady state of every schedule against the FP64 oracle, all outputs.

At 2^26 samples the persistent two-pass schedule gives every block of its cooperative grid
20 or more chunks, so its shared-memory stage ring, its pass-A-to-pass-B lag and its ring of
per-row incoming pairs wrap many times; the cascade kernels run tens of thousands of chunks in
ticket order. Errors are compared on the device against the FP64 oracle (the reference's golden
path, tools/ref_generate.py:89). Tolerances: the reference's gate max|err| <= 1e-4 * max|ref|
(src/test_accuracy.cu:178-188), and max|err| / RMS(ref) <= 1e-5 (orders 2-8) or 2e-5 (order 16).
"""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import Plan

pytestmark = pytest.mark.gpu


def _butter(order, cutoff):
    from scipy import signal
    return signal.butter(order, cutoff, output="sos")


class _Ref:
    def __init__(self, sos, x):
        _, ref = oracle.reference_golden(sos, x)
        self.ref = torch.from_numpy(ref).cuda()
        self.maxabs = float(self.ref.abs().max())
        self.rms = float(self.ref.square().mean().sqrt())

    def check(self, y, rms_bar, what):
        assert bool(torch.isfinite(y).all()), what
        err = float((y.double() - self.ref).abs().max())
        assert err <= 1e-4 * self.maxabs, (what, err / self.maxabs)
        assert err <= rms_bar * self.rms, (what, err / self.rms)


@pytest.fixture(scope="module")
def long_signal():
    n = (1 << 26) + 12345
    x = np.random.default_rng(11).uniform(-1, 1, n).astype(np.float32)
    return x, torch.from_numpy(x).cuda()


@pytest.mark.parametrize("geom", [(32, 32), (32, 64), (32, 128), (64, 64)], ids=lambda g: f"{g[0]}x{g[1]}")
def test_two_pass_schedule_long(geom, long_signal, cuda_device):
    x, xt = long_signal
    sos = _butter(2, 0.1)
    ref = _Ref(sos, x)
    y = torch.empty_like(xt)
    for kernel in ("PH", "STCR", "STCR_UNROLL", "DTCR", "DTCR_UNROLL"):
        plan = Plan(sos, kernel, *geom, max_n=x.size)
        info = plan.info()
        chunk = 8192 if geom[1] != 32 or kernel.startswith("STCR") else 4096
        assert x.size / chunk / info["grid"] >= 20, (kernel, info)  # every block runs >= 20 chunks
        plan(xt, y)
        plan(xt, y)  # a second launch: new epoch over the same carry slots
        plan.check()
        ref.check(y, 1e-5, (kernel, geom))
        plan.close()


@pytest.mark.parametrize("order", (8, 16))
def test_cascades_long(order, long_signal, cuda_device):
    x, xt = long_signal
    sos = _butter(order, 0.1)
    ref = _Ref(sos, x)
    y = torch.empty_like(xt)
    for kernel, b, nb in (("PH", 32, 64), ("STCR_UNROLL", 32, 64), ("DTCR_UNROLL", 32, 64), ("STCR", 32, 64),
                          ("TC", 0, 0)):
        plan = Plan(sos, kernel, b, nb, max_n=x.size)
        plan(xt, y)
        plan.check()
        ref.check(y, 2e-5 if order == 16 else 1e-5, (kernel, order))
        plan.close()
