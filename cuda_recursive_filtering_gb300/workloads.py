"""Seeded synthetic workloads (the reference benchmarks on synthetic signals only).

  plain_order2_small   butter(2, 0.1) SOS, 2^16 samples uniform[-1,1], seed 0
  plain_sweep          butter(order, 0.1) SOS, orders 2/4/8/16, 2^25 or 2^28 samples
                       uniform[-1,1], seed 1
  precision            butter(8|16, 0.05), 2^28 samples N(0,1) + 8 sinusoids at frequencies
                       U[0, 0.5) (cycles/sample) with amplitudes spanning 60 dB, seed 2
  multichannel_mixed   4096 channels, lengths log-uniform in [2^10, 2^20], each its own filter:
                       order in {2, 4, 8, 16}, butter or cheby1 (1 dB ripple), cutoff U[0.02, 0.45],
                       seed 3
  streaming_poisson    1024 streams, each an order-8 butter with cutoff U[0.05, 0.4]; chunk lengths
                       uniform in [256, 65536]; Poisson arrivals at 2e9 samples/s in aggregate, seed 4
Large inputs are generated on the device with torch (plumbing only) so a 2^28-sample signal
does not need a host round trip.
"""
from __future__ import annotations

import numpy as np
import torch


def butter_sos(order: int, cutoff: float) -> np.ndarray:
    from scipy import signal
    return signal.butter(order, cutoff, output="sos")


def uniform_signal(n: int, seed: int, device="cuda") -> torch.Tensor:
    """float32 i.i.d. uniform[-1, 1)."""
    if device == "cpu" or n <= (1 << 22):
        x = np.random.default_rng(seed).uniform(-1.0, 1.0, n).astype(np.float32)
        t = torch.from_numpy(x)
        return t if device == "cpu" else t.to(device)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    return torch.rand(n, generator=g, device=device, dtype=torch.float32).mul_(2.0).sub_(1.0)


def noise_plus_tones(n: int, seed: int, device="cuda") -> torch.Tensor:
    """N(0,1) noise plus 8 sinusoids, frequencies U[0, 0.5) cycles/sample, amplitudes
    log-spaced over 60 dB (1 .. 1e-3), random phases."""
    rng = np.random.default_rng(seed)
    freqs = rng.uniform(0.0, 0.5, 8)
    amps = 10.0 ** (-3.0 * rng.permutation(np.linspace(0.0, 1.0, 8)))
    phases = rng.uniform(0.0, 2 * np.pi, 8)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    x = torch.randn(n, generator=g, device=device, dtype=torch.float32)
    i = torch.arange(n, device=device, dtype=torch.float64)
    for f, a, p in zip(freqs, amps, phases):
        # phase reduced in float64 before the float32 sin
        ph = torch.remainder(2.0 * np.pi * f * i + p, 2.0 * np.pi)
        x += (a * torch.sin(ph)).to(torch.float32)
    return x


def plain_order2_small(device="cuda"):
    return butter_sos(2, 0.1), uniform_signal(1 << 16, 0, device)


def plain_sweep(order: int, log2n: int, device="cuda"):
    return butter_sos(order, 0.1), uniform_signal(1 << log2n, 1, device)


def precision(order: int, log2n: int = 28, device="cuda"):
    return butter_sos(order, 0.05), noise_plus_tones(1 << log2n, 2, device)


def multichannel_mixed(n_channels: int = 4096, seed: int = 3):
    """Returns (filters, lengths): one SOS array per channel and the channel lengths."""
    from scipy import signal
    rng = np.random.default_rng(seed)
    orders = rng.choice([2, 4, 8, 16], n_channels)
    kinds = rng.choice(["butter", "cheby1"], n_channels)
    cut = rng.uniform(0.02, 0.45, n_channels)
    lens = np.exp(rng.uniform(np.log(2 ** 10), np.log(2 ** 20), n_channels)).astype(np.int64)
    filters = [signal.butter(int(o), float(c), output="sos") if k == "butter"
               else signal.cheby1(int(o), 1.0, float(c), output="sos") for o, k, c in zip(orders, kinds, cut)]
    return filters, lens


def streaming_poisson(n_streams: int = 1024, seed: int = 4):
    """Returns (filters, params): one order-8 butter per stream and the load parameters
    (aggregate samples/s, chunk length range, seed) for serving.run_poisson_load."""
    from scipy import signal
    rng = np.random.default_rng(seed)
    filters = [signal.butter(8, float(c), output="sos") for c in rng.uniform(0.05, 0.4, n_streams)]
    return filters, {"rate_sps": 2e9, "chunk_lo": 256, "chunk_hi": 65536, "seed": seed}
