"""Batched segments (iir_batch_*): many independent signals with their own filters in one
launch, streams continued across launches through device-resident state, against the FP64
oracle. Tolerance: the reference's gate max|err| <= 1e-4 * max|ref| (src/test_accuracy.cu:178-188)
and max|err| / RMS(ref) <= 1e-5 at orders 2-8, 2e-5 at order 16.
"""
import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import Batch, IirError
from cuda_recursive_filtering_gb300._lib import IIR_ERR_LOOKBACK_TIMEOUT

pytestmark = pytest.mark.gpu

RMS_TOL = {2: 1e-5, 4: 1e-5, 6: 1e-5, 8: 1e-5, 16: 2e-5}


def _filters():
    from scipy import signal
    out = []
    for order, cutoff in ((2, 0.1), (4, 0.2), (8, 0.1), (16, 0.1), (2, 0.4), (8, 0.3)):
        out.append((order, signal.butter(order, cutoff, output="sos")))
    for order, cutoff in ((4, 0.15), (6, 0.3)):
        out.append((order, signal.cheby1(order, 1.0, cutoff, output="sos")))
    return out


def _check(y, x, sos, order, what):
    _, ref = oracle.reference_golden(sos, x)
    e = oracle.errors(y, ref)
    assert e["finite"], (what, e)
    assert e["rel_max"] <= 1e-4, (what, e)
    if x.size >= 64:
        assert e["rel_rms"] <= RMS_TOL[order], (what, e)


def test_many_channels_uneven_lengths(cuda_device):
    filters = _filters()
    batch = Batch([s for _, s in filters])
    rng = np.random.default_rng(11)
    lengths = [0, 1, 2, 3, 31, 4095, 4096, 4097, 3 * 4096 + 7, 40 * 4096 + 1]
    lengths += [int(v) for v in np.exp(rng.uniform(np.log(1 << 8), np.log(1 << 17), 40)).astype(int)]
    chans = []
    for i, n in enumerate(lengths):
        f = int(rng.integers(len(filters)))
        x = rng.uniform(-1, 1, n).astype(np.float32)
        xt = torch.from_numpy(x).cuda()
        chans.append((x, xt, torch.full_like(xt, float("nan")), f))
    batch([(xt, yt, f) for _, xt, yt, f in chans])
    batch.check()
    for i, (x, _, yt, f) in enumerate(chans):
        if x.size:
            _check(yt.cpu().numpy(), x, filters[f][1], filters[f][0], ("channel", i, x.size, f))


def test_stream_in_pieces_matches_whole(cuda_device):
    """One stream cut into random pieces, filtered launch after launch with the state kept on
    the device (zi of a piece = zf of the one before): the pieces join into the whole-signal
    output."""
    filters = _filters()
    batch = Batch([s for _, s in filters])
    rng = np.random.default_rng(12)
    for f in (0, 2, 3, 6):
        n = 150_000
        x = rng.uniform(-1, 1, n).astype(np.float32)
        xt = torch.from_numpy(x).cuda()
        yt = torch.empty_like(xt)
        st = [torch.zeros(batch.state_size(f), device="cuda") for _ in range(2)]
        pos, turn = 0, 0
        cuts = [1, 2, 1, 4096, 4097, 3, 10000]
        while pos < n:
            m = cuts.pop(0) if cuts else int(rng.integers(1, 20000))
            m = min(m, n - pos)
            batch([(xt[pos:pos + m], yt[pos:pos + m], f, st[turn], st[turn ^ 1])])
            pos += m
            turn ^= 1
        batch.check()
        _check(yt.cpu().numpy(), x, filters[f][1], filters[f][0], ("stream", f))


def test_interleaved_streams_continuous_batching(cuda_device):
    """Several live streams with different filters; every launch takes the next piece of a
    random subset of them (continuous batching). Each stream joins into its whole output."""
    filters = _filters()
    batch = Batch([s for _, s in filters])
    rng = np.random.default_rng(13)
    streams = []
    for sidx in range(8):
        f = sidx % len(filters)
        n = int(rng.integers(20_000, 80_000))
        x = rng.uniform(-1, 1, n).astype(np.float32)
        xt = torch.from_numpy(x).cuda()
        streams.append({"f": f, "x": x, "xt": xt, "yt": torch.empty_like(xt), "pos": 0, "turn": 0,
                        "st": [torch.zeros(batch.state_size(f), device="cuda") for _ in range(2)]})
    while any(s["pos"] < s["x"].size for s in streams):
        segs = []
        for s in streams:
            if s["pos"] >= s["x"].size or rng.random() < 0.3:
                continue
            m = min(int(rng.integers(1, 9000)), s["x"].size - s["pos"])
            p0 = s["pos"]
            segs.append((s["xt"][p0:p0 + m], s["yt"][p0:p0 + m], s["f"], s["st"][s["turn"]], s["st"][s["turn"] ^ 1]))
            s["pos"] += m
            s["turn"] ^= 1
        if segs:
            batch(segs)
    batch.check()
    for i, s in enumerate(streams):
        _check(s["yt"].cpu().numpy(), s["x"], filters[s["f"]][1], filters[s["f"]][0], ("stream", i))


def test_batch_withheld_carry_times_out_and_recovers(cuda_device):
    filters = _filters()
    batch = Batch([s for _, s in filters])
    batch.set_timeout_ns(20_000_000)
    rng = np.random.default_rng(14)
    x = rng.uniform(-1, 1, 50 * 4096).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    batch.debug_withhold(5)
    batch([(xt, yt, 2)])
    with pytest.raises(IirError) as ei:
        batch.check()
    assert ei.value.status == IIR_ERR_LOOKBACK_TIMEOUT
    batch([(xt, yt, 2)])
    batch.check()
    _check(yt.cpu().numpy(), x, filters[2][1], filters[2][0], "recovered")
