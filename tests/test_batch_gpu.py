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


def test_packed_segments_match_list_call(cuda_device):
    """The array-built segment table (Batch.packed) gives the same output as the list call,
    including per-segment states in the rows of a (segments, state) tensor."""
    filters = _filters()
    batch = Batch([s for _, s in filters])
    rng = np.random.default_rng(15)
    lens = rng.integers(0, 30_000, 37)
    off = np.concatenate([[0], np.cumsum(lens)])
    flt = rng.integers(0, len(filters), lens.size)
    x = torch.from_numpy(rng.uniform(-1, 1, int(off[-1])).astype(np.float32)).cuda()
    width = max(batch.state_size(int(f)) for f in flt)
    zi = torch.from_numpy(rng.uniform(-0.5, 0.5, (lens.size, width)).astype(np.float32)).cuda()
    zf1 = torch.zeros_like(zi)
    zf2 = torch.zeros_like(zi)
    y1 = torch.empty_like(x)
    y2 = torch.empty_like(x)
    batch.packed(x, y1, off, flt, zi=zi, zf=zf1)
    segs = [(x[off[i]:off[i + 1]], y2[off[i]:off[i + 1]], int(flt[i]),
             zi[i, :batch.state_size(int(flt[i]))], zf2[i, :batch.state_size(int(flt[i]))]) for i in range(lens.size)]
    batch(segs)
    batch.check()
    assert torch.allclose(y1, y2, rtol=0, atol=1e-5 * float(y2.abs().max()))
    nz = torch.from_numpy(lens > 0).cuda()
    assert torch.allclose(zf1[nz], zf2[nz], rtol=0, atol=1e-5 * float(zf2.abs().max() + 1))


def test_bound_batch_replays_in_a_cuda_graph(cuda_device):
    """A bound segment table launches with one kernel launch per call; captured into a CUDA
    graph and replayed it gives the same output as the uncaptured launch."""
    filters = _filters()
    batch = Batch([s for _, s in filters])
    rng = np.random.default_rng(16)
    lens = rng.integers(1, 20_000, 24)
    off = np.concatenate([[0], np.cumsum(lens)])
    flt = rng.integers(0, len(filters), lens.size)
    x = torch.from_numpy(rng.uniform(-1, 1, int(off[-1])).astype(np.float32)).cuda()
    y_direct = torch.empty_like(x)
    y_graph = torch.zeros_like(x)
    batch.packed(x, y_direct, off, flt)
    batch.check()
    bound = batch.bind(x, y_graph, off, flt)
    bound()
    torch.cuda.synchronize()
    assert torch.allclose(y_graph, y_direct, rtol=0, atol=1e-6 * float(y_direct.abs().max()))
    y_graph.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        bound()
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    batch.check()
    assert torch.allclose(y_graph, y_direct, rtol=0, atol=1e-6 * float(y_direct.abs().max()))
    bound.close()


def _resonator(w, r):
    """Band-pass biquad with poles r e^(+-i pi w): its state decays as r^n."""
    g = (1.0 - r * r) / 2.0
    return np.array([[g, 0.0, -g, 1.0, -2.0 * r * np.cos(np.pi * w), r * r]])


def _mixed_filters():
    """Filters on both schedules. Most decay within half a chunk (tail aggregate). Two take the
    per-section lookback at every shape: a resonator of pole radius 0.996 (12 pieces of 512
    samples to decay to 1e-10, more than the 8 the schedule allows) alone and behind a
    butter(14, 0.6). Their poles are away from z = 1, so float32 filters them as well as any
    other filter here (a sequential float32 cascade is within 2e-6 RMS of FP64); a low-cutoff
    filter with the same decay, butter(2, 0.003), is not (1.7e-4 sequentially)."""
    from scipy import signal
    res = _resonator(0.5, 0.996)
    return _filters() + [(2, res), (16, np.vstack([signal.butter(14, 0.6, output="sos"), res]))]


SCHEDULES = ["per_section", "tail"]


def _schedule(monkeypatch, schedule):
    """The batch's schedule for later launches: the per-section lookback (default) or, for every
    segment whose filter's state decays within half a chunk, the tail aggregate."""
    if schedule == "tail":
        monkeypatch.setenv("IIR_GB300_BATCH_TAIL_CHUNKS", "1")
    else:
        monkeypatch.delenv("IIR_GB300_BATCH_TAIL_CHUNKS", raising=False)


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("shape", [(128, 64), (128, 32), (128, 16), (64, 16)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_every_chunk_shape(shape, schedule, monkeypatch, cuda_device):
    """Every compiled chunk shape of the persistent batch kernel, channels of many lengths around
    the chunk size, with both schedules, two launches in a row (new epoch, same slots)."""
    _schedule(monkeypatch, schedule)
    filters = _mixed_filters()
    batch = Batch([s for _, s in filters])
    batch.set_shape(*shape)
    sh = batch.shape()
    assert (sh["rows"], sh["samples_per_row"]) == shape and sh["blocks_per_sm"] > 0
    chunk = sh["chunk"]
    rng = np.random.default_rng(shape[1])
    lengths = [1, 5, chunk - 1, chunk, chunk + 1, 3 * chunk + 17, 20 * chunk + 5]
    lengths += [int(v) for v in rng.integers(1, 30 * chunk, 24)]
    chans = []
    for i, n in enumerate(lengths):
        f = i % len(filters)
        x = rng.uniform(-1, 1, n).astype(np.float32)
        xt = torch.from_numpy(x).cuda()
        chans.append((x, xt, torch.empty_like(xt), f))
    for launch in range(2):
        for _, _, yt, _ in chans:
            yt.fill_(float("nan"))
        batch([(xt, yt, f) for _, xt, yt, f in chans])
        batch.check()
        for i, (x, _, yt, f) in enumerate(chans):
            _check(yt.cpu().numpy(), x, filters[f][1], filters[f][0], (shape, launch, i, x.size, f))


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("shape", [(128, 64), (64, 16)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_streamed_state_both_schedules(shape, schedule, monkeypatch, cuda_device):
    """A stream in random pieces with its state carried on the device, with both schedules, for a
    filter whose state decays within half a chunk and one whose state does not (it keeps the
    per-section lookback either way), at the largest and smallest chunk shapes."""
    _schedule(monkeypatch, schedule)
    filters = _mixed_filters()
    batch = Batch([s for _, s in filters])
    batch.set_shape(*shape)
    rng = np.random.default_rng(7)
    for f in (2, len(filters) - 2):
        n = 120_000
        x = rng.uniform(-1, 1, n).astype(np.float32)
        xt = torch.from_numpy(x).cuda()
        yt = torch.empty_like(xt)
        st = [torch.zeros(batch.state_size(f), device="cuda") for _ in range(2)]
        pos, turn = 0, 0
        while pos < n:
            m = min(int(rng.integers(1, 30000)), n - pos)
            batch([(xt[pos:pos + m], yt[pos:pos + m], f, st[turn], st[turn ^ 1])])
            pos += m
            turn ^= 1
        batch.check()
        _check(yt.cpu().numpy(), x, filters[f][1], filters[f][0], ("stream", shape, f))


def test_tail_and_per_section_schedules_agree(monkeypatch, cuda_device):
    """The same channels with the tail-aggregate schedule (IIR_GB300_BATCH_TAIL_CHUNKS=1) and with
    the per-section lookback everywhere (the default, and IIR_GB300_TAIL=0, read when a shape is
    prepared): all meet the gate and agree to 1e-5 of the signal's peak."""
    filters = _mixed_filters()
    rng = np.random.default_rng(8)
    lengths = [int(v) for v in rng.integers(1, 200_000, 30)]
    xs = [rng.uniform(-1, 1, n).astype(np.float32) for n in lengths]
    outs = []
    for mode in ("tail", "default", "tail_off"):
        _schedule(monkeypatch, "tail" if mode != "default" else "per_section")
        if mode == "tail_off":
            monkeypatch.setenv("IIR_GB300_TAIL", "0")
        batch = Batch([s for _, s in filters])
        ys = [torch.empty(x.size, device="cuda") for x in xs]
        batch([(torch.from_numpy(x).cuda(), y, i % len(filters)) for i, (x, y) in enumerate(zip(xs, ys))])
        batch.check()
        outs.append([y.cpu().numpy() for y in ys])
    for i, x in enumerate(xs):
        order, sos = filters[i % len(filters)]
        _, ref = oracle.reference_golden(sos, x)
        scale = float(np.max(np.abs(ref))) or 1.0
        for k in (1, 2):
            assert np.max(np.abs(outs[0][i] - outs[k][i])) <= 1e-5 * scale, (i, k)
        _check(outs[0][i], x, sos, order, ("tail", i))
        _check(outs[1][i], x, sos, order, ("per-section", i))


def test_tune_batch_picks_a_shape_and_filters_correctly(cuda_device):
    """The batching tuner times every compiled shape in the order the occupancy model proposes
    and leaves the fastest set; the batch still filters correctly with it."""
    from cuda_recursive_filtering_gb300 import autotune
    filters = _mixed_filters()
    batch = Batch([s for _, s in filters])
    rng = np.random.default_rng(9)
    lengths = rng.integers(500, 3000, 2000)
    off = np.concatenate([[0], np.cumsum(lengths)])
    x = torch.from_numpy(rng.uniform(-1, 1, int(off[-1])).astype(np.float32)).cuda()
    y = torch.empty_like(x)
    flt = (np.arange(lengths.size) % len(filters)).astype(np.int32)
    res = autotune.tune_batch(batch, x, y, off, flt, reps=2)
    assert len(res["table"]) == 4 and all(t["gsps"] > 0 for t in res["table"])
    assert [batch.shape()["rows"], batch.shape()["samples_per_row"]] == res["shape"]
    # short segments: the model ranks the biggest chunk, mostly padding here, last
    assert res["model_order"][-1] == [128, 64]
    batch.packed(x, y, off, flt)
    batch.check()
    yh = y.cpu().numpy()
    for i in rng.choice(lengths.size, 12, replace=False):
        f = int(flt[i])
        _check(yh[off[i]:off[i + 1]], x[off[i]:off[i + 1]].cpu().numpy(), filters[f][1], filters[f][0], ("tuned", i))


@pytest.mark.parametrize("shape", [(128, 64), (128, 32), (128, 16), (64, 16)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_segments_at_every_float_offset(shape, cuda_device):
    """Segments packed into one input and one output buffer at every offset modulo 16 bytes, the
    input and output offsets independent, with lengths at and around whole chunks (whole chunks of
    a segment that is not 16-byte aligned move as shifted 16-byte loads and stores). Every segment
    meets the gate, and the output samples between segments keep their sentinel."""
    filters = _mixed_filters()
    batch = Batch([s for _, s in filters])
    batch.set_shape(*shape)
    chunk = batch.shape()["chunk"]
    rng = np.random.default_rng(31 + shape[1])
    lengths = [chunk, chunk + 1, chunk + 3, chunk + 4, chunk + 5, 2 * chunk, 2 * chunk + 2, 3 * chunk + 3,
               5 * chunk + 1, chunk - 1, 7, 4 * chunk + 4]
    lengths = [n for n in lengths for _ in range(2)]
    xo, yo, px, py = [], [], 0, 0
    for i, n in enumerate(lengths):
        px += i % 4          # input offsets cycle through every residue mod 4 floats
        py += int(rng.integers(0, 6))
        xo.append(px)
        yo.append(py)
        px += n
        py += n
    x = rng.uniform(-1, 1, px + 8).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    yt = torch.full((py + 8,), float("nan"), device="cuda")
    segs = [(xt[a:a + n], yt[b:b + n], i % len(filters)) for i, (a, b, n) in enumerate(zip(xo, yo, lengths))]
    assert {t[0].data_ptr() % 16 for t in segs} == {0, 4, 8, 12}
    assert len({t[1].data_ptr() % 16 for t in segs}) > 1
    batch(segs)
    batch.check()
    yh = yt.cpu().numpy()
    covered = np.zeros(yh.size, bool)
    for i, (a, b, n) in enumerate(zip(xo, yo, lengths)):
        f = i % len(filters)
        _check(yh[b:b + n], x[a:a + n], filters[f][1], filters[f][0], (shape, i, n, a % 4, b % 4))
        covered[b:b + n] = True
    assert np.isnan(yh[~covered]).all()


@pytest.mark.parametrize("shape", [(128, 64), (64, 16)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_segments_from_rest_at_every_offset_carry_their_state(shape, cuda_device):
    """Segments that start at rest (no zi) at every offset modulo 16 bytes, with a final state:
    such a segment is chunked on its input's 16-byte grid, its first chunk padded with leading
    zeros. A second launch continues each one from its zf over the rest of its signal (that
    launch's segments have a zi, so they keep the segment-aligned chunking), and the two pieces
    join into the whole-signal output."""
    filters = _mixed_filters()
    batch = Batch([s for _, s in filters])
    batch.set_shape(*shape)
    chunk = batch.shape()["chunk"]
    rng = np.random.default_rng(41 + shape[1])
    firsts = [1, 2, 3, 5, chunk - 3, chunk - 1, chunk, chunk + 2, 3 * chunk + 1, 4 * chunk - 2]
    firsts = [n for n in firsts for _ in range(2)]
    rests = [int(v) for v in rng.integers(1, 3 * chunk, len(firsts))]
    xo, p = [], 0
    for i, (a, b) in enumerate(zip(firsts, rests)):
        p += 1 + i % 4
        xo.append(p)
        p += a + b
    x = rng.uniform(-1, 1, p + 8).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    yt = torch.full_like(xt, float("nan"))
    fl = [i % len(filters) for i in range(len(firsts))]
    st = [torch.full((batch.state_size(f),), float("nan"), device="cuda") for f in fl]
    batch([(xt[o:o + a], yt[o:o + a], f, None, z) for o, a, f, z in zip(xo, firsts, fl, st)])
    assert {xt[o:].data_ptr() % 16 for o in xo} == {0, 4, 8, 12}
    batch([(xt[o + a:o + a + b], yt[o + a:o + a + b], f, z) for o, a, b, f, z in zip(xo, firsts, rests, fl, st)])
    batch.check()
    yh = yt.cpu().numpy()
    for i, (o, a, b, f) in enumerate(zip(xo, firsts, rests, fl)):
        _check(yh[o:o + a + b], x[o:o + a + b], filters[f][1], filters[f][0], (shape, i, a, b, o % 4))
