"""Serving form: live streams send chunks; a continuous-batching loop filters whatever has
arrived in one launch per step, keeping each stream's state on the device. Chunked output must
match whole-stream filtering (FP64 oracle, the reference's gate max|err| <= 1e-4 * max|ref| and
max|err| / RMS(ref) <= 1e-5)."""
import numpy as np
import pytest

import oracle
from cuda_recursive_filtering_gb300.serving import StreamServer, run_poisson_load

pytestmark = pytest.mark.gpu


def _filters():
    from scipy import signal
    return [signal.butter(8, c, output="sos") for c in (0.05, 0.1, 0.25, 0.4)] + [signal.butter(2, 0.2, output="sos")]


def test_streams_in_chunks_match_whole(cuda_device):
    filters = _filters()
    srv = StreamServer(filters, max_batch=64)
    rng = np.random.default_rng(21)
    sigs, reqs = {}, {}
    for i in range(10):
        sid = srv.open_stream(i % len(filters))
        sigs[sid] = rng.standard_normal(int(rng.integers(5_000, 60_000))).astype(np.float32)
        reqs[sid] = []
    pos = {sid: 0 for sid in sigs}
    while any(pos[s] < sigs[s].size for s in sigs):
        for sid in sigs:
            if pos[sid] < sigs[sid].size and rng.random() < 0.6:
                m = min(int(rng.integers(1, 7000)), sigs[sid].size - pos[sid])
                reqs[sid].append(srv.submit(sid, sigs[sid][pos[sid]:pos[sid] + m]))
                pos[sid] += m
        srv.step()
        srv.poll()
    srv.drain()
    for sid, x in sigs.items():
        y = np.concatenate([r.out.numpy() for r in reqs[sid]])
        _, ref = oracle.reference_golden(filters[srv.streams[sid].filter], x)
        e = oracle.errors(y, ref)
        assert e["rel_max"] <= 1e-4 and e["rel_rms"] <= 1e-5, (sid, e)
    assert all(r.latency is not None and r.latency >= 0 for rs in reqs.values() for r in rs)


def test_poisson_load_reports_latency(cuda_device):
    filters = _filters()
    srv = StreamServer(filters, max_batch=256)
    streams = [srv.open_stream(i % len(filters)) for i in range(64)]
    out = run_poisson_load(srv, streams, rate_sps=2e8, duration_s=0.3, chunk_lo=256, chunk_hi=8192, seed=4)
    assert out["requests"] > 0 and out["samples"] > 0
    assert out["p50_us"] is not None and out["p99_us"] >= out["p50_us"] > 0


def test_burst_of_chunks_is_one_segment(cuda_device):
    """Chunks that queue up on a stream between steps go out in one step as one segment (they
    are consecutive pieces of the stream's signal); the result equals whole-stream filtering."""
    filters = _filters()
    srv = StreamServer(filters, max_batch=16, max_stream_samples=1 << 20)
    rng = np.random.default_rng(5)
    sigs, reqs = {}, {}
    for i in range(6):
        sid = srv.open_stream(i % len(filters))
        x = rng.standard_normal(int(rng.integers(20_000, 90_000))).astype(np.float32)
        cuts = np.sort(rng.choice(np.arange(1, x.size), 11, replace=False))
        sigs[sid] = x
        reqs[sid] = [srv.submit(sid, piece) for piece in np.split(x, cuts)]
    assert srv.step() == sum(len(r) for r in reqs.values())  # every queued chunk in one launch
    srv.drain()
    for sid, x in sigs.items():
        y = np.concatenate([r.out.numpy() for r in reqs[sid]])
        _, ref = oracle.reference_golden(filters[srv.streams[sid].filter], x)
        e = oracle.errors(y, ref)
        assert e["rel_max"] <= 1e-4 and e["rel_rms"] <= 1e-5, (sid, e)


def test_admission_by_free_device_memory(cuda_device):
    """Streams and requests are admitted only while the device keeps the server's reserve free:
    taking device memory below the reserve makes open_stream and submit raise AdmissionError,
    and giving it back admits them again. The stream table's size is a second limit."""
    import time

    import torch

    from cuda_recursive_filtering_gb300.serving import AdmissionError
    filters = _filters()
    srv = StreamServer(filters, max_batch=16, max_streams=3)
    sid = srv.open_stream(0)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()  # the hog below must take new device memory, not cached blocks
    free_now = torch.cuda.mem_get_info()[0]
    srv.reserve = free_now - (2 << 30)  # 2 GiB of headroom above the reserve
    hog = torch.empty(3 << 30, dtype=torch.uint8, device="cuda")  # takes 3 GiB: below the reserve
    time.sleep(0.02)  # the server re-reads free memory at most every 5 ms
    with pytest.raises(AdmissionError):
        srv.open_stream(1)
    with pytest.raises(AdmissionError):
        srv.submit(sid, np.zeros(1000, np.float32))
    del hog
    torch.cuda.empty_cache()
    time.sleep(0.02)
    sid2 = srv.open_stream(1)
    req = srv.submit(sid2, np.ones(1000, np.float32))
    srv.drain()
    assert req.out is not None and req.out.numel() == 1000
    srv.open_stream(2)
    with pytest.raises(AdmissionError):  # the stream table holds 3
        srv.open_stream(3)
    srv.close_stream(sid)
    srv.open_stream(3)


def test_stream_alone_and_in_a_mix_agree(cuda_device):
    """One stream's chunks served alone and the same chunks served among 15 other live streams
    (other filters, other lengths, sharing every launch) give the same output, and both match
    whole-stream FP64 filtering."""
    filters = _filters()
    rng = np.random.default_rng(33)
    x = rng.standard_normal(150_000).astype(np.float32)
    cuts = np.sort(rng.choice(np.arange(1, x.size), 24, replace=False))
    pieces = np.split(x, cuts)

    def serve(mix: bool):
        srv = StreamServer(filters, max_batch=64)
        sid = srv.open_stream(1)
        others = [srv.open_stream(i % len(filters)) for i in range(15)] if mix else []
        orng = np.random.default_rng(7)
        reqs = []
        for piece in pieces:  # one piece per step, with whatever the others send
            reqs.append(srv.submit(sid, piece))
            for o in others:
                srv.submit(o, orng.standard_normal(int(orng.integers(100, 20_000))).astype(np.float32))
            srv.step()
            srv.poll()
        srv.drain()
        return np.concatenate([r.out.numpy() for r in reqs])

    alone, mixed = serve(False), serve(True)
    _, ref = oracle.reference_golden(filters[1], x)
    for y in (alone, mixed):
        e = oracle.errors(y, ref)
        assert e["rel_max"] <= 1e-4 and e["rel_rms"] <= 1e-5, e
    assert np.max(np.abs(alone - mixed)) <= 1e-6 * np.max(np.abs(ref))
