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
