"""Streaming service with continuous batching over iir_batch_* (the serving form).

Live streams send chunks of samples as they arrive. Every stream keeps its filter state on the
device between chunks (two state buffers used in turn: zi of a chunk is zf of the chunk before),
so chunked output equals whole-stream filtering. A serving step takes the oldest waiting chunk of
every stream that has one and filters them all in one launch (continuous batching: the batch is
rebuilt every step from whatever has arrived). Host chunks are copied to the device and results
back on one CUDA stream, so a request is complete when its step's device-to-host copy is.
Streams and requests are admitted while the device keeps `reserve_bytes` free.

The reference has no serving path: its kernels filter one zero-state signal per launch
(src/test_accuracy.cu:136-159); its per-sample state hooks (xi1/xi2/yi1/yi2,
include/ph_kernels.cuh:45,251-253) are what a stream carries here between chunks.
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np
import torch

from .api import Batch

__all__ = ["StreamServer", "Request", "AdmissionError"]


class AdmissionError(RuntimeError):
    """The device has too little free memory to admit a stream or a request."""


@dataclasses.dataclass
class Request:
    stream: int
    samples: int
    t_arrival: float
    t_done: float | None = None
    out: torch.Tensor | None = None  # pinned host copy of the filtered chunk

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.t_arrival


class _Stream:
    def __init__(self, filt: int, size: int, device):
        self.filter = filt
        self.state = [torch.zeros(size, device=device), torch.zeros(size, device=device)]
        self.turn = 0
        self.queue: collections.deque = collections.deque()


class StreamServer:
    """Continuous-batching filter service for many live streams (one GPU).

    ``filters``: SOS arrays (one per distinct filter). ``max_batch``: chunks per launch.
    ``reserve_bytes``: device memory left free when admitting streams and requests.
    """

    def __init__(self, filters, max_batch: int = 1024, reserve_bytes: int = 1 << 30, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        with torch.cuda.device(self.device):
            self.batch = Batch(filters, max_segments=max_batch, max_chunks=1 << 16, device=self.device)
            self.cuda_stream = torch.cuda.Stream(self.device)
        self.max_batch = max_batch
        self.reserve = reserve_bytes
        self.streams: dict[int, _Stream] = {}
        self._next_id = 0
        self._inflight: collections.deque = collections.deque()  # (event, requests, buffers)
        self.completed: list[Request] = []
        self.samples_done = 0

    # ---------------------------------------------------------------- admission
    def _free(self) -> int:
        free, _ = torch.cuda.mem_get_info(self.device)
        return free

    def open_stream(self, filter_index: int) -> int:
        size = self.batch.state_size(filter_index)
        if self._free() < self.reserve + 8 * size:
            raise AdmissionError("not enough free device memory for a new stream")
        sid = self._next_id
        self._next_id += 1
        self.streams[sid] = _Stream(filter_index, size, self.device)
        return sid

    def close_stream(self, sid: int) -> None:
        self.streams.pop(sid)

    def state(self, sid: int) -> torch.Tensor:
        """The stream's current device state (x[-2], x[-1], per section y[-2], y[-1])."""
        s = self.streams[sid]
        return s.state[s.turn]

    def submit(self, sid: int, chunk: np.ndarray | torch.Tensor, t_arrival: float | None = None) -> Request:
        """Queues a host chunk (float32) of stream ``sid``; returns its request record."""
        s = self.streams[sid]
        host = torch.as_tensor(np.ascontiguousarray(chunk, np.float32)) if not torch.is_tensor(chunk) else chunk
        if self._free() < self.reserve + 8 * host.numel():
            raise AdmissionError("not enough free device memory for the request")
        req = Request(sid, int(host.numel()), time.perf_counter() if t_arrival is None else t_arrival)
        s.queue.append((req, host))
        return req

    # ---------------------------------------------------------------- serving loop
    def step(self) -> int:
        """One launch over the oldest waiting chunk of every stream that has one (at most
        ``max_batch``). Returns the number of chunks launched."""
        picked = []
        for sid, s in self.streams.items():
            if s.queue:
                picked.append((sid, s, s.queue.popleft()))
                if len(picked) == self.max_batch:
                    break
        if not picked:
            return 0
        total = sum(req.samples for _, _, (req, _) in picked)
        with torch.cuda.device(self.device), torch.cuda.stream(self.cuda_stream):
            xin = torch.empty(max(total, 1), device=self.device)
            yout = torch.empty_like(xin)
            yhost = torch.empty(max(total, 1), pin_memory=True)
            segs, reqs, pos = [], [], 0
            for sid, s, (req, host) in picked:
                n = req.samples
                if n:
                    xin[pos:pos + n].copy_(host, non_blocking=True)
                    segs.append((xin[pos:pos + n], yout[pos:pos + n], s.filter, s.state[s.turn], s.state[s.turn ^ 1]))
                    s.turn ^= 1
                req.out = yhost[pos:pos + n]
                reqs.append(req)
                pos += n
            if segs:
                self.batch(segs, stream=self.cuda_stream)
            yhost[:total].copy_(yout[:total], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.cuda_stream)
        self._inflight.append((ev, reqs, (xin, yout, yhost)))
        return len(reqs)

    def poll(self, block: bool = False) -> int:
        """Completes requests whose step has finished; returns how many completed."""
        done = 0
        while self._inflight:
            ev, reqs, _ = self._inflight[0]
            if block:
                ev.synchronize()
            elif not ev.query():
                break
            t = time.perf_counter()
            for r in reqs:
                r.t_done = t
                self.samples_done += r.samples
            self.completed.extend(reqs)
            self._inflight.popleft()
            done += len(reqs)
        return done

    def drain(self) -> None:
        while any(s.queue for s in self.streams.values()):
            self.step()
        self.poll(block=True)
        self.batch.check(self.cuda_stream)

    def latency_percentiles(self, qs=(50, 99)) -> dict:
        lat = np.array([r.latency for r in self.completed if r.latency is not None])
        if lat.size == 0:
            return {f"p{q}_us": None for q in qs}
        return {f"p{q}_us": float(np.percentile(lat, q) * 1e6) for q in qs}


def run_poisson_load(server: StreamServer, streams: list[int], rate_sps: float, duration_s: float,
                     chunk_lo: int, chunk_hi: int, seed: int = 4, signals: dict | None = None) -> dict:
    """Drives ``server`` with Poisson chunk arrivals at ``rate_sps`` samples per second in
    aggregate (chunk lengths uniform in [chunk_lo, chunk_hi], streams chosen uniformly) for
    ``duration_s`` seconds of wall clock, serving continuously. ``signals`` (optional) maps a
    stream to a host array its chunks are taken from, in order, for correctness checks.
    Returns throughput and latency percentiles."""
    rng = np.random.default_rng(seed)
    mean_chunk = 0.5 * (chunk_lo + chunk_hi)
    rate_req = rate_sps / mean_chunk
    t0 = time.perf_counter()
    next_t = t0 + rng.exponential(1.0 / rate_req)
    positions = {sid: 0 for sid in streams}
    submitted = 0
    while True:
        now = time.perf_counter()
        while next_t <= now and next_t - t0 < duration_s:
            sid = streams[int(rng.integers(len(streams)))]
            m = int(rng.integers(chunk_lo, chunk_hi + 1))
            if signals is not None:
                src = signals[sid]
                p0 = positions[sid]
                m = min(m, src.size - p0)
                chunk = src[p0:p0 + m]
                positions[sid] = p0 + m
            else:
                chunk = rng.standard_normal(m).astype(np.float32)
            server.submit(sid, chunk, t_arrival=next_t)
            submitted += m
            next_t += rng.exponential(1.0 / rate_req)
        server.step()
        server.poll()
        if next_t - t0 >= duration_s and not any(s.queue for s in server.streams.values()):
            break
    server.poll(block=True)
    elapsed = time.perf_counter() - t0
    out = {"requests": len(server.completed), "samples": int(server.samples_done), "seconds": elapsed,
           "gsps": server.samples_done / elapsed / 1e9, "offered_gsps": rate_sps / 1e9}
    out.update(server.latency_percentiles())
    return out
