"""Streaming service with continuous batching over iir_batch_* (the serving form).

Live streams send chunks of samples as they arrive. Every stream keeps its filter state on the
device between chunks (two state buffers used in turn: zi of a chunk is zf of the chunk before),
so chunked output equals whole-stream filtering. A serving step takes the oldest waiting chunk of
every stream that has one and filters them all in one launch (continuous batching: the batch is
rebuilt every step from whatever has arrived). Host chunks are copied to the device and results
back on one CUDA stream, so a request is complete when its step's device-to-host copy is.
A stream's waiting chunks are consecutive pieces of one signal, so a step takes all of them (up to
``max_stream_samples``) as one segment: a burst on one stream costs one step, not one per chunk.
Streams and requests are admitted while the device keeps `reserve_bytes` free.

The reference has no serving path: its kernels filter one zero-state signal per launch
(src/test_accuracy.cu:136-159); its per-sample state hooks (xi1/xi2/yi1/yi2,
include/ph_kernels.cuh:45,251-253) are what a stream carries here between chunks.
"""
from __future__ import annotations

import collections
import dataclasses
import gc
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
    out: torch.Tensor | None = None  # host copy of the filtered chunk (when the server keeps outputs)

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.t_arrival


class _Stream:
    def __init__(self, filt: int, slot: int):
        self.filter = filt
        self.slot = slot  # row of the server's state tensor
        self.turn = 0
        self.queue: collections.deque = collections.deque()


class StreamServer:
    """Continuous-batching filter service for many live streams (one GPU).

    ``filters``: SOS arrays (one per distinct filter). ``max_batch``: chunks per launch.
    ``max_streams``: open streams at a time (their states live in one device tensor).
    ``reserve_bytes``: device memory left free when admitting streams and requests.
    """

    def __init__(self, filters, max_batch: int = 1024, max_streams: int = 4096, reserve_bytes: int = 1 << 30,
                 device=None, keep_outputs: bool = True, max_stream_samples: int = 1 << 22,
                 max_step_samples: int = 1 << 23, step_slots: int = 3):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        with torch.cuda.device(self.device):
            self.batch = Batch(filters, max_segments=max_batch, max_chunks=1 << 16, device=self.device)
            self.cuda_stream = torch.cuda.Stream(self.device)
            self.width = max(self.batch.state_size(f) for f in range(len(self.batch.n_sections)))
            # [turn][slot][state]: a stream's chunk reads [turn] and writes [turn ^ 1]
            self.states = torch.zeros(2, max_streams, self.width, device=self.device)
        self.max_batch = max_batch
        self.max_streams = max_streams
        self.max_stream_samples = max_stream_samples  # per stream and step (more chunks wait a step)
        self.max_step_samples = max_step_samples  # per step: bounds the step's buffers and latency
        # step buffers, allocated once: pinned host input / output and device input / output of
        # max_step_samples each, for up to step_slots steps in flight (no allocation while serving)
        with torch.cuda.device(self.device):
            self._slots = [{"xh": torch.empty(max_step_samples, pin_memory=True),
                            "yh": torch.empty(max_step_samples, pin_memory=True),
                            "xd": torch.empty(max_step_samples, device=self.device),
                            "yd": torch.empty(max_step_samples, device=self.device), "busy": False}
                           for _ in range(step_slots)]
        self.keep_outputs = keep_outputs  # copy each request's result out of the step's pinned buffer
        self.reserve = reserve_bytes
        self.streams: dict[int, _Stream] = {}
        self._sid: dict[int, int] = {}  # id(stream record) -> stream id
        self._free_slots = list(range(max_streams - 1, -1, -1))
        self._next_id = 0
        self._inflight: collections.deque = collections.deque()  # (event, requests, slot, request offsets)
        self._free_bytes, self._free_t = 0, -1.0
        self.completed: list[Request] = []
        self.samples_done = 0

    # ---------------------------------------------------------------- admission
    def _free(self) -> int:
        # device free memory, re-read at most every 5 ms (the query is a driver call)
        now = time.perf_counter()
        if now - self._free_t > 5e-3:
            self._free_bytes, _ = torch.cuda.mem_get_info(self.device)
            self._free_t = now
        return self._free_bytes

    def open_stream(self, filter_index: int) -> int:
        if not self._free_slots:
            raise AdmissionError("stream table full")
        if self._free() < self.reserve:
            raise AdmissionError("not enough free device memory for a new stream")
        sid = self._next_id
        self._next_id += 1
        slot = self._free_slots.pop()
        self.states[:, slot].zero_()
        self.streams[sid] = _Stream(filter_index, slot)
        self._sid[id(self.streams[sid])] = sid
        return sid

    def close_stream(self, sid: int) -> None:
        s = self.streams.pop(sid)
        self._sid.pop(id(s), None)
        self._free_slots.append(s.slot)

    def state(self, sid: int) -> torch.Tensor:
        """The stream's current device state (x[-2], x[-1], per section y[-2], y[-1])."""
        s = self.streams[sid]
        return self.states[s.turn, s.slot, :self.batch.state_size(s.filter)]

    def submit(self, sid: int, chunk, t_arrival: float | None = None) -> Request:
        """Queues a host chunk (float32) of stream ``sid``; returns its request record."""
        s = self.streams[sid]
        host = np.ascontiguousarray(chunk.numpy() if torch.is_tensor(chunk) else chunk, dtype=np.float32)
        if host.size > self.max_step_samples:
            raise AdmissionError("chunk longer than the server's step capacity")
        if self._free() < self.reserve:
            raise AdmissionError("not enough free device memory for the request")
        req = Request(sid, int(host.size), time.perf_counter() if t_arrival is None else t_arrival)
        s.queue.append((req, host))
        return req

    # ---------------------------------------------------------------- serving loop
    def step(self) -> int:
        """One launch over every stream that has waiting chunks (at most ``max_batch`` streams):
        each stream's waiting chunks, concatenated in order, are one segment. One host-to-device
        copy of all of them, one batch launch, one copy of the results back. Returns the number
        of requests launched."""
        picked, reqs, chunks, lens = [], [], [], []
        total = 0
        for s in self.streams.values():
            if not s.queue:
                continue
            if picked and total + s.queue[0][0].samples > self.max_step_samples:
                break  # the step is full; this stream goes first next time (dict order rotates below)
            n = 0
            while s.queue and (n == 0 or (n + s.queue[0][0].samples <= self.max_stream_samples and
                                          total + n + s.queue[0][0].samples <= self.max_step_samples)):
                req, host = s.queue.popleft()
                reqs.append(req)
                chunks.append(host)
                n += req.samples
            picked.append(s)
            lens.append(n)
            total += n
            if len(picked) == self.max_batch:
                break
        if not picked:
            return 0
        if any(s.queue for s in self.streams.values()):
            # streams left waiting: the picked ones go to the back of the order (round robin)
            for s in picked:
                sid = self._sid[id(s)]
                self.streams[sid] = self.streams.pop(sid)
        k = len(picked)
        lens = np.asarray(lens, dtype=np.int64)
        off = np.zeros(k + 1, dtype=np.int64)
        np.cumsum(lens, out=off[1:])
        req_off = np.zeros(len(reqs) + 1, dtype=np.int64)
        np.cumsum(np.fromiter((r.samples for r in reqs), dtype=np.int64, count=len(reqs)), out=req_off[1:])
        slots = np.fromiter((s.slot for s in picked), dtype=np.int64, count=k)
        turns = np.fromiter((s.turn for s in picked), dtype=np.int64, count=k)
        filt = np.fromiter((s.filter for s in picked), dtype=np.int32, count=k)
        for s in picked:
            s.turn ^= 1
        slot = next((sl for sl in self._slots if not sl["busy"]), None)
        if slot is None:  # every step buffer is in flight: complete the oldest step first
            self.poll(block=True)
            slot = next(sl for sl in self._slots if not sl["busy"])
        slot["busy"] = True
        xhost, yhost, xin, yout = slot["xh"], slot["yh"], slot["xd"], slot["yd"]
        with torch.cuda.device(self.device), torch.cuda.stream(self.cuda_stream):
            np.concatenate(chunks, out=xhost.numpy()[:total])
            xin[:total].copy_(xhost[:total], non_blocking=True)
            tab = self.batch.segment_table(k)
            tab["x"][:k] = xin.data_ptr() + 4 * off[:-1]
            tab["y"][:k] = yout.data_ptr() + 4 * off[:-1]
            tab["n"][:k] = lens
            tab["filter"][:k] = filt
            row = 4 * self.width
            base = self.states.data_ptr()
            tab["zi"][:k] = base + row * (turns * self.max_streams + slots)
            tab["zf"][:k] = base + row * ((turns ^ 1) * self.max_streams + slots)
            self.batch.execute_table(tab, k, stream=self.cuda_stream)
            yhost[:total].copy_(yout[:total], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.cuda_stream)
        self._inflight.append((ev, reqs, slot, req_off))
        return len(reqs)

    def poll(self, block: bool = False) -> int:
        """Completes requests whose step has finished; returns how many completed."""
        done = 0
        while self._inflight:
            ev, reqs, slot, off = self._inflight[0]
            if block:
                ev.synchronize()
            elif not ev.query():
                break
            t = time.perf_counter()
            yhost = slot["yh"]
            for i, r in enumerate(reqs):
                r.t_done = t
                if self.keep_outputs:
                    r.out = yhost[off[i]:off[i + 1]].clone()
                self.samples_done += r.samples
            slot["busy"] = False  # results taken: the step's buffers may be reused
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
            return {**{f"p{q}_us": None for q in qs}, "max_us": None}
        out = {f"p{q}_us": float(np.percentile(lat, q) * 1e6) for q in qs}
        out["max_us"] = float(lat.max() * 1e6)
        return out


def run_poisson_load(server: StreamServer, streams: list[int], rate_sps: float, duration_s: float,
                     chunk_lo: int, chunk_hi: int, seed: int = 4, signals: dict | None = None) -> dict:
    """Drives ``server`` with Poisson chunk arrivals at ``rate_sps`` samples per second in
    aggregate (chunk lengths uniform in [chunk_lo, chunk_hi], streams chosen uniformly) for
    ``duration_s`` seconds of wall clock, serving continuously. ``signals`` (optional) maps a
    stream to a host array its chunks are taken from, in order, for correctness checks.
    Returns throughput and latency percentiles."""
    rng = np.random.default_rng(seed)
    pool = rng.standard_normal(1 << 22).astype(np.float32)  # chunk data: slices of one pool
    # The loop creates tens of thousands of request records a second; a cyclic-GC pass over them
    # stalls the serving loop for tens of milliseconds, so the collector is paused for the run.
    gc_was_enabled = gc.isenabled()
    gc.collect()
    gc.disable()
    try:
        return _poisson_loop(server, streams, rate_sps, duration_s, chunk_lo, chunk_hi, rng, pool, signals)
    finally:
        if gc_was_enabled:
            gc.enable()


def _poisson_loop(server, streams, rate_sps, duration_s, chunk_lo, chunk_hi, rng, pool, signals) -> dict:
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
                o = int(rng.integers(0, pool.size - m + 1))
                chunk = pool[o:o + m]
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
