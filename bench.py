#!/usr/bin/env python3
"""Throughput benchmark: cascaded-biquad IIR filtering on GB300.

Workload (one step = one filtering pass over the whole signal): Butterworth lowpass
(scipy butter, cutoff 0.1 x Nyquist, SOS form) over 2^28 float32 samples i.i.d.
uniform[-1, 1) from seed 1 — the plain roofline sweep the reference benchmarks
(GS/s, P20 of batches in src/test_performance.cu / include/measure.cuh). Headline: the DTCR
realization at order 2 (geometry 32x64). The signal (1 GiB in + 1 GiB out) is far larger
than L2, so no flush is needed between steps.

Every row of the sweep (realization x order x geometry, at 2^28 and 2^25 samples; order 2 at
2^16) carries {gsps, frac, rel_max, rel_rms}: frac against the measured HBM roof (8 bytes per
sample), and the error of ALL of that row's outputs against the FP64 oracle (the reference's
golden path, tools/ref_generate.py:89), compared on the device. The precision form is
measured at orders 8..16 on its own workload with the same full-length error.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-sweep]

Prints one JSON line (rank 0). Under torchrun every rank filters its own replica of the
workload on its own GPU (the path has no exchange step between GPUs: replicas only).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GS/s (fp32 samples per second through the cascaded-biquad filter)"
UNIT = "GS/s"
LOG2N = 28
HEADLINE = {"kernel": "DTCR_UNROLL", "order": 2, "block_size": 32, "n_blocks": 64}
# the reference's geometry set BLOCK_SIZE x N_BLOCKS (stcr_kernels.cuh:3613-3624)
_GEOMS = [(32, 32), (32, 64), (32, 128), (64, 64)]
SWEEP_GEOM = {"PH": _GEOMS, "STCR": _GEOMS, "STCR_UNROLL": _GEOMS, "DTCR": _GEOMS, "DTCR_UNROLL": _GEOMS,
              "PLR": [(0, 0)]}
BYTES_PER_SAMPLE = 8  # 4 read + 4 written (algorithmic)
L2_BYTES = 129 * 1024 * 1024
GATE = 1e-4           # the reference's accuracy gate, max|err| <= 1e-4 max|ref| (src/test_accuracy.cu:178-188)
CPU_PIECE = 1 << 21   # samples per piece of the CPU baselines (one piece per host thread)


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic_per_launch() -> dict | None:
    """DRAM bytes (read + write) of one launch of the headline kernel at 2^28 samples, from the
    committed one-pass ncu capture of that launch (profiles/dtcr_unroll_order2_traffic_2p28.md)."""
    path = os.path.join(ROOT, "profiles", "dtcr_unroll_order2_traffic_2p28.md")
    if not os.path.exists(path):
        return None
    vals = {}
    for line in open(path):
        if ":" in line and line.split(":")[0].strip() in ("dram_bytes_read", "dram_bytes_write", "samples"):
            k, v = line.split(":", 1)
            vals[k.strip()] = float(v.split()[0])
    if "dram_bytes_read" not in vals or "dram_bytes_write" not in vals:
        return None
    return {"bytes": vals["dram_bytes_read"] + vals["dram_bytes_write"], "read": vals["dram_bytes_read"],
            "write": vals["dram_bytes_write"], "samples": vals.get("samples")}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def time_plan(plan, x, y, steps: int, warmup: int, stream, per_launch: bool = False):
    """ms per launch: the CUDA-event time of `steps` back-to-back launches after `warmup`. With
    per_launch, every launch is bracketed by its own pair of events and the median launch is
    returned, so that a host thread descheduled between two launches (the sweep computes its
    FP64 goldens on host threads meanwhile) leaves the GPU idle outside every timed interval."""
    import torch
    for _ in range(warmup):
        plan(x, y, stream=stream)
    plan.check(stream)
    torch.cuda.synchronize()
    if per_launch:
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for s, e in ev:
            s.record(stream)
            plan(x, y, stream=stream)
            e.record(stream)
        torch.cuda.synchronize()
        plan.check(stream)
        return statistics.median(s.elapsed_time(e) for s, e in ev)
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(steps):
        plan(x, y, stream=stream)
    e.record(stream)
    e.synchronize()
    torch.cuda.synchronize()
    plan.check(stream)
    return s.elapsed_time(e) / steps


class _RefAsPlan:
    """A reference kernel module (oracle/refgpu.RefKernel) with the calls time_rotating makes."""

    def __init__(self, rk):
        self.rk = rk

    def __call__(self, x, y, stream=None):
        self.rk(x, y, stream)

    def check(self, stream=None):
        import torch
        torch.cuda.synchronize()


def time_rotating(plan, xs, ys, batches: int, per_batch: int, stream) -> list[float]:
    """The reference's timing method (include/measure.cuh:37-110): launches cycle through
    several identical input / output buffers whose total exceeds L2; `batches` batches of
    `per_batch` launches, each timed with CUDA events. Returns ms per launch of each batch."""
    import torch
    nb = len(xs)
    for i in range(min(3 * nb, 600)):
        plan(xs[i % nb], ys[i % nb], stream=stream)
    plan.check(stream)
    out = []
    k = 0
    for _ in range(batches):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(per_batch):
            plan(xs[k % nb], ys[k % nb], stream=stream)
            k += 1
        e.record(stream)
        e.synchronize()
        out.append(s.elapsed_time(e) / per_batch)
    plan.check(stream)
    return out


def host_threads() -> int:
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


# ------------------------------------------------------------------------------------------
# FP64 oracle outputs, computed on the host in background threads (the C oracle releases the
# GIL) and compared with the device output on the device
# ------------------------------------------------------------------------------------------
class Golden:
    """FP64 oracle output of a workload, prefetched a few jobs ahead on host threads."""

    def __init__(self, jobs, ahead: int = 3):
        self.jobs = list(jobs)          # (key, sos, x_host_f32)
        self.ahead = ahead
        self.pool = cf.ThreadPoolExecutor(ahead)
        self.fut = {}
        self.next = 0
        self._fill()

    def _fill(self):
        while self.next < len(self.jobs) and len(self.fut) < self.ahead:
            key, sos, xh = self.jobs[self.next]
            self.fut[key] = self.pool.submit(self._run, sos, xh)
            self.next += 1

    @staticmethod
    def _run(sos, xh):
        import oracle
        return oracle.reference_golden(sos, xh)[1]

    def get(self, key):
        ref = self.fut.pop(key).result()
        self._fill()
        return ref

    def close(self):
        self.pool.shutdown(wait=False, cancel_futures=True)


class DeviceRef:
    """An FP64 oracle output on the device with its scale (max|ref|, RMS(ref))."""

    def __init__(self, ref_host, dev):
        import torch
        self.ref = torch.from_numpy(ref_host).to(dev)
        self.maxabs = float(self.ref.abs().max())
        self.rms = float(self.ref.square().mean().sqrt())

    def errors(self, y, n: int | None = None) -> dict:
        """max|y - ref| over the first n outputs, relative to max|ref| (the reference's gate) and
        to RMS(ref); non-finite output gives inf."""
        import torch
        n = y.numel() if n is None else n
        err = 0.0
        step = 1 << 26
        for i in range(0, n, step):
            d = (y[i:min(n, i + step)].double() - self.ref[i:min(n, i + step)]).abs().max()
            err = max(err, float(d))
        if not (err == err) or err == float("inf") or not bool(torch.isfinite(y[:n]).all()):
            return {"rel_max": float("inf"), "rel_rms": float("inf")}
        if n == self.ref.numel():
            mref, rms = self.maxabs, self.rms
        else:
            r = self.ref[:n]
            mref, rms = float(r.abs().max()), float(r.square().mean().sqrt())
        return {"rel_max": err / max(mref, 1e-300), "rel_rms": err / max(rms, 1e-300)}


def row_entry(gsps: float, hbm_gbs: float, e: dict) -> dict:
    return {"gsps": round(gsps, 1), "frac": round(gsps * BYTES_PER_SAMPLE / hbm_gbs, 4),
            "rel_max": float(f"{e['rel_max']:.3g}"), "rel_rms": float(f"{e['rel_rms']:.3g}"),
            "gate": "pass" if e["rel_max"] <= GATE else "fail"}


# ------------------------------------------------------------------------------------------
# CPU baselines (the reference's CPU golden path and the float32 sequential cascade)
# ------------------------------------------------------------------------------------------
def cpu_pieces(x_host, threads: int):
    """One piece of CPU_PIECE samples per host thread, cut from the start of the workload's
    signal; each piece is filtered as an independent signal from zero state (the recurrence
    within a signal is serial, so the host's cores are used across pieces)."""
    import numpy as np
    n = min(x_host.size, CPU_PIECE * threads)
    return [np.ascontiguousarray(p) for p in np.array_split(x_host[:n], threads)]


def cpu_pass(fn, pieces, threads: int) -> float:
    """Wall time of one pass of fn over every piece, the pieces spread over `threads` threads
    (fn must release the GIL: the C oracle through ctypes, scipy's sosfilt)."""
    t0 = time.perf_counter()
    if threads == 1:
        for p in pieces:
            fn(p)
    else:
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(fn, pieces))
    return time.perf_counter() - t0


def cpu_kernels(sos):
    """The CPU implementations timed: the oracle's C port of the FP64 golden path, scipy's own
    sosfilt (the call tools/ref_generate.py:89 makes) and the float32 sequential cascade."""
    import numpy as np
    from scipy import signal

    import oracle
    oracle.build()
    norm, g = oracle.normalise_sos(sos)
    sos_f32 = norm.astype(np.float32)
    s64 = np.asarray(sos, np.float64)
    return {
        "port": lambda p: oracle.sosfilt_f64(s64, p),
        "scipy_sosfilt": lambda p: signal.sosfilt(s64, p),
        "float32_cascade": lambda p: oracle.cascade_f32(p.astype(np.float32) * np.float32(g), sos_f32),
    }


def cpu_baseline_sample(sos, x_host, budget_s: float = 10.0) -> dict:
    """The reference's CPU path on a bounded sample of the workload, on all host threads:
    one 2^21-sample piece per thread (each an independent zero-state signal), passes repeated
    for about `budget_s` seconds per implementation. Same pieces and piece size as the
    reference arm (--impl reference)."""
    import numpy as np
    threads = host_threads()
    xs = np.ascontiguousarray(x_host[:CPU_PIECE * threads], dtype=np.float64)
    pieces = cpu_pieces(xs, threads)
    sample = sum(p.size for p in pieces)
    fns = cpu_kernels(sos)
    rates = {}
    for name, fn in fns.items():
        done, spent = 0, 0.0
        cpu_pass(fn, pieces[:1], 1)  # warm-up
        while spent < budget_s / len(fns):
            spent += cpu_pass(fn, pieces, threads)
            done += sample
        rates[name] = {"gsps": round(done / spent / 1e9, 4), "seconds": round(spent, 2)}
    one = cpu_pass(fns["scipy_sosfilt"], pieces[:1], 1)
    return {"value": rates["port"]["gsps"], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample} samples per pass: the first {sample} samples of the workload in {threads} pieces "
                      f"of {CPU_PIECE} (one per host thread, each an independent zero-state signal); value = the "
                      f"oracle's C port of the FP64 golden cascade",
            "implementations": rates,
            "scipy_sosfilt_1_thread_gsps": round(pieces[0].size / one / 1e9, 4)}


def run_reference(args, rank: int, world: int) -> None:
    """Reference arm: the reference's own CPU implementation of the path (its golden
    generator's FP64 sosfilt cascade, restated in C under oracle/) on all host threads, on the
    same pieces as the in-line CPU baseline; scipy's sosfilt itself is timed beside it."""
    if rank != 0:
        return
    import numpy as np
    from scipy import signal
    sos = signal.butter(HEADLINE["order"], 0.1, output="sos")
    threads = host_threads()
    sample = CPU_PIECE * threads
    x = np.random.default_rng(1).uniform(-1, 1, sample).astype(np.float32).astype(np.float64)
    pieces = cpu_pieces(x, threads)
    fns = cpu_kernels(sos)
    for _ in range(args.warmup):
        cpu_pass(fns["port"], pieces, threads)
    spent = sum(cpu_pass(fns["port"], pieces, threads) for _ in range(args.steps))
    dt = spent / args.steps
    value = sample / dt / 1e9
    sp = min(cpu_pass(fns["scipy_sosfilt"], pieces, threads) for _ in range(3))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"butter order {HEADLINE['order']} cutoff 0.1, uniform[-1,1) seed 1; "
                               f"step = {sample} samples of the 2^{LOG2N}-sample workload in {threads} pieces "
                               f"of {CPU_PIECE} (one per host thread, each an independent zero-state signal)",
                   "n_samples_per_step": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{sample} samples per step in {threads} independent pieces of {CPU_PIECE}, "
                                   "FP64 cascade (the oracle's C port of scipy's sosfilt as "
                                   "tools/ref_generate.py:89 calls it)",
                         "scipy_sosfilt_gsps": round(sample / sp / 1e9, 4)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------------------------
# forms (batching, serving, precision)
# ------------------------------------------------------------------------------------------
def run_batching(dev) -> dict:
    """Many channels of uneven length, each with its own filter, in one persistent launch; the
    chunk shape chosen by autotune.tune_batch (every compiled shape timed, in the order the
    occupancy model proposes); then the launch over a bound segment table is captured in a CUDA
    graph, and 10 replays are timed with CUDA events (device-resident); a few channels are
    checked against the oracle."""
    import numpy as np
    import torch

    import oracle
    from cuda_recursive_filtering_gb300 import Batch, autotune, workloads

    filters, lens = workloads.multichannel_mixed()
    batch = Batch(filters, max_segments=len(filters), max_chunks=int(lens.sum() // 1024 + len(filters)), device=dev)
    off = np.concatenate([[0], np.cumsum(lens)])
    x = workloads.uniform_signal(int(off[-1]), 3, device=dev)
    y = torch.empty_like(x)
    flt = np.arange(len(filters), dtype=np.int32)
    tuned = autotune.tune_batch(batch, x, y, off, flt, reps=3)
    # the tuned shape's launch over a bound segment table, captured in a CUDA graph and replayed
    bound = batch.bind(x, y, off, flt)
    bound()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        bound()
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(True), torch.cuda.Event(True)
    s.record()
    for _ in range(10):
        graph.replay()
    e.record()
    torch.cuda.synchronize()
    batch.check()
    ms = s.elapsed_time(e) / 10
    worst = 0.0
    for i in np.random.default_rng(0).choice(len(filters), 8, replace=False):
        xi = x[off[i]:off[i + 1]].cpu().numpy()
        _, ref = oracle.reference_golden(filters[i], xi)
        worst = max(worst, oracle.errors(y[off[i]:off[i + 1]].cpu().numpy(), ref)["rel_max"])
    return {"workload": "4096 channels, lengths log-uniform [2^10, 2^20], own filter each: order {2,4,8,16}, "
                        "butter / cheby1 (1 dB), cutoff U[0.02, 0.45], seed 3; one persistent launch of the "
                        "tuned chunk shape over a bound segment table, replayed from a captured CUDA graph",
            "value": round(float(off[-1]) / (ms * 1e-3) / 1e9, 1), "unit": "GS/s", "ms_per_launch": ms,
            "samples": int(off[-1]), "check_rel_max_8_channels": worst, "shape": batch.shape(),
            "tuner": tuned}


def run_precision(dev, log2n: int, hbm_gbs: float) -> dict:
    """Precision form (kernel TC: the chunk solve as tcgen05 GEMMs with split products; TC is the
    default operand form, TC_TF32 / TC_BF16x6 / TC_BF16x3 force GEMM 1's)
    against the plain PH and STCR_UNROLL realizations on the precision workload: butter(order,
    0.05) on N(0,1) noise plus 8 tones spanning 60 dB (seed 2), orders 8..16, device-resident,
    CUDA events over 5 launches each; max|err| / RMS(ref) over ALL outputs against the FP64
    oracle. `tc_vs_plain_at_1e-5` compares TC with the fastest plain row whose error is within
    the 1e-5 RMS-relative bar."""
    import torch

    from cuda_recursive_filtering_gb300 import Plan, workloads

    n = 1 << log2n
    x = workloads.noise_plus_tones(n, 2, device=dev)
    y = torch.empty_like(x)
    xh = x.cpu().numpy()
    stream = torch.cuda.current_stream()
    orders = (8, 10, 12, 14, 16)
    gold = Golden([(o, workloads.butter_sos(o, 0.05), xh) for o in orders], ahead=3)
    out = {"workload": f"butter(order, 0.05) SOS on 2^{log2n} samples of N(0,1) noise + 8 tones (60 dB span), "
                       "seed 2; error = max|err| / RMS(ref) over all outputs"}
    try:
        for order in orders:
            sos = workloads.butter_sos(order, 0.05)
            ref = DeviceRef(gold.get(order), dev)
            row = {}
            for kname, b, nb in (("TC", 0, 0), ("TC_TF32", 0, 0), ("TC_BF16x6", 0, 0), ("TC_BF16x3", 0, 0), ("PH", 32, 64),
                                 ("STCR_UNROLL", 32, 64)):
                # TC_TF32: GEMM 1 with TF32 hi / lo operands; TC_BF16x6 / x3: with BF16 operands,
                # three parts and six products / two parts and three products (IIR_GB300_TC_BF16,
                # read when the plan is created; the default takes BF16x6 for 5..8 states)
                bf = ("0" if kname == "TC_TF32" else
                      kname.split("x")[-1] if kname.startswith("TC_BF16") else None)
                if bf:
                    os.environ["IIR_GB300_TC_BF16"] = bf
                try:
                    pl = Plan(sos, "TC" if bf else kname, b, nb, max_n=n, device=dev)
                finally:
                    os.environ.pop("IIR_GB300_TC_BF16", None)
                t = time_plan(pl, x, y, 5, 2, stream, per_launch=True)
                pl.check()
                pl.close()
                row[kname] = row_entry(n / (t * 1e-3) / 1e9, hbm_gbs, ref.errors(y))
            plain = [row[k]["gsps"] for k in ("PH", "STCR_UNROLL") if row[k]["rel_rms"] <= 1e-5]
            row["tc_vs_ph"] = round(row["TC"]["gsps"] / row["PH"]["gsps"], 2)
            row["tc_vs_plain_at_1e-5"] = (round(row["TC"]["gsps"] / max(plain), 2)
                                          if plain and row["TC"]["rel_rms"] <= 1e-5 else None)
            out[f"order{order}"] = row
            del ref
    finally:
        gold.close()
    del x, y
    return out


def median_p99_run(results: list[dict]) -> dict:
    """The run with the median p99 latency (upper median for an even count), with every run's
    GS/s, p50, p99 and maximum latency listed under "runs"."""
    order = sorted(range(len(results)), key=lambda i: results[i]["p99_us"] or 0.0)
    out = dict(results[order[len(results) // 2]])
    out["runs"] = [{k: (round(r[k], 3) if r.get(k) is not None else None) for k in ("gsps", "p50_us", "p99_us", "max_us")}
                   for r in results]
    return out


def run_serving(dev, seconds: float = 4.0, runs: int = 3) -> dict:
    """Continuous-batching stream server under Poisson arrivals (host chunks in, results back
    on the host): achieved GS/s and request latency percentiles. The load runs ``runs`` times;
    the top-level figures are the run with the median p99, and every run is listed (a rare
    host-side stall of tens to hundreds of milliseconds sets the p99 of the run it falls in)."""
    from cuda_recursive_filtering_gb300 import workloads
    from cuda_recursive_filtering_gb300.serving import StreamServer, run_poisson_load

    filters, load = workloads.streaming_poisson()
    srv = StreamServer(filters, max_batch=1024, max_streams=len(filters), device=dev, keep_outputs=False)
    streams = [srv.open_stream(i) for i in range(len(filters))]
    # warm-up at the full rate, so that the first measured run finds every buffer at its working size
    run_poisson_load(srv, streams, rate_sps=load["rate_sps"], duration_s=1.0, chunk_lo=load["chunk_lo"],
                     chunk_hi=load["chunk_hi"], seed=1)
    results = []
    for k in range(runs):
        srv.completed.clear()
        srv.samples_done = 0
        results.append(run_poisson_load(srv, streams, rate_sps=load["rate_sps"], duration_s=seconds,
                                        chunk_lo=load["chunk_lo"], chunk_hi=load["chunk_hi"], seed=load["seed"] + k))
    out = median_p99_run(results)
    out["workload"] = ("1024 streams, order-8 butter cutoff U[0.05, 0.4] each; chunks U[256, 65536]; "
                       f"Poisson arrivals {load['rate_sps']:.0e} samples/s; {runs} runs of {seconds:g} s "
                       "(top level: the run with the median p99); host chunks in and out")
    return out


# ------------------------------------------------------------------------------------------
# the sweep: realization x order x geometry
# ------------------------------------------------------------------------------------------
def sweep_keys(order: int):
    for kname, geoms in SWEEP_GEOM.items():
        if kname == "PLR" and order > 8:
            continue  # float32 direct form: non-finite at order 16 (plr_emulator.py:228-248)
        for b, nb in geoms:
            yield kname, b, nb, f"order{order}_{kname}" + (f"_{b}x{nb}" if b else "")


def run_sweep(dev, x, xh, steps: int, hbm_gbs: float) -> dict:
    """Every realization x order x geometry at 2^LOG2N samples (and, with rotating buffers past
    L2, at 2^25), each with the error of all its outputs against the FP64 oracle."""
    import torch
    from scipy import signal

    from cuda_recursive_filtering_gb300 import Plan

    n = x.numel()
    stream = torch.cuda.current_stream()
    y = torch.empty_like(x)
    n25 = min(n, 1 << 25)
    nbuf = max(4, -(-2 * L2_BYTES // (4 * n25)))
    xs25 = [x[:n25].clone() for _ in range(nbuf)]
    ys25 = [torch.empty(n25, device=dev) for _ in range(nbuf)]
    orders = (2, 4, 8, 16)
    gold = Golden([(o, signal.butter(o, 0.1, output="sos"), xh) for o in orders], ahead=3)
    rows_full, rows_25, rows_refk = {}, {}, {}
    try:
        for order in orders:
            s_o = signal.butter(order, 0.1, output="sos")
            ref = DeviceRef(gold.get(order), dev)
            rows_refk.update(run_reference_kernels(dev, x, y, s_o, order, ref, hbm_gbs, stream))
            for kname, b, nb, key in sweep_keys(order):
                try:
                    pl = Plan(s_o, kname, b, nb, max_n=n, device=dev)
                    t = time_plan(pl, x, y, max(3, steps // 2), 2, stream, per_launch=True)
                    rows_full[key] = row_entry(n / (t * 1e-3) / 1e9, hbm_gbs, ref.errors(y))
                    if n25 < n:
                        ms = time_rotating(pl, xs25, ys25, 5, 2 * nbuf, stream)
                        rows_25[key] = row_entry(n25 / (statistics.median(ms) * 1e-3) / 1e9, hbm_gbs,
                                                 ref.errors(ys25[0], n25))
                    pl.close()
                except Exception as exc:  # report, do not hide
                    rows_full[key] = f"error: {exc}"
            del ref
    finally:
        gold.close()
    del xs25, ys25, y
    out = {f"2^{n.bit_length() - 1}": rows_full}
    for key, row in rows_refk.items():  # the same realization and geometry of this library, and the ratio
        ours = rows_full.get(key.replace("reference_", ""))
        if isinstance(row, dict) and isinstance(ours, dict):
            row["ours_gsps"] = ours["gsps"]
            row["ours_vs_reference"] = round(ours["gsps"] / row["gsps"], 1)
    out["reference_kernels"] = rows_refk
    if rows_25:
        out["2^25"] = rows_25
        out["2^25_method"] = (f"{nbuf} identical input and output buffers (> 2x L2) cycled, 5 batches of "
                              f"{2 * nbuf} launches, median batch")
    return out


def run_reference_kernels(dev, x, y, sos, order: int, ref, hbm_gbs: float, stream) -> dict:
    """The reference's own GPU kernels, PH_32, STCR_32_LOOP, STCR_32_UNROLL_64, DTCR_32_LOOP and
    DTCR_32_UNROLL_64 (include/{ph,stcr,dtcr}_kernels.cuh), built from its sources into device code
    (oracle/refgpu.py) and launched on this GPU under its own launch contract, on the same signal
    (times the cascade's gain, as its drivers give it) with the same timing as this library's rows;
    every output against the same FP64 oracle."""
    import numpy as np
    import torch

    import oracle
    from oracle import refgpu
    if not refgpu.available():
        return {f"reference_order{order}": "unavailable: the reference kernels' cubins (oracle/_ref) are absent"}
    sn, g = oracle.normalise_sos(sos)
    xs = (x * np.float32(g)).contiguous()
    rows = {}
    for kname in refgpu.KERNELS:
        rk = refgpu.RefKernel(kname, sn, x.numel(), device=dev)
        for _ in range(3):
            rk(xs, y)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        for a, b in ev:
            a.record(stream)
            rk(xs, y, stream)
            b.record(stream)
        torch.cuda.synchronize()
        ms = statistics.median(a.elapsed_time(b) for a, b in ev)
        rows[f"reference_order{order}_{kname}_32x64"] = row_entry(x.numel() / (ms * 1e-3) / 1e9, hbm_gbs,
                                                                  ref.errors(y))
        rk.close()
    del xs
    return rows


def run_small(dev, hbm_gbs: float) -> dict:
    """The latency regime (2^16 samples, butter(2, 0.1), uniform[-1,1) seed 0): the reference's
    timing method — 1032 identical buffers (2 x L2) cycled, 20 batches of 200 launches, the
    20th-percentile and median batch (include/measure.cuh:70-109) — with the error of the
    output against the FP64 oracle (gate max|err| / RMS <= 1e-5)."""
    import numpy as np
    import torch
    from scipy import signal

    import oracle
    from cuda_recursive_filtering_gb300 import Plan, workloads

    n = 1 << 16
    sos = signal.butter(2, 0.1, output="sos")
    x = workloads.uniform_signal(n, 0, device=dev)
    _, ref = oracle.reference_golden(sos, x.cpu().numpy())
    nbuf = -(-2 * L2_BYTES // (4 * n))
    xs = [x.clone() for _ in range(nbuf)]
    ys = [torch.empty(n, device=dev) for _ in range(nbuf)]
    stream = torch.cuda.current_stream()
    rows = {}
    for kname, b, nb in (("PH", 32, 64), ("DTCR", 32, 64), ("DTCR_UNROLL", 32, 64), ("STCR", 32, 64),
                         ("STCR_UNROLL", 32, 64), ("PLR", 0, 0), ("TC", 0, 0)):
        pl = Plan(sos, kname, b, nb, max_n=n, device=dev)
        ms = time_rotating(pl, xs, ys, 20, 200, stream)
        e = oracle.errors(ys[0].cpu().numpy(), ref)
        pl.close()
        ms_sorted = sorted(ms)
        p20 = ms_sorted[len(ms_sorted) // 5]
        key = f"order2_{kname}" + (f"_{b}x{nb}" if b else "")
        rows[key] = dict(row_entry(n / (p20 * 1e-3) / 1e9, hbm_gbs, e),
                         gsps_median=round(n / (statistics.median(ms) * 1e-3) / 1e9, 1),
                         us_per_launch_p20=round(p20 * 1e3, 2))
    # the same launches from a captured CUDA graph (200 launches over the rotating buffers per
    # replay, 20 replays): the host's launch cost leaves the measured time
    for kname, b, nb in (("PH", 32, 64), ("DTCR_UNROLL", 32, 64)):
        pl = Plan(sos, kname, b, nb, max_n=n, device=dev)
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            for i in range(3):
                pl(xs[i % nbuf], ys[i % nbuf])
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            for i in range(200):
                pl(xs[i % nbuf], ys[i % nbuf])
        graph.replay()
        torch.cuda.synchronize()
        ms = []
        for _ in range(20):
            s0, e0 = torch.cuda.Event(True), torch.cuda.Event(True)
            s0.record(stream)
            graph.replay()
            e0.record(stream)
            torch.cuda.synchronize()
            ms.append(s0.elapsed_time(e0) / 200)
        pl.check()
        e = oracle.errors(ys[0].cpu().numpy(), ref)
        del graph
        pl.close()
        p20 = sorted(ms)[len(ms) // 5]
        rows[f"order2_{kname}_{b}x{nb}_graph"] = dict(
            row_entry(n / (p20 * 1e-3) / 1e9, hbm_gbs, e),
            gsps_median=round(n / (statistics.median(ms) * 1e-3) / 1e9, 1), us_per_launch_p20=round(p20 * 1e3, 2))
    # the reference's own kernels on the same buffers and timing (oracle/refgpu.py)
    from oracle import refgpu
    if refgpu.available():
        sn, g = oracle.normalise_sos(sos)
        xsg = [(t * np.float32(g)).contiguous() for t in xs]
        for kname in refgpu.KERNELS:
            rk = refgpu.RefKernel(kname, sn, n, device=dev)
            ms = time_rotating(_RefAsPlan(rk), xsg, ys, 20, 200, stream)
            e = oracle.errors(ys[0].cpu().numpy(), ref)
            rk.close()
            p20 = sorted(ms)[len(ms) // 5]
            rows[f"reference_order2_{kname}_32x64"] = dict(
                row_entry(n / (p20 * 1e-3) / 1e9, hbm_gbs, e),
                gsps_median=round(n / (statistics.median(ms) * 1e-3) / 1e9, 1), us_per_launch_p20=round(p20 * 1e3, 2))
        del xsg
    del xs, ys
    return {"rows": rows, "method": f"{nbuf} identical input and output buffers cycled, 20 batches of 200 launches; "
                                    "gsps = 20th-percentile batch, gsps_median = median batch; *_graph rows: the "
                                    "200 launches of a batch replayed from a captured CUDA graph"}


def run_ours(args, rank: int, world: int, local_rank: int) -> None:
    import torch
    from scipy import signal

    import cuda_recursive_filtering_gb300 as pkg
    from cuda_recursive_filtering_gb300 import Plan, workloads

    torch.cuda.set_device(local_rank)
    pkg.load_library()
    dev = torch.device("cuda", local_rank)
    n = 1 << LOG2N
    stream = torch.cuda.current_stream()
    x = workloads.uniform_signal(n, 1, device=dev)
    xh = x.cpu().numpy()
    y = torch.empty_like(x)
    pk = peaks()

    # ---- headline: device-resident throughput ----
    sos = signal.butter(HEADLINE["order"], 0.1, output="sos")
    plan = Plan(sos, HEADLINE["kernel"], HEADLINE["block_size"], HEADLINE["n_blocks"], max_n=n, device=dev)
    for _ in range(2):
        plan(x, y)
    torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.15)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ms = time_plan(plan, x, y, args.steps, args.warmup, stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n / (ms * 1e-3) / 1e9
    achieved = BYTES_PER_SAMPLE * n / (ms * 1e-3) / 1e9
    # correctness of this exact run: every output of the last timed launch against the oracle
    # (computed on host threads only now, so that nothing competes with the timed launches)
    gold = Golden([("headline", sos, xh)], ahead=1)
    head_ref = DeviceRef(gold.get("headline"), dev)
    gold.close()
    chk = head_ref.errors(y)
    del head_ref

    # ---- end to end: host buffers through the public API (C ABI), copies inside ----
    # iir_plan_execute_host: pinned host input and output; the copies of the signal's pieces
    # overlap the filtering on three streams, each piece starting from the previous one's state.
    e2e = None
    if rank == 0 or world > 1:
        xhp = torch.empty(n, dtype=torch.float32, pin_memory=True)
        xhp.copy_(torch.from_numpy(xh))
        yh = torch.empty(n, dtype=torch.float32, pin_memory=True)
        hplan = Plan(sos, HEADLINE["kernel"], HEADLINE["block_size"], HEADLINE["n_blocks"], max_n=n)
        e2e_steps = max(2, min(args.steps, 5))
        for _ in range(2):
            hplan.filter_host(xhp, out=yh)
        hplan.check()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            hplan.filter_host(xhp, out=yh)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / e2e_steps
        hplan.check()
        e2e = {"value": world * n / dt / 1e9, "unit": UNIT, "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n,
               "ms_per_step": dt * 1e3, "api": "iir_plan_execute_host, pieces of 2^24 samples",
               "check_max_abs_diff_vs_device_output": float((yh.to(dev) - y).abs().max())}
        hplan.close()
        del xhp, yh

    # ---- sweep rows with full-length errors, the latency regime, the forms ----
    sweep = {}
    if not args.no_sweep:
        try:
            sweep = run_sweep(dev, x, xh, args.steps, pk["hbm_gbs"])
        except Exception as exc:  # report, do not hide
            sweep = {"error": str(exc)}
        try:
            sweep["2^16"] = run_small(dev, pk["hbm_gbs"])
        except Exception as exc:
            sweep["2^16"] = {"error": str(exc)}
    del y
    forms = {}
    if not args.no_forms:
        try:
            forms["precision"] = run_precision(dev, LOG2N, pk["hbm_gbs"])
        except Exception as exc:  # report, do not hide
            forms["precision"] = {"error": str(exc)}
        try:
            forms["batching"] = run_batching(dev)
        except Exception as exc:  # report, do not hide
            forms["batching"] = {"error": str(exc)}
        try:
            forms["serving"] = run_serving(dev)
        except Exception as exc:
            forms["serving"] = {"error": str(exc)}
    if rank != 0:
        return
    cpu = cpu_baseline_sample(sos, xh, budget_s=args.cpu_seconds)
    traffic = ncu_traffic_per_launch()
    tr = None
    if traffic is not None:
        tr = traffic["bytes"] * (n / traffic["samples"] if traffic.get("samples") else 1.0)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"plain roofline sweep: butter order {HEADLINE['order']} cutoff 0.1 (SOS), "
                               f"2^{LOG2N} float32 samples uniform[-1,1) seed 1, zero initial state",
                   "kernel": HEADLINE["kernel"], "geometry": f"{HEADLINE['block_size']}x{HEADLINE['n_blocks']}",
                   "n_samples": n, "order": HEADLINE["order"],
                   "l2": "inputs (1 GiB) larger than L2 (129 MB): no flush between steps",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": tr,
                     "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 2^28 "
                                        "(profiles/dtcr_unroll_order2_traffic_2p28.md)") if tr else None,
                     "peak_source": pk["source"] + " (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": args.steps * plan.launches_per_execute(),
        "clocks": clk,
        "check": {"rel_max": float(f"{chk['rel_max']:.3g}"), "rel_rms": float(f"{chk['rel_rms']:.3g}"),
                  "samples": n, "what": "all outputs of the last timed launch against the FP64 oracle"},
        "sweep": sweep,
    }
    out.update(forms)
    print(json.dumps(out), flush=True)


def run_only_batch(args, spec: str) -> None:
    """The batching form alone (a short command to profile its kernel): BATCH[:ROWSxN] is the mixed
    multichannel workload with channel lengths scaled by 2^(LOG2N - 28) (at least 64 samples each),
    BATCH1:ORDER[:ROWSxN] one segment of 2^LOG2N samples with butter(ORDER, 0.1); chunk shape ROWSxN
    (default 128x64), a bound segment table launched args.steps times after args.warmup."""
    import numpy as np
    import torch

    import cuda_recursive_filtering_gb300 as pkg
    from cuda_recursive_filtering_gb300 import Batch, workloads
    parts = spec.split(":")
    single = parts[0] == "BATCH1"  # BATCH1:ORDER[:ROWSxN]: one segment of 2^LOG2N, butter(ORDER, 0.1)
    k = 2 if single else 1
    shape_part = parts[k] if len(parts) > k else None
    rows, n_per_row = (int(v) for v in shape_part.split("x")) if shape_part else (128, 64)
    pkg.load_library()
    dev = torch.device("cuda", 0)
    if single:
        from scipy import signal
        filters, lens = [signal.butter(int(parts[1]), 0.1, output="sos")], np.array([1 << LOG2N], dtype=np.int64)
    else:
        filters, lens = workloads.multichannel_mixed()
        lens = np.maximum(64, (lens.astype(np.float64) * 2.0 ** (LOG2N - 28)).astype(np.int64))
    batch = Batch(filters, max_segments=len(filters), max_chunks=int(lens.sum() // 1024 + len(filters)), device=dev)
    batch.set_shape(rows, n_per_row)
    off = np.concatenate([[0], np.cumsum(lens)])
    x = workloads.uniform_signal(int(off[-1]), 3, device=dev)
    y = torch.empty_like(x)
    bound = batch.bind(x, y, off, np.arange(len(filters), dtype=np.int32))
    for _ in range(args.warmup):
        bound()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(True), torch.cuda.Event(True)
    s.record()
    for _ in range(args.steps):
        bound()
    e.record()
    torch.cuda.synchronize()
    batch.check()
    ms = s.elapsed_time(e) / args.steps
    print(json.dumps({"only": spec, "shape": batch.shape(), "samples": int(off[-1]), "ms_per_launch": ms,
                      "gsps": round(float(off[-1]) / (ms * 1e-3) / 1e9, 1)}), flush=True)


def run_only(args, spec: str) -> None:
    """One realization / order / geometry on the plain workload at 2^LOG2N samples, timed like the
    headline and nothing else (a short command to profile one kernel): spec = KERNEL:ORDER[:BxN],
    or BATCH[:ROWSxN] for the batching form (run_only_batch)."""
    import torch
    from scipy import signal

    import cuda_recursive_filtering_gb300 as pkg
    from cuda_recursive_filtering_gb300 import Plan, workloads
    if spec.split(":")[0] in ("BATCH", "BATCH1"):
        run_only_batch(args, spec)
        return
    parts = spec.split(":")
    kernel, order = parts[0], int(parts[1])
    b, nb = (int(v) for v in parts[2].split("x")) if len(parts) > 2 else (0, 0)
    pkg.load_library()
    dev = torch.device("cuda", 0)
    n = 1 << LOG2N
    x = workloads.uniform_signal(n, 1, device=dev)
    y = torch.empty_like(x)
    plan = Plan(signal.butter(order, 0.1, output="sos"), kernel, b, nb, max_n=n, device=dev)
    ms = time_plan(plan, x, y, args.steps, args.warmup, torch.cuda.current_stream())
    print(json.dumps({"only": spec, "plan": plan.info(), "n": n, "ms_per_launch": ms,
                      "gsps": round(n / (ms * 1e-3) / 1e9, 1)}), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the precision, batching and serving legs")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--log2n", type=int, default=LOG2N,
                    help="signal length 2^k (the bench line is quoted at 2^28; smaller k is for profiling)")
    ap.add_argument("--only", default=None, metavar="KERNEL:ORDER[:BxN] | BATCH[:ROWSxN] | BATCH1:ORDER[:ROWSxN]",
                    help="time one realization / order / geometry and print only that (for profiling)")
    args = ap.parse_args()
    globals()["LOG2N"] = args.log2n
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        elif args.only:
            run_only(args, args.only)
        else:
            run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
