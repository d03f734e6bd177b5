"""Autotuner for the realizations: picks realization and BLOCK_SIZE x N_BLOCKS geometry
for a filter and signal length by timing the candidates on this GPU (CUDA events, device-
resident data) and checking each against the FP64 reference filter on a prefix.

The candidate order is a prior taken from measurements on GB300: at order 2 the two-pass
single-section kernels, PH first; for cascades the precision form (TC) first, then PH with 64
samples per row. (The reference
picks its launch shape from an occupancy model, gpu_specs.hpp:57-116; here the resident-block
count comes from the CUDA occupancy query and the rest is measured.) Results are cached per
(device, order, filter, signal-length bucket) in memory and, optionally, in a JSON file.
"""
from __future__ import annotations

import json
import os

import numpy as np
import torch

from .api import Plan

__all__ = ["tune", "tuned_plan", "GB300", "supply_blocks_per_sm", "demand_blocks_per_sm", "rank_batch_shapes",
           "tune_batch"]

_CANDIDATES_ORDER2 = [("PH", 32, 64), ("PH", 32, 32), ("STCR_UNROLL", 32, 64), ("STCR_UNROLL", 32, 32),
                      ("DTCR_UNROLL", 32, 128), ("DTCR_UNROLL", 32, 64), ("PH", 32, 128), ("PLR", 0, 0)]
_CANDIDATES_CASCADE = [("TC", 0, 0), ("PH", 32, 64), ("PH", 32, 32), ("STCR_UNROLL", 32, 64), ("DTCR_UNROLL", 32, 64),
                       ("PH", 32, 128), ("STCR_UNROLL", 32, 32)]
_memo: dict = {}


def _key(sos: np.ndarray, n: int, device) -> str:
    name = torch.cuda.get_device_name(device)
    digest = np.asarray(sos, np.float32).tobytes().hex()[:32]
    return f"{name}|{sos.shape[0]}|{digest}|{max(10, int(np.log2(max(n, 1))))}"


def _reference_check(sos, x: np.ndarray) -> np.ndarray:
    from scipy import signal
    s = np.asarray(sos, np.float64)
    return signal.sosfilt(s, x.astype(np.float64))


def tune(sos, n: int, candidates=None, reps: int = 5, device=None, cache_path: str | None = None) -> dict:
    """Times every candidate (realization, block_size, n_blocks) on a signal of
    min(n, 2^26) samples and returns {"kernel", "block_size", "n_blocks", "gsps", "table"}.
    Candidates whose output on a 2^16-sample prefix misses max|err| <= 1e-4 max|ref| (the
    reference's gate) are skipped."""
    sos = np.asarray(sos, dtype=np.float32).reshape(-1, 6)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    key = _key(sos, n, dev)
    if key in _memo:
        return _memo[key]
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            disk = json.load(f)
        if key in disk:
            _memo[key] = disk[key]
            return disk[key]
    if candidates is None:
        candidates = _CANDIDATES_ORDER2 if sos.shape[0] == 1 else _CANDIDATES_CASCADE
    m = int(min(max(n, 1 << 16), 1 << 26))
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    x = torch.rand(m, generator=g, device=dev).mul_(2).sub_(1)
    y = torch.empty_like(x)
    prefix = x[: 1 << 16].cpu().numpy()
    ref = _reference_check(sos, prefix)
    scale = float(np.max(np.abs(ref))) or 1.0
    table = []
    for kernel, b, nb in candidates:
        try:
            plan = Plan(sos, kernel, b, nb, max_n=m, device=dev)
        except Exception:
            continue
        plan(x, y)
        plan.check()
        err = float(np.max(np.abs(y[: 1 << 16].cpu().numpy() - ref)))
        if not np.isfinite(err) or err > 1e-4 * scale:
            table.append({"kernel": kernel, "block_size": b, "n_blocks": nb, "gsps": None, "rejected": err / scale})
            plan.close()
            continue
        for _ in range(2):
            plan(x, y)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(True), torch.cuda.Event(True)
        s.record()
        for _ in range(reps):
            plan(x, y)
        e.record()
        torch.cuda.synchronize()
        ms = s.elapsed_time(e) / reps
        table.append({"kernel": kernel, "block_size": b, "n_blocks": nb, "gsps": m / (ms * 1e-3) / 1e9})
        plan.close()
    timed = [t for t in table if t["gsps"] is not None]
    if not timed:
        raise RuntimeError("no candidate passed the accuracy gate")
    best = max(timed, key=lambda t: t["gsps"])
    result = dict(best, table=table)
    _memo[key] = result
    if cache_path:
        disk = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                disk = json.load(f)
        disk[key] = result
        with open(cache_path, "w") as f:
            json.dump(disk, f, indent=1)
    return result


def tuned_plan(sos, n: int, **kw) -> Plan:
    """A Plan with the tuned realization and geometry for this filter and signal length."""
    best = tune(sos, n, **{k: v for k, v in kw.items() if k in ("candidates", "reps", "device", "cache_path")})
    return Plan(sos, best["kernel"], best["block_size"], best["n_blocks"], max_n=n, device=kw.get("device"))


# ------------------------------------------------------------------------------------------------
# Batching form: the chunk shape, chosen by timing, in the order an occupancy model proposes
# ------------------------------------------------------------------------------------------------
# The reference sizes its launches with an occupancy model of its two GPUs (gpu_specs.hpp:16-46 has
# GTX 1070 and RTX 3060 profiles only, and compiling elsewhere silently uses the RTX 3060 one).
# GB300 profile (sm_103a): 228 KB of shared memory per SM with 1 KB reserved per resident block,
# 227 KB per block at most, 64 Ki registers, 2048 threads, 64 warps and 32 blocks per SM.
# chunk_overhead_samples: the fixed cost of one chunk of the batch kernel (draw, segment search,
# barriers, lookback) in sample-equivalents, fitted on GB300 to one 2^28-sample segment filtered
# with each shape: a block's time per chunk is about 3.5 us + 0.97 ns per sample of the chunk.
GB300 = {"name": "GB300 (sm_103a)", "num_sms": 152, "registers_per_sm": 65536, "shared_mem_per_sm": 228 * 1024,
         "reserved_shared_mem_per_tb": 1024, "max_shared_mem_per_tb": 227 * 1024, "max_threads_per_sm": 2048,
         "max_warps_per_sm": 64, "max_tbs_per_sm": 32, "max_threads_per_tb": 1024, "warp_size": 32,
         "register_alloc_unit": 256, "chunk_overhead_samples": 3600}


def supply_blocks_per_sm(threads: int, regs_per_thread: int, smem_bytes: int, prof: dict = GB300) -> int:
    """Resident blocks per SM the hardware allows (the supply side): gpu_specs.hpp:57-74
    (compute_supply_tb_per_sm) restated with the kernel's own footprint instead of the
    reference's estimate from BLOCK_SIZE x N_BLOCKS: the minimum over shared memory, registers
    (allocated per warp in units of 256), threads, warps and the block cap."""
    warps = -(-threads // prof["warp_size"])
    unit = prof["register_alloc_unit"]
    regs_per_warp = -(-regs_per_thread * prof["warp_size"] // unit) * unit
    limits = [prof["shared_mem_per_sm"] // (smem_bytes + prof["reserved_shared_mem_per_tb"]),
              prof["registers_per_sm"] // max(1, regs_per_warp * warps),
              prof["max_threads_per_sm"] // threads,
              prof["max_warps_per_sm"] // warps,
              prof["max_tbs_per_sm"]]
    return max(0, min(limits))


def demand_blocks_per_sm(chunks: int, prof: dict = GB300) -> int:
    """Blocks per SM the launch asks for when its chunks spread evenly over the SMs
    (gpu_specs.hpp:83-86, compute_demand_tb_per_sm)."""
    return -(-chunks // prof["num_sms"])


def rank_batch_shapes(shapes: list[dict], lengths, prof: dict = GB300) -> list[dict]:
    """Orders candidate chunk shapes for segments of the given lengths, fastest predicted first.
    A shape's launch keeps `resident` = min(supply, demand) blocks per SM busy (the reference's
    effective residency, gpu_specs.hpp:100-104); each block takes chunks one after another at
    (chunk_overhead_samples + chunk) sample-times per chunk, padding past a segment's end
    included. Predicted time = chunks / (resident x SMs) waves of that; score = the segments'
    samples / predicted time, normalised to the best shape. `useful` is the unpadded fraction."""
    lengths = np.asarray(lengths, dtype=np.int64)
    total = int(lengths.sum())
    rows = []
    for sh in shapes:
        chunk = sh["chunk"]
        chunks = int(np.sum(-(-lengths // chunk)))
        supply = supply_blocks_per_sm(sh["threads"], sh["regs_per_thread"], sh["smem_bytes"], prof)
        resident = min(supply, demand_blocks_per_sm(chunks, prof))
        slots = max(1, resident * prof["num_sms"])
        waves = max(1.0, chunks / slots)
        rows.append(dict(sh, chunks=chunks, supply=supply, resident=resident,
                         useful=total / max(1, chunks * chunk),
                         predicted=waves * (prof["chunk_overhead_samples"] + chunk)))
    best = min(r["predicted"] for r in rows) or 1.0
    for r in rows:
        r["score"] = best / r["predicted"]
    return sorted(rows, key=lambda r: -r["score"])


def tune_batch(batch, x, y, offsets, filters, reps: int = 3, prof: dict | None = None) -> dict:
    """Chooses the chunk shape of `batch` for segments packed in x / y at `offsets` (filters[i] for
    segment i): every compiled shape, in the order rank_batch_shapes proposes, is timed over
    `reps` launches (CUDA events, after one warm-up launch), and the fastest is left set.
    Returns {"shape", "gsps", "table"} with the model's figures beside each measurement."""
    from .api import Batch
    prof = dict(GB300 if prof is None else prof)
    prof["num_sms"] = torch.cuda.get_device_properties(batch.device).multi_processor_count
    offsets = np.asarray(offsets, dtype=np.int64)
    lengths = np.diff(offsets)
    shapes = []
    for rows_, n_ in Batch.SHAPES:
        batch.set_shape(rows_, n_)
        shapes.append(batch.shape())
    table = []
    for cand in rank_batch_shapes(shapes, lengths, prof):
        batch.set_shape(cand["rows"], cand["samples_per_row"])
        batch.packed(x, y, offsets, filters)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(True), torch.cuda.Event(True)
        s.record()
        for _ in range(reps):
            batch.packed(x, y, offsets, filters)
        e.record()
        torch.cuda.synchronize()
        batch.check()
        ms = s.elapsed_time(e) / reps
        table.append({k: cand[k] for k in ("rows", "samples_per_row", "chunk", "chunks", "supply", "resident",
                                           "blocks_per_sm", "useful", "score")}
                     | {"gsps": round(int(lengths.sum()) / (ms * 1e-3) / 1e9, 1)})
    best = max(table, key=lambda t: t["gsps"])
    batch.set_shape(best["rows"], best["samples_per_row"])
    return {"shape": [best["rows"], best["samples_per_row"]], "gsps": best["gsps"], "table": table,
            "model_order": [[t["rows"], t["samples_per_row"]] for t in table]}

