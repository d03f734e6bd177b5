"""The batching tuner's occupancy and cost model (autotune.py), on the CPU: the GB300 restatement
of the reference's supply / demand residency (include/gpu_specs.hpp:57-116) and the ranking of
chunk shapes it seeds the timed search with."""
import numpy as np

from cuda_recursive_filtering_gb300 import autotune

# footprints of the four compiled batch shapes (threads, registers per thread, shared memory)
SHAPES = [dict(rows=128, samples_per_row=64, chunk=8192, threads=160, regs_per_thread=64, smem_bytes=33644),
          dict(rows=128, samples_per_row=32, chunk=4096, threads=160, regs_per_thread=64, smem_bytes=17260),
          dict(rows=128, samples_per_row=16, chunk=2048, threads=160, regs_per_thread=64, smem_bytes=9068),
          dict(rows=64, samples_per_row=16, chunk=1024, threads=96, regs_per_thread=95, smem_bytes=4972)]


def test_supply_blocks_per_sm():
    g = autotune.GB300
    # 160 threads x 64 registers: 5 warps x 2048 registers = 10240 per block -> 6 by registers;
    # 33644 + 1024 bytes of shared memory -> 6 by shared memory
    assert autotune.supply_blocks_per_sm(160, 64, 33644, g) == 6
    # 1024 threads per block: 2 by threads
    assert autotune.supply_blocks_per_sm(1024, 32, 0, g) == 2
    # 32 threads, tiny footprint: the 32-block cap
    assert autotune.supply_blocks_per_sm(32, 16, 0, g) == 32
    # a block that does not fit
    assert autotune.supply_blocks_per_sm(160, 64, 230 * 1024, g) == 0


def test_demand_blocks_per_sm():
    assert autotune.demand_blocks_per_sm(1, autotune.GB300) == 1
    assert autotune.demand_blocks_per_sm(152 * 3 + 1, autotune.GB300) == 4


def test_rank_long_segments_prefers_big_chunks():
    lengths = np.exp(np.random.default_rng(3).uniform(np.log(1 << 10), np.log(1 << 20), 4096)).astype(np.int64)
    order = autotune.rank_batch_shapes(SHAPES, lengths)
    assert order[0]["chunk"] == 8192 and order[0]["score"] == 1.0
    assert all(0 < r["score"] <= 1.0 and 0 < r["useful"] <= 1.0 for r in order)


def test_rank_short_segments_prefers_small_chunks():
    lengths = np.random.default_rng(9).integers(500, 3000, 2000)
    order = autotune.rank_batch_shapes(SHAPES, lengths)
    assert order[0]["chunk"] <= 4096 and order[-1]["chunk"] == 8192  # most of an 8192 chunk is padding
    # a single segment shorter than every chunk: the smallest chunk pads least
    assert autotune.rank_batch_shapes(SHAPES, [700])[0]["chunk"] == 1024


def test_rank_few_chunks_is_limited_by_demand():
    # 152 chunks of 8192 fill one block per SM: residency is the demand, not the supply
    order = {r["chunk"]: r for r in autotune.rank_batch_shapes(SHAPES, [8192 * 152])}
    assert order[8192]["resident"] == 1 and order[8192]["supply"] == 6
