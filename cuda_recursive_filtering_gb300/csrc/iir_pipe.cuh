// iir_pipe.cuh — warp-specialized persistent pipeline for single-section filters (order 2).
//
// The grid is launched cooperatively (all blocks co-resident) and block b filters chunks
// b, b + G, b + 2G, ... The reference takes chunks from a ticket counter at block start
// (ph_kernels.cuh:227-229); with co-residency guaranteed a static order is equally
// deadlock-free (the lowest chunk without an inclusive carry always belongs to a running
// block whose earlier chunks are done) and a block knows its next chunks in advance.
// Every chunk goes through
//   LOAD   one TMA tensor load into one of S shared-memory stages      (TMA warp)
//   P1     zero-state solve: the chunk filtered with zero state at its  (row warps)
//          start, per-row zero-state incoming pairs, the chunk aggregate
//   CARRY  publish the aggregate, two-level lookback, publish the       (lookback warp)
//          inclusive carry
//   P2     correction by the response to the chunk's incoming state     (row warps)
//   STORE  one TMA tensor store                                         (TMA warp)
// Row warps run P1(k) and then P2(k - LAG), so the lookback of chunk k overlaps LAG chunk
// solves of the same block: its latency (set by the predecessors' progress, microseconds)
// leaves the critical path. Roles hand stages over through mbarriers:
//   full[s]  TMA load landed (or, for element-wise chunks, the stage is free)
//   part[s]  P1 done, aggregate in partv[s]
//   xrdy[s]  incoming state of the chunk in xv[s]
//   done[s]  P2 done, stage holds the output
// Every wait is bounded by the plan's timeout; a wait that runs out records an error and
// makes the block skip its remaining work, after it has waited (bounded) for its own copies.
#pragma once
#include "iir_device.cuh"

namespace iirgb {

// Per-chunk phase timestamps for performance analysis (IIR_PROFILE builds only):
// prof[(block * 16 + k) * 8 + slot] for the block's first 16 chunks.
#ifdef IIR_PROFILE
#define PIPE_STAMP(k, slot)                                                                            \
    do {                                                                                               \
        if (p.prof && (k) < 16u) p.prof[(static_cast<size_t>(blockIdx.x) * 16 + (k)) * 8 + (slot)] = globaltimer_ns(); \
    } while (0)
#else
#define PIPE_STAMP(k, slot) \
    do {                    \
    } while (0)
#endif

// Lookback of the persistent pipeline: 1 = two-level decoupled lookback over chunk and group
// slots (inclusive carries published by every chunk), 0 = window of the G-1 preceding
// aggregates plus the block's own previous carry.
#ifndef IIR_PIPE_HIER
#define IIR_PIPE_HIER 1
#endif

struct PipeAux {
    unsigned long long full[8];
    unsigned long long part[8];
    unsigned long long xrdy[8];
    unsigned long long done[8];
    float partv[8][2];
    float xv[8][2];
    float wtot[16][2][2];
    unsigned int epoch;
    int bail;      // lookback gave up: no more stores
    int abandon;   // an mbarrier wait ran out: skip every remaining wait
    int pad;
};

template <int ROWS, int N, int S>
struct PipeGeom {
    static constexpr int CHUNK = ROWS * N;
    static constexpr int LINES = CHUNK / 32;
    static_assert(N == 16 || N == 32 || N == 64 || N == 128, "samples per row");
    static_assert(LINES <= 256, "one TMA box per chunk");
    static_assert(S >= 2 && S <= 8, "stages");
    static constexpr size_t DATA_BYTES = static_cast<size_t>(CHUNK) * sizeof(float);
    static constexpr size_t ZIN_BYTES = static_cast<size_t>(ROWS) * 2 * sizeof(float);
    static constexpr size_t HIST_BYTES = 128;  // the 32 input samples before the chunk
    // table cache: C^(r+1) (r < ROWS), G^(t+1) (t < 32), Q^l and Q^(32 l) (l <= 32), A^(N/2)
    static constexpr int TC_CPOW = 0, TC_GPOW = ROWS, TC_QC = ROWS + 32, TC_QG = ROWS + 65, TC_HALF = ROWS + 98,
                         TC_LEN = ROWS + 100;
    static constexpr size_t TC_BYTES = static_cast<size_t>(TC_LEN) * 16;
    static constexpr size_t SMEM_BYTES =
        1024 + S * (DATA_BYTES + ZIN_BYTES + HIST_BYTES) + TC_BYTES + sizeof(PipeAux);
    // resident blocks per SM that shared memory allows (1 KB reserved per block)
    static constexpr int BLOCKS_BY_SMEM = static_cast<int>((227 * 1024) / (SMEM_BYTES + 1024));
    static constexpr int min_blocks(int threads) {
        const int by_thr = 2048 / threads;
        const int b = BLOCKS_BY_SMEM < by_thr ? BLOCKS_BY_SMEM : by_thr;
        return b < 1 ? 1 : b;
    }
};

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded mbarrier wait that gives up at once after any earlier wait of the block ran out.
// Its limit is four lookback limits: a stage wait is downstream of a lookback, so a chunk
// whose predecessor never publishes reports the lookback timeout (the cause), not this.
__device__ __forceinline__ bool pipe_wait(PipeAux* aux, unsigned long long* bar, uint32_t parity,
                                          const IirParams& p, uint32_t epoch) {
    if (*reinterpret_cast<volatile int*>(&aux->abandon)) return false;
    const long long limit = p.timeout_ns < (1ll << 60) ? 4 * p.timeout_ns : p.timeout_ns;
    if (wait_mbar_bounded(bar, parity, limit)) return true;
    *reinterpret_cast<volatile int*>(&aux->abandon) = 1;
    raise_error(p.state, epoch, IIR_DEV_ERR_MBARRIER);
    return false;
}

// Last block out advances the launch epoch (every block of a persistent launch runs to the
// end, so the ticket counter is not used).
__device__ __forceinline__ void pipe_finish(IirLaunchState* st, uint32_t epoch) {
    __threadfence();
    const unsigned prev = atomicAdd(&st->done, 1u);
    if (prev == gridDim.x - 1) {
        atomicExch(&st->done, 0u);
        atomicExch(&st->ticket, static_cast<unsigned long long>(epoch + 1u) << 32);
        __threadfence();
    }
}

// Incoming state of chunk c = k G + b (the block's chunk after c - G, G = gridDim.x):
//   X_c = sum_{t < n} Q^t part(c-1-t) + [c >= G] Q^(G-1) full(c-G),   n = min(c, G-1),
// with full(c-G) = part(c-G) + Q X_{c-G} known to the block itself. Only aggregates are read,
// and every block publishes those right after its zero-state pass, so no chunk waits for
// another chunk's lookback. Lane l owns the distances t = l + 32 m and adds its terms from
// the oldest (largest m) to the newest in that fixed order, so the result does not depend on
// arrival order. The terms with t >= b belong to earlier waves of chunks and are added before
// the block's own aggregate is ready (window_open); the b newest ones after it (window_close).
struct WindowAcc {
    float acc0, acc1;
    int m;  // next term of this lane (descending)
};

// Adds this lane's terms down to m_stop (exclusive below), polling until they are published.
__device__ __forceinline__ bool window_terms(const IirParams& p, const unsigned long long* slots, uint32_t c,
                                             uint32_t epoch, int m_stop, WindowAcc& w) {
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u;
    const uint64_t t_start = globaltimer_ns();
    uint32_t spin = 64;
    while (true) {
        // up to 8 independent loads in flight, then add while present, in order
        constexpr int BATCH = 8;
        const int m0 = w.m;
        unsigned long long w0[BATCH], w1[BATCH];
#pragma unroll
        for (int i = 0; i < BATCH; ++i) {
            const int mi = m0 - i;
            w0[i] = w1[i] = 0ull;
            if (mi >= m_stop)
                ld_relaxed_v2(slots + static_cast<size_t>(c - 1u - static_cast<uint32_t>(lane + 32 * mi)) * 4, w0[i],
                              w1[i]);
        }
        bool stalled = false;
#pragma unroll
        for (int i = 0; i < BATCH; ++i) {
            const int mi = m0 - i;
            if (mi < m_stop || stalled) continue;
            if (word_flag(w0[i]) != pf || word_flag(w1[i]) != pf) {
                stalled = true;
                continue;
            }
            float t0, t1;
            mv2(p.qpow[lane + 32 * mi], word_val(w0[i]), word_val(w1[i]), t0, t1);
            w.acc0 += t0;
            w.acc1 += t1;
            w.m = mi - 1;
        }
        if (!__any_sync(FULL_MASK, w.m >= m_stop)) return true;
        if (__any_sync(FULL_MASK, stalled)) {
            int give_up = 0;
            if (lane == 0) give_up = lookback_give_up(p, epoch, t_start) ? 1 : 0;
            if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
            backoff(spin);
        }
    }
}

// First phase for chunk c: the terms of earlier waves (t >= b).
__device__ __forceinline__ bool window_open(const IirParams& p, const unsigned long long* slots, uint32_t c,
                                            uint32_t epoch, WindowAcc& w) {
    const int lane = threadIdx.x & 31;
    const uint32_t G = gridDim.x, b = c % G;
    const uint32_t n = c < G - 1 ? c : G - 1;
    w.acc0 = w.acc1 = 0.f;
    w.m = static_cast<int>((n + 31u) / 32u) - 1;
    if (w.m >= 0 && static_cast<uint32_t>(lane + 32 * w.m) >= n) --w.m;
    // lowest m of this lane with t = lane + 32 m >= b
    const int m_lo = (static_cast<int>(b) - lane + 31) / 32 > 0 ? (static_cast<int>(b) - lane + 31) / 32 : 0;
    return window_terms(p, slots, c, epoch, m_lo, w);
}

// Second phase: the b newest terms, then the block's own previous carry.
__device__ __forceinline__ bool window_close(const IirParams& p, const unsigned long long* slots, uint32_t c,
                                             uint32_t epoch, WindowAcc& w, float fp0, float fp1, float& X0,
                                             float& X1) {
    const uint32_t G = gridDim.x;
    if (!window_terms(p, slots, c, epoch, 0, w)) return false;
    X0 = warp_sum(w.acc0);
    X1 = warp_sum(w.acc1);
    if (c >= G) {
        float f0, f1;
        mv2(p.qpow[G - 1], fp0, fp1, f0, f1);
        X0 += f0;
        X1 += f1;
    }
    return true;
}

// R provides: ROWS, N, NW (row warps);
//   p1(p, buf, hist, tc, zin, aux, slot, c, w, lane)  zero-state solve; one thread writes
//        aux->partv[slot]; called by every row thread (may use barrier 1). hist = the 32 input
//        samples before the chunk, tc = the table cache (PipeGeom::TC_*).
//   p2(p, buf, tc, zin, X0, X1, c, w, lane)  correction by the response to incoming state X;
//        may be skipped per thread, so no barriers
// S = shared-memory stages, LAG = chunks between a chunk's P1 and its P2 (S >= LAG + 2).
// Warp 0 is the TMA warp, warp 1 the lookback warp, the rest the row warps.
template <class R, int S, int LAG>
__device__ __forceinline__ void run_pipeline(const IirParams& p, unsigned char* smem_raw) {
    constexpr int ROWS = R::ROWS, N = R::N, NW = R::NW;
    static_assert(S >= LAG + 2, "a stage for the chunk being loaded and one being stored");
    using G = PipeGeom<ROWS, N, S>;
    const uint32_t a = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((a + 1023u) & ~1023u) - a);
    // [S data stages (1024-aligned) | S history lines | table cache | S zin arrays | aux]
    float* bufs = reinterpret_cast<float*>(base);
    float* hists = reinterpret_cast<float*>(base + S * G::DATA_BYTES);
    float4* tc = reinterpret_cast<float4*>(base + S * (G::DATA_BYTES + G::HIST_BYTES));
    float(*zins)[2] = reinterpret_cast<float(*)[2]>(base + S * (G::DATA_BYTES + G::HIST_BYTES) + G::TC_BYTES);
    PipeAux* aux =
        reinterpret_cast<PipeAux*>(base + S * (G::DATA_BYTES + G::HIST_BYTES + G::ZIN_BYTES) + G::TC_BYTES);
    auto buf_of = [&](int s) { return bufs + static_cast<size_t>(s) * G::CHUNK; };
    auto hist_of = [&](int s) { return hists + static_cast<size_t>(s) * 32; };
    auto zin_of = [&](int s) { return zins + static_cast<size_t>(s) * ROWS; };

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t nb = gridDim.x;
    const uint32_t nk = (p.nchunks > blockIdx.x) ? (p.nchunks - blockIdx.x + nb - 1) / nb : 0;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&aux->full[s], 1);
            mbar_init(&aux->part[s], 1);
            mbar_init(&aux->xrdy[s], 1);
            mbar_init(&aux->done[s], 1);
        }
        fence_mbar_init();
        aux->epoch = static_cast<uint32_t>(*reinterpret_cast<volatile unsigned long long*>(&p.state->ticket) >> 32);
        aux->bail = 0;
        aux->abandon = 0;
    }
    for (int i = tid; i < G::TC_LEN; i += blockDim.x) {
        int src;
        if (i < G::TC_GPOW) src = IIR_TAB_CPOW + i;
        else if (i < G::TC_QC) src = IIR_TAB_GPOW + (i - G::TC_GPOW);
        else if (i < G::TC_QG) src = IIR_TAB_QC + (i - G::TC_QC);
        else if (i < G::TC_HALF) src = IIR_TAB_QG + (i - G::TC_QG);
        else src = IIR_TAB_HALF + (i - G::TC_HALF);
        tc[i] = p.tables[src];
    }
    __syncthreads();
    const uint32_t epoch = aux->epoch;
    auto chunk_of = [&](uint32_t k) { return blockIdx.x + k * nb; };
    auto bulk_of = [&](uint32_t c) { return p.use_tma && (static_cast<long long>(c) + 1) * (ROWS * N) <= p.n; };
    auto par = [](uint32_t k) { return (k / S) & 1u; };

    if (warp == 0) {
        // --------------------------------- TMA warp ---------------------------------
        // Issues loads S chunks ahead and stores each chunk once its P2 is done. For an
        // element-wise chunk, `full` only says that the stage is free again.
        auto load = [&](uint32_t k) {
            const int s = k % S;
            const uint32_t c = chunk_of(k);
            if (lane == 0) {
                PIPE_STAMP(k, 0);
                if (bulk_of(c)) {
                    mbar_arrive_expect_tx(&aux->full[s], static_cast<uint32_t>(G::DATA_BYTES + G::HIST_BYTES));
                    tma_load_2d(buf_of(s), &p.tmap_x, 0, static_cast<int>(c) * G::LINES, &aux->full[s]);
                    // line before the chunk (zero fill before the signal's start)
                    tma_load_2d(hist_of(s), &p.tmap_h, 0, static_cast<int>(c) * G::LINES - 1, &aux->full[s]);
                } else {
                    mbar_arrive(&aux->full[s]);
                }
            }
        };
        uint32_t issued = 0;  // chunks [0, issued) have had their load issued
        for (; issued < nk && issued < static_cast<uint32_t>(S); ++issued) load(issued);
        for (uint32_t k = 0; k < nk; ++k) {
            const int s = k % S;
            const uint32_t c = chunk_of(k);
            const bool ok = pipe_wait(aux, &aux->done[s], par(k), p, epoch);
            if (lane == 0 && ok && bulk_of(c) && !*reinterpret_cast<volatile int*>(&aux->bail)) {
                tma_store_2d(&p.tmap_y, 0, static_cast<int>(c) * G::LINES, buf_of(s));
                bulk_commit();
            }
            if (k + S < nk && ok) {
                if (lane == 0) {
                    bulk_wait_read_all();  // the stage's store has read the buffer
                    PIPE_STAMP(k, 7);
                }
                __syncwarp();
                load(k + S);
                issued = k + S + 1;
            }
        }
        if (lane == 0) bulk_wait_all();
        // After a failed wait some loads may not have been waited for: they must land before
        // the block exits (at most one per stage is outstanding).
        if (*reinterpret_cast<volatile int*>(&aux->abandon) && lane == 0) {
            const uint32_t first = issued > static_cast<uint32_t>(S) ? issued - S : 0;
            for (uint32_t k = first; k < issued; ++k)
                (void)wait_mbar_bounded(&aux->full[k % S], par(k), p.timeout_ns);
        }
    } else if (warp == 1) {
        // ------------------------------- lookback warp -------------------------------
        // Resolves the block's chunks in order; the aggregates were published by the row warps.
        unsigned long long* slots = p.carry;
        const float4 Q = tc[G::TC_QC + 1];
        float fp0 = 0.f, fp1 = 0.f;  // inclusive carry of the block's previous chunk
        bool failed = false;
        for (uint32_t k = 0; k < nk; ++k) {
            const int s = k % S;
            const uint32_t c = chunk_of(k);
            float X0 = 0.f, X1 = 0.f;
#if !IIR_PIPE_HIER
            WindowAcc win;
            bool opened = true;
            if (!failed && c > 0) opened = window_open(p, slots, c, epoch, win);
#endif
            bool ok = pipe_wait(aux, &aux->part[s], par(k), p, epoch);
            // warp-uniform: the lookback is a full-warp routine
            ok = __all_sync(FULL_MASK, ok && !failed);
#if !IIR_PIPE_HIER
            ok = ok && opened;
#endif
            if (lane == 0) PIPE_STAMP(k, 3);
            if (ok) {
                const float a0 = aux->partv[s][0], a1 = aux->partv[s][1];
#if IIR_PIPE_HIER
                const bool withhold = static_cast<long long>(c) == p.withhold_chunk;
                unsigned long long* gslots = slots + static_cast<size_t>(p.carry_cap) * 4;
                if (c > 0)
                    ok = lookback_hier(p, slots, gslots, tc + G::TC_QC, tc + G::TC_QG, c, epoch, a0, a1, withhold, X0, X1);
                float q0, q1;
                mv2(Q, X0, X1, q0, q1);
                fp0 = a0 + q0;
                fp1 = a1 + q1;
                if (lane == 0 && ok && !withhold) {
                    const uint32_t ff = 2u * epoch + 2u;
                    publish2(slots + static_cast<size_t>(c) * 4 + 2, ff, fp0, fp1);
                    if ((c & 31u) == 31u) publish2(gslots + static_cast<size_t>(c >> 5) * 4 + 2, ff, fp0, fp1);
                }
#else
                if (c > 0) ok = window_close(p, slots, c, epoch, win, fp0, fp1, X0, X1);
                float q0, q1;
                mv2(Q, X0, X1, q0, q1);
                fp0 = a0 + q0;
                fp1 = a1 + q1;
#endif
                if (!ok) {
                    failed = true;
                    if (lane == 0) *reinterpret_cast<volatile int*>(&aux->bail) = 1;
                }
            }
            if (lane == 0) {
                aux->xv[s][0] = X0;
                aux->xv[s][1] = X1;
                PIPE_STAMP(k, 4);
                mbar_arrive(&aux->xrdy[s]);  // release: xv is visible to the waiting row warps
            }
            __syncwarp();
        }
    } else {
        // --------------------------------- row warps ---------------------------------
        const int w = warp - 2;
        const int rt = tid - 64;  // row-thread index
        const uint32_t pf = 2u * epoch + 1u;
        for (uint32_t k = 0; k < nk + LAG; ++k) {
            if (k < nk) {
                const int s = k % S;
                const uint32_t c = chunk_of(k);
                const bool ok = pipe_wait(aux, &aux->full[s], par(k), p, epoch);
                if (rt == 0) PIPE_STAMP(k, 1);
                // (barriers below depend on uniform conditions only; `ok` may differ per thread)
                if (!bulk_of(c)) {
                    const long long cs = static_cast<long long>(c) * G::CHUNK;
                    float* b = buf_of(s);
                    if (ok) {
                        for (int i = rt; i < G::CHUNK; i += NW * 32) {
                            const long long g = cs + i;
                            b[swz<N>(i / N, i % N)] = (g < p.n) ? p.x[g] : 0.f;
                        }
                        if (rt < 32) hist_of(s)[rt] = (cs - 32 + rt >= 0) ? p.x[cs - 32 + rt] : 0.f;
                    }
                    named_barrier_rows(NW);
                }
                R::p1(p, buf_of(s), hist_of(s), tc, zin_of(s), aux, s, c, w, lane);
                named_barrier_rows(NW);
                if (rt == 0) {
                    // publish the aggregate at once: successors' lookbacks need it, whatever
                    // this block's own lookbacks are waiting for
                    if (static_cast<long long>(c) != p.withhold_chunk)
                        publish2(p.carry + static_cast<size_t>(c) * 4, pf, aux->partv[s][0], aux->partv[s][1]);
                    PIPE_STAMP(k, 2);
                    mbar_arrive(&aux->part[s]);
                }
            }
            if (k >= static_cast<uint32_t>(LAG)) {
                const uint32_t kp = k - LAG;
                const int s = kp % S;
                const uint32_t c = chunk_of(kp);
                const bool ok = pipe_wait(aux, &aux->xrdy[s], par(kp), p, epoch);
                if (rt == 0) PIPE_STAMP(kp, 5);
                // warp-uniform, so p2 may use full-warp shuffles
                const bool live = __all_sync(FULL_MASK, ok && !*reinterpret_cast<volatile int*>(&aux->bail));
                if (live) R::p2(p, buf_of(s), tc, zin_of(s), aux->xv[s][0], aux->xv[s][1], c, w, lane);
                if (!bulk_of(c)) {
                    named_barrier_rows(NW);
                    const long long cs = static_cast<long long>(c) * G::CHUNK;
                    const float* b = buf_of(s);
                    if (live) {
                        for (int i = rt; i < G::CHUNK; i += NW * 32) {
                            const long long g = cs + i;
                            if (g < p.n) p.y[g] = b[swz<N>(i / N, i % N)];
                        }
                    }
                }
                fence_proxy_async_smem();  // generic writes -> visible to the TMA store
                named_barrier_rows(NW);
                if (rt == 0) {
                    PIPE_STAMP(kp, 6);
                    mbar_arrive(&aux->done[s]);
                }
            }
        }
    }
    __syncthreads();
    if (tid == 0) pipe_finish(p.state, epoch);
}

}  // namespace iirgb
