// iir_batch.cu — batched segments: many independent signals in one persistent launch.
//
// A segment is one signal (a channel, or the next chunk of a live stream) with its own
// cascade (any number of sections up to IIR_MAX_SECTIONS), an optional state in (zi) and an
// optional state out (zf). The launch's chunks are the concatenation of every segment's
// chunks; that list is the launch's work queue. A persistent grid (every block resident: the
// occupancy of the chosen kernel times the SMs) draws chunks from it in ticket order, one atomic
// per chunk, finds each chunk's segment with a 32-way search of the segment start table, and
// runs the PH section solve (iir_ph.cuh) with the decoupled lookback restricted to the segment:
// a segment's first chunk starts from zi, and the lookback treats zi as the state before the
// segment. The block that holds a segment's last sample writes zf. A chunk only ever waits for
// a chunk drawn before it, which a running block holds, so the queue cannot deadlock.
//
// Two schedules:
//   * per-section lookback (the default): each section publishes the chunk's zero-state
//     aggregate and waits for its predecessor's (control(); two block barriers per section);
//   * tail aggregate (iir_tail.cuh), for segments of at least IIR_GB300_BATCH_TAIL_CHUNKS chunks
//     whose filter's cascade state decays within half a chunk: the chunk's aggregate of every
//     section comes from its last pieces, published at once; the chunk reads its predecessor's
//     and the row warps run every section with one barrier each.
//
// The chunk shape (rows x samples per row) is a run-time choice among compiled instantiations
// (iir_batch_set_shape): long channels favour big chunks (fewer lookbacks per sample), short ones
// small chunks (less padding past a segment's end). The tuner in autotune.py picks it, seeded
// by an occupancy model of GB300.
//
// The reference filters one signal with one compile-time filter per launch
// (ph_kernels.cuh:151-200, src/test_accuracy.cu:146); this is the batching form that design
// cannot express.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/iir_gb300.h"
#include "iir_host_internal.h"
#include "iir_ph.cuh"
#include "iir_registry.h"
#include "iir_tail.cuh"

// Resident blocks per SM the batch kernel is compiled for (its register budget), at most what
// shared memory allows.
#ifndef IIR_BATCH_MIN_BLOCKS
#define IIR_BATCH_MIN_BLOCKS 6
#endif

namespace iirgb {

struct BatchAux {
    unsigned int chunk, seg;  // the chunk the block drew, and its segment
    int more;                 // the draw found a chunk of this launch
    unsigned int epoch;
    int bail;
    float wtot[16][2][2];
    float X[2];
    float Xs[IIR_MAX_SECTIONS][2];                           // tail schedule: incoming states
    float tpiece[IIR_TAIL_MAX_PIECES][IIR_MAX_SECTIONS][2];  // tail schedule: pieces' end states
};

template <int N_, int ROWS_>
struct BatchBlock {
    static constexpr int N = N_, ROWS = ROWS_, NW = ROWS / 32, THREADS = 32 + ROWS, WARPS = THREADS / 32;
    static constexpr int CHUNK = ROWS * N;
    static_assert(ROWS % 32 == 0 && ROWS <= IIR_BATCH_MAX_ROWS, "rows per chunk");
    using Ph = PhBlock<32, N, ROWS>;
    static constexpr size_t SMEM_BYTES = CHUNK * sizeof(float) + sizeof(BatchAux) + 16;
    // resident blocks per SM the kernel is compiled for (registers), at most what shared memory allows
    static constexpr int SMEM_BLOCKS = static_cast<int>((228 * 1024) / (SMEM_BYTES + 1024));
    static constexpr int MIN_BLOCKS = SMEM_BLOCKS < IIR_BATCH_MIN_BLOCKS ? SMEM_BLOCKS : IIR_BATCH_MIN_BLOCKS;
    // tail pieces a chunk of this shape takes: one per warp, at most half of the chunk
    static constexpr int MAX_PIECES_RAW = WARPS < IIR_TAIL_MAX_PIECES ? WARPS : IIR_TAIL_MAX_PIECES;
    static constexpr int MAX_PIECES = MAX_PIECES_RAW < CHUNK / (2 * IIR_TAIL_PIECE) ? MAX_PIECES_RAW
                                                                                   : CHUNK / (2 * IIR_TAIL_PIECE);

    // Per-section schedule: incoming state of the segment's chunk lc for section `sec`.
    __device__ static bool control(const IirBatchParams& p, BatchAux* aux, const IirBatchSegment& sg, int sec,
                                   uint32_t lc, uint32_t epoch, const float4* tab, float4 Gw) {
        const int lane = threadIdx.x & 31;
        float t0 = 0.f, t1 = 0.f;
#pragma unroll 4
        for (int w = 0; w < NW; ++w) {
            float n0, n1;
            mv2(Gw, t0, t1, n0, n1);
            t0 = n0 + aux->wtot[w][0][0];
            t1 = n1 + aux->wtot[w][0][1];
        }
        const float z0 = sg.zi ? sg.zi[2 + 2 * sec] : 0.f;
        const float z1 = sg.zi ? sg.zi[3 + 2 * sec] : 0.f;
        unsigned long long* level = p.carry + static_cast<size_t>(sec) * p.carry_stride;
        unsigned long long* slots = level + static_cast<size_t>(sg.chunk0) * 4;
        unsigned long long* gslots = level + static_cast<size_t>(p.carry_cap) * 4 + static_cast<size_t>(sg.group0) * 4;
        const bool withhold = static_cast<long long>(sg.chunk0 + lc) == p.withhold_chunk;
        const uint32_t pf = 2u * epoch + 1u, ff = 2u * epoch + 2u;
        if (lane == 0 && !withhold) publish2(slots + static_cast<size_t>(lc) * 4, pf, t0, t1);
        float X0 = z0, X1 = z1;
        bool ok = true;
        const int depth = static_cast<int>(tab[IIR_BT_LBD].x);  // truncated lookback depth (0: two-level)
        if (lc > 0)
            ok = depth > 0 ? lookback_trunc2(p, slots, tab + IIR_BT_QC, lc, epoch, depth, X0, X1, z0, z1)
                           : lookback_hier(p, slots, gslots, tab + IIR_BT_QC, tab + IIR_BT_QG, lc, epoch, t0, t1,
                                           withhold, X0, X1, z0, z1);
        if (lane == 0) {
            if (ok && !withhold) {
                float f0, f1;
                mv2(tab[IIR_BT_QC + 1], X0, X1, f0, f1);
                publish2(slots + static_cast<size_t>(lc) * 4 + 2, ff, t0 + f0, t1 + f1);
                if ((lc & 31u) == 31u) publish2(gslots + static_cast<size_t>(lc >> 5) * 4 + 2, ff, t0 + f0, t1 + f1);
            }
            aux->X[0] = X0;
            aux->X[1] = X1;
            aux->bail = ok ? 0 : 1;
        }
        return ok;
    }

    // Bulk L2 prefetch of chunk c's whole 16-byte granules (those inside its segment).
    __device__ static void prefetch_chunk(const IirBatchParams& p, uint32_t c) {
        const IirBatchSegment& sg = p.segs[__ldg(p.chunk_seg + c)];
        const long long cs = static_cast<long long>(c - sg.chunk0) * CHUNK - sg.lead;
        const long long ce = cs + CHUNK < sg.n ? cs + CHUNK : sg.n;
        const uintptr_t a = (reinterpret_cast<uintptr_t>(sg.x + (cs > 0 ? cs : 0)) + 15u) & ~static_cast<uintptr_t>(15u);
        const uintptr_t b = reinterpret_cast<uintptr_t>(sg.x + ce) & ~static_cast<uintptr_t>(15u);
        if (b > a) prefetch_l2_bulk(reinterpret_cast<const void*>(a), static_cast<uint32_t>(b - a));
    }

    // Warp 0: draws the block's next chunk from the launch's queue and finds its segment: the
    // last s with chunk_start[s] <= c (empty segments share their start with the next one, so
    // the last such index is the non-empty one). 32-way search: each round the lanes probe 32
    // evenly spaced starts of [lo, hi).
    __device__ static void draw(const IirBatchParams& p, BatchAux* aux, int lane) {
        uint32_t c = 0;
        if (lane == 0) c = static_cast<uint32_t>(atomicAdd(&p.state->ticket, 1ull) & 0xffffffffull);
        c = __shfl_sync(FULL_MASK, c, 0);
        const bool more = c < p.nchunks;
        uint32_t lo = 0;
        if (more && p.chunk_seg) {
            lo = __ldg(p.chunk_seg + c);  // a bound table's precomputed map
        } else if (more) {
            uint32_t hi = p.nsegs;  // answer in [lo, hi)
            while (hi - lo > 1) {
                const uint32_t span = hi - lo;
                const uint32_t probe = lo + static_cast<uint32_t>((static_cast<unsigned long long>(span) * lane) / 32);
                const bool le = p.chunk_start[probe] <= c;
                const unsigned m = __ballot_sync(FULL_MASK, le);  // lanes 0..k-1 hold (starts ascend)
                const int k = 32 - __clz(m);                        // highest lane with start <= c, + 1
                const uint32_t nlo = lo + static_cast<uint32_t>((static_cast<unsigned long long>(span) * (k - 1)) / 32);
                const uint32_t nhi = (k < 32) ? lo + static_cast<uint32_t>((static_cast<unsigned long long>(span) * k) / 32)
                                              : hi;
                lo = nlo;
                hi = nhi > nlo ? nhi : nlo + 1;
            }
        }
        if (lane == 0) {
            aux->chunk = c;
            aux->seg = lo;
            aux->more = more ? 1 : 0;
        }
    }

    // Whole chunk of a segment that does not start on a 16-byte boundary: granule j of the chunk
    // (samples 4j..4j+3, 16-byte aligned in shared memory) as two 8-byte or four 4-byte cp.async
    // copies, as the source's alignment allows. Every copy stays within the chunk.
    template <bool EIGHT>
    __device__ static void stage_unaligned(const float* src, float* buf, int tid) {
#pragma unroll 4
        for (int j = tid; j < CHUNK / 4; j += THREADS) {
            float* dst = buf + swz<N, ROWS, true>((4 * j) / N, (4 * j) % N);
            if constexpr (EIGHT) cp_async16_from8(dst, src + 4 * j);
            else cp_async16_from4(dst, src + 4 * j);
        }
    }

    // Whole chunk written to dst, B floats past a 16-byte boundary (B = 1..3): the aligned granule k
    // of the output (chunk samples 4k - B .. 4k - B + 3) is the last B floats of the chunk's granule
    // k - 1 and the first 4 - B of its granule k, one 16-byte store. The two end granules hold
    // samples of the neighbouring chunks: only this chunk's samples in them are written.
    template <int B>
    __device__ static void store_shifted(float* dst, const float* buf, int tid) {
        float4* g = reinterpret_cast<float4*>(dst - B);
        const float4* s = reinterpret_cast<const float4*>(buf);
#pragma unroll 1
        for (int k = tid; k <= CHUNK / 4; k += THREADS) {
            if (k == 0) {
                for (int t = 0; t < 4 - B; ++t) dst[t] = buf[swz<N, ROWS, true>(0, t)];
            } else if (k == CHUNK / 4) {
                for (int t = CHUNK - B; t < CHUNK; ++t) dst[t] = buf[swz<N, ROWS, true>(t / N, t % N)];
            } else {
                const float4 u = s[swz<N, ROWS, true>((4 * k - 4) / N, (4 * k - 4) % N) >> 2];
                const float4 w = s[swz<N, ROWS, true>((4 * k) / N, (4 * k) % N) >> 2];
                if constexpr (B == 1) g[k] = make_float4(u.w, w.x, w.y, w.z);
                else if constexpr (B == 2) g[k] = make_float4(u.z, u.w, w.x, w.y);
                else g[k] = make_float4(u.y, u.z, u.w, w.x);
            }
        }
    }

    // All threads: start copying chunk c of segment `seg` into buf (cp.async, no registers held),
    // zero before the segment's start (a first chunk's leading zeros) and past its end. A chunk on
    // the 16-byte grid moves its whole granules as 16-byte copies; a whole chunk off the grid (a
    // segment with an initial state, not 16-byte aligned) as 8- or 4-byte copies per granule; the
    // rest sample by sample. Completion: the caller's cp_async_wait and barrier.
    __device__ static void stage(const IirBatchParams& p, uint32_t c, uint32_t seg, float* buf, int tid) {
        const IirBatchSegment& sg = p.segs[seg];
        // chunk position i holds segment sample cs + i (cs < 0: the first chunk's leading zeros)
        const long long cs = static_cast<long long>(c - sg.chunk0) * CHUNK - sg.lead;
        const long long nrem = sg.n - cs;  // > 0
        const uintptr_t mis = (reinterpret_cast<uintptr_t>(sg.x) + static_cast<uintptr_t>(4 * cs)) & 15u;
        if ((cs < 0 || nrem < CHUNK) && mis == 0) {
            // a segment's first chunk with leading zeros, or its last chunk, on a 16-byte boundary:
            // whole granules inside the segment as 16-byte copies, granules outside it zeroed, the
            // granules it cuts sample by sample
#pragma unroll 1
            for (int g = tid; g < CHUNK / 4; g += THREADS) {
                float* dst = buf + swz<N, ROWS, true>((4 * g) / N, (4 * g) % N);
                const long long i0 = 4 * g;
                if (i0 >= -cs && i0 + 3 < nrem) {
                    cp_async16(dst, sg.x + (cs + i0));
                } else if (i0 + 3 < -cs || i0 >= nrem) {
                    *reinterpret_cast<float4*>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
                } else {
                    for (int t = 0; t < 4; ++t) {
                        const bool in = i0 + t >= -cs && i0 + t < nrem;
                        cp_async4(dst + t, in ? sg.x + (cs + i0 + t) : sg.x, in ? 4 : 0);
                    }
                }
            }
            return;
        }
        if (cs < 0) {
#pragma unroll 4
            for (int i = tid; i < CHUNK; i += THREADS) {
                const bool in = i >= -cs && i < nrem;
                cp_async4(buf + swz<N, ROWS, true>(i / N, i % N), in ? sg.x + (cs + i) : sg.x, in ? 4 : 0);
            }
            return;
        }
        const float* src = sg.x + cs;
        if (nrem >= CHUNK && mis == 0) {
#pragma unroll 4
            for (int i = tid; i < CHUNK / 4; i += THREADS)
                cp_async16(buf + swz<N, ROWS, true>((4 * i) / N, (4 * i) % N), src + 4 * i);
        } else if (nrem >= CHUNK && (mis & 3u) == 0) {
            if (mis == 8) stage_unaligned<true>(src, buf, tid);
            else stage_unaligned<false>(src, buf, tid);
        } else {
#pragma unroll 4
            for (int i = tid; i < CHUNK; i += THREADS) {
                const bool in = i < nrem;
                cp_async4(buf + swz<N, ROWS, true>(i / N, i % N), in ? src + i : src, in ? 4 : 0);
            }
        }
    }

    // One chunk (all threads), already staged in buf. Returns false when a wait of this launch
    // gave up (uniform).
    __device__ static bool chunk(const IirBatchParams& p, float* buf, BatchAux* aux, uint32_t c, uint32_t seg, int tid,
                                 int warp, int lane) {
        const uint32_t epoch = aux->epoch;
        const IirBatchSegment sg = p.segs[seg];
        const IirBatchFilter flt = p.filters[sg.filter];
        const uint32_t lc = c - sg.chunk0;
        const long long cs = static_cast<long long>(lc) * CHUNK - sg.lead;  // segment sample at position 0
        const long long nrem = sg.n - cs;  // samples of the segment from this chunk's start (> 0)

        const bool row_warp = warp > 0;
        const int K = flt.n_sections;
        const bool tail = flt.tail > 0 && sg.tail_ok;  // the segment's schedule (uniform in the block)
        if (tail) {
            // the chunk's aggregate from its last pieces (not for the segment's last chunk)
            const bool has_succ = nrem > CHUNK;
            if (has_succ && warp < flt.tail) {
                const TailFilter f{p.secs + flt.sec0, p.tables + static_cast<size_t>(flt.sec0) * IIR_BT_STRIDE,
                                   IIR_BT_STRIDE, IIR_BT_TAIL, K, flt.gain};
                tail_piece<N, ROWS, true>(f, flt.tail, buf, aux->tpiece, warp);
            }
            __syncthreads();  // the pieces are in aux; the staged chunk may now be changed
            if (!row_warp) {
                unsigned long long* slot = p.carry + static_cast<size_t>(sg.chunk0 + lc) * 4;  // section 0's
                const uint32_t pf = 2u * epoch + 1u;
                if (has_succ && static_cast<long long>(c) != p.withhold_chunk)
                    tail_join_publish(p.phi + static_cast<size_t>(sg.filter) * IIR_BT_PHI_FLOATS, aux->tpiece, K,
                                      flt.tail, slot, p.carry_stride, pf);
                float X0 = 0.f, X1 = 0.f;
                bool ok = true;
                if (lc > 0) {
                    ok = tail_poll(p, slot - 4, p.carry_stride, K, epoch, X0, X1);
                } else if (sg.zi && lane < K) {
                    X0 = sg.zi[2 + 2 * lane];  // the segment's initial state
                    X1 = sg.zi[3 + 2 * lane];
                }
                if (lane < K) {
                    aux->Xs[lane][0] = X0;
                    aux->Xs[lane][1] = X1;
                }
                if (lane == 0) aux->bail = ok ? 0 : 1;
            }
        }

        const int w = warp - 1;
        const int r = w * 32 + lane;
        // A row warp whose rows all lie past the segment's end (padding of its last chunk) only
        // takes part in the barriers: nothing there is stored, and the chunk's aggregate (the
        // segment's last) has no reader.
        const bool live = row_warp && static_cast<long long>(w) * 32 * N < nrem;
        const float gain = flt.gain;
        float xh2 = 0.f, xh1 = 0.f;
        if (row_warp) {
            if (r > 0) {
                xh2 = buf[swz<N, ROWS, true>(r - 1, N - 2)];
                xh1 = buf[swz<N, ROWS, true>(r - 1, N - 1)];
            } else if (lc > 0) {
                xh2 = sg.x[cs - 2];
                xh1 = sg.x[cs - 1];
            } else if (sg.zi) {
                xh2 = sg.zi[0];
                xh1 = sg.zi[1];
            }
            xh2 *= gain;
            xh1 *= gain;
            named_barrier_rows(NW);  // histories read before the first pass overwrites rows (it applies the gain)
        }
        // Control warp, idle until the row warps' first filter pass ends: with a bound table (every
        // chunk's segment known), the chunk one grid ahead in the queue, which some block draws
        // about one chunk's time from now, goes into L2, so that its copy-in waits for L2 rather
        // than for memory.
        if (!row_warp && lane == 0 && p.chunk_seg && static_cast<unsigned long long>(c) + gridDim.x < p.nchunks)
            prefetch_chunk(p, c + gridDim.x);
        // positions of the segment's last two samples relative to this chunk
        const long long m1 = nrem - 1, m2 = nrem - 2;  // in [0, CHUNK) when inside this chunk
        float pa1 = 0.f, pa2 = 0.f, d2 = 0.f, d1 = 0.f;
        for (int sec = 0; sec < K; ++sec) {
            const IirSection& q = p.secs[flt.sec0 + sec];
            const float4* tab = p.tables + static_cast<size_t>(flt.sec0 + sec) * IIR_BT_STRIDE;
            const float4 Gw = tab[IIR_BT_GPOW + 31];
            const int wb = tail ? (sec & 1) : 0;  // the tail schedule alternates the totals' buffers
            float s0 = 0.f, s1 = 0.f, in0 = 0.f, in1 = 0.f;
            if (live) {
                if (sec == 0)
                    Ph::template filter_pass<false>(buf, r, q.b1, q.b2, q.a1, q.a2, 0.f, 0.f, 0.f, 0.f, xh2, xh1, s0, s1,
                                                    gain);
                else
                    Ph::template filter_pass<true>(buf, r, q.b1, q.b2, q.a1, q.a2, pa1, pa2, d2, d1, xh2, xh1, s0, s1);
                warp_scan2<32, 1>(s0, s1, q.M, lane);
            }
            if (row_warp && lane == 31) {
                aux->wtot[w][wb][0] = s0;
                aux->wtot[w][wb][1] = s1;
            }
            // (A); with the tail schedule the control warp is done after the first section's
            if (!tail || sec == 0) __syncthreads();
            else if (row_warp) named_barrier_rows(NW);
            if (live) {
                warp_incoming(aux, w, wb, Gw, in0, in1);
                if (w > 0) {
                    float e0, e1;
                    mv2(tab[IIR_BT_GPOW + lane], in0, in1, e0, e1);
                    s0 += e0;
                    s1 += e1;
                }
            } else if (!row_warp && !tail) {
                control(p, aux, sg, sec, lc, epoch, tab, Gw);
            }
            if (!tail) __syncthreads();  // (B)
            if (aux->bail) return false;
            if (live) {
                const float X0 = tail ? aux->Xs[sec][0] : aux->X[0], X1 = tail ? aux->Xs[sec][1] : aux->X[1];
                float P0, P1;
                mv2(tab[IIR_BT_CPOW + r], X0, X1, P0, P1);
                const float T0 = s0 + P0, T1 = s1 + P1;
                float i0 = __shfl_up_sync(FULL_MASK, T0, 1);
                float i1 = __shfl_up_sync(FULL_MASK, T1, 1);
                if (lane == 0) {
                    if (r == 0) {
                        i0 = X0;
                        i1 = X1;
                    } else {
                        float q0, q1;
                        mv2(tab[IIR_BT_CPOW + r - 1], X0, X1, q0, q1);
                        i0 = in0 + q0;
                        i1 = in1 + q1;
                    }
                }
                if (sg.zf) {
                    // this section's true output at the segment's last two samples: the row's
                    // zero-state value + the response to the row's incoming pair (i0, i1)
                    const long long rs = static_cast<long long>(r) * N;
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        const long long m = t == 0 ? m2 : m1;
                        if (m >= rs && m < rs + N) {
                            float e2 = i0, e1 = i1, dn = 0.f;
                            for (int k = 0; k <= static_cast<int>(m - rs); ++k) {
                                dn = fmaf(q.a1, e1, q.a2 * e2);
                                e2 = e1;
                                e1 = dn;
                            }
                            sg.zf[2 + 2 * sec + t] = buf[swz<N, ROWS, true>(r, static_cast<int>(m - rs))] + dn;
                        }
                    }
                    // the second-to-last sample in the previous chunk: the chunk's incoming y[-1]
                    if (r == 0 && lane == 0 && m2 == -1) sg.zf[2 + 2 * sec] = X1;
                }
                pa1 = q.a1;
                pa2 = q.a2;
                d2 = i0;
                d1 = i1;
                xh2 = i0;
                xh1 = i1;
            }
        }
        if (live) Ph::correct_pass(buf, r, pa1, pa2, d2, d1);
        __syncthreads();
        const long long cnt = nrem < CHUNK ? nrem : CHUNK;
        const uintptr_t ymis = (reinterpret_cast<uintptr_t>(sg.y) + static_cast<uintptr_t>(4 * cs)) & 15u;
        if ((cs < 0 || cnt < CHUNK) && ymis == 0) {
            // a first chunk with leading zeros or a last chunk on a 16-byte boundary: whole
            // granules of the segment's samples as 16-byte stores, the granules it cuts sample by
            // sample
            for (int g = tid; g < CHUNK / 4; g += THREADS) {
                const long long i0 = 4 * g;
                if (i0 + 3 < -cs || i0 >= cnt) continue;
                const float4 v = *reinterpret_cast<const float4*>(buf + swz<N, ROWS, true>((4 * g) / N, (4 * g) % N));
                if (i0 >= -cs && i0 + 3 < cnt) {
                    *reinterpret_cast<float4*>(sg.y + (cs + i0)) = v;
                } else {
                    const float e[4] = {v.x, v.y, v.z, v.w};
                    for (int t = 0; t < 4; ++t)
                        if (i0 + t >= -cs && i0 + t < cnt) sg.y[cs + i0 + t] = e[t];
                }
            }
        } else if (cs < 0) {  // the first chunk of a segment with leading zeros: its own samples only
            for (long long i = tid - cs; i < cnt; i += THREADS)
                sg.y[cs + i] = buf[swz<N, ROWS, true>(static_cast<int>(i) / N, static_cast<int>(i) % N)];
        } else if (cnt == CHUNK && ymis == 0) {
            float4* dst = reinterpret_cast<float4*>(sg.y + cs);
            for (int i = tid; i < CHUNK / 4; i += THREADS)
                dst[i] = *reinterpret_cast<const float4*>(buf + swz<N, ROWS, true>((4 * i) / N, (4 * i) % N));
        } else if (cnt == CHUNK && (ymis & 3u) == 0) {
            if (ymis == 4) store_shifted<1>(sg.y + cs, buf, tid);
            else if (ymis == 8) store_shifted<2>(sg.y + cs, buf, tid);
            else store_shifted<3>(sg.y + cs, buf, tid);
        } else {
            for (int i = tid; i < cnt; i += THREADS) sg.y[cs + i] = buf[swz<N, ROWS, true>(i / N, i % N)];
        }
        if (sg.zf && tid == 0 && nrem <= CHUNK) {
            // input history after the segment (raw)
            sg.zf[1] = sg.x[sg.n - 1];
            sg.zf[0] = sg.n >= 2 ? sg.x[sg.n - 2] : (sg.zi ? sg.zi[1] : 0.f);
        }
        return true;
    }

    // Persistent block: chunks from the launch's queue until it is empty (or a wait gave up);
    // the last block to leave re-arms the queue for the next launch with the next epoch. A block
    // starts filtering every chunk it draws at once: a drawn chunk that waited for its block
    // (to prefetch it, say) would hold up its segment's later chunks, which wait for its carries.
    // The copy-in latency is hidden by the other resident blocks instead (the kernel is compiled
    // for several per SM, and its staging holds no registers).
    __device__ static void run(const IirBatchParams& p, unsigned char* smem) {
        float* buf = reinterpret_cast<float*>(smem);
        BatchAux* aux = reinterpret_cast<BatchAux*>(smem + CHUNK * sizeof(float));
        const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
        if (tid == 0)  // tickets only add to the low word within a launch: the high word is the epoch
            aux->epoch = static_cast<uint32_t>(*reinterpret_cast<volatile unsigned long long*>(&p.state->ticket) >> 32);
        while (true) {
            if (warp == 0) draw(p, aux, lane);
            __syncthreads();  // also: the previous chunk's store has read the buffer
            if (!aux->more) break;
            const uint32_t c = aux->chunk, seg = aux->seg;
            stage(p, c, seg, buf, tid);
            cp_async_commit();
            cp_async_wait<0>();
            __syncthreads();
            if (!chunk(p, buf, aux, c, seg, tid, warp, lane)) break;
        }
        __syncthreads();
        if (tid == 0) pipe_finish(p.state, aux->epoch);
    }
};

template <int N, int ROWS>
__global__ void __launch_bounds__(BatchBlock<N, ROWS>::THREADS, BatchBlock<N, ROWS>::MIN_BLOCKS) iir_batch_kernel(const __grid_constant__ IirBatchParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    BatchBlock<N, ROWS>::run(p, smem);
}

}  // namespace iirgb

// -------------------------------------------------------------------------------------------
// host side
// -------------------------------------------------------------------------------------------
using namespace iirgb;
using namespace iirhost;

namespace {

// A compiled chunk shape of the batch kernel.
struct ShapeDef {
    int rows, n;
    const void* fn;
    int threads;
    size_t smem;
    int max_pieces;
};

template <int N, int ROWS>
ShapeDef shape_def() {
    using Blk = BatchBlock<N, ROWS>;
    return ShapeDef{ROWS, N, reinterpret_cast<const void*>(iir_batch_kernel<N, ROWS>), Blk::THREADS, Blk::SMEM_BYTES,
                    Blk::MAX_PIECES};
}

// chunks of 8192, 4096, 2048 and 1024 samples (the first is the default)
const std::vector<ShapeDef>& shapes() {
    static const std::vector<ShapeDef> s = {shape_def<64, 128>(), shape_def<32, 128>(), shape_def<16, 128>(),
                                            shape_def<16, 64>()};
    return s;
}

// Per-shape device data: the sections' scalars and lane tables (both depend on the samples per
// row) and the filters (with each filter's schedule for this shape), built when the shape is
// first used; the occupancy of its kernel.
struct ShapeData {
    bool ready = false;
    IirSection* d_secs = nullptr;
    float4* d_tables = nullptr;
    IirBatchFilter* d_filters = nullptr;
    int blocks_per_sm = 0;
    int regs = 0;  // registers per thread of the shape's kernel
};

}  // namespace

struct iir_batch {
    int device = 0;
    int sms = 0;
    int n_filters = 0;
    int max_sections = 0;
    // filters on the host: normalised sections, gains, sections per filter, tail pieces needed
    std::vector<SectionF32> sec32;
    std::vector<IirBatchFilter> filters;
    std::vector<int> tail_need;  // least number of tail pieces for the filter's state to decay (0: > 8)
    float* d_phi = nullptr;
    std::vector<ShapeData> shape_data;
    int shape = 0;  // index into shapes()
    IirLaunchState* d_state = nullptr;
    unsigned long long* d_carry = nullptr;
    size_t carry_cap = 0, gcap = 0, carry_bytes = 0;
    IirBatchSegment* d_segs = nullptr;
    unsigned int* d_starts = nullptr;
    size_t seg_cap = 0;
    // pinned staging for the segment table, two buffers used in turn (an event guards reuse)
    unsigned char* h_stage[2] = {nullptr, nullptr};
    cudaEvent_t stage_done[2] = {nullptr, nullptr};
    int stage_turn = 0;
    std::vector<int> filter_sections;
    long long timeout_ns = 1000000000ll;
    long long withhold = -1;
    unsigned long long launches = 0;
};

namespace {

size_t stage_bytes(size_t segs) { return segs * sizeof(IirBatchSegment) + (segs + 1) * sizeof(unsigned int) + 64; }

void batch_free_segments(iir_batch* b) {
    if (b->d_segs) cudaFree(b->d_segs);
    if (b->d_starts) cudaFree(b->d_starts);
    for (int i = 0; i < 2; ++i) {
        if (b->h_stage[i]) cudaFreeHost(b->h_stage[i]);
        b->h_stage[i] = nullptr;
    }
    b->d_segs = nullptr;
    b->d_starts = nullptr;
    b->seg_cap = 0;
}

int batch_alloc_segments(iir_batch* b, size_t segs) {
    batch_free_segments(b);
    segs = std::max<size_t>(segs, 16);
    int st = cuda_status(cudaMalloc(&b->d_segs, segs * sizeof(IirBatchSegment)));
    if (!st) st = cuda_status(cudaMalloc(&b->d_starts, (segs + 1) * sizeof(unsigned int)));
    for (int i = 0; i < 2 && !st; ++i) st = cuda_status(cudaMallocHost(&b->h_stage[i], stage_bytes(segs)));
    if (st) return st;
    b->seg_cap = segs;
    return IIR_OK;
}

int batch_alloc_carry(iir_batch* b, size_t chunks, size_t segs) {
    if (b->d_carry) cudaFree(b->d_carry);
    b->d_carry = nullptr;
    chunks = std::max<size_t>(chunks, 64);
    const size_t gcap = chunks / IIR_GROUP + segs + 2;
    const size_t words = 4 * (chunks + gcap);
    const size_t bytes = words * sizeof(unsigned long long) * static_cast<size_t>(b->max_sections);
    int st = cuda_status(cudaMalloc(&b->d_carry, bytes));
    if (!st) st = cuda_status(cudaMemset(b->d_carry, 0, bytes));
    if (!st) st = cuda_status(cudaMemset(b->d_state, 0, IIR_STATE_RESET_BYTES));
    if (st) return st;
    b->carry_cap = chunks;
    b->gcap = gcap;
    b->carry_bytes = bytes;
    b->launches = 0;
    return IIR_OK;
}

void batch_free(iir_batch* b) {
    if (!b) return;
    cudaDeviceSynchronize();
    batch_free_segments(b);
    for (int i = 0; i < 2; ++i)
        if (b->stage_done[i]) cudaEventDestroy(b->stage_done[i]);
    for (ShapeData& d : b->shape_data) {
        if (d.d_secs) cudaFree(d.d_secs);
        if (d.d_tables) cudaFree(d.d_tables);
        if (d.d_filters) cudaFree(d.d_filters);
    }
    if (b->d_phi) cudaFree(b->d_phi);
    if (b->d_state) cudaFree(b->d_state);
    if (b->d_carry) cudaFree(b->d_carry);
    delete b;
}

// Tail-aggregate schedule for batched filters (IIR_GB300_TAIL=0 turns it off, as for plans).
bool batch_tail_enabled() {
    if (std::getenv("IIR_GB300_FULL_LOOKBACK")) return false;
    const char* e = std::getenv("IIR_GB300_TAIL");
    return !(e && std::atoi(e) == 0);
}

// Least number of chunks for a segment to take its filter's tail-aggregate schedule
// (IIR_GB300_BATCH_TAIL_CHUNKS; by default none does). In the persistent batch kernel the
// per-section lookback is the faster schedule at every segment length measured on GB300 (a
// single 2^27-sample segment of butter(16, 0.1): 201 against 189 GS/s; the mixed 4096-channel
// workload: 299 against 280): the other resident blocks fill the lookback waits, while the tail
// pieces add up to half a chunk of filtering to every chunk.
size_t batch_tail_min_chunks() {
    const char* e = std::getenv("IIR_GB300_BATCH_TAIL_CHUNKS");
    if (!e) return ~static_cast<size_t>(0);
    const long long v = std::atoll(e);
    return v > 0 ? static_cast<size_t>(v) : 1;
}

// Builds shape k's lane tables and filter records (once) and its occupancy.
int shape_prepare(iir_batch* b, int k) {
    ShapeData& d = b->shape_data[static_cast<size_t>(k)];
    if (d.ready) return IIR_OK;
    const ShapeDef& sd = shapes()[static_cast<size_t>(k)];
    std::vector<float4> tabs(b->sec32.size() * IIR_BT_STRIDE, make_float4(0, 0, 0, 0));
    std::vector<IirSection> secs(b->sec32.size());
    std::vector<float4> full(IIR_TAB_STRIDE);
    for (size_t s = 0; s < b->sec32.size(); ++s) {
        IirSection& q = secs[s];
        const int st = precompute_section(b->sec32[s], IIR_KIND_PH, sd.rows, sd.n, q, full.data());
        if (st) return st;
        float4* t = tabs.data() + s * IIR_BT_STRIDE;
        for (int r = 0; r < sd.rows; ++r) t[IIR_BT_CPOW + r] = full[IIR_TAB_CPOW + r];
        for (int i = 0; i < 32; ++i) t[IIR_BT_GPOW + i] = full[IIR_TAB_GPOW + i];
        for (int l = 0; l <= 32; ++l) {
            t[IIR_BT_QC + l] = full[IIR_TAB_QC + l];
            t[IIR_BT_QG + l] = full[IIR_TAB_QG + l];
        }
        t[IIR_BT_LBD] = full[IIR_TAB_LBD];
        for (int l = 0; l < 32; ++l) t[IIR_BT_TAIL + l] = full[IIR_TAB_TAIL + l];
    }
    std::vector<IirBatchFilter> flt = b->filters;
    const bool tail_on = batch_tail_enabled();
    for (size_t f = 0; f < flt.size(); ++f) {
        const int need = b->tail_need[f];
        flt[f].tail = (tail_on && need > 0 && need <= sd.max_pieces) ? need : 0;
    }
    int st = cuda_status(cudaMalloc(&d.d_secs, secs.size() * sizeof(IirSection)));
    if (!st) st = cuda_status(cudaMemcpy(d.d_secs, secs.data(), secs.size() * sizeof(IirSection), cudaMemcpyHostToDevice));
    if (!st) st = cuda_status(cudaMalloc(&d.d_tables, tabs.size() * sizeof(float4)));
    if (!st) st = cuda_status(cudaMemcpy(d.d_tables, tabs.data(), tabs.size() * sizeof(float4), cudaMemcpyHostToDevice));
    if (!st) st = cuda_status(cudaMalloc(&d.d_filters, flt.size() * sizeof(IirBatchFilter)));
    if (!st)
        st = cuda_status(cudaMemcpy(d.d_filters, flt.data(), flt.size() * sizeof(IirBatchFilter), cudaMemcpyHostToDevice));
    if (!st)
        st = cuda_status(
            cudaFuncSetAttribute(sd.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sd.smem)));
    if (!st) st = cuda_status(cudaFuncSetAttribute(sd.fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int nb = 0;
    if (!st) st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sd.fn, sd.threads, sd.smem));
    cudaFuncAttributes fa{};
    if (!st) st = cuda_status(cudaFuncGetAttributes(&fa, sd.fn));
    if (st) return st;
    if (nb <= 0) return IIR_ERR_UNSUPPORTED;
    d.blocks_per_sm = nb;
    d.regs = fa.numRegs;
    d.ready = true;
    return IIR_OK;
}

// Parameters of a launch over `nchunks` chunks with shape k (segment tables already on the device).
IirBatchParams batch_params(const iir_batch* b, int k, const IirBatchSegment* segs, const unsigned int* starts,
                            unsigned int nsegs, unsigned int nchunks, long long withhold) {
    IirBatchParams q{};
    q.segs = segs;
    q.chunk_start = starts;
    q.filters = b->shape_data[static_cast<size_t>(k)].d_filters;
    q.secs = b->shape_data[static_cast<size_t>(k)].d_secs;
    q.tables = b->shape_data[static_cast<size_t>(k)].d_tables;
    q.phi = b->d_phi;
    q.carry = b->d_carry;
    q.state = b->d_state;
    q.carry_stride = 4 * (b->carry_cap + b->gcap);
    q.timeout_ns = b->timeout_ns;
    q.withhold_chunk = withhold;
    q.nsegs = nsegs;
    q.nchunks = nchunks;
    q.carry_cap = static_cast<unsigned int>(b->carry_cap);
    q.max_sections = b->max_sections;
    return q;
}

// The persistent launch: at most every resident block of shape k's kernel.
int batch_launch(const iir_batch* b, int k, IirBatchParams& q, cudaStream_t stream) {
    const ShapeDef& sd = shapes()[static_cast<size_t>(k)];
    const size_t resident = static_cast<size_t>(b->shape_data[static_cast<size_t>(k)].blocks_per_sm) * b->sms;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>(q.nchunks, resident));
    void* args[] = {&q};
    return cuda_status(cudaLaunchKernel(sd.fn, dim3(grid), dim3(sd.threads), args, sd.smem, stream));
}

// chunks of a segment of n samples with shape k
// Leading zeros of a segment's first chunk: a segment that starts at rest (no zi) with x not on
// a 16-byte boundary is chunked on x's 16-byte grid, its first chunk starting 1..3 zero samples
// before it (zero input from a zero state leaves the state zero, so the zeros change nothing). Its
// later chunks then start 16-byte aligned and move by the 16-byte copies.
int seg_lead(const iir_segment& s) {
    if (s.zi || s.n == 0) return 0;
    return static_cast<int>((reinterpret_cast<uintptr_t>(s.x) >> 2) & 3u);
}

size_t seg_chunks(const iir_segment& s, int k) {
    const ShapeDef& sd = shapes()[static_cast<size_t>(k)];
    const size_t chunk = static_cast<size_t>(sd.rows) * sd.n;
    const size_t n = s.n == 0 ? 0 : s.n + static_cast<size_t>(seg_lead(s));
    return (n + chunk - 1) / chunk;
}

}  // namespace

extern "C" {

int iir_batch_create(iir_batch** out, const float* sos, const int* n_sections, int n_filters, size_t max_segments,
                     size_t max_chunks) {
    if (!out || !sos || !n_sections || n_filters < 1) return IIR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    iir_batch* b = new iir_batch();
    b->n_filters = n_filters;
    b->filters.resize(static_cast<size_t>(n_filters));
    b->tail_need.assign(static_cast<size_t>(n_filters), 0);
    std::vector<float> phi(static_cast<size_t>(n_filters) * IIR_BT_PHI_FLOATS, 0.f);
    int max_sec = 1;
    size_t off = 0;
    for (int f = 0; f < n_filters; ++f) {
        const int ns = n_sections[f];
        if (ns < 1 || ns > IIR_MAX_SECTIONS) {
            delete b;
            return IIR_ERR_INVALID_ARGUMENT;
        }
        SectionF32 s32[IIR_MAX_SECTIONS];
        double gain = 1.0;
        int st = normalise_sos(sos + 6 * off, ns, s32, gain);
        if (st) {
            delete b;
            return st;
        }
        // the sections' scalars and lane tables depend on the chunk shape: shape_prepare builds them
        b->filters[static_cast<size_t>(f)] =
            IirBatchFilter{static_cast<float>(gain), ns, static_cast<int>(b->sec32.size()), 0};
        for (int k = 0; k < ns; ++k) b->sec32.push_back(s32[k]);
        // tail-aggregate schedule: pieces for the cascade's state to decay, and Phi^512
        std::vector<float> pf;
        b->tail_need[static_cast<size_t>(f)] = tail_pieces(s32, ns, IIR_TAIL_MAX_PIECES, pf);
        std::copy(pf.begin(), pf.end(), phi.begin() + static_cast<size_t>(f) * IIR_BT_PHI_FLOATS);
        max_sec = std::max(max_sec, ns);
        off += static_cast<size_t>(ns);
    }
    b->max_sections = max_sec;
    b->filter_sections.assign(n_sections, n_sections + n_filters);
    b->shape_data.resize(shapes().size());
    int st = cuda_status(cudaGetDevice(&b->device));
    if (!st) st = cuda_status(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
    if (!st) st = cuda_status(cudaMalloc(&b->d_phi, phi.size() * sizeof(float)));
    if (!st) st = cuda_status(cudaMemcpy(b->d_phi, phi.data(), phi.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (!st) st = cuda_status(cudaMalloc(&b->d_state, sizeof(IirLaunchState)));
    if (!st) st = cuda_status(cudaMemset(b->d_state, 0, sizeof(IirLaunchState)));
    if (!st) st = batch_alloc_segments(b, max_segments);
    if (!st) st = batch_alloc_carry(b, max_chunks, b->seg_cap);
    for (int i = 0; i < 2 && !st; ++i) st = cuda_status(cudaEventCreateWithFlags(&b->stage_done[i], cudaEventDisableTiming));
    if (!st) st = shape_prepare(b, 0);
    if (st) {
        batch_free(b);
        return st;
    }
    *out = b;
    return IIR_OK;
}

int iir_batch_set_shape(iir_batch* b, int rows, int samples_per_row) {
    if (!b) return IIR_ERR_INVALID_ARGUMENT;
    for (size_t k = 0; k < shapes().size(); ++k) {
        if (shapes()[k].rows == rows && shapes()[k].n == samples_per_row) {
            const int st = shape_prepare(b, static_cast<int>(k));
            if (st) return st;
            b->shape = static_cast<int>(k);
            return IIR_OK;
        }
    }
    return IIR_ERR_UNSUPPORTED;
}

int iir_batch_get_shape(const iir_batch* b, int* rows, int* samples_per_row, int* threads, int* regs_per_thread,
                        int* smem_bytes, int* blocks_per_sm) {
    if (!b) return IIR_ERR_INVALID_ARGUMENT;
    const ShapeDef& sd = shapes()[static_cast<size_t>(b->shape)];
    const ShapeData& d = b->shape_data[static_cast<size_t>(b->shape)];
    if (rows) *rows = sd.rows;
    if (samples_per_row) *samples_per_row = sd.n;
    if (threads) *threads = sd.threads;
    if (regs_per_thread) *regs_per_thread = d.regs;
    if (smem_bytes) *smem_bytes = static_cast<int>(sd.smem);
    if (blocks_per_sm) *blocks_per_sm = d.blocks_per_sm;
    return IIR_OK;
}

int iir_batch_execute(iir_batch* b, const iir_segment* segs, int n_segs, void* stream_) {
    if (!b || n_segs < 0 || (n_segs > 0 && !segs)) return IIR_ERR_INVALID_ARGUMENT;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const int k = b->shape;
    // validate and count chunks
    size_t total = 0, groups = 0;
    for (int i = 0; i < n_segs; ++i) {
        const iir_segment& s = segs[i];
        if (s.filter < 0 || s.filter >= b->n_filters) return IIR_ERR_INVALID_ARGUMENT;
        if (s.n > 0 && (!s.x || !s.y)) return IIR_ERR_INVALID_ARGUMENT;
        if (s.n > (1ull << 40)) return IIR_ERR_TOO_LARGE;
        const char* xb = reinterpret_cast<const char*>(s.x);
        const char* yb = reinterpret_cast<const char*>(s.y);
        if (s.n > 0 && xb < yb + s.n * sizeof(float) && yb < xb + s.n * sizeof(float)) return IIR_ERR_INVALID_ARGUMENT;
        const size_t ch = seg_chunks(s, k);
        total += ch;
        groups += (ch + IIR_GROUP - 1) / IIR_GROUP;
    }
    if (total == 0) return IIR_OK;
    if (total > 0x7fffffffull) return IIR_ERR_TOO_LARGE;
    if (static_cast<size_t>(n_segs) > b->seg_cap) {
        cudaStreamSynchronize(stream);
        const int st = batch_alloc_segments(b, static_cast<size_t>(n_segs) * 2);
        if (st) return st;
    }
    if (total > b->carry_cap || groups > b->gcap) {
        cudaStreamSynchronize(stream);
        const int st = batch_alloc_carry(b, std::max(total, b->carry_cap * 2), std::max<size_t>(n_segs, groups));
        if (st) return st;
    }
    if (++b->launches >= (1ull << 30)) {
        int st = cuda_status(cudaMemsetAsync(b->d_carry, 0, b->carry_bytes, stream));
        if (!st) st = cuda_status(cudaMemsetAsync(b->d_state, 0, IIR_STATE_RESET_BYTES, stream));
        if (st) return st;
        b->launches = 1;
    }
    // segment table into a pinned staging buffer (wait until its previous copy has left)
    const int turn = b->stage_turn;
    b->stage_turn ^= 1;
    int st = cuda_status(cudaEventSynchronize(b->stage_done[turn]));
    if (st) return st;
    IirBatchSegment* hs = reinterpret_cast<IirBatchSegment*>(b->h_stage[turn]);
    unsigned int* hstart = reinterpret_cast<unsigned int*>(b->h_stage[turn] + n_segs * sizeof(IirBatchSegment));
    unsigned int chunk0 = 0, group0 = 0;
    const size_t tail_min = batch_tail_min_chunks();
    for (int i = 0; i < n_segs; ++i) {
        const iir_segment& s = segs[i];
        const unsigned int ch = static_cast<unsigned int>(seg_chunks(s, k));
        hs[i] = IirBatchSegment{s.x, s.y, static_cast<long long>(s.n), s.zi, s.zf, chunk0, group0, s.filter,
                                ch >= tail_min ? 1 : 0, seg_lead(s), 0};
        hstart[i] = chunk0;
        chunk0 += ch;
        group0 += (ch + IIR_GROUP - 1) / IIR_GROUP;
    }
    hstart[n_segs] = chunk0;
    st = cuda_status(cudaMemcpyAsync(b->d_segs, hs, n_segs * sizeof(IirBatchSegment), cudaMemcpyHostToDevice, stream));
    if (!st)
        st = cuda_status(cudaMemcpyAsync(b->d_starts, hstart, (n_segs + 1) * sizeof(unsigned int),
                                         cudaMemcpyHostToDevice, stream));
    if (!st) st = cuda_status(cudaEventRecord(b->stage_done[turn], stream));
    if (st) return st;
    IirBatchParams q = batch_params(b, k, b->d_segs, b->d_starts, static_cast<unsigned int>(n_segs),
                                    static_cast<unsigned int>(total), b->withhold);
    b->withhold = -1;
    return batch_launch(b, k, q, stream);
}

struct iir_batch_bound {
    iir_batch* b = nullptr;
    int shape = 0;
    IirBatchSegment* d_segs = nullptr;
    unsigned int* d_starts = nullptr;
    unsigned int* d_chunk_seg = nullptr;  // each chunk's segment: no search in the launch
    IirBatchParams params{};
    unsigned int nchunks = 0;
};

int iir_batch_bind(iir_batch* b, const iir_segment* segs, int n_segs, iir_batch_bound** out) {
    if (!b || !out || n_segs < 0 || (n_segs > 0 && !segs)) return IIR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const int k = b->shape;
    std::vector<IirBatchSegment> hs(static_cast<size_t>(std::max(n_segs, 1)));
    std::vector<unsigned int> starts(static_cast<size_t>(n_segs) + 1);
    size_t chunk0 = 0, group0 = 0;
    const size_t tail_min = batch_tail_min_chunks();
    for (int i = 0; i < n_segs; ++i) {
        const iir_segment& s = segs[i];
        if (s.filter < 0 || s.filter >= b->n_filters) return IIR_ERR_INVALID_ARGUMENT;
        if (s.n > 0 && (!s.x || !s.y)) return IIR_ERR_INVALID_ARGUMENT;
        if (s.n > (1ull << 40)) return IIR_ERR_TOO_LARGE;
        const char* xb = reinterpret_cast<const char*>(s.x);
        const char* yb = reinterpret_cast<const char*>(s.y);
        if (s.n > 0 && xb < yb + s.n * sizeof(float) && yb < xb + s.n * sizeof(float)) return IIR_ERR_INVALID_ARGUMENT;
        const size_t ch = seg_chunks(s, k);
        hs[i] = IirBatchSegment{s.x, s.y, static_cast<long long>(s.n), s.zi, s.zf, static_cast<unsigned int>(chunk0),
                                static_cast<unsigned int>(group0), s.filter, ch >= tail_min ? 1 : 0, seg_lead(s), 0};
        starts[i] = static_cast<unsigned int>(chunk0);
        chunk0 += ch;
        group0 += (ch + IIR_GROUP - 1) / IIR_GROUP;
        if (chunk0 > 0x7fffffffull) return IIR_ERR_TOO_LARGE;
    }
    starts[n_segs] = static_cast<unsigned int>(chunk0);
    // each chunk's segment (the last of equal starts: empty segments have no chunks)
    std::vector<unsigned int> cseg(std::max<size_t>(chunk0, 1), 0u);
    for (int i = 0; i < n_segs; ++i)
        for (unsigned int c = starts[i]; c < starts[i + 1]; ++c) cseg[c] = static_cast<unsigned int>(i);
    int st = cuda_status(cudaDeviceSynchronize());
    if (st) return st;
    if (chunk0 > b->carry_cap || group0 > b->gcap) {
        st = batch_alloc_carry(b, std::max(chunk0, b->carry_cap * 2), std::max<size_t>(n_segs, group0));
        if (st) return st;
    }
    iir_batch_bound* h = new iir_batch_bound();
    h->b = b;
    h->shape = k;
    h->nchunks = static_cast<unsigned int>(chunk0);
    st = cuda_status(cudaMalloc(&h->d_segs, hs.size() * sizeof(IirBatchSegment)));
    if (!st) st = cuda_status(cudaMalloc(&h->d_starts, starts.size() * sizeof(unsigned int)));
    if (!st) st = cuda_status(cudaMalloc(&h->d_chunk_seg, cseg.size() * sizeof(unsigned int)));
    if (!st)
        st = cuda_status(
            cudaMemcpy(h->d_chunk_seg, cseg.data(), cseg.size() * sizeof(unsigned int), cudaMemcpyHostToDevice));
    if (!st)
        st = cuda_status(cudaMemcpy(h->d_segs, hs.data(), hs.size() * sizeof(IirBatchSegment), cudaMemcpyHostToDevice));
    if (!st)
        st = cuda_status(
            cudaMemcpy(h->d_starts, starts.data(), starts.size() * sizeof(unsigned int), cudaMemcpyHostToDevice));
    if (st) {
        if (h->d_segs) cudaFree(h->d_segs);
        if (h->d_starts) cudaFree(h->d_starts);
        if (h->d_chunk_seg) cudaFree(h->d_chunk_seg);
        delete h;
        return st;
    }
    h->params = batch_params(b, k, h->d_segs, h->d_starts, static_cast<unsigned int>(n_segs), h->nchunks, -1);
    h->params.chunk_seg = h->d_chunk_seg;
    *out = h;
    return IIR_OK;
}

int iir_batch_launch_bound(iir_batch_bound* h, void* stream_) {
    if (!h) return IIR_ERR_INVALID_ARGUMENT;
    if (h->nchunks == 0) return IIR_OK;
    iir_batch* b = h->b;
    // the carry slots must still be the ones bound (a later execute that grew them rebinds)
    if (h->params.carry != b->d_carry) return IIR_ERR_INVALID_ARGUMENT;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    if (++b->launches >= (1ull << 30)) {
        int st = cuda_status(cudaMemsetAsync(b->d_carry, 0, b->carry_bytes, stream));
        if (!st) st = cuda_status(cudaMemsetAsync(b->d_state, 0, IIR_STATE_RESET_BYTES, stream));
        if (st) return st;
        b->launches = 1;
    }
    return batch_launch(b, h->shape, h->params, stream);
}

int iir_batch_unbind(iir_batch_bound* h) {
    if (!h) return IIR_ERR_INVALID_ARGUMENT;
    cudaDeviceSynchronize();
    cudaFree(h->d_segs);
    cudaFree(h->d_starts);
    cudaFree(h->d_chunk_seg);
    delete h;
    return IIR_OK;
}

int iir_batch_check(iir_batch* b, void* stream_) {
    if (!b) return IIR_ERR_INVALID_ARGUMENT;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    int st = cuda_status(cudaStreamSynchronize(stream));
    if (st) return st;
    IirLaunchState hs;
    st = cuda_status(cudaMemcpy(&hs, b->d_state, sizeof(hs), cudaMemcpyDeviceToHost));
    if (st) return st;
    if (hs.error == 0ull) return IIR_OK;
    const unsigned long long zero = 0ull;
    cudaMemcpy(reinterpret_cast<char*>(b->d_state) + offsetof(IirLaunchState, error), &zero, sizeof(zero),
               cudaMemcpyHostToDevice);
    return device_error_status(hs.error);
}

int iir_batch_set_timeout_ns(iir_batch* b, long long timeout_ns) {
    if (!b || timeout_ns <= 0) return IIR_ERR_INVALID_ARGUMENT;
    b->timeout_ns = timeout_ns;
    return IIR_OK;
}

int iir_batch_debug_withhold(iir_batch* b, long long chunk) {
    if (!b) return IIR_ERR_INVALID_ARGUMENT;
    b->withhold = chunk;
    return IIR_OK;
}

int iir_batch_filter_sections(const iir_batch* b, int filter) {
    if (!b || filter < 0 || filter >= b->n_filters) return IIR_ERR_INVALID_ARGUMENT;
    return b->filter_sections[static_cast<size_t>(filter)];
}

int iir_batch_destroy(iir_batch* b) {
    if (!b) return IIR_ERR_INVALID_ARGUMENT;
    batch_free(b);
    return IIR_OK;
}

}  // extern "C"
