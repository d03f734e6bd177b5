// iir_twopass.cuh — persistent two-pass pipeline for single-section filters (order 2).
//
// Every chunk is read twice: once to compute its zero-state aggregate (pass A) and, D chunks
// of the block later, again to filter it with its incoming state already known (pass B).
// The second read comes from L2: between the two reads the whole grid streams about
// D * G * 32 KB (a few tens of MB), far below the 129 MB L2, so HBM still sees 4 bytes read
// and 4 written per sample. What this buys: the lookback of chunk k (microseconds of L2
// round trips) overlaps D chunks of work and never stalls the filtering, and shared memory
// holds only chunks in flight, not chunks waiting for their carries.
//
// The grid is launched cooperatively (all blocks co-resident) and block b owns chunks
// b, b + G, b + 2G, ... (G = gridDim.x); every dependency points to a lower chunk index, so
// the static order cannot deadlock. Roles:
//   TMA warp       loads chunk data (and the 32 samples before it) for the items A(k), B(k)
//                  in the order the row warps consume them, S stages ahead; stores B items;
//   lookback warp  two-level decoupled lookback of chunk k once A(k) published its aggregate;
//   row warps      A(k) then B(k - D) for k = 0, 1, ...:
//                  A: zero-state pass over the chunk (one or two threads per row), scan of the
//                     row tails; keeps the per-row zero-state incoming pairs for B (PH) and
//                     publishes the chunk aggregate at once;
//                  B: the realization's own solve of the chunk with its incoming state.
// Every wait is bounded (iir_pipe.cuh: pipe_wait, lookback_hier / lookback_trunc2).
#pragma once
#include "iir_pipe.cuh"

namespace iirgb {

// Items consumed by the row warps, in order: step k emits A(k) (k < nk), then B(k - D) (k >= D).
struct TwoPassSeq {
    uint32_t nk, D, k = 0;
    int phase = 0;
    __device__ TwoPassSeq(uint32_t nk_, uint32_t D_) : nk(nk_), D(D_) {}
    __device__ bool next(bool& is_b, uint32_t& kk) {
        while (k < nk + D) {
            if (phase == 0) {
                phase = 1;
                if (k < nk) {
                    is_b = false;
                    kk = k;
                    return true;
                }
            } else {
                phase = 0;
                const uint32_t kb = k++;
                if (kb >= D) {
                    is_b = true;
                    kk = kb - D;
                    return true;
                }
            }
        }
        return false;
    }
};

// Inclusive scan over the RW rows of a warp (TPR lanes per row, the row's state in its last
// lane) of S_r = C S_{r-1} + s_r, with C^(2^k) = tc[2^k - 1].
template <int RW, int TPR>
__device__ __forceinline__ void warp_scan_rows(float& s0, float& s1, const float4* tc, int row) {
#pragma unroll
    for (int k = 0; (1 << k) < RW; ++k) {
        const int d = 1 << k;
        const float o0 = __shfl_up_sync(FULL_MASK, s0, d * TPR);
        const float o1 = __shfl_up_sync(FULL_MASK, s1, d * TPR);
        if (row >= d) {
            const float4 m = tc[d - 1];
            s0 = fmaf(m.x, o0, fmaf(m.y, o1, s0));
            s1 = fmaf(m.z, o0, fmaf(m.w, o1, s1));
        }
    }
}

// Pass A: zero-state aggregate of the chunk in `buf` (not modified). TPR lanes per row, each
// filtering N / TPR samples with zero state; the halves of a row are joined with A^(N/2).
// Writes the per-row zero-state incoming pairs to zin and the aggregate to aux->partv[slot].
template <int N, int ROWS, int TPR, int NW>
__device__ __forceinline__ void pass_aggregate(const IirParams& p, const float* buf, const float* hist,
                                               const float4* tc, float (*zin)[2], PipeAux* aux, int slot, int w,
                                               int lane) {
    using Geo = PipeGeom<ROWS, N, 2>;
    constexpr int RW = 32 / TPR, SPAN = N / TPR;
    static_assert(NW * RW == ROWS, "rows per block");
    const int rl = lane / TPR, p0 = lane % TPR, r = w * RW + rl, n0 = p0 * SPAN;
    const IirSection& q = p.sec[0];
    float xh2, xh1;
    if (n0 > 0) {
        xh2 = buf[swz<N, ROWS, two_planes(N)>(r, n0 - 2)];
        xh1 = buf[swz<N, ROWS, two_planes(N)>(r, n0 - 1)];
    } else if (r > 0) {
        xh2 = buf[swz<N, ROWS, two_planes(N)>(r - 1, N - 2)];
        xh1 = buf[swz<N, ROWS, two_planes(N)>(r - 1, N - 1)];
    } else {
        xh2 = hist[30];
        xh1 = hist[31];
    }
    // The aggregate is linear in the input: the recurrence runs on the raw samples and the
    // gain scales its end pair once.
    float y1 = 0.f, y2 = 0.f;
#pragma unroll 4
    for (int j = 0; j < SPAN / 4; ++j) {
        const float4 v = *reinterpret_cast<const float4*>(buf + swz<N, ROWS, two_planes(N)>(r, n0 + 4 * j));
        const float xs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float wv = fmaf(q.b2, xh2, fmaf(q.b1, xh1, xs[k]));
            const float y = fmaf(q.a1, y1, fmaf(q.a2, y2, wv));
            xh2 = xh1;
            xh1 = xs[k];
            y2 = y1;
            y1 = y;
        }
    }
    float s0 = y2 * p.gain, s1 = y1 * p.gain;
    if (TPR == 2) {
        // row tail = A^(N/2) (first half's tail) + second half's zero-state tail
        const float t0 = __shfl_xor_sync(FULL_MASK, s0, 1);
        const float t1 = __shfl_xor_sync(FULL_MASK, s1, 1);
        if (p0) {
            float h0, h1;
            mv2(tc[Geo::TC_HALF], t0, t1, h0, h1);
            s0 += h0;
            s1 += h1;
        }
    }
    warp_scan_rows<RW, TPR>(s0, s1, tc, rl);
    if (lane == 31) {
        aux->wtot[w][0][0] = s0;
        aux->wtot[w][0][1] = s1;
    }
    named_barrier_rows(NW);
    float in0 = 0.f, in1 = 0.f;
    if (w > 0) {
        warp_incoming(aux, w, 0, tc[RW - 1], in0, in1);  // C^RW across a warp's rows
        float e0, e1;
        mv2(tc[rl], in0, in1, e0, e1);  // C^(rl+1)
        s0 += e0;
        s1 += e1;
    }
    // zero-state incoming pair of row r = zero-state tail of row r - 1
    float i0 = __shfl_up_sync(FULL_MASK, s0, TPR);
    float i1 = __shfl_up_sync(FULL_MASK, s1, TPR);
    if (rl == 0) {
        i0 = in0;
        i1 = in1;
    }
    if (p0 == TPR - 1) {
        zin[r][0] = i0;
        zin[r][1] = i1;
        if (r == ROWS - 1) {
            aux->partv[slot][0] = s0;
            aux->partv[slot][1] = s1;
        }
    }
}

template <int ROWS, int N, int S, int D>
struct TwoPassGeom {
    using G = PipeGeom<ROWS, N, S>;
    static constexpr size_t SMEM_BYTES =
        1024 + S * (G::DATA_BYTES + G::HIST_BYTES) + G::TC_BYTES + (D + 1) * G::ZIN_BYTES + sizeof(PipeAux);
    static constexpr int min_blocks(int threads) {
        const int by_smem = static_cast<int>((227 * 1024) / (SMEM_BYTES + 1024));
        const int by_thr = 2048 / threads;
        const int b = by_smem < by_thr ? by_smem : by_thr;
        return b < 1 ? 1 : b;
    }
};

// R provides: ROWS, N, NW (row warps), TPR (threads per row);
//   b_pass(p, buf, hist, tc, zin, aux, X0, X1, w, lane): the output of the chunk in buf given
//        its incoming state X and pass A's per-row zero-state incoming pairs zin; called by
//        every row thread (may use barrier 1 and aux->wtot); ends with the output in buf.
// S = shared-memory stages, D = chunks between a chunk's pass A and its pass B.
template <class R, int S, int D>
__device__ __forceinline__ void run_twopass(const IirParams& p, unsigned char* smem_raw) {
    constexpr int ROWS = R::ROWS, N = R::N, NW = R::NW, RING = D + 1;
    static_assert(S >= 2 && S <= 8 && RING <= 8 && D >= 1, "stages and lag");
    using G = PipeGeom<ROWS, N, S>;
    const uint32_t a = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((a + 1023u) & ~1023u) - a);
    // [S data stages (1024-aligned) | S history lines | table cache | RING zin arrays | aux]
    float* bufs = reinterpret_cast<float*>(base);
    float* hists = reinterpret_cast<float*>(base + S * G::DATA_BYTES);
    float4* tc = reinterpret_cast<float4*>(base + S * (G::DATA_BYTES + G::HIST_BYTES));
    float(*zins)[2] = reinterpret_cast<float(*)[2]>(base + S * (G::DATA_BYTES + G::HIST_BYTES) + G::TC_BYTES);
    PipeAux* aux = reinterpret_cast<PipeAux*>(base + S * (G::DATA_BYTES + G::HIST_BYTES) + G::TC_BYTES +
                                              RING * G::ZIN_BYTES);
    auto buf_of = [&](int s) { return bufs + static_cast<size_t>(s) * G::CHUNK; };
    auto hist_of = [&](int s) { return hists + static_cast<size_t>(s) * 32; };
    auto zin_of = [&](uint32_t k) { return zins + static_cast<size_t>(k % RING) * ROWS; };

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t nb = gridDim.x;
    const uint32_t nk = (p.nchunks > blockIdx.x) ? (p.nchunks - blockIdx.x + nb - 1) / nb : 0;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&aux->full[s], 1);
            mbar_init(&aux->done[s], 1);
        }
        for (int s = 0; s < RING; ++s) {
            mbar_init(&aux->part[s], 1);
            mbar_init(&aux->xrdy[s], 1);
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
    const uint32_t items = 2u * nk;
    auto chunk_of = [&](uint32_t k) { return blockIdx.x + k * nb; };
    auto bulk_of = [&](uint32_t c) { return p.use_tma && (static_cast<long long>(c) + 1) * (ROWS * N) <= p.n; };
    auto spar = [](uint32_t q) { return (q / S) & 1u; };
    auto rpar = [](uint32_t k) { return (k / RING) & 1u; };

    if (warp == 0) {
        // --------------------------------- TMA warp ---------------------------------
        TwoPassSeq ld(nk, D), dn(nk, D);
        auto load = [&](uint32_t q) {
            bool is_b;
            uint32_t k;
            ld.next(is_b, k);
            const int s = q % S;
            const uint32_t c = chunk_of(k);
            if (lane == 0) {
                if (bulk_of(c)) {
                    mbar_arrive_expect_tx(&aux->full[s], static_cast<uint32_t>(G::DATA_BYTES + G::HIST_BYTES));
                    tma_load_chunk<ROWS, N, two_planes(N)>(buf_of(s), &p.tmap_x, c, &aux->full[s]);
                    tma_load_2d(hist_of(s), &p.tmap_h, 0, static_cast<int>(c) * G::LINES - 1, &aux->full[s]);
                } else {
                    mbar_arrive(&aux->full[s]);  // element-wise chunk: the stage is free
                }
            }
        };
        uint32_t issued = 0;
        for (; issued < items && issued < static_cast<uint32_t>(S); ++issued) load(issued);
        for (uint32_t q = 0; q < items; ++q) {
            bool is_b;
            uint32_t k;
            dn.next(is_b, k);
            const int s = q % S;
            const uint32_t c = chunk_of(k);
            const bool ok = pipe_wait(aux, &aux->done[s], spar(q), p, epoch);
            const bool stored = is_b && ok && bulk_of(c) && !*reinterpret_cast<volatile int*>(&aux->bail);
            if (lane == 0 && stored) {
                tma_store_chunk<ROWS, N, two_planes(N)>(&p.tmap_y, c, buf_of(s));
                bulk_commit();
            }
            if (q + S < items && ok) {
                if (lane == 0 && stored) bulk_wait_read_all();  // the stage's store has read the buffer
                __syncwarp();
                load(q + S);
                issued = q + S + 1;
            }
        }
        if (lane == 0) bulk_wait_all();
        if (*reinterpret_cast<volatile int*>(&aux->abandon) && lane == 0) {
            const uint32_t first = issued > static_cast<uint32_t>(S) ? issued - S : 0;
            for (uint32_t q = first; q < issued; ++q) (void)wait_mbar_bounded(&aux->full[q % S], spar(q), p.timeout_ns);
        }
    } else if (warp == 1) {
        // ------------------------------- lookback warp -------------------------------
        unsigned long long* slots = p.carry;
        unsigned long long* gslots = slots + static_cast<size_t>(p.carry_cap) * 4;
        const float4 Q = tc[G::TC_QC + 1];
        const int lb_depth = static_cast<int>(p.tables[IIR_TAB_LBD].x);  // truncated lookback depth (0: two-level)
        const float z0 = p.zi ? p.zi[2] : 0.f, z1 = p.zi ? p.zi[3] : 0.f;
        const uint32_t ff = 2u * epoch + 2u;
        bool failed = false;
        for (uint32_t k = 0; k < nk; ++k) {
            const int s = k % RING;
            const uint32_t c = chunk_of(k);
            // chunk 0 starts from the signal's initial state (y[-2], y[-1]) (zero unless given)
            float X0 = z0, X1 = z1;
            bool ok = pipe_wait(aux, &aux->part[s], rpar(k), p, epoch);
            ok = __all_sync(FULL_MASK, ok && !failed);  // warp-uniform: lookback_hier is a full-warp routine
            if (ok) {
                const float a0 = aux->partv[s][0], a1 = aux->partv[s][1];
                const bool withhold = static_cast<long long>(c) == p.withhold_chunk;
                if (c > 0)
                    ok = lb_depth > 0 ? lookback_trunc2(p, slots, tc + G::TC_QC, c, epoch, lb_depth, X0, X1, z0, z1)
                                      : lookback_hier(p, slots, gslots, tc + G::TC_QC, tc + G::TC_QG, c, epoch, a0, a1,
                                                      withhold, X0, X1, z0, z1);
                if (lane == 0 && ok && !withhold) {
                    float q0, q1;
                    mv2(Q, X0, X1, q0, q1);
                    publish2(slots + static_cast<size_t>(c) * 4 + 2, ff, a0 + q0, a1 + q1);
                    if ((c & 31u) == 31u) publish2(gslots + static_cast<size_t>(c >> 5) * 4 + 2, ff, a0 + q0, a1 + q1);
                }
                if (!ok) {
                    failed = true;
                    if (lane == 0) *reinterpret_cast<volatile int*>(&aux->bail) = 1;
                }
            }
            if (lane == 0) {
                aux->xv[s][0] = X0;
                aux->xv[s][1] = X1;
                mbar_arrive(&aux->xrdy[s]);  // release: xv is visible to the waiting row warps
            }
            __syncwarp();
        }
    } else {
        // --------------------------------- row warps ---------------------------------
        const int w = warp - 2;
        const int rt = tid - 64;
        const uint32_t pf = 2u * epoch + 1u;
        TwoPassSeq seq(nk, D);
        bool is_b;
        uint32_t k;
        for (uint32_t q = 0; seq.next(is_b, k); ++q) {
            const int s = q % S;
            const uint32_t c = chunk_of(k);
            const bool ok = pipe_wait(aux, &aux->full[s], spar(q), p, epoch);
            // (barriers depend on uniform conditions only; `ok` may differ per thread)
            if (!bulk_of(c)) {
                const long long cs = static_cast<long long>(c) * G::CHUNK;
                float* b = buf_of(s);
                if (ok) {
                    for (int i = rt; i < G::CHUNK; i += NW * 32) {
                        const long long g = cs + i;
                        b[swz<N, ROWS, two_planes(N)>(i / N, i % N)] = (g < p.n) ? p.x[g] : 0.f;
                    }
                    if (rt < 32) hist_of(s)[rt] = (cs - 32 + rt >= 0) ? p.x[cs - 32 + rt] : 0.f;
                }
                named_barrier_rows(NW);
            }
            if (c == 0 && p.zi) {
                // the two input samples before the signal come from the initial state
                if (rt == 0) {
                    hist_of(s)[30] = p.zi[0];
                    hist_of(s)[31] = p.zi[1];
                    fence_proxy_async_smem();  // before the stage is refilled by a tensor copy
                }
                named_barrier_rows(NW);
            }
            if (!is_b) {
                pass_aggregate<N, ROWS, R::TPR, NW>(p, buf_of(s), hist_of(s), tc, zin_of(k), aux, k % RING, w, lane);
                named_barrier_rows(NW);  // the stage has been read; partv is written
                if (rt == 0) {
                    if (static_cast<long long>(c) != p.withhold_chunk)
                        publish2(p.carry + static_cast<size_t>(c) * 4, pf, aux->partv[k % RING][0],
                                 aux->partv[k % RING][1]);
                    mbar_arrive(&aux->part[k % RING]);
                    mbar_arrive(&aux->done[s]);
                }
            } else {
                (void)pipe_wait(aux, &aux->xrdy[k % RING], rpar(k), p, epoch);
                // (after a failed wait the pass still runs, so every barrier is met; the
                // chunk is not stored)
                R::b_pass(p, buf_of(s), hist_of(s), tc, zin_of(k), aux, aux->xv[k % RING][0], aux->xv[k % RING][1],
                          w, lane);
                if (!bulk_of(c)) {
                    named_barrier_rows(NW);
                    const long long cs = static_cast<long long>(c) * G::CHUNK;
                    const float* b = buf_of(s);
                    if (!*reinterpret_cast<volatile int*>(&aux->bail)) {
                        for (int i = rt; i < G::CHUNK; i += NW * 32) {
                            const long long g = cs + i;
                            if (g < p.n) p.y[g] = b[swz<N, ROWS, two_planes(N)>(i / N, i % N)];
                        }
                    }
                }
                fence_proxy_async_smem();  // generic writes -> visible to the TMA store
                named_barrier_rows(NW);
                if (rt == 0) mbar_arrive(&aux->done[s]);
            }
        }
    }
    __syncthreads();
    if (tid == 0) pipe_finish(p.state, epoch);
}

}  // namespace iirgb
