// iir_ph.cuh — PH realization (partial LU + correction vectors) for sm_103a.
//
// Reference: PH_32 / PH_64, include/ph_kernels.cuh:208-820. Per section, every row (thread)
//   1. runs FIR + recurrence over its N samples with zero row state (ph_kernels.cuh:265-287);
//   2. the rows' tail pairs (y[N-2], y[N-1]) are combined by an inclusive scan of the affine
//      map s_r = C s_{r-1} + local_r, C = A^N (ph_kernels.cuh:293-382 does it with shuffled
//      C_cross powers; here a Kogge-Stone scan with uniform C^(2^k) inside a warp and a
//      shared-memory composition across the block's warps, as PH_64 does for its two warps,
//      ph_kernels.cuh:680-771);
//   3. the block aggregate is published and its incoming state X resolved by the decoupled
//      lookback (control warp, iir_device.cuh; reference ph_kernels.cuh:384-451);
//   4. true tails T_r = s_r + C^(r+1) X (ph_kernels.cuh:456-459, C_inner);
//   5. the row body is corrected by the homogeneous response to the row's incoming state
//      T_{r-1} (ph_kernels.cuh:471-480 uses h1/h2 tables; here the response is generated by
//      the section's own recurrence and applied on the fly while the next section's filter
//      pass reads the row, so each section costs one read and one write of the row).
// GB300 layout: rows stay in the block's (TMA-staged, swizzled) shared-memory buffer rather
// than in registers. A thread needs ~30 registers, so up to a dozen blocks share an SM and
// their loads and lookback waits overlap each other's filtering (the lookback latency is
// set by the slowest predecessor's load, so concurrency, not a faster poll, hides it).
// With TAIL (iir_tail.cuh), the control warp resolves every section's incoming state once per
// chunk from the predecessor's tail aggregate, and steps 3 and 4 read it from shared memory: the
// row warps meet at one barrier per section (among themselves) instead of two around a lookback.
#pragma once
#include "iir_device.cuh"
#include "iir_tail.cuh"
#include "iir_twopass.cuh"

namespace iirgb {

template <int B_, int N_, int ROWS_, bool TAIL = false>
struct PhBlock {
    static constexpr int B = B_, N = N_, ROWS = ROWS_;
    static constexpr int NW = ROWS / 32;           // row warps
    static constexpr int THREADS = 32 + ROWS;      // + control warp
    static_assert(ROWS % 32 == 0 && ROWS <= IIR_MAX_ROWS && NW <= 16, "rows per block");

    __device__ static void run(const IirParams& p, unsigned char* smem) {
        float* buf = chunk_buffer<ROWS, N>(smem);
        BlockAux* aux = block_aux<ROWS, N>(smem);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (warp == 0) block_begin<ROWS, N>(p, buf, aux);
        __syncthreads();
        const uint32_t c = aux->chunk, epoch = aux->epoch;
        if (!block_acquire<ROWS, N, THREADS>(p, buf, aux, c, epoch)) return;
        const bool ok = filter_block(p, buf, aux, c, epoch, warp, lane);
        // output written to shared memory + fence.proxy.async by the row warps
        __syncthreads();
        if (ok) block_store<ROWS, N, THREADS>(p, buf, c);
    }

    // One pass over the row: x = stored value (+ correction of the previous section, whose
    // recurrence is (pa1, pa2) and whose incoming state is (d2, d1); or, for the first section,
    // times the cascade's input gain g), then FIR + recurrence with zero row state; the
    // zero-state output overwrites the row. Returns the row's zero-state tail pair in (s0, s1).
    template <bool CORRECT>
    __device__ static void filter_pass(float* buf, int r, float b1, float b2, float a1, float a2, float pa1,
                                       float pa2, float d2, float d1, float& xh2, float& xh1, float& s0,
                                       float& s1, float g = 1.f) {
        float y1 = 0.f, y2 = 0.f;
#pragma unroll
        for (int j = 0; j < N / 4; ++j) {
            float4* ptr = reinterpret_cast<float4*>(buf + swz<N, ROWS, true>(r, 4 * j));
            const float4 q = *ptr;
            const float xs[4] = {q.x, q.y, q.z, q.w};
            float ys[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float xv = xs[k];
                if (CORRECT) {
                    const float dn = fmaf(pa1, d1, pa2 * d2);
                    d2 = d1;
                    d1 = dn;
                    xv += dn;
                } else {
                    xv *= g;
                }
                const float wv = fmaf(b2, xh2, fmaf(b1, xh1, xv));
                const float y = fmaf(a1, y1, fmaf(a2, y2, wv));
                xh2 = xh1;
                xh1 = xv;
                y2 = y1;
                y1 = y;
                ys[k] = y;
            }
            *ptr = make_float4(ys[0], ys[1], ys[2], ys[3]);
        }
        s0 = y2;
        s1 = y1;
    }

    // Final correction pass (last section): row += response to the incoming state.
    __device__ static void correct_pass(float* buf, int r, float a1, float a2, float d2, float d1) {
#pragma unroll
        for (int j = 0; j < N / 4; ++j) {
            float4* ptr = reinterpret_cast<float4*>(buf + swz<N, ROWS, true>(r, 4 * j));
            const float4 q = *ptr;
            float v[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float dn = fmaf(a1, d1, a2 * d2);
                d2 = d1;
                d1 = dn;
                v[k] += dn;
            }
            *ptr = make_float4(v[0], v[1], v[2], v[3]);
        }
    }

    // All warps: warp 0 resolves carries, warps 1.. filter one row per thread.
    __device__ static bool filter_block(const IirParams& p, float* buf, BlockAux* aux, uint32_t c, uint32_t epoch,
                                        int warp, int lane) {
        const bool row_warp = warp > 0;
        if constexpr (TAIL) {
            bool ok = true;
            if (!tail_begin<N, ROWS, true>(p, buf, aux, c, epoch, warp, ok)) return ok;  // control warp
        }
        const int w = warp - 1;
        const int r = w * 32 + lane;  // row index (row warps)
        float xh2 = 0.f, xh1 = 0.f;   // input history of this row
        const float gain = p.gain;
        if (row_warp) {
            if (r > 0) {
                xh2 = buf[swz<N, ROWS, true>(r - 1, N - 2)];
                xh1 = buf[swz<N, ROWS, true>(r - 1, N - 1)];
            } else if (c > 0) {
                const long long cs = static_cast<long long>(c) * (ROWS * N);
                xh2 = __ldg(p.x + cs - 2);
                xh1 = __ldg(p.x + cs - 1);
            }
            xh2 *= gain;
            xh1 *= gain;
            // Every row has read its neighbour's history before any row is overwritten (the
            // first section's pass applies the gain as it reads the raw samples).
            named_barrier_rows(NW);
        }
        float pa1 = 0.f, pa2 = 0.f, d2 = 0.f, d1 = 0.f;  // previous section's correction
        for (int sec = 0; sec < p.n_sections; ++sec) {
            const IirSection& q = p.sec[sec];
            const float4* tab = p.tables + sec * IIR_TAB_STRIDE;
            const float4 Gw = tab[IIR_TAB_GPOW + 31];
            float s0 = 0.f, s1 = 0.f, in0 = 0.f, in1 = 0.f;
            if (row_warp) {
                if (sec == 0)
                    filter_pass<false>(buf, r, q.b1, q.b2, q.a1, q.a2, 0.f, 0.f, 0.f, 0.f, xh2, xh1, s0, s1, gain);
                else
                    filter_pass<true>(buf, r, q.b1, q.b2, q.a1, q.a2, pa1, pa2, d2, d1, xh2, xh1, s0, s1);
                // scan of row tails (zero block state)
                warp_scan2<32, 1>(s0, s1, q.M, lane);
                if (lane == 31) {
                    aux->wtot[w][TAIL ? (sec & 1) : 0][0] = s0;
                    aux->wtot[w][TAIL ? (sec & 1) : 0][1] = s1;
                }
            }
            // (A); the tail schedule alternates the warp totals' buffers, so one barrier per section
            // separates a section's reads from the next section's writes
            if (!TAIL || sec == 0) __syncthreads();
            else named_barrier_rows(NW);
            if (row_warp) {
                warp_incoming(aux, w, TAIL ? (sec & 1) : 0, Gw, in0, in1);  // zero-state tail before this warp
                if (w > 0) {
                    float e0, e1;
                    mv2(tab[IIR_TAB_GPOW + lane], in0, in1, e0, e1);
                    s0 += e0;
                    s1 += e1;
                }
            }
            if (!TAIL) {
                if (!row_warp) control_section<NW, 1>(p, aux, sec, c, epoch, tab, Gw);
                __syncthreads();  // (B)
            }
            if (aux->bail) return false;
            if (row_warp) {
                const float X0 = TAIL ? aux->Xs[sec][0] : aux->X[0], X1 = TAIL ? aux->Xs[sec][1] : aux->X[1];
                // true tails and the true incoming state of this row
                float P0, P1;
                mv2(tab[IIR_TAB_CPOW + r], X0, X1, P0, P1);
                const float T0 = s0 + P0, T1 = s1 + P1;
                float i0 = __shfl_up_sync(FULL_MASK, T0, 1);
                float i1 = __shfl_up_sync(FULL_MASK, T1, 1);
                if (lane == 0) {
                    if (r == 0) {
                        i0 = X0;
                        i1 = X1;
                    } else {
                        float q0, q1;
                        mv2(tab[IIR_TAB_CPOW + r - 1], X0, X1, q0, q1);
                        i0 = in0 + q0;
                        i1 = in1 + q1;
                    }
                }
                // the correction of this section is applied by the next pass
                pa1 = q.a1;
                pa2 = q.a2;
                d2 = i0;
                d1 = i1;
                xh2 = i0;  // next section's input history = this section's true outputs
                xh1 = i1;
            }
        }
        if (row_warp) {
            correct_pass(buf, r, pa1, pa2, d2, d1);
            fence_proxy_async_smem();
        }
        return true;
    }
};

// Single-section PH on the two-pass pipeline (iir_twopass.cuh): pass B runs the true
// recurrence over each row from its true incoming pair (pass A's zero-state incoming pair +
// C^r X), one pass over the row.
template <int N_, int ROWS_>
struct PhTwo {
    static constexpr int N = N_, ROWS = ROWS_, NW = ROWS / 32, TPR = 1;
    static_assert(ROWS % 32 == 0 && NW <= 16, "rows per block");

    __device__ static void b_pass(const IirParams& p, float* buf, const float* hist, const float4* tc,
                                  const float (*zin)[2], PipeAux*, float X0, float X1, int w, int lane) {
        const int r = w * 32 + lane;
        const IirSection& q = p.sec[0];
        const float gain = p.gain;
        float xh2, xh1;
        if (r > 0) {
            xh2 = buf[swz<N, ROWS, two_planes(N)>(r - 1, N - 2)];
            xh1 = buf[swz<N, ROWS, two_planes(N)>(r - 1, N - 1)];
        } else {
            xh2 = hist[30];
            xh1 = hist[31];
        }
        xh2 *= gain;
        xh1 *= gain;
        float y2 = X0, y1 = X1;  // true incoming pair (y[-2], y[-1]) of the row
        if (r > 0) {
            float q0, q1;
            mv2(tc[r - 1], X0, X1, q0, q1);  // C^r X
            y2 = zin[r][0] + q0;
            y1 = zin[r][1] + q1;
        }
        named_barrier_rows(NW);  // every row has its input history before rows are overwritten
#pragma unroll 4
        for (int j = 0; j < N / 4; ++j) {
            float4* ptr = reinterpret_cast<float4*>(buf + swz<N, ROWS, two_planes(N)>(r, 4 * j));
            const float4 v = *ptr;
            const float xs[4] = {v.x * gain, v.y * gain, v.z * gain, v.w * gain};
            float ys[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float wv = fmaf(q.b2, xh2, fmaf(q.b1, xh1, xs[k]));
                const float y = fmaf(q.a1, y1, fmaf(q.a2, y2, wv));
                xh2 = xh1;
                xh1 = xs[k];
                y2 = y1;
                y1 = y;
                ys[k] = y;
            }
            *ptr = make_float4(ys[0], ys[1], ys[2], ys[3]);
        }
    }
};

}  // namespace iirgb
