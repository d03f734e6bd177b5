// iir_cr.cuh — cyclic-reduction row solver shared by the STCR and DTCR realizations.
//
// Reference algorithm (include/stcr_kernels.cuh:279-605, include/dtcr_kernels.cuh:291-657,
// factors stcr_kernels.cuh:93-147), restated. For the section recurrence
//     y[n] + e y[n-1] + f y[n-2] = w[n],   e = -a1, f = -a2,  w = FIR(x),
// one double-sided round multiplies by (1 - e z^-1 + f z^-2):
//     y[n] + e1 y[n-2] + f1 y[n-4] = v1[n],  v1 = w[n] - e w[n-1] + f w[n-2],
// which decouples the even and odd samples (DTCR runs the two halves on two threads of a
// row; STCR runs both halves in one thread). Each half of M = N/2 samples (half index m,
// row position 2m + p) is then reduced by L-1 levels (L = log2 N); level k has half-stride
// h = 2^(k-1) and coefficients (e_k, f_k) of the stride-2^k recurrence. In every group of
// 2h half positions, the dropped position d = g + h - 1 keeps
//     u[d] = v[d] - (f_k / e_k) v[d - h]
// and the kept position q = d + h becomes  v'[q] = v[q] - e_k u[d]
// (the LU-split elimination; v[d - h] is the previous group's kept value before this level,
// and for the first group the previous row's). After the last level the half's last sample
// (row position N-2+p) obeys the cross-row recurrence Y_t + e_L Y_{t-1} + f_L Y_{t-2} = V_t
// (the reference's "block filtering", here a Kogge-Stone scan per parity). Back-substitution
// then recovers the dropped positions level by level:
//     y[d] = u[d] - c_k y[d - h] - d_k y[d - 3h],   c_k = e_k - f_k/e_k,  d_k = -f_k^2/e_k.
// In the cascade kernels this runs in the zero-padded tile (zero state before the tile) and
// the response to the tile's incoming state is added afterwards (PH-style correction), since
// that state is only known after the lookback. The two-pass kernels know it before the solve
// and put it into the first row's right-hand sides instead (solve_tile, Y2 / Y1). The
// reference folds the state into the back-substitution with its h/g/p/q factors
// (stcr_kernels.cuh:479-585).
//
// UNROLL selects the straight-line form (every reduction level spelled out; the reference's
// hand-unrolled kernels) or the loop form (a run-time loop over the reduction levels; the
// reference's *_LOOP kernels). Both keep the row's halves in registers, as the reference's loop
// kernels do ("all loop bounds and indices are compile-time constants after full unrolling, so
// in_reg[] stays register-resident", stcr_kernels.cuh back-substitution): the loop form's
// level loop dispatches each iteration to that level's body, whose indices are compile-time
// constants. Both execute the same operations in the same order, so they are bit-identical.
//
// With TAIL (iir_tail.cuh) the cascade kernel resolves every section's incoming state once per
// chunk from the predecessor's tail aggregate, before the first section's join; the row warps
// then join tiles with one barrier among themselves per section instead of two around a lookback.
#pragma once
#include <type_traits>
#include "iir_device.cuh"
#include "iir_tail.cuh"
#include "iir_twopass.cuh"

namespace iirgb {

// One parity half of a row. u[] holds the half's values (half index m), in registers.
template <int M>
struct CrHalf {
    static constexpr int L1 = (M == 8) ? 3 : (M == 16) ? 4 : (M == 32) ? 5 : (M == 64) ? 6 : 0;  // log2(M)
    static_assert(L1 > 0, "half length");

    // Elimination level k (half-stride h), prev = previous row's kept tail before this level.
    template <class U>
    __device__ __forceinline__ static void eliminate(U&& u, int h, float rk, float ek, float prev) {
        float old = prev;  // level-(k-1) value of the previous group's kept position
#pragma unroll
        for (int g = 0; g < M; g += 2 * h) {
            const int d = g + h - 1, q = d + h;
            const float ud = fmaf(-rk, old, u[d]);
            const float vq = u[q];
            u[d] = ud;
            u[q] = fmaf(-ek, ud, vq);
            old = vq;
        }
    }
    // Back-substitution level k: ym1 = y at half position -1 (previous row's tail),
    // yfar = y at half position -1 - 2h (previous row's, or two rows back for h = M/2).
    template <class U>
    __device__ __forceinline__ static void backsub(U&& u, int h, float ck, float dk, float ym1, float yfar) {
#pragma unroll
        for (int g = 0; g < M; g += 2 * h) {
            const int d = g + h - 1;
            const float a1 = u[g > 0 ? g - 1 : 0];
            const float a3 = u[g >= 4 * h ? g - 1 - 2 * h : 0];
            const float y1 = (g == 0) ? ym1 : a1;
            const float y3 = (g == 0) ? yfar : ((g == 2 * h) ? ym1 : a3);
            u[d] = fmaf(-dk, y3, fmaf(-ck, y1, u[d]));
        }
    }
};

}  // namespace iirgb

namespace iirgb {

constexpr int ilog2_c(int v) { return v <= 1 ? 0 : 1 + ilog2_c(v / 2); }

// STCR (SPLIT = false): one thread per row holds both parity halves.
// DTCR (SPLIT = true): the two halves of a row run on two neighbouring lanes (dim3(B, 2) in
// the reference, dtcr_kernels.cuh:56), interleaved so a row's pair shares a warp.
//
// A tile is BLOCK_SIZE = B rows, the reference's cyclic-reduction unit (its thread block):
// WT = B * TPR / 32 warps. Each tile is solved zero-padded (zero state before the tile): the
// cross-row values of the elimination, the top-level scan and the back-substitution move by
// warp shuffles inside a warp and, when the tile spans several warps (STCR at B = 64, DTCR at
// B = 32 and 64, like the reference's two-warp tiles with their neighbour exchange,
// stcr_kernels.cuh:2674-2706, dtcr_kernels.cuh:2625-2636), from the last row of one warp to the
// first row of the next through shared memory, one barrier among the row warps per level.
// Tiles are then joined like chunks: tile t's true incoming state is
// S_t = C^(B t) X + sum_{v<t} C^(B (t-1-v)) P_v (P_v = tile v's zero-state end pair,
// X = the chunk's incoming state from the lookback), and every row adds the response of the
// section recurrence to its own incoming pair C^(row in tile) S_t.
template <bool SPLIT, int B_, int N_, int ROWS_, bool UNROLL, bool PLANES = true, bool TAIL = false>
struct CrBlock {
    static constexpr int B = B_, N = N_, ROWS = ROWS_, M = N_ / 2, L = ilog2_c(N_);
    static constexpr int TPR = SPLIT ? 2 : 1;   // threads per row
    static constexpr int NPAR = SPLIT ? 1 : 2;  // parity halves per thread
    static constexpr int RW = 32 / TPR;         // rows per warp (tile)
    static constexpr int NW = ROWS * TPR / 32;  // row warps
    static constexpr int THREADS = 32 + NW * 32;
    static_assert(ROWS % RW == 0 && NW <= 16 && ROWS <= IIR_MAX_ROWS, "rows per chunk");
    static constexpr int TW = B;               // rows per tile (BLOCK_SIZE)
    static constexpr int WT = TW * TPR / 32;   // warps per tile
    static constexpr int NT = NW / WT;         // tiles per chunk
    static_assert(WT >= 1 && NW % WT == 0 && TW <= 32 * WT, "whole tiles of whole warps per chunk");
    static_assert(WT == 1 || NT <= 14, "a named barrier per tile (ids 2..15)");
    using Half = CrHalf<M>;
    static constexpr size_t SMEM_BYTES = BlockGeom<ROWS, N>::SMEM_BYTES;
    // occupancy target: both forms keep NPAR * M values per thread in registers
    static constexpr int REGS_WANTED = NPAR * M + 48;
    static constexpr int MIN_BLOCKS_REGS = 65536 / (THREADS * (REGS_WANTED < 64 ? 64 : REGS_WANTED));
    static constexpr int MIN_BLOCKS = min_blocks_for(SMEM_BYTES, THREADS) < MIN_BLOCKS_REGS
                                          ? min_blocks_for(SMEM_BYTES, THREADS)
                                          : (MIN_BLOCKS_REGS < 1 ? 1 : MIN_BLOCKS_REGS);

    __device__ static void run(const IirParams& p, unsigned char* smem) {
        float* buf = chunk_buffer<ROWS, N>(smem);
        BlockAux* aux = block_aux<ROWS, N>(smem);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (warp == 0) block_begin<ROWS, N>(p, buf, aux);
        __syncthreads();
        const uint32_t c = aux->chunk, epoch = aux->epoch;
        if (!block_acquire<ROWS, N, THREADS>(p, buf, aux, c, epoch)) return;
        const bool ok = filter_block(p, buf, aux, c, epoch, warp, lane);
        __syncthreads();
        if (ok) block_store<ROWS, N, THREADS>(p, buf, c);
    }

    // A row's halves in registers (compile-time indices keep them there).
    struct Row {
        float v[NPAR][M];
        __device__ __forceinline__ auto operator[](int hh) -> float (&)[M] { return v[hh]; }
    };

    // Where a row sits: rl = row in its warp, jw = warp in its tile, w = row warp in the block,
    // p0 = first parity it holds; and the shared memory that carries a tile's cross-warp terms.
    struct TilePos {
        int rl, jw, w, p0, tt;  // ... and tt = the tile of the chunk
        float* xch;          // [2][16][2]: alternating per-level buffers, [warp][parity or half]
        float* xscan;        // [16][2][2]: top-level scan totals, [warp][parity or half][pair]
        const float4* gpow;  // G^(t+1), t < 32 (top-level companion powers)
        int tog;
        __device__ __forceinline__ bool tile_first_row() const { return rl == 0 && jw == 0; }
    };

    // Barrier among the warps of tile tt only (named barrier 2 + tt): the tiles of a chunk do not
    // wait for each other.
    __device__ __forceinline__ static void tile_barrier(int tt) {
        asm volatile("bar.sync %0, %1;" ::"r"(2 + tt), "r"(WT * 32) : "memory");
    }

    // The previous row's value (same parity) of each half in v, within the tile: shuffled inside
    // the warp, passed from the previous warp of the tile through shared memory, zero before the
    // tile's first row. Every row thread of the tile takes part (one barrier when WT > 1).
    __device__ __forceinline__ static void prev_rows(const float (&v)[NPAR], float (&o)[NPAR], TilePos& t) {
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) o[hh] = __shfl_up_sync(FULL_MASK, v[hh], TPR);
        if constexpr (WT > 1) {
            float* slot = t.xch + (t.tog & 1) * 32;
            if (t.rl == RW - 1) {
#pragma unroll
                for (int hh = 0; hh < NPAR; ++hh) slot[t.w * 2 + (SPLIT ? t.p0 : hh)] = v[hh];
            }
            tile_barrier(t.tt);
            if (t.rl == 0 && t.jw > 0) {
#pragma unroll
                for (int hh = 0; hh < NPAR; ++hh) o[hh] = slot[(t.w - 1) * 2 + (SPLIT ? t.p0 : hh)];
            }
            t.tog ^= 1;
        }
        if (t.tile_first_row()) {
#pragma unroll
            for (int hh = 0; hh < NPAR; ++hh) o[hh] = 0.f;
        }
    }

    // Top-level scan of a tile that spans several warps: each warp's scan started from zero;
    // warp jw adds G^(rl+1) times the tile's state after its earlier warps.
    __device__ __forceinline__ static void tile_scan_join(float (&s0)[NPAR], float (&s1)[NPAR], TilePos& t) {
        if constexpr (WT > 1) {
            if (t.rl == RW - 1) {
#pragma unroll
                for (int hh = 0; hh < NPAR; ++hh) {
                    const int k = t.w * 2 + (SPLIT ? t.p0 : hh);
                    t.xscan[2 * k] = s0[hh];
                    t.xscan[2 * k + 1] = s1[hh];
                }
            }
            tile_barrier(t.tt);
            if (t.jw > 0) {
                const float4 Gw = t.gpow[RW - 1];  // G^RW across one warp's rows
                const float4 Gr = t.gpow[t.rl];    // G^(rl+1)
#pragma unroll
                for (int hh = 0; hh < NPAR; ++hh) {
                    float i0 = 0.f, i1 = 0.f;
                    for (int v = t.w - t.jw; v < t.w; ++v) {
                        float n0, n1;
                        mv2(Gw, i0, i1, n0, n1);
                        const int k = v * 2 + (SPLIT ? t.p0 : hh);
                        i0 = n0 + t.xscan[2 * k];
                        i1 = n1 + t.xscan[2 * k + 1];
                    }
                    float e0, e1;
                    mv2(Gr, i0, i1, e0, e1);
                    s0[hh] += e0;
                    s1[hh] += e1;
                }
            }
        }
    }

    // Elimination level K (half-stride 2^(K-1)) of this thread's parity halves.
    template <int K, class UA>
    __device__ __forceinline__ static void eliminate_level(UA&& u, const IirSection& q, TilePos& t) {
        constexpr int h = 1 << (K - 1);
        float v[NPAR], prev[NPAR];
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) v[hh] = u[hh][M - 1];
        prev_rows(v, prev, t);
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) Half::eliminate(u[hh], h, q.cr_r[K], q.cr_e[K], prev[hh]);
    }
    // Back-substitution level K; s0 = each half's top-level y at half position -1.
    template <int K, class UA>
    __device__ __forceinline__ static void backsub_level(UA&& u, const IirSection& q, TilePos& t, const float* s0) {
        constexpr int h = 1 << (K - 1);
        // y at half position -1 - 2h: the previous row's, or two rows back at the top
        float v[NPAR], far[NPAR];
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) v[hh] = (2 * h == M) ? s0[hh] : u[hh][M - 1 - 2 * h];
        prev_rows(v, far, t);
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) Half::backsub(u[hh], h, q.cr_c[K], q.cr_d[K], s0[hh], far[hh]);
    }
    // Straight-line form: levels 1 .. L-1, then L-1 .. 1.
    template <class UA, int... I>
    __device__ __forceinline__ static void eliminate_levels(UA&& u, const IirSection& q, TilePos& t,
                                                            std::integer_sequence<int, I...>) {
        (eliminate_level<I + 1>(u, q, t), ...);
    }
    template <class UA, int... I>
    __device__ __forceinline__ static void backsub_levels(UA&& u, const IirSection& q, TilePos& t, const float* s0,
                                                          std::integer_sequence<int, I...>) {
        (backsub_level<L - 1 - I>(u, q, t, s0), ...);
    }
    // Loop form: one iteration of the run-time level loop (levels 1 .. 6 for rows of up to 128).
    template <bool ELIM, class UA>
    __device__ __forceinline__ static void level_dispatch(int k, UA&& u, const IirSection& q, TilePos& t,
                                                          const float* s0) {
        switch (k) {
#define IIR_CR_LEVEL(K)                                             \
    case K:                                                         \
        if constexpr (K < L) {                                      \
            if constexpr (ELIM) eliminate_level<K>(u, q, t);        \
            else backsub_level<K>(u, q, t, s0);                     \
        }                                                           \
        break;
            IIR_CR_LEVEL(1)
            IIR_CR_LEVEL(2)
            IIR_CR_LEVEL(3)
            IIR_CR_LEVEL(4)
            IIR_CR_LEVEL(5)
            IIR_CR_LEVEL(6)
#undef IIR_CR_LEVEL
            default: break;
        }
    }

    // Zero-padded tile solve of one section for this thread's row (parity halves): FIR +
    // first double-sided round, elimination levels, top-level scan across the tile's rows,
    // back-substitution. (P0, P1) = the tile's zero-state end pair (valid in its last row).
    // Xp0/Xp1: the previous section's incoming state (row-0 input history for sec > 0).
    // h2, h1: the two input samples before the chunk (row 0's history in section 0).
    // (Y2, Y1) = (y[-2], y[-1]) before the tile's first row: zero for the zero-padded tile; a
    // known incoming pair enters the stride-2 system through its first four right-hand sides
    //     v[0] = y[0],  v[1] = y[1],  v[2] -= f_1 y[-2],  v[3] -= f_1 y[-1]
    // (y[0], y[1] from the section recurrence), after which the zero-padded solve returns the
    // true output of the tile.
    // u: the row's halves, float[NPAR][M] in registers; buf is only read.
    template <class UA>
    __device__ __forceinline__ static void solve_tile(const IirParams& p, const float* buf, const IirSection& q, int sec,
                                                      float h2, float h1, int r, TilePos& t, float Xp0, float Xp1,
                                                      float Y2, float Y1, UA&& u, float& P0, float& P1) {
        const int p0 = t.p0;
        float s0[NPAR], s1[NPAR];
        // ---- FIR + first double-sided round -> u (own parity halves) ----
        const float g = (sec == 0) ? p.gain : 1.f;
        if (SPLIT) {
            // One lane per parity: v1[n] = g (x[n] + fir5 . (x[n-1], .., x[n-4])) only at its own
            // parities n = 2m + p0, as six taps over x[2m-4 .. 2m+1] whose coefficients depend on
            // the lane only (no per-sample selects).
            float m4, m3, m2, m1;  // raw x[-4], x[-3], x[-2], x[-1] of this row
            if (r > 0) {
                m4 = buf[swz<N, ROWS, PLANES>(r - 1, N - 4)];
                m3 = buf[swz<N, ROWS, PLANES>(r - 1, N - 3)];
                m2 = buf[swz<N, ROWS, PLANES>(r - 1, N - 2)];
                m1 = buf[swz<N, ROWS, PLANES>(r - 1, N - 1)];
            } else {
                m4 = m3 = 0.f;
                m2 = (sec == 0) ? h2 : Xp0;
                m1 = (sec == 0) ? h1 : Xp1;
            }
            const float c0 = g, c1 = g * q.fir5[0], c2 = g * q.fir5[1], c3 = g * q.fir5[2], c4 = g * q.fir5[3];
            const float d0 = p0 ? 0.f : c4, d1 = p0 ? c4 : c3, d2 = p0 ? c3 : c2, d3 = p0 ? c2 : c1,
                        d4 = p0 ? c1 : c0, d5 = p0 ? c0 : 0.f;
            const float xm2 = m2, xm1 = m1;
            float xr0 = 0.f, xr1 = 0.f;  // raw x[0], x[1] of the row
#pragma unroll
            for (int j = 0; j < N / 4; ++j) {
                const float4 v4 = *reinterpret_cast<const float4*>(buf + swz<N, ROWS, PLANES>(r, 4 * j));
                if (j == 0) {
                    xr0 = v4.x;
                    xr1 = v4.y;
                }
                u[0][2 * j] = fmaf(d5, v4.y, fmaf(d4, v4.x, fmaf(d3, m1, fmaf(d2, m2, fmaf(d1, m3, d0 * m4)))));
                u[0][2 * j + 1] =
                    fmaf(d5, v4.w, fmaf(d4, v4.z, fmaf(d3, v4.y, fmaf(d2, v4.x, fmaf(d1, m1, d0 * m2)))));
                m4 = v4.x;
                m3 = v4.y;
                m2 = v4.z;
                m1 = v4.w;
            }
            if (t.tile_first_row()) {
                // first row of the tile: y[0] = w[0] + a1 y[-1] + a2 y[-2], y[1] = w[1] + a1 y[0] + a2 y[-1]
                // (v[0], v[1] of the system that is zero before the tile), and f_1 y[n-4] moved out of
                // v[2], v[3]
                const float w0 = g * fmaf(q.b2, xm2, fmaf(q.b1, xm1, xr0));
                const float w1 = g * fmaf(q.b2, xm1, fmaf(q.b1, xr0, xr1));
                const float y0 = fmaf(q.a1, Y1, fmaf(q.a2, Y2, w0));
                const float y1 = fmaf(q.a1, y0, fmaf(q.a2, Y1, w1));
                u[0][0] = p0 ? y1 : y0;
                u[0][1] = fmaf(q.ha2, p0 ? Y1 : Y2, u[0][1]);
            }
        } else {
            float x1, x2, x3, x4;  // x[-1], x[-2], x[-3], x[-4] of this row
            if (r > 0) {
                x4 = buf[swz<N, ROWS, PLANES>(r - 1, N - 4)] * g;
                x3 = buf[swz<N, ROWS, PLANES>(r - 1, N - 3)] * g;
                x2 = buf[swz<N, ROWS, PLANES>(r - 1, N - 2)] * g;
                x1 = buf[swz<N, ROWS, PLANES>(r - 1, N - 1)] * g;
            } else if (sec == 0) {
                x4 = x3 = 0.f;
                x2 = h2 * g;
                x1 = h1 * g;
            } else {
                x4 = x3 = 0.f;
                x2 = Xp0;
                x1 = Xp1;
            }
            const float b1 = q.b1, b2 = q.b2, e = q.e0, f = q.f0;
            // w[-2], w[-1]: zero before the tile (zero-padded system), else the FIR
            const bool first = t.tile_first_row();
            float w2 = !first ? fmaf(b2, x4, fmaf(b1, x3, x2)) : 0.f;
            float w1 = !first ? fmaf(b2, x3, fmaf(b1, x2, x1)) : 0.f;
#pragma unroll
            for (int j = 0; j < N / 4; ++j) {
                const float4 v4 = *reinterpret_cast<const float4*>(buf + swz<N, ROWS, PLANES>(r, 4 * j));
                const float xs[4] = {v4.x * g, v4.y * g, v4.z * g, v4.w * g};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int n = 4 * j + k;
                    const float wn = fmaf(b2, x2, fmaf(b1, x1, xs[k]));
                    u[n & 1][n >> 1] = fmaf(f, w2, fmaf(-e, w1, wn));
                    x2 = x1;
                    x1 = xs[k];
                    w2 = w1;
                    w1 = wn;
                }
            }
            if (first) {
                // first row of the tile: v[0] = y[0], v[1] = y[1] and f_1 y[n-4] moved out of v[2], v[3]
                // (the loop above left v[0] = w[0], v[1] = w[1] + a1 w[0])
                const float dy0 = fmaf(q.a1, Y1, q.a2 * Y2);
                u[0][0] += dy0;
                u[1][0] = fmaf(q.a1, dy0, fmaf(q.a2, Y1, u[1][0]));
                u[0][1] = fmaf(q.ha2, Y2, u[0][1]);
                u[1][1] = fmaf(q.ha2, Y1, u[1][1]);
            }
        }
        // ---- elimination levels 1 .. L-1 (previous row's kept tail by shuffle) ----
        if constexpr (UNROLL) {
            eliminate_levels(u, q, t, std::make_integer_sequence<int, L - 1>{});
        } else {
#pragma unroll 1
            for (int k = 1; k < L; ++k) level_dispatch<true>(k, u, q, t, s0);
        }
        // ---- top level across the tile's rows: Y_t + e_L Y_{t-1} + f_L Y_{t-2} = V_t ----
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) {
            s0[hh] = 0.f;
            s1[hh] = u[hh][M - 1];
            warp_scan2<RW, TPR>(s0[hh], s1[hh], q.M, t.rl);
        }
        tile_scan_join(s0, s1, t);
#pragma unroll
        for (int hh = 0; hh < NPAR; ++hh) u[hh][M - 1] = s1[hh];
        // ---- back-substitution L-1 .. 1 (zero-padded tile) ----
        if constexpr (UNROLL) {
            backsub_levels(u, q, t, s0, std::make_integer_sequence<int, L - 1>{});
        } else {
#pragma unroll 1
            for (int k = L - 1; k >= 1; --k) level_dispatch<false>(k, u, q, t, s0);
        }
        // tile end pair (y[N-2], y[N-1]) of the last row
        if (SPLIT) {
            const float mine = u[0][M - 1];
            const float other = __shfl_xor_sync(FULL_MASK, mine, 1);
            P0 = p0 ? other : mine;
            P1 = p0 ? mine : other;
        } else {
            P0 = u[0][M - 1];
            P1 = u[1][M - 1];
        }
    }

    // u += response of the section recurrence to the row's incoming pair (d2, d1) =
    // (delta[-2], delta[-1]). DTCR: each parity runs the stride-2 recurrence of its half.
    template <class UA>
    __device__ __forceinline__ static void add_response(UA&& u, const IirSection& q, int p0, float d2, float d1) {
        const float a1 = q.a1, a2 = q.a2;
        if (SPLIT) {
            // stride-2 recurrence of this parity: delta[2m+p] from (delta[p], delta[p+2])
            const float e0s = fmaf(a1, d1, a2 * d2);    // delta[0]
            const float e1s = fmaf(a1, e0s, a2 * d1);   // delta[1]
            const float e2s = fmaf(a1, e1s, a2 * e0s);  // delta[2]
            const float e3s = fmaf(a1, e2s, a2 * e1s);  // delta[3]
            float dm2 = p0 ? e1s : e0s, dm1 = p0 ? e3s : e2s;
            const float al1 = q.ha1, al2 = q.ha2;  // -e_1, -f_1
            u[0][0] += dm2;
            u[0][1] += dm1;
#pragma unroll
            for (int m = 2; m < M; ++m) {
                const float dn = fmaf(al1, dm1, al2 * dm2);
                dm2 = dm1;
                dm1 = dn;
                u[0][m] += dn;
            }
        } else {
#pragma unroll
            for (int n = 0; n < N; ++n) {
                const float dn = fmaf(a1, d1, a2 * d2);
                d2 = d1;
                d1 = dn;
                u[n & 1][n >> 1] += dn;
            }
        }
    }

    // Row r from this thread's halves into the swizzled buffer (DTCR: each lane stores its own
    // parity's samples).
    template <class UA>
    __device__ __forceinline__ static void write_row(float* buf, UA&& u, int r, int p0) {
        if (SPLIT) {
            // The row's lane pair holds the even (p0 = 0) and odd (p0 = 1) samples. Float4 j is
            // (e[2j], o[2j], e[2j+1], o[2j+1]); the even lane stores the even j, the odd lane the
            // odd j. For each pair (j, j+1) each lane sends the two values its partner needs:
            // the even lane e[2j+2], e[2j+3], the odd lane o[2j], o[2j+1].
#pragma unroll
            for (int j = 0; j < N / 4; j += 2) {
                const float s0 = p0 ? u[0][2 * j] : u[0][2 * j + 2];
                const float s1 = p0 ? u[0][2 * j + 1] : u[0][2 * j + 3];
                const float r0 = __shfl_xor_sync(FULL_MASK, s0, 1);
                const float r1 = __shfl_xor_sync(FULL_MASK, s1, 1);
                const int jj = j + p0;  // the float4 this lane stores
                const float4 v = p0 ? make_float4(r0, u[0][2 * j + 2], r1, u[0][2 * j + 3])
                                    : make_float4(u[0][2 * j], r0, u[0][2 * j + 1], r1);
                *reinterpret_cast<float4*>(buf + swz<N, ROWS, PLANES>(r, 4 * jj)) = v;
            }
        } else {
#pragma unroll
            for (int j = 0; j < N / 4; ++j)
                *reinterpret_cast<float4*>(buf + swz<N, ROWS, PLANES>(r, 4 * j)) =
                    make_float4(u[0][2 * j], u[1][2 * j], u[0][2 * j + 1], u[1][2 * j + 1]);
        }
    }

    __device__ static bool filter_block(const IirParams& p, float* buf, BlockAux* aux, uint32_t c, uint32_t epoch,
                                        int warp, int lane) {
        const bool row_warp = warp > 0;
        if constexpr (TAIL) {
            bool ok = true;
            if (!tail_begin<N, ROWS, PLANES>(p, buf, aux, c, epoch, warp, ok)) return ok;  // control warp
        }
        const int w = warp - 1;
        const int rl = SPLIT ? (lane >> 1) : lane;  // row within the warp
        const int r = w * RW + rl;                    // row within the chunk
        const int p0 = SPLIT ? (lane & 1) : 0;        // first parity handled
        const int tt = w / WT, jw = w % WT;           // tile of the chunk, warp within the tile
        const int rlt = jw * RW + rl;                 // row within the tile
        typename CrBlock::Row u;  // (register form: written by the first solve before any read)
        float Xp0 = 0.f, Xp1 = 0.f;  // previous section's incoming state (row-0 input history)
        float h2 = 0.f, h1 = 0.f;    // input samples before the chunk
        if (row_warp && r == 0 && c > 0) {
            const long long cs = static_cast<long long>(c) * (ROWS * N);
            h2 = __ldg(p.x + cs - 2);
            h1 = __ldg(p.x + cs - 1);
        }
        for (int sec = 0; sec < p.n_sections; ++sec) {
            const IirSection& q = p.sec[sec];
            const float4* tab = p.tables + sec * IIR_TAB_STRIDE;
            const float4 Ct = tab[IIR_TAB_CPOW + TW - 1];  // tile transition C^B
            float P0 = 0.f, P1 = 0.f;  // tile zero-state end pair (valid in the tile's last row)
            if (row_warp) {
                TilePos tp{rl, jw, w, p0, tt, &aux->xch[0][0][0], &aux->xscan[0][0][0], tab + IIR_TAB_GPOW, 0};
                solve_tile(p, buf, q, sec, h2, h1, r, tp, Xp0, Xp1, 0.f, 0.f, u, P0, P1);
                if (lane == 31 && jw == WT - 1) {
                    aux->wtot[tt][TAIL ? (sec & 1) : 0][0] = P0;
                    aux->wtot[tt][TAIL ? (sec & 1) : 0][1] = P1;
                }
            }
            if (!TAIL || sec == 0) __syncthreads();  // (A)
            else named_barrier_rows(NW);
            float in0 = 0.f, in1 = 0.f;  // zero-state incoming pair of this tile
            if (row_warp) {
                warp_incoming(aux, tt, TAIL ? (sec & 1) : 0, Ct, in0, in1);
            } else if (!TAIL) {
                control_section<NT, 1>(p, aux, sec, c, epoch, tab, Ct);
            }
            if (!TAIL) __syncthreads();  // (B)
            if (aux->bail) return false;
            const float X0 = TAIL ? aux->Xs[sec][0] : aux->X[0], X1 = TAIL ? aux->Xs[sec][1] : aux->X[1];
            if (row_warp) {
                // true incoming pair of the tile, then of this row
                float S0 = X0, S1 = X1;
                if (tt > 0) {
                    float t0, t1;
                    mv2(tab[IIR_TAB_CPOW + TW * tt - 1], X0, X1, t0, t1);
                    S0 = t0 + in0;
                    S1 = t1 + in1;
                }
                float d2 = S0, d1 = S1;  // (delta[-2], delta[-1]) at the row start
                if (rlt > 0) mv2(tab[IIR_TAB_CPOW + rlt - 1], S0, S1, d2, d1);
                add_response(u, q, p0, d2, d1);
                write_row(buf, u, r, p0);
                Xp0 = X0;
                Xp1 = X1;
                named_barrier_rows(NW);  // rows written before the next section reads histories
            }
        }
        if (row_warp) fence_proxy_async_smem();
        return true;
    }
};


// Single-section STCR / DTCR on the two-pass pipeline (iir_twopass.cuh): pass B is CrBlock's
// tile solve with the tile's true incoming pair known from the start. Pass A left every row's
// zero-state incoming pair (zin), so tile w starts from S_w = zin[RW w] + C^(RW w) X; the solve
// takes S_w in its first row's right-hand sides and returns the true output, which each row
// writes once (no tile join, no response added afterwards).
template <bool SPLIT, int B, int N_, int ROWS_, bool UNROLL>
struct CrTwo {
    using Blk = CrBlock<SPLIT, B, N_, ROWS_, UNROLL, two_planes(N_)>;
    static constexpr int N = N_, ROWS = ROWS_, M = Blk::M, NPAR = Blk::NPAR, RW = Blk::RW, NW = Blk::NW;
    static constexpr int TPR = Blk::TPR, TW = Blk::TW, WT = Blk::WT;

    __device__ static void b_pass(const IirParams& p, float* buf, const float* hist, const float4* tc,
                                  const float (*zin)[2], PipeAux* aux, float X0, float X1, int w, int lane) {
        using G = PipeGeom<ROWS, N, 2>;
        const int rl = SPLIT ? (lane >> 1) : lane;
        const int r = w * RW + rl;
        const int p0 = SPLIT ? (lane & 1) : 0;
        const int tt = w / WT, jw = w % WT;  // tile of the chunk, warp within the tile
        const IirSection& q = p.sec[0];
        float S0 = X0, S1 = X1;  // (y[-2], y[-1]) before the tile's first row
        if (tt > 0) {
            float t0, t1;
            mv2(tc[TW * tt - 1], X0, X1, t0, t1);  // C^(B t)
            S0 = t0 + zin[TW * tt][0];
            S1 = t1 + zin[TW * tt][1];
        }
        typename Blk::Row u;
        float P0, P1;
        typename Blk::TilePos tp{rl, jw, w, p0, tt, &aux->xch[0][0][0], &aux->xscan[0][0][0], tc + G::TC_GPOW, 0};
        Blk::solve_tile(p, buf, q, 0, hist[30], hist[31], r, tp, 0.f, 0.f, S0, S1, u, P0, P1);
        named_barrier_rows(NW);  // every row has read its input history
        Blk::write_row(buf, u, r, p0);
    }
};

}  // namespace iirgb
