// iir_tail.cuh — the tail-aggregate schedule of the cascade kernels.
//
// In the per-section schedule (iir_device.cuh: control_section), every section of a chunk
// publishes its zero-state aggregate only after its own filter pass and waits for its
// predecessor's, so a chunk of K sections makes K lookbacks, each between two block barriers,
// and chunk c's section s waits on chunk c-1's section s (which waited on c-2's section s-1, and
// so on). The reference has the same shape (one lookback per section, ph_kernels.cuh:384-469).
//
// When the cascade's state decays within a chunk, one lookback per chunk suffices. The planner
// finds, in FP64, the least number P of 512-sample pieces with ||Phi^(512 P)||_inf <= 1e-10,
// where Phi is the cascade's one-sample state transition (all sections' (y[n-2], y[n-1]),
// coupled through each section's FIR of its predecessor's output). Then
//   * the zero-state aggregate of chunk c (every section's end state, the reference's partcarry)
//     equals, to that bound, the cascade run over the chunk's last 512 P samples from rest (the
//     input history before them is kept, exactly);
//   * the incoming state of chunk c + 1 equals that aggregate: older chunks contribute Phi^L
//     times theirs, which is smaller still (L = the chunk length >= 1024 P).
//
// The tail is cut into P pieces of 32 lanes x 16 samples. At the start of the block every warp
// t < P computes piece t from rest with the PH algorithm on the staged chunk (each lane filters
// its samples from rest, applying the previous section's correction as it reads them, as
// PhBlock::filter_pass does; a warp scan with (A^16)^(2^k) joins the lane tails; each lane's true
// incoming pair feeds the next section), and leaves the piece's end state of every section.
// After one block barrier the row warps start their first section while the control warp joins
// the pieces, S = Phi^512 S + s_t (exact: each piece's zero-state end state plus the earlier
// pieces' state carried across it), publishes S for every section in the chunk's carry slots
// (the same launch-versioned flag|value words as the per-section lookback), reads chunk c - 1's
// and hands the incoming states of all sections to the row warps at the first section's join.
// The row warps then run their sections back to back, one barrier among themselves per section,
// with no wait on another block.
#pragma once
#include "iir_device.cuh"
#include "iir_twopass.cuh"

namespace iirgb {

constexpr int TAIL_LANE = IIR_TAIL_PIECE / 32;  // samples per lane of a tail piece

// One section over a lane's samples v[] from rest, applying the previous section's correction
// (recurrence pa1, pa2 from the lane's incoming pair (d2, d1)) to each input on the fly;
// (xh2, xh1) = the FIR history. Leaves the zero-state output in v and its tail in (s0, s1).
template <bool CORRECT>
__device__ __forceinline__ void tail_lane_pass(float (&v)[TAIL_LANE], float b1, float b2, float a1, float a2,
                                               float pa1, float pa2, float d2, float d1, float xh2, float xh1,
                                               float& s0, float& s1) {
    float y1 = 0.f, y2 = 0.f;
#pragma unroll
    for (int j = 0; j < TAIL_LANE; ++j) {
        float xv = v[j];
        if (CORRECT) {
            const float dn = fmaf(pa1, d1, pa2 * d2);
            d2 = d1;
            d1 = dn;
            xv += dn;
        }
        const float wv = fmaf(b2, xh2, fmaf(b1, xh1, xv));
        const float y = fmaf(a1, y1, fmaf(a2, y2, wv));
        xh2 = xh1;
        xh1 = xv;
        y2 = y1;
        y1 = y;
        v[j] = y;
    }
    s0 = y2;
    s1 = y1;
}

// The filter a tail piece runs: K sections (per-section scalars sec[s]), their lane tables
// (section s at tables + s * tab_stride, (A^16)^(l+1) at offset tail_off), the input gain.
struct TailFilter {
    const IirSection* sec;
    const float4* tables;
    int tab_stride, tail_off, K;
    float gain;
};

// Warp t of the block: the zero-state end state of every section over tail piece t (of
// `pieces`) of the chunk staged in buf (rows of N samples, swizzled layout swz<N, ROWS, PLANES>),
// into tp[t]. The staged chunk is only read.
template <int N, int ROWS, bool PLANES>
__device__ __forceinline__ void tail_piece(const TailFilter& f, int pieces, const float* buf,
                                           float (*tp)[IIR_MAX_SECTIONS][2], int t) {
    static_assert(N % TAIL_LANE == 0 || TAIL_LANE % N == 0, "a lane's samples in whole float4s of a row");
    const int lane = threadIdx.x & 31;
    const int K = f.K;
    const float g = f.gain;
    const int first = ROWS * N - pieces * IIR_TAIL_PIECE + t * IIR_TAIL_PIECE + lane * TAIL_LANE;
    float v[TAIL_LANE];
#pragma unroll
    for (int j = 0; j < TAIL_LANE / 4; ++j) {
        const int i = first + 4 * j;
        const float4 q4 = *reinterpret_cast<const float4*>(buf + swz<N, ROWS, PLANES>(i / N, i % N));
        v[4 * j] = q4.x * g;
        v[4 * j + 1] = q4.y * g;
        v[4 * j + 2] = q4.z * g;
        v[4 * j + 3] = q4.w * g;
    }
    // section 0's FIR history: the two input samples before the lane (exact; first >= 2)
    float xh2 = buf[swz<N, ROWS, PLANES>((first - 2) / N, (first - 2) % N)] * g;
    float xh1 = buf[swz<N, ROWS, PLANES>((first - 1) / N, (first - 1) % N)] * g;
    float pa1 = 0.f, pa2 = 0.f, d2 = 0.f, d1 = 0.f;
    for (int s = 0; s < K; ++s) {
        const IirSection& q = f.sec[s];
        const float4* tt = f.tables + static_cast<size_t>(s) * f.tab_stride + f.tail_off;  // (A^16)^(l+1)
        float s0, s1;
        if (s == 0)
            tail_lane_pass<false>(v, q.b1, q.b2, q.a1, q.a2, 0.f, 0.f, 0.f, 0.f, xh2, xh1, s0, s1);
        else
            tail_lane_pass<true>(v, q.b1, q.b2, q.a1, q.a2, pa1, pa2, d2, d1, xh2, xh1, s0, s1);
        warp_scan_rows<32, 1>(s0, s1, tt, lane);  // zero state before the piece: true tails
        float i0 = __shfl_up_sync(FULL_MASK, s0, 1);
        float i1 = __shfl_up_sync(FULL_MASK, s1, 1);
        if (lane == 0) {
            i0 = 0.f;
            i1 = 0.f;
        }
        if (lane == 31) {
            tp[t][s][0] = s0;
            tp[t][s][1] = s1;
        }
        // the next section's input is this section's output: its correction is applied by the
        // next pass, and its FIR history is this section's incoming pair
        pa1 = q.a1;
        pa2 = q.a2;
        d2 = i0;
        d1 = i1;
        xh2 = i0;
        xh1 = i1;
    }
}

// Control warp: joins the pieces tp[0..pieces) into the chunk's aggregate, S = Phi S + s_t with
// phi = Phi^512 row-major over the 2K-vector (y_0[-2], y_0[-1], y_1[-2], ...), and publishes
// section s's pair at slot + s * stride (the chunk's carry slot of that section), flag pf.
__device__ __forceinline__ void tail_join_publish(const float* phi, const float (*tp)[IIR_MAX_SECTIONS][2], int K,
                                                  int pieces, unsigned long long* slot, size_t stride, uint32_t pf) {
    const int lane = threadIdx.x & 31;
    const int D = 2 * K;
    const int i = lane < D ? lane : 0;
    float S = tp[0][i >> 1][i & 1];
    for (int t = 1; t < pieces; ++t) {
        float Sn = 0.f;
        for (int j = 0; j < D; ++j) Sn = fmaf(__ldg(phi + i * D + j), __shfl_sync(FULL_MASK, S, j), Sn);
        S = Sn + tp[t][i >> 1][i & 1];
    }
    const float a0 = __shfl_sync(FULL_MASK, S, (2 * lane) & 31);
    const float a1 = __shfl_sync(FULL_MASK, S, (2 * lane + 1) & 31);
    if (lane < K) publish2(slot + static_cast<size_t>(lane) * stride, pf, a0, a1);
}

// Control warp: section `lane`'s pair (X0, X1) from the slots slot + s * stride (the predecessor
// chunk's, flag pf), bounded by the launch's wait limit. false if the wait gave up.
template <class P>
__device__ __forceinline__ bool tail_poll(const P& p, const unsigned long long* slot, size_t stride, int K,
                                          uint32_t epoch, float& X0, float& X1) {
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u;
    const unsigned long long* mine = slot + static_cast<size_t>(lane) * stride;
    const uint64_t t_start = globaltimer_ns();
    uint32_t spin = 32;
    while (true) {
        bool got = true;
        if (lane < K) {
            unsigned long long a, b;
            ld_relaxed_v2(mine, a, b);
            got = word_flag(a) == pf && word_flag(b) == pf;
            X0 = word_val(a);
            X1 = word_val(b);
        }
        if (__all_sync(FULL_MASK, got)) return true;
        int give_up = 0;
        if (lane == 0) give_up = lookback_give_up(p, epoch, t_start) ? 1 : 0;
        if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
        backoff(spin);
    }
}

// Control warp of a tail-schedule block over chunk c, after the pieces are in aux (block
// barrier): joins and publishes the chunk's aggregate for every section (unless the chunk is the
// last, which has no successor), then resolves the incoming states X_s = aggregate of chunk
// c - 1 (rest for chunk 0), leaving them in aux->Xs with aux->bail. Phi^512 follows the
// sections' lane tables. Every wait is bounded by the plan's limit.
__device__ __forceinline__ bool tail_control(const IirParams& p, BlockAux* aux, uint32_t c, uint32_t epoch) {
    const int lane = threadIdx.x & 31;
    const int K = p.n_sections;
    const uint32_t pf = 2u * epoch + 1u;
    if (c + 1u < p.nchunks && static_cast<long long>(c) != p.withhold_chunk)
        tail_join_publish(reinterpret_cast<const float*>(p.tables + static_cast<size_t>(K) * IIR_TAB_STRIDE),
                          aux->tpiece, K, p.tail_pieces, p.carry + static_cast<size_t>(c) * 4, p.carry_stride, pf);
    float X0 = 0.f, X1 = 0.f;
    bool ok = true;
    if (c > 0) ok = tail_poll(p, p.carry + static_cast<size_t>(c - 1) * 4, p.carry_stride, K, epoch, X0, X1);
    if (lane < K) {
        aux->Xs[lane][0] = X0;
        aux->Xs[lane][1] = X1;
    }
    if (lane == 0) aux->bail = ok ? 0 : 1;
    return ok;
}

// The tail schedule's start of a block (all threads, after the chunk is staged): warps
// t < tail_pieces compute their piece (not for the last chunk, which has no successor), then a
// block barrier; the control warp then joins, publishes and looks back, and meets the row warps
// at their first section's join (its own __syncthreads). Returns false for the control warp
// (whose part ends here) after that barrier with the bail flag folded in; true for row warps.
template <int N, int ROWS, bool PLANES>
__device__ __forceinline__ bool tail_begin(const IirParams& p, const float* buf, BlockAux* aux, uint32_t c,
                                           uint32_t epoch, int warp, bool& ok) {
    if (c + 1u < p.nchunks && warp < p.tail_pieces) {
        const TailFilter f{p.sec, p.tables, IIR_TAB_STRIDE, IIR_TAB_TAIL, p.n_sections, p.gain};
        tail_piece<N, ROWS, PLANES>(f, p.tail_pieces, buf, aux->tpiece, warp);
    }
    __syncthreads();  // the pieces are in aux; the staged chunk may now be overwritten
    if (warp == 0) {
        tail_control(p, aux, c, epoch);
        __syncthreads();  // the first section's join: every section's incoming state is in aux
        ok = aux->bail == 0;
        return false;
    }
    return true;
}

}  // namespace iirgb
