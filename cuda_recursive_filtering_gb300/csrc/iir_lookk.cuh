// iir_lookk.cuh — two-level decoupled lookback for a K-dimensional carry (K <= 16), used by
// the PLR direct-form realization (state = the last K outputs). Same protocol as the 2-state
// version in iir_device.cuh: per chunk (and per group of 32 chunks) a slot of 2K words
//   [0, K) part words, [K, 2K) full words, each (flag << 32) | float bits,
// part_flag = 2*epoch+1, full_flag = 2*epoch+2 (reference: plr_kernels.cuh:813-887 with
// partcarry / fullcarry[chunk * order + i] and one status word per chunk).
// Composition: X = Phi^(j-1-f) full(f) + sum Phi^(j-1-i) part(i) inside the group, or
// X = Phi^j Xg + sum_{i<j} Phi^(j-1-i) part(i) with Xg from the group slots (Phi^32 powers).
// Matrices (K x K, row-major) live in global memory: Pc[l] = Phi^l, Pg[l] = Phi^(32 l), l <= 32.
#pragma once
#include "iir_device.cuh"

namespace iirgb {

template <int K>
struct VecK {
    float v[K];
};

// y = M x (K x K row-major matrix in global memory)
template <int K>
__device__ __forceinline__ void matvec(const float* __restrict__ M, const float (&x)[K], float (&y)[K]) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
        float a = 0.f;
#pragma unroll
        for (int j = 0; j < K; ++j) a = fmaf(__ldg(M + i * K + j), x[j], a);
        y[i] = a;
    }
}

template <int K>
__device__ __forceinline__ void publishk(unsigned long long* slot, uint32_t flag, const float (&v)[K]) {
#pragma unroll
    for (int i = 0; i < K; i += 2) st_relaxed_v2(slot + i, pack_word(flag, v[i]), pack_word(flag, v[i + 1]));
}

// Reads part / full words of one slot. ok flags are true only if every word carries the flag.
template <int K>
__device__ __forceinline__ void read_slotk(const unsigned long long* s, uint32_t pf, uint32_t ff, bool& part,
                                           bool& full, float (&pv)[K], float (&fv)[K]) {
    part = true;
    full = true;
#pragma unroll
    for (int i = 0; i < K; i += 2) {
        unsigned long long a, b, c2, d;
        ld_relaxed_v2(s + i, a, b);
        ld_relaxed_v2(s + K + i, c2, d);
        part = part && word_flag(a) == pf && word_flag(b) == pf;
        full = full && word_flag(c2) == ff && word_flag(d) == ff;
        pv[i] = word_val(a);
        pv[i + 1] = word_val(b);
        fv[i] = word_val(c2);
        fv[i + 1] = word_val(d);
    }
}

template <int K>
__device__ __forceinline__ void warp_sumk(float (&v)[K]) {
#pragma unroll
    for (int i = 0; i < K; ++i) v[i] = warp_sum(v[i]);
}

// Truncated lookback (one full warp): when ||Phi^m|| <= 1e-10 (FP64, checked by the plan), the
// incoming state of chunk c is X = sum_{i < min(m, c)} Phi^i part(c - 1 - i) (zero state before
// the signal): lane i polls the part words of chunk c - 1 - i, and no chain of inclusive carries
// is needed.
template <int K, class P>
__device__ bool lookback_trunc_k(const P& p, const unsigned long long* slots, const float* Pc, uint32_t c,
                                 uint32_t epoch, int m, float (&X)[K]) {
    constexpr int SW = 2 * K;
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u;
    const bool mine = lane < m && static_cast<uint32_t>(lane) < c;
    float v[K];
#pragma unroll
    for (int i = 0; i < K; ++i) v[i] = 0.f;
    const uint64_t t_start = globaltimer_ns();
    uint32_t spin = 32;
    while (true) {
        bool ok = true;
        if (mine) {
            const unsigned long long* s = slots + static_cast<size_t>(c - 1 - lane) * SW;
#pragma unroll
            for (int i = 0; i < K; i += 2) {
                unsigned long long a, b;
                ld_relaxed_v2(s + i, a, b);
                ok = ok && word_flag(a) == pf && word_flag(b) == pf;
                v[i] = word_val(a);
                v[i + 1] = word_val(b);
            }
        }
        if (__all_sync(FULL_MASK, ok)) break;
        int give_up = 0;
        if (lane == 0) give_up = lookback_give_up(p, epoch, t_start) ? 1 : 0;
        if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
        backoff(spin);
    }
    float t[K];
    if (mine && lane > 0) {
        matvec<K>(Pc + static_cast<size_t>(lane) * K * K, v, t);  // Phi^lane part(c - 1 - lane)
    } else {
#pragma unroll
        for (int i = 0; i < K; ++i) t[i] = v[i];  // lane 0: Phi^0 = I (others: zero)
    }
    warp_sumk<K>(t);
#pragma unroll
    for (int i = 0; i < K; ++i) X[i] = t[i];
    return true;
}

// One full warp. own = this chunk's part (needed for the group aggregate of a group's last chunk).
template <int K, class P>
__device__ bool lookback_hier_k(const P& p, unsigned long long* slots, unsigned long long* gslots,
                                const float* Pc, const float* Pg, uint32_t c, uint32_t epoch, const float (&own)[K],
                                bool withhold, float (&X)[K]) {
    constexpr int SW = 2 * K;  // words per slot
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u, ff = 2u * epoch + 2u;
    const int j = static_cast<int>(c & 31u);
    const long long g = static_cast<long long>(c >> 5);
    const uint64_t t_start = globaltimer_ns();
    bool gpart_done = (j != 31) || withhold;
    uint32_t spin = 64;
    while (true) {
        bool cpart = false, cfull = false;
        float cp[K], cf[K];
#pragma unroll
        for (int i = 0; i < K; ++i) cp[i] = cf[i] = 0.f;
        if (lane < j) read_slotk<K>(slots + (static_cast<size_t>(g) * 32 + lane) * SW, pf, ff, cpart, cfull, cp, cf);
        bool gpart = true, gfull = true;
        float gp[K], gfv[K];
#pragma unroll
        for (int i = 0; i < K; ++i) gp[i] = gfv[i] = 0.f;
        const long long gm = g - 1 - lane;
        if (gm >= 0) read_slotk<K>(gslots + static_cast<size_t>(gm) * SW, pf, ff, gpart, gfull, gp, gfv);
        // group aggregate of a group's last chunk
        if (!gpart_done && __ballot_sync(FULL_MASK, lane < j && !cpart) == 0u) {
            float t[K];
            if (lane < j) matvec<K>(Pc + static_cast<size_t>(31 - lane) * K * K, cp, t);
            else
#pragma unroll
                for (int i = 0; i < K; ++i) t[i] = 0.f;
            warp_sumk<K>(t);
#pragma unroll
            for (int i = 0; i < K; ++i) t[i] += own[i];
            if (lane == 0) publishk<K>(gslots + static_cast<size_t>(g) * SW, pf, t);
            gpart_done = true;
        }
        const unsigned fm = __ballot_sync(FULL_MASK, lane < j && cfull);
        bool resolved = false;
        if (fm != 0u) {
            const int f = 31 - __clz(fm);
            if (__ballot_sync(FULL_MASK, lane > f && lane < j && !cpart) == 0u) {
                float t[K];
#pragma unroll
                for (int i = 0; i < K; ++i) t[i] = 0.f;
                if (lane >= f && lane < j) matvec<K>(Pc + static_cast<size_t>(j - 1 - lane) * K * K, lane == f ? cf : cp, t);
                warp_sumk<K>(t);
#pragma unroll
                for (int i = 0; i < K; ++i) X[i] = t[i];
                resolved = true;
            }
        } else {
            const unsigned nr = __ballot_sync(FULL_MASK, lane < j && !cpart);
            const unsigned gfm = __ballot_sync(FULL_MASK, gfull);
            const int h = gfm ? (__ffs(gfm) - 1) : 32;
            const unsigned gnr = __ballot_sync(FULL_MASK, lane < h && !gpart);
            if (nr == 0u && gnr == 0u && h < 32) {
                float t[K], xg[K];
#pragma unroll
                for (int i = 0; i < K; ++i) t[i] = 0.f;
                if (lane <= h) matvec<K>(Pg + static_cast<size_t>(lane) * K * K, lane == h ? gfv : gp, t);
                warp_sumk<K>(t);  // Xg
#pragma unroll
                for (int i = 0; i < K; ++i) xg[i] = t[i];
                matvec<K>(Pc + static_cast<size_t>(j) * K * K, xg, t);  // Phi^j Xg (all lanes alike)
                float u[K];
#pragma unroll
                for (int i = 0; i < K; ++i) u[i] = 0.f;
                if (lane < j) matvec<K>(Pc + static_cast<size_t>(j - 1 - lane) * K * K, cp, u);
                warp_sumk<K>(u);
#pragma unroll
                for (int i = 0; i < K; ++i) X[i] = t[i] + u[i];
                resolved = true;
            }
            // (h == 32: no group carry within 32 groups = 1024 chunks; the nearer groups
            //  publish theirs shortly, so keep polling)
        }
        if (resolved && gpart_done) return true;
        int give_up = 0;
        if (lane == 0) give_up = lookback_give_up(p, epoch, t_start) ? 1 : 0;
        if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
        backoff(spin);
        if (resolved) {
            // X is final; only the group aggregate is outstanding: poll for it alone
            float Xs[K];
#pragma unroll
            for (int i = 0; i < K; ++i) Xs[i] = X[i];
            while (!gpart_done) {
                bool cp2 = false, cf2 = false;
                float a[K], b[K];
#pragma unroll
                for (int i = 0; i < K; ++i) a[i] = b[i] = 0.f;
                if (lane < j) read_slotk<K>(slots + (static_cast<size_t>(g) * 32 + lane) * SW, pf, ff, cp2, cf2, a, b);
                if (__ballot_sync(FULL_MASK, lane < j && !cp2) == 0u) {
                    float t[K];
#pragma unroll
                    for (int i = 0; i < K; ++i) t[i] = 0.f;
                    if (lane < j) matvec<K>(Pc + static_cast<size_t>(31 - lane) * K * K, a, t);
                    warp_sumk<K>(t);
#pragma unroll
                    for (int i = 0; i < K; ++i) t[i] += own[i];
                    if (lane == 0) publishk<K>(gslots + static_cast<size_t>(g) * SW, pf, t);
                    gpart_done = true;
                    break;
                }
                int gu = 0;
                if (lane == 0) gu = lookback_give_up(p, epoch, t_start) ? 1 : 0;
                if (__shfl_sync(FULL_MASK, gu, 0)) return false;
                backoff(spin);
            }
#pragma unroll
            for (int i = 0; i < K; ++i) X[i] = Xs[i];
            return true;
        }
    }
}

}  // namespace iirgb
