// iir_device.cuh — sm_103a building blocks shared by every realization:
//   * inline-PTX wrappers for mbarrier, bulk async copies (TMA engine), proxy fences,
//     relaxed gpu-scope 64-bit accesses and %globaltimer;
//   * the launch-versioned, two-level decoupled lookback over flag|value words;
//   * the block driver (one TMA tensor load / store of a swizzled chunk per block).
//
// Reference protocol being replaced (include/ph_kernels.cuh:384-469): a chunk publishes
// partcarry, __threadfence(), sets status = part_flag; predecessors are polled through
// `volatile int` flags with an unbounded spin; carries are read after a second fence.
// Here each carry component is stored in the low half of a 64-bit word whose high half is
// the launch-versioned flag, so one relaxed 64-bit store publishes value and flag together
// (no fences), a reader validates every word it uses, chunks are grouped 32 to a group so a
// single poll sees both the chunk's own group and 32 preceding groups (the inclusive-carry
// frontier advances ~1024 chunks per round trip instead of 32), the composition is a
// parallel warp reduction with precomputed powers, and every wait is bounded.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "iir_params.h"

namespace iirgb {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Optional per-block accumulators for performance analysis (compiled in with -DIIR_PROFILE).
#define IIR_PROF_STRIDE 16
#ifdef IIR_PROFILE
#define IIR_PROF_ADD(p, slot, val)                                                                    \
    do {                                                                                              \
        if ((p).prof) (p).prof[static_cast<size_t>(blockIdx.x) * IIR_PROF_STRIDE + (slot)] += (val); \
    } while (0)
#else
#define IIR_PROF_ADD(p, slot, val) \
    do {                           \
    } while (0)
#endif

// ------------------------------------------------------------------------------------
// PTX wrappers
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// global -> shared bulk copy; completion is signalled on `bar` (transaction bytes)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// shared -> global bulk copy, tracked by this thread's bulk async-groups
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Asynchronous global -> shared copies that bypass registers (completion: cp_async_commit /
// cp_async_wait, then a barrier). cp_async16 wants both addresses 16-byte aligned. cp_async4
// copies `bytes` (4 or 0) of src and zero-fills the rest of the 4-byte destination; src must
// point into the source buffer even when nothing is read.
__device__ __forceinline__ void cp_async16(void* dst_smem, const void* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst_smem, const void* src, int bytes) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
// Four floats (16 bytes) to a 16-byte-aligned destination from a source aligned to 8 bytes
// (two 8-byte copies) or only to 4 (four 4-byte copies).
__device__ __forceinline__ void cp_async16_from8(void* dst_smem, const void* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
    asm volatile(
        "cp.async.ca.shared.global [%0], [%1], 8;\n\t"
        "cp.async.ca.shared.global [%0+8], [%1+8], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16_from4(void* dst_smem, const void* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
    asm volatile(
        "cp.async.ca.shared.global [%0], [%1], 4;\n\t"
        "cp.async.ca.shared.global [%0+4], [%1+4], 4;\n\t"
        "cp.async.ca.shared.global [%0+8], [%1+8], 4;\n\t"
        "cp.async.ca.shared.global [%0+12], [%1+12], 4;" ::"r"(d), "l"(src) : "memory");
}
// Bulk prefetch of [src, src + bytes) into L2 (one instruction, no completion to wait for):
// src 16-byte aligned, bytes a multiple of 16, the range inside the source buffer.
__device__ __forceinline__ void prefetch_l2_bulk(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory"); }
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void st_relaxed_v2(unsigned long long* p, unsigned long long a, unsigned long long b) {
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
__device__ __forceinline__ void ld_relaxed_v2(const unsigned long long* p, unsigned long long& a,
                                              unsigned long long& b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pack_word(uint32_t flag, float v) {
    return (static_cast<unsigned long long>(flag) << 32) | __float_as_uint(v);
}
__device__ __forceinline__ uint32_t word_flag(unsigned long long w) { return static_cast<uint32_t>(w >> 32); }
__device__ __forceinline__ float word_val(unsigned long long w) {
    return __uint_as_float(static_cast<uint32_t>(w & 0xffffffffull));
}

// ------------------------------------------------------------------------------------
// Launch state / errors
// ------------------------------------------------------------------------------------
__device__ __forceinline__ bool launch_failed(const IirLaunchState* st, uint32_t epoch) {
    const unsigned long long e = ld_relaxed_u64(&st->error);
    return e != 0ull && static_cast<uint32_t>(e >> 32) == epoch;
}
// Records a failure of launch `epoch`. The first failure of a launch is kept (it is the cause:
// a withheld carry times out its successors' lookbacks first, and their blocks' later waits
// give up after it); the word also goes to the host-mapped copy, if the plan has one.
__device__ __forceinline__ void raise_error(IirLaunchState* st, uint32_t epoch, uint32_t code) {
    const unsigned long long w = (static_cast<unsigned long long>(epoch) << 32) | code;
    unsigned long long cur = ld_relaxed_u64(&st->error);
    while (true) {
        if (cur != 0ull && static_cast<uint32_t>(cur >> 32) == epoch) return;  // already recorded
        const unsigned long long prev = atomicCAS(&st->error, cur, w);
        if (prev == cur) break;
        cur = prev;
    }
    unsigned long long* h = *reinterpret_cast<unsigned long long* volatile*>(&st->host_error);
    if (h) *reinterpret_cast<volatile unsigned long long*>(h) = w;  // seen by the host without a sync
}

// Takes the block's ticket: one atomic returns the launch epoch (high word) and the chunk
// id (low word). The block that draws the last chunk re-arms the counter for the next
// launch on the stream (every other block of this launch has already drawn its ticket).
__device__ __forceinline__ uint32_t take_ticket(IirLaunchState* st, uint32_t nchunks, uint32_t& epoch) {
    const unsigned long long old = atomicAdd(&st->ticket, 1ull);
    epoch = static_cast<uint32_t>(old >> 32);
    const uint32_t c = static_cast<uint32_t>(old & 0xffffffffull);
    if (c == nchunks - 1u) atomicExch(&st->ticket, static_cast<unsigned long long>(epoch + 1u) << 32);
    return c;
}

// Back-off between polls of a carry slot: a sleep of `cycles` / 2 ns, doubling up to
// IIR_BACKOFF_CAP / 2 ns. The warp sleeps rather than spins, so it takes no issue slots from the
// warps that compute. Every poll is an L2 round trip (several hundred ns) anyway; a short cap
// keeps the time between a predecessor's publish and its observation close to that (measured at
// 2^28 samples, PH 32x64 orders 4 / 8 / 16: 609 / 389 / 221 GS/s with a 512 ns cap, 621 / 400 /
// 228 with 32 ns).
#ifndef IIR_BACKOFF_CAP
#define IIR_BACKOFF_CAP 64u
#endif
__device__ __forceinline__ void backoff(uint32_t& cycles) {
    __nanosleep(cycles >> 1);
    if (cycles < IIR_BACKOFF_CAP) cycles <<= 1;
}

// Barrier among the row warps only (named barrier 1; the control warp is not involved).
__device__ __forceinline__ void named_barrier_rows(int row_warps) {
    asm volatile("bar.sync 1, %0;" ::"r"(row_warps * 32) : "memory");
}

// Waits for an mbarrier phase with a wall-clock bound (never hangs the device).
__device__ __forceinline__ bool wait_mbar_bounded(unsigned long long* bar, uint32_t parity, long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    uint32_t spins = 0;
    while (!mbar_try_wait(bar, parity)) {
        if ((++spins & 63u) == 0u && globaltimer_ns() - t0 > static_cast<uint64_t>(limit_ns)) return false;
    }
    return true;
}

// ------------------------------------------------------------------------------------
// 2x2 helpers (row-major float4 {m00, m01, m10, m11})
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void mv2(const float4 m, float v0, float v1, float& o0, float& o1) {
    o0 = fmaf(m.x, v0, m.y * v1);
    o1 = fmaf(m.z, v0, m.w * v1);
}
__device__ __forceinline__ float4 mm2(const float4 a, const float4 b) {
    return make_float4(fmaf(a.x, b.x, a.y * b.z), fmaf(a.x, b.y, a.y * b.w), fmaf(a.z, b.x, a.w * b.z),
                       fmaf(a.z, b.y, a.w * b.w));
}

// Kogge-Stone inclusive scan of the affine recurrence S_r = G S_{r-1} + s_r over the rows
// held by one warp (row index `row`, LANE_STRIDE lanes per row). Round k combines with
// G^(2^k) = M[k]. Zero state before the warp's first row.
template <int ROWS_IN_WARP, int LANE_STRIDE>
__device__ __forceinline__ void warp_scan2(float& s0, float& s1, const float (*M)[4], int row) {
#pragma unroll
    for (int k = 0; (1 << k) < ROWS_IN_WARP; ++k) {
        const int d = 1 << k;
        const float o0 = __shfl_up_sync(FULL_MASK, s0, d * LANE_STRIDE);
        const float o1 = __shfl_up_sync(FULL_MASK, s1, d * LANE_STRIDE);
        if (row >= d) {
            s0 = fmaf(M[k][0], o0, fmaf(M[k][1], o1, s0));
            s1 = fmaf(M[k][2], o0, fmaf(M[k][3], o1, s1));
        }
    }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

// ------------------------------------------------------------------------------------
// Carry slots. Per chunk (and per group of IIR_GROUP chunks), 32 bytes:
//   [0] part0  [1] part1  [2] full0  [3] full1    each word = (flag << 32) | float bits
// part = zero-state aggregate (the reference's partcarry), full = inclusive carry
// (fullcarry); part_flag = 2*epoch+1, full_flag = 2*epoch+2 (ph_kernels.cuh:16-24).
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void publish2(unsigned long long* slot, uint32_t flag, float v0, float v1) {
    st_relaxed_v2(slot, pack_word(flag, v0), pack_word(flag, v1));
}

struct SlotView {
    bool part, full;
    float p0, p1, f0, f1;
};
__device__ __forceinline__ SlotView read_slot(const unsigned long long* s, uint32_t pf, uint32_t ff) {
    unsigned long long w0, w1, w2, w3;
    ld_relaxed_v2(s, w0, w1);
    ld_relaxed_v2(s + 2, w2, w3);
    SlotView v;
    v.part = word_flag(w0) == pf && word_flag(w1) == pf;
    v.full = word_flag(w2) == ff && word_flag(w3) == ff;
    v.p0 = word_val(w0);
    v.p1 = word_val(w1);
    v.f0 = word_val(w2);
    v.f1 = word_val(w3);
    return v;
}

template <class P>
__device__ __forceinline__ bool lookback_give_up(const P& p, uint32_t epoch, uint64_t t_start) {
    if (launch_failed(p.state, epoch)) return true;
    if (globaltimer_ns() - t_start > static_cast<uint64_t>(p.timeout_ns)) {
        raise_error(p.state, epoch, IIR_DEV_ERR_TIMEOUT);
        return true;
    }
    return false;
}

// Two-level decoupled lookback (one full warp). Chunk c sits at position j = c % 32 of group
// g = c / 32. One poll reads the slots of the j preceding chunks of its own group (lane l:
// chunk 32g + l) and of the 32 preceding groups (lane l: group g - 1 - l).
//   * nearest inclusive carry inside the group at position f:
//       X = Q^(j-1-f) full(f) + sum_{f<i<j} Q^(j-1-i) part(i)
//   * otherwise, with all j partials present and group carries back to the nearest group
//     inclusive carry h (group -1 = zero state):
//       Xg = Qg^h gfull(g-1-h) + sum_{l<h} Qg^l gpart(g-1-l),  Qg = Q^32
//       X  = Q^j Xg + sum_{i<j} Q^(j-1-i) part(i)
// The last chunk of a group (j = 31) publishes the group aggregate
// gpart(g) = sum_{i<=31} Q^(31-i) part(i) as soon as its group's partials are visible; its
// own inclusive carry is the group's (published by the caller).
// Tables: Qc[l] = Q^l (l <= 32), Qg[l] = Q^(32 l) (l <= 32). (z0, z1) is the state before
// chunk 0 (the incoming state of a stream segment; zero for a signal that starts at rest).
// Truncated lookback (one warp) for a 2-state carry: X = sum_{i<m} Q^i part(c-1-i), chunks before
// the signal contributing nothing. The host sets m only when ||Q^m||_inf <= 1e-10 (FP64), so the
// neglected term Q^m X(c-m) is far below float32 resolution and a chunk waits for the aggregates
// of its m predecessors only, never for a chain of inclusive carries. Lane i polls chunk c-1-i.
// (z0, z1): the state before chunk 0 (a batched segment's initial state), whose term Q^c z is
// kept while c < m.
template <class P>
__device__ bool lookback_trunc2(const P& p, const unsigned long long* slots, const float4* Qc, uint32_t c,
                                uint32_t epoch, int m, float& X0, float& X1, float z0 = 0.f, float z1 = 0.f) {
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u;
    const bool mine = lane < m && static_cast<uint32_t>(lane) < c;
    float v0 = 0.f, v1 = 0.f;
    const uint64_t t_start = globaltimer_ns();
    uint32_t spin = 32;
    while (true) {
        bool ok = true;
        if (mine) {
            unsigned long long a, b;
            ld_relaxed_v2(slots + static_cast<size_t>(c - 1 - lane) * 4, a, b);
            ok = word_flag(a) == pf && word_flag(b) == pf;
            v0 = word_val(a);
            v1 = word_val(b);
        }
        if (__all_sync(FULL_MASK, ok)) break;
        int give_up = 0;
        if (lane == 0) give_up = lookback_give_up(p, epoch, t_start) ? 1 : 0;
        if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
        backoff(spin);
    }
    float u0 = 0.f, u1 = 0.f;
    if (mine) {
        if (lane > 0) {
            mv2(Qc[lane], v0, v1, u0, u1);  // Q^lane
        } else {
            u0 = v0;
            u1 = v1;
        }
    }
    if (lane == 0 && c < static_cast<uint32_t>(m)) {
        float w0, w1;
        mv2(Qc[c], z0, z1, w0, w1);  // Q^c z
        u0 += w0;
        u1 += w1;
    }
    X0 = warp_sum(u0);
    X1 = warp_sum(u1);
    return true;
}

template <class P>
__device__ bool lookback_hier(const P& p, const unsigned long long* slots, unsigned long long* gslots,
                              const float4* Qc, const float4* Qg, uint32_t c, uint32_t epoch, float own0, float own1,
                              bool withhold, float& X0, float& X1, float z0 = 0.f, float z1 = 0.f) {
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u, ff = 2u * epoch + 2u;
    const int j = static_cast<int>(c & 31u);
    const long long g = static_cast<long long>(c >> 5);
    const uint64_t t_start = globaltimer_ns();
    bool gpart_done = (j != 31) || withhold;
    uint32_t spin = 64;
    // Q^(j-1-lane) for the chunk terms (only lanes < j use it)
    const float4 qc = Qc[(j - 1 - lane) & 31];
    long long gbase = g - 1;               // group window start (nearest group first)
    float4 gscale = make_float4(1.f, 0.f, 0.f, 1.f);  // Qg^(32 w) for extended group windows
    float gacc0 = 0.f, gacc1 = 0.f;        // group-level partial sum over earlier windows
    while (true) {
        // ---- one poll: own-group chunks + one window of groups ----
        SlotView cs;
        cs.part = cs.full = false;
        cs.p0 = cs.p1 = cs.f0 = cs.f1 = 0.f;
        if (lane < j) cs = read_slot(slots + (static_cast<size_t>(g) * 32 + lane) * 4, pf, ff);
        SlotView gs;
        const long long gm = gbase - lane;
        if (gm >= 0) {
            gs = read_slot(gslots + static_cast<size_t>(gm) * 4, pf, ff);
        } else {
            // before the signal: the state at its start, (z0, z1) (zero unless given)
            gs.part = gs.full = true;
            gs.p0 = gs.p1 = 0.f;
            gs.f0 = z0;
            gs.f1 = z1;
        }
        IIR_PROF_ADD(p, 6, lane == 0 ? 1ull : 0ull);
        // group aggregate of a group's last chunk
        if (!gpart_done) {
            const unsigned np = __ballot_sync(FULL_MASK, lane < j && !cs.part);
            if (np == 0u) {
                float t0 = 0.f, t1 = 0.f;
                if (lane < j) {
                    const float4 q = Qc[31 - lane];  // Q^(31 - lane)
                    mv2(q, cs.p0, cs.p1, t0, t1);
                }
                t0 = warp_sum(t0);
                t1 = warp_sum(t1);
                if (lane == 0) publish2(gslots + static_cast<size_t>(g) * 4, pf, t0 + own0, t1 + own1);
                gpart_done = true;
            }
        }
        // ---- nearest inclusive carry inside the group ----
        const unsigned fm = __ballot_sync(FULL_MASK, lane < j && cs.full);
        bool resolved = false;
        if (fm != 0u) {
            const int f = 31 - __clz(fm);  // highest (nearest) position with a full carry
            const unsigned nr = __ballot_sync(FULL_MASK, lane > f && lane < j && !cs.part);
            if (nr == 0u) {
                float t0 = 0.f, t1 = 0.f;
                if (lane == f) mv2(qc, cs.f0, cs.f1, t0, t1);
                else if (lane > f && lane < j) mv2(qc, cs.p0, cs.p1, t0, t1);
                X0 = warp_sum(t0);
                X1 = warp_sum(t1);
                resolved = true;
            }
        } else {
            const unsigned nr = __ballot_sync(FULL_MASK, lane < j && !cs.part);
            const unsigned gfm = __ballot_sync(FULL_MASK, gs.full);
            const int h = gfm ? (__ffs(gfm) - 1) : 32;
            const unsigned gnr = __ballot_sync(FULL_MASK, lane < h && !gs.part);
            if (nr == 0u && gnr == 0u) {
                // group-level terms of this window, scaled by the window offset
                float u0 = 0.f, u1 = 0.f;
                if (lane < h) mv2(Qg[lane], gs.p0, gs.p1, u0, u1);
                else if (lane == h) mv2(Qg[lane], gs.f0, gs.f1, u0, u1);
                float w0, w1;
                mv2(gscale, u0, u1, w0, w1);
                gacc0 += warp_sum(w0);
                gacc1 += warp_sum(w1);
                if (h < 32) {
                    // X = Q^j Xg + sum_{i<j} Q^(j-1-i) part(i)
                    float t0 = 0.f, t1 = 0.f;
                    if (lane < j) mv2(qc, cs.p0, cs.p1, t0, t1);
                    t0 = warp_sum(t0);
                    t1 = warp_sum(t1);
                    float z0, z1;
                    mv2(Qc[j], gacc0, gacc1, z0, z1);
                    X0 = z0 + t0;
                    X1 = z1 + t1;
                    resolved = true;
                } else {
                    // no group carry in this window: move the window back by 32 groups
                    gscale = mm2(gscale, Qg[32]);
                    gbase -= 32;
                    continue;
                }
            }
        }
        if (resolved && gpart_done) return true;
        // ---- not ready: bounded wait ----
        int give_up = 0;
        if (lane == 0) give_up = lookback_give_up(p, epoch, t_start) ? 1 : 0;
        if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
        if (resolved) {
            // only the group aggregate is outstanding: its partials are already visible
            // through this warp's reads on the next poll; keep X
            const float k0 = X0, k1 = X1;
            backoff(spin);
            while (!gpart_done) {
                SlotView cs2;
                cs2.part = false;
                cs2.p0 = cs2.p1 = 0.f;
                if (lane < j) cs2 = read_slot(slots + (static_cast<size_t>(g) * 32 + lane) * 4, pf, ff);
                const unsigned np = __ballot_sync(FULL_MASK, lane < j && !cs2.part);
                if (np == 0u) {
                    float t0 = 0.f, t1 = 0.f;
                    if (lane < j) mv2(Qc[31 - lane], cs2.p0, cs2.p1, t0, t1);
                    t0 = warp_sum(t0);
                    t1 = warp_sum(t1);
                    if (lane == 0) publish2(gslots + static_cast<size_t>(g) * 4, pf, t0 + own0, t1 + own1);
                    gpart_done = true;
                    break;
                }
                int gu = 0;
                if (lane == 0) gu = lookback_give_up(p, epoch, t_start) ? 1 : 0;
                if (__shfl_sync(FULL_MASK, gu, 0)) return false;
                backoff(spin);
            }
            X0 = k0;
            X1 = k1;
            return true;
        }
        backoff(spin);
        gacc0 = 0.f;  // the window is re-read from the nearest group
        gacc1 = 0.f;
        gbase = g - 1;
        gscale = make_float4(1.f, 0.f, 0.f, 1.f);
    }
}

// ------------------------------------------------------------------------------------
// Block driver for the row-major realizations (PH, STCR, DTCR).
//
// A block filters one chunk: ROWS consecutive rows of N samples (ROWS = tiles x BLOCK_SIZE;
// a tile is the reference's chunk, thread t owning samples [t*N, (t+1)*N),
// ph_kernels.cuh:236-241). Warp 0 is the control warp: it takes the block's ticket (chunk
// order = ticket order = block start order, the forward-progress argument of
// ph_kernels.cuh:227-229), starts ONE 2D TMA tensor load of the chunk (the signal viewed as
// 32-float lines; 128-byte swizzle, so row-wise float4 reads hit distinct banks), resolves
// every section's carry and publishes the chunk's carries; the row warps filter, keeping
// rows in the shared-memory buffer (few registers per thread, so many blocks share an SM
// and hide each other's load and lookback latency). Results are written back in place
// (same swizzle) and stored with one TMA tensor store. Carries between the tiles of a
// chunk are resolved in shared memory (the same algebra as the lookback). Ragged last
// chunks and unaligned buffers use element-wise staging into the same layout.
// ------------------------------------------------------------------------------------
struct BlockAux {
    unsigned long long mbar;
    unsigned int chunk;
    unsigned int epoch;
    int bail;
    int pad;
    float wtot[16][2][2];  // per row warp, per scan q (tail schedule: per section parity): zero-state warp totals
    float X[2];            // lookback result (incoming state of the chunk)
    float Xs[IIR_MAX_SECTIONS][2];    // tail schedule: incoming state of the chunk, every section
    float tpiece[IIR_TAIL_MAX_PIECES][IIR_MAX_SECTIONS][2];  // tail schedule: pieces' end states
    float xch[2][16][2];    // cyclic-reduction tiles over several warps: per-level row hand-off
    float xscan[16][2][2];  // and the warps' top-level scan totals
};

// Occupancy target of the row-major kernels (registers left for the lookback's state).
#ifndef IIR_MAX_BLOCKS_PER_SM
#define IIR_MAX_BLOCKS_PER_SM 8
#endif

template <int ROWS, int N>
struct BlockGeom {
    static_assert(N == 16 || N == 32 || N == 64 || N == 128, "samples per row");
    static constexpr int CHUNK = ROWS * N;
    static constexpr int LINES = CHUNK / 32;          // 128-byte lines per chunk
    static_assert((N >= 32 ? ROWS : LINES) <= 256, "TMA box of at most 256 rows");
    static constexpr size_t DATA_BYTES = static_cast<size_t>(CHUNK) * sizeof(float);
    static constexpr size_t SMEM_BYTES = 1024 + DATA_BYTES + sizeof(BlockAux);  // + swizzle alignment
    // resident blocks per SM that shared memory (227 KB) and threads (2048) allow
    static constexpr int min_blocks(int threads) {
        const int by_smem = static_cast<int>((227 * 1024) / SMEM_BYTES);
        const int by_thr = 2048 / threads;
        int b = by_smem < by_thr ? by_smem : by_thr;
        if (b > IIR_MAX_BLOCKS_PER_SM) b = IIR_MAX_BLOCKS_PER_SM;
        return b < 1 ? 1 : b;
    }
};

// Resident blocks per SM that shared memory (227 KB), threads (2048) and the occupancy
// target allow: the __launch_bounds__ minimum for a kernel of `threads` threads.
constexpr int min_blocks_for(size_t smem_bytes, int threads) {
    const int by_smem = static_cast<int>((227 * 1024) / smem_bytes);
    const int by_thr = 2048 / threads;
    int b = by_smem < by_thr ? by_smem : by_thr;
    if (b > IIR_MAX_BLOCKS_PER_SM) b = IIR_MAX_BLOCKS_PER_SM;
    return b < 1 ? 1 : b;
}

// Float index of sample n of row r in the swizzled chunk buffer (128B swizzle: the 16-byte
// unit u of line L lives at unit u ^ (L & 7)). Two layouts:
//   PLANES  rows of 32 or more samples stored as N / 32 planes of 32-sample columns,
//           plane-major ([N/32][ROWS][32]): line L = plane * ROWS + r, so L & 7 = r & 7 and the
//           32 rows a warp reads at one column fall on 8 distinct units (four wavefronts per
//           128-bit access, no bank conflict). Each plane is one tensor copy.
//   lines   the chunk as it lies in memory, CHUNK / 32 lines of 32 samples: L = r * N / 32 +
//           n / 32, one tensor copy per chunk. For N = 64 (128) only 4 (2) of the 8 units are
//           used at a column: 2-way (4-way) conflicts for a warp of rows.
// Rows of 16 samples share a line (two rows per line) in both.
template <int N, int ROWS, bool PLANES>
__device__ __forceinline__ int swz(int r, int n) {
    static_assert(ROWS % 8 == 0, "whole swizzle atoms per plane");
    int L, u;
    if constexpr (N >= 32) {
        L = PLANES ? (n >> 5) * ROWS + r : r * (N / 32) + (n >> 5);
        u = (n & 31) >> 2;
    } else {
        L = r >> 1;
        u = ((r & 1) << 2) + (n >> 2);
    }
    return (L << 5) + ((u ^ (L & 7)) << 2) + (n & 3);
}

template <int ROWS, int N>
__device__ __forceinline__ bool chunk_is_bulk(const IirParams& p, uint32_t c) {
    return p.use_tma && (static_cast<long long>(c) + 1) * (ROWS * N) <= p.n;
}

// Shared-memory carve-up: 1024-aligned chunk buffer, then the aux block.
template <int ROWS, int N>
__device__ __forceinline__ float* chunk_buffer(unsigned char* smem) {
    const uint32_t a = smem_u32(smem);
    return reinterpret_cast<float*>(smem + (((a + 1023u) & ~1023u) - a));
}
template <int ROWS, int N>
__device__ __forceinline__ BlockAux* block_aux(unsigned char* smem) {
    return reinterpret_cast<BlockAux*>(chunk_buffer<ROWS, N>(smem) + BlockGeom<ROWS, N>::CHUNK);
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}

// Chunk c between global memory and its swizzled buffer. PLANES: one tensor copy per plane
// (the map views the signal as rows of N samples, box 32 x ROWS); lines: one copy of CHUNK / 32
// lines (the map views the signal as 32-sample lines). 128B swizzle in both.
template <int ROWS, int N, bool PLANES>
__device__ __forceinline__ void tma_load_chunk(float* buf, const CUtensorMap* map, uint32_t c,
                                               unsigned long long* bar) {
    if constexpr (PLANES && N >= 32) {
#pragma unroll
        for (int h = 0; h < N / 32; ++h) tma_load_2d(buf + h * ROWS * 32, map, 32 * h, static_cast<int>(c) * ROWS, bar);
    } else {
        tma_load_2d(buf, map, 0, static_cast<int>(c) * (ROWS * N / 32), bar);
    }
}
template <int ROWS, int N, bool PLANES>
__device__ __forceinline__ void tma_store_chunk(const CUtensorMap* map, uint32_t c, const float* buf) {
    if constexpr (PLANES && N >= 32) {
#pragma unroll
        for (int h = 0; h < N / 32; ++h) tma_store_2d(map, 32 * h, static_cast<int>(c) * ROWS, buf + h * ROWS * 32);
    } else {
        tma_store_2d(map, 0, static_cast<int>(c) * (ROWS * N / 32), buf);
    }
}

// Control warp: takes the ticket and starts the chunk's TMA load.
template <int ROWS, int N>
__device__ __forceinline__ void block_begin(const IirParams& p, float* buf, BlockAux* aux) {
    if ((threadIdx.x & 31) == 0) {
        mbar_init(&aux->mbar, 1);
        fence_mbar_init();
        uint32_t epoch;
        const uint32_t c = take_ticket(p.state, p.nchunks, epoch);
        aux->chunk = c;
        aux->epoch = epoch;
        aux->bail = 0;
        if (chunk_is_bulk<ROWS, N>(p, c)) {
            mbar_arrive_expect_tx(&aux->mbar, static_cast<uint32_t>(BlockGeom<ROWS, N>::DATA_BYTES));
            tma_load_chunk<ROWS, N, true>(buf, &p.tmap_x, c, &aux->mbar);
        }
    }
}

// All threads: make the chunk's input available in `buf`. Returns false on a failed wait.
template <int ROWS, int N, int THREADS>
__device__ __forceinline__ bool block_acquire(const IirParams& p, float* buf, BlockAux* aux, uint32_t c,
                                              uint32_t epoch) {
    if (chunk_is_bulk<ROWS, N>(p, c)) {
        bool arrived = true;
        if (threadIdx.x >= 32) arrived = wait_mbar_bounded(&aux->mbar, 0, p.timeout_ns);
        if (__syncthreads_or(arrived ? 0 : 1)) {
            if (threadIdx.x == 0) raise_error(p.state, epoch, IIR_DEV_ERR_MBARRIER);
            return false;
        }
    } else {
        const long long cs = static_cast<long long>(c) * (ROWS * N);
        for (int i = threadIdx.x; i < ROWS * N; i += THREADS) {
            const long long g = cs + i;
            buf[swz<N, ROWS, true>(i / N, i % N)] = (g < p.n) ? p.x[g] : 0.f;
        }
        __syncthreads();
    }
    return true;
}

// All threads, after the rows hold the output (fence.proxy.async by the writers, then
// __syncthreads).
template <int ROWS, int N, int THREADS>
__device__ __forceinline__ void block_store(const IirParams& p, float* buf, uint32_t c) {
    if (chunk_is_bulk<ROWS, N>(p, c)) {
        if (threadIdx.x == 0) {
            tma_store_chunk<ROWS, N, true>(&p.tmap_y, c, buf);
            bulk_commit();
            bulk_wait_read_all();  // shared memory must outlive the copy's reads
        }
    } else {
        const long long cs = static_cast<long long>(c) * (ROWS * N);
        for (int i = threadIdx.x; i < ROWS * N; i += THREADS) {
            const long long g = cs + i;
            if (g < p.n) p.y[g] = buf[swz<N, ROWS, true>(i / N, i % N)];
        }
    }
}

// Control warp, per section (between barriers (A) and (B) of the caller): composes the
// chunk's zero-state aggregate from the row warps' totals (NQ independent 2-state scans,
// warp transition Gw = G^(rows per warp)), publishes it, resolves the incoming state X by
// the two-level lookback, publishes full = aggregate + Q X (also the group's inclusive
// carry when the chunk closes a group) and leaves X in aux. Returns false on failure.
template <int NW, int NQ, class P>
__device__ __forceinline__ bool control_section(const P& p, BlockAux* aux, int sec, uint32_t c, uint32_t epoch,
                                                const float4* tab, float4 Gw) {
    const int lane = threadIdx.x & 31;
    float t[NQ][2];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        t[q][0] = 0.f;
        t[q][1] = 0.f;
    }
#pragma unroll 4
    for (int w = 0; w < NW; ++w) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float n0, n1;
            mv2(Gw, t[q][0], t[q][1], n0, n1);
            t[q][0] = n0 + aux->wtot[w][q][0];
            t[q][1] = n1 + aux->wtot[w][q][1];
        }
    }
    // chunk state pair: PH keeps the pair itself; the CR forms scan (Y_{t-1}, Y_t) per parity
    const float a0 = (NQ == 1) ? t[0][0] : t[0][1];
    const float a1 = (NQ == 1) ? t[0][1] : t[NQ - 1][1];
    unsigned long long* slots = p.carry + static_cast<size_t>(sec) * p.carry_stride;
    unsigned long long* gslots = slots + static_cast<size_t>(p.carry_cap) * 4;
    const bool withhold = static_cast<long long>(c) == p.withhold_chunk;
    const uint32_t pf = 2u * epoch + 1u, ff = 2u * epoch + 2u;
    if (lane == 0 && !withhold) publish2(slots + static_cast<size_t>(c) * 4, pf, a0, a1);
    float X0 = 0.f, X1 = 0.f;
    bool ok = true;
#ifdef IIR_PROFILE
    const uint64_t tl = globaltimer_ns();
#endif
    const int depth = static_cast<int>(tab[IIR_TAB_LBD].x);  // truncated lookback depth (0: full)
    if (c > 0)
        ok = depth > 0 ? lookback_trunc2(p, slots, tab + IIR_TAB_QC, c, epoch, depth, X0, X1)
                       : lookback_hier(p, slots, gslots, tab + IIR_TAB_QC, tab + IIR_TAB_QG, c, epoch, a0, a1,
                                       withhold, X0, X1);
#ifdef IIR_PROFILE
    if (lane == 0) IIR_PROF_ADD(p, 5, globaltimer_ns() - tl);
#endif
    if (lane == 0) {
        if (ok && !withhold) {
            float f0, f1;
            mv2(tab[IIR_TAB_QC + 1], X0, X1, f0, f1);  // Q (chunk transition)
            publish2(slots + static_cast<size_t>(c) * 4 + 2, ff, a0 + f0, a1 + f1);
            if ((c & 31u) == 31u) publish2(gslots + static_cast<size_t>(c >> 5) * 4 + 2, ff, a0 + f0, a1 + f1);
        }
        aux->X[0] = X0;
        aux->X[1] = X1;
        aux->bail = ok ? 0 : 1;
    }
    return ok;
}

// Row warps: zero-state incoming state of warp `w` (row-warp index) for scan q.
template <class Aux>
__device__ __forceinline__ void warp_incoming(const Aux* aux, int w, int q, float4 Gw, float& i0, float& i1) {
    i0 = 0.f;
    i1 = 0.f;
    for (int v = 0; v < w; ++v) {
        float n0, n1;
        mv2(Gw, i0, i1, n0, n1);
        i0 = n0 + aux->wtot[v][q][0];
        i1 = n1 + aux->wtot[v][q][1];
    }
}

}  // namespace iirgb
