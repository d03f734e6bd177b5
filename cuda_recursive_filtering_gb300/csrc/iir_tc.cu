// iir_tc.cu — precision form: the cascade's chunk solve as tcgen05 tensor-core GEMMs.
//
// The signal is cut into chunks of L = 64 samples and tiles of NB = 128 chunks. For a cascade
// of K sections (D = 2K carried output states y_s[-2], y_s[-1], plus the input history
// x[-2], x[-1] that the first section's FIR reads), every chunk j obeys
//     y_j      = T x_j + H S_j + Hx xh_j                (L outputs of the last section)
//     S_{j+1}  = Phi S_j + Phix xh_j + B x_j            (D carried states)
// with T the L x L lower-triangular Toeplitz matrix of the cascade's impulse response (gain
// included), B the zero-state end states, H / Hx the responses to unit states and Phi / Phix
// the chunk transitions; all are computed on the host in FP64 by running the cascade.
//   GEMM 1 (tcgen05.mma kind::tf32, M = 128, N = 128 chunks, K = 64): [T; B] X -> TMEM; rows
//          0..63 are the zero-state outputs, rows 64..64+D-1 the zero-state end states B x_j.
//   scan   the D-state recurrence over the tile's 128 chunks on CUDA cores: 16 sub-blocks of 8
//          chunks scanned in parallel from zero, joined, then rescanned from their true states;
//          tiles are joined by the D-dimensional decoupled lookback (iir_lookk.cuh) with the
//          tile transition Q = Phi^128.
//   GEMM 2 (K = 32): TMEM += [H | Hx] [S_j | xh_j], then the epilogue reads the outputs.
// Operands are split TF32 hi / lo (hi = the nearest TF32 value, lo = the nearest TF32 value of
// the rest) and multiplied as hi*hi + hi*lo + lo*hi with FP32 accumulation in TMEM, which keeps
// float32 accuracy. The reference has no such form; its chunk work is scalar float32
// (ph_kernels.cuh:265-480), which this replaces by two GEMMs whose cost does not grow with the
// order (M = L + D rows).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/iir_gb300.h"
#include "iir_host_internal.h"
#include "iir_lookk.cuh"
#include "iir_pipe.cuh"

namespace iirgb {

constexpr int TC_L = 64;                 // samples per chunk (GEMM K)
constexpr int TC_NB = 128;               // chunks per tile (GEMM N)
constexpr int TC_TILE = TC_L * TC_NB;    // samples per tile
constexpr int TC_THREADS = 256;
constexpr int TC_GROUPS = 16;            // scan sub-blocks (half-warps)
constexpr int TC_SUB = TC_NB / TC_GROUPS;
constexpr int TC_DMAX = 16;              // carried states (order <= 16)
constexpr int TC_KB = 32 * 128;          // floats of one swizzled [128 rows x 32] block

struct TcParams {
    CUtensorMap tmap_x;          // x as [n/64 rows][64], box {32, 128}, 128-byte swizzle
    const float* x;
    float* y;
    long long n;
    IirLaunchState* state;
    unsigned long long* carry;   // per tile slot 2*KD words, then per group of 32 tiles
    const float* a1img;          // [hi | lo] x [2 k-blocks] x TC_KB, swizzled smem images
    const float* a2img;          // [hi | lo] x TC_KB
    const float* phi;            // 16 x 16 (row-major, zero beyond D)
    const float* phix;           // 16 x 2
    const float* phi_grp;        // Phi^(8 g), g < 16: 16 x 16 x 16
    const float* pc;             // Q^l (l <= 32), KD x KD
    const float* pg;             // Q^(32 l) (l <= 32), KD x KD
    long long timeout_ns;
    long long withhold_chunk;
    unsigned int ntiles;
    unsigned int carry_cap;
    int D;
    int use_tma;
    unsigned long long* prof;
};

struct TcAux {
    unsigned long long mb_tma, mb_g1, mb_g2;
    uint32_t tmem;
    uint32_t epoch;
    int bail;
    float agg[2][TC_DMAX];           // tile aggregates (zero incoming state), per slot
    float X[TC_DMAX];                // incoming state of the tile being finished
    float Ag[TC_GROUPS][TC_DMAX];    // sub-block aggregates (zero start) of the current tile
    float Ig0[2][TC_GROUPS][TC_DMAX];  // zero-start incoming state of each sub-block, per slot
    float xh[2][TC_NB][2];           // input history of each chunk, per slot
    float Z[2][TC_NB][TC_DMAX];      // GEMM 1 end-state rows, per slot
};

struct TcSmem {
    static constexpr size_t A1 = 0;                        // hi, lo: 2 x 2 x TC_KB floats
    static constexpr size_t A2 = A1 + 4 * TC_KB * 4;       // hi, lo: 2 x TC_KB
    static constexpr size_t XH = A2 + 2 * TC_KB * 4;       // x tile hi (TMA target): 2 x TC_KB
    static constexpr size_t XL = XH + 2 * TC_KB * 4;       // x tile lo
    static constexpr size_t B2H = XL + 2 * TC_KB * 4;      // state operand hi: TC_KB
    static constexpr size_t B2L = B2H + TC_KB * 4;         // lo
    static constexpr size_t AUX = B2L + TC_KB * 4;
    static constexpr size_t BYTES = 1024 + AUX + sizeof(TcAux);
};

__device__ __forceinline__ int swz32(int r, int c) { return (r << 5) + ((((c >> 2) ^ (r & 7))) << 2) + (c & 3); }
// Nearest TF32 value of v (ties away from zero): round the magnitude at mantissa bit 13. The
// tensor core reads only the top 19 bits of an operand, so the split v = hi + lo with
// hi = tf32(v), lo = tf32(v - hi) loses about 2^-22 |v| (the lo * lo product is dropped too).
__device__ __forceinline__ float tf32_hi(float v) { return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u); }

// K-major, 128-byte swizzled operand: rows of 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFF) | (static_cast<uint64_t>(1) << 16) |
           (static_cast<uint64_t>(1024 >> 4) << 32) | (static_cast<uint64_t>(1) << 46) | (static_cast<uint64_t>(2) << 61);
}
// kind::tf32, D f32, A / B tf32 K-major, M = 128, N = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((TC_NB >> 3) << 17) | ((128 >> 4) << 24);

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(TC_IDESC), "r"(acc));
}
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

template <int KD>
__global__ void __launch_bounds__(TC_THREADS, 1) iir_tc_kernel(const __grid_constant__ TcParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t a0 = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((a0 + 1023u) & ~1023u) - a0);
    float* a1 = reinterpret_cast<float*>(base + TcSmem::A1);
    float* a2 = reinterpret_cast<float*>(base + TcSmem::A2);
    float* xhb = reinterpret_cast<float*>(base + TcSmem::XH);
    float* xlb = reinterpret_cast<float*>(base + TcSmem::XL);
    float* b2h = reinterpret_cast<float*>(base + TcSmem::B2H);
    float* b2l = reinterpret_cast<float*>(base + TcSmem::B2L);
    TcAux* aux = reinterpret_cast<TcAux*>(base + TcSmem::AUX);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int D = p.D;
    const uint32_t G = gridDim.x;
    const uint32_t nk = (p.ntiles > blockIdx.x) ? (p.ntiles - blockIdx.x + G - 1) / G : 0;

    // ---- setup: operand images, zeroed state operand, TMEM, barriers ----
    {
        const float4* s1 = reinterpret_cast<const float4*>(p.a1img);
        float4* d1 = reinterpret_cast<float4*>(a1);
        for (int i = tid; i < TC_KB; i += TC_THREADS) d1[i] = __ldg(s1 + i);  // 4 blocks = TC_KB float4
        const float4* s2 = reinterpret_cast<const float4*>(p.a2img);
        float4* d2 = reinterpret_cast<float4*>(a2);
        for (int i = tid; i < TC_KB / 2; i += TC_THREADS) d2[i] = __ldg(s2 + i);
        float4* z = reinterpret_cast<float4*>(b2h);
        for (int i = tid; i < TC_KB / 2; i += TC_THREADS) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // b2h, b2l
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&aux->tmem)),
                     "r"(256));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 32) {
        mbar_init(&aux->mb_tma, 1);
        mbar_init(&aux->mb_g1, 1);
        mbar_init(&aux->mb_g2, 1);
        fence_mbar_init();
        aux->epoch = static_cast<uint32_t>(*reinterpret_cast<volatile unsigned long long*>(&p.state->ticket) >> 32);
        aux->bail = 0;
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = aux->tmem, epoch = aux->epoch;

    // this thread's state row d of Phi, Phix (scan: half-warp groups, lane d = state component)
    const int grp = tid >> 4, d = tid & 15;
    float phi_row[TC_DMAX], phix_row[2];
#pragma unroll
    for (int e = 0; e < TC_DMAX; ++e) phi_row[e] = __ldg(p.phi + d * TC_DMAX + e);
    phix_row[0] = __ldg(p.phix + d * 2);
    phix_row[1] = __ldg(p.phix + d * 2 + 1);

    unsigned long long* slots = p.carry;
    unsigned long long* gslots = p.carry + static_cast<size_t>(p.carry_cap) * 2 * KD;
    const uint32_t pf = 2u * epoch + 1u, ff = 2u * epoch + 2u;
    uint32_t ph_tma = 0, ph_g1 = 0, ph_g2 = 0;
    bool live1 = false, pend1 = false, pend2 = false;

    for (uint32_t k = 0; k <= nk; ++k) {
        const int slot = k & 1;
        const uint32_t t = blockIdx.x + k * G;  // tile of this iteration (k < nk)
        if (k < nk) {
            // ---- 1. load the tile (chunks as rows, samples as K) and split it hi / lo ----
            const long long ts = static_cast<long long>(t) * TC_TILE;
            const bool bulk = p.use_tma && ts + TC_TILE <= p.n;
            if (bulk) {
                if (tid == 0) {
                    mbar_arrive_expect_tx(&aux->mb_tma, 2u * TC_KB * 4u);
                    tma_load_2d(xhb, &p.tmap_x, 0, static_cast<int>(t) * TC_NB, &aux->mb_tma);
                    tma_load_2d(xhb + TC_KB, &p.tmap_x, 32, static_cast<int>(t) * TC_NB, &aux->mb_tma);
                }
                if (!wait_mbar_bounded(&aux->mb_tma, ph_tma, p.timeout_ns) && tid == 0) {
                    aux->bail = 1;
                    raise_error(p.state, epoch, IIR_DEV_ERR_MBARRIER);
                }
                ph_tma ^= 1u;
            } else {
                for (int i = tid; i < TC_TILE; i += TC_THREADS) {
                    const int j = i / TC_L, c = i % TC_L;
                    const long long g = ts + i;
                    xhb[(c >> 5) * TC_KB + swz32(j, c & 31)] = (g < p.n) ? p.x[g] : 0.f;
                }
            }
            __syncthreads();
            // input history of each chunk: the two samples before it
            if (tid < TC_NB) {
                float h2, h1;
                if (tid > 0) {
                    h2 = xhb[TC_KB + swz32(tid - 1, 30)];
                    h1 = xhb[TC_KB + swz32(tid - 1, 31)];
                } else if (ts > 0) {
                    h2 = p.x[ts - 2];
                    h1 = p.x[ts - 1];
                } else {
                    h2 = h1 = 0.f;
                }
                aux->xh[slot][tid][0] = h2;
                aux->xh[slot][tid][1] = h1;
            }
            __syncthreads();
            for (int i = tid; i < 2 * TC_KB; i += TC_THREADS) {
                const float v = xhb[i];
                const float h = tf32_hi(v);
                xhb[i] = h;
                xlb[i] = tf32_hi(v - h);
            }
            fence_proxy_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            live1 = !aux->bail;  // every thread reads it after the same barrier
            // ---- 2. GEMM 1: [T; B] X -> TMEM slot ----
            if (tid == 0 && live1) {
                const uint32_t dt = tmem + slot * TC_NB;
                uint32_t acc = 0;
#pragma unroll
                for (int kb = 0; kb < 2; ++kb) {
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {
                        const uint32_t oa = (kb * TC_KB) * 4 + ks * 32;
                        const uint64_t ah = umma_desc(smem_u32(a1) + oa);
                        const uint64_t al = umma_desc(smem_u32(a1) + 2 * TC_KB * 4 + oa);
                        const uint64_t bh = umma_desc(smem_u32(xhb) + oa);
                        const uint64_t bl = umma_desc(smem_u32(xlb) + oa);
                        umma_tf32(dt, ah, bh, acc);
                        umma_tf32(dt, ah, bl, 1u);
                        umma_tf32(dt, al, bh, 1u);
                        acc = 1u;
                    }
                }
                umma_commit(&aux->mb_g1);
            }
        }
        // ---- 3. lookback of the previous tile (its aggregate was published one iteration ago) ----
        if (k >= 1 && warp == 0) {
            const uint32_t tp = blockIdx.x + (k - 1) * G;
            float own[KD], X[KD];
#pragma unroll
            for (int e = 0; e < KD; ++e) {
                own[e] = aux->agg[slot ^ 1][e];
                X[e] = 0.f;
            }
            const bool withhold = static_cast<long long>(tp) == p.withhold_chunk;
            bool ok = true;
            if (tp > 0 && !aux->bail) ok = lookback_hier_k<KD>(p, slots, gslots, p.pc, p.pg, tp, epoch, own, withhold, X);
            if (lane == 0) {
                if (ok && !withhold && !aux->bail) {
                    float f[KD];
                    matvec<KD>(p.pc + KD * KD, X, f);  // Q X
#pragma unroll
                    for (int e = 0; e < KD; ++e) f[e] += own[e];
                    publishk<KD>(slots + static_cast<size_t>(tp) * 2 * KD + KD, ff, f);
                    if ((tp & 31u) == 31u) publishk<KD>(gslots + static_cast<size_t>(tp >> 5) * 2 * KD + KD, ff, f);
                }
                if (!ok) aux->bail = 1;
#pragma unroll
                for (int e = 0; e < TC_DMAX; ++e) aux->X[e] = e < KD ? X[e] : 0.f;
            }
        }
        if (k < nk) {
            // ---- 4. GEMM 1 done: end-state rows (TMEM lanes 64 ..) to shared memory ----
            if (live1) {
                if (!wait_mbar_bounded(&aux->mb_g1, ph_g1, p.timeout_ns)) {
                    pend1 = true;  // waited for again (bounded) before TMEM is freed
                    if (tid == 0) {
                        aux->bail = 1;
                        raise_error(p.state, epoch, IIR_DEV_ERR_MBARRIER);
                    }
                } else {
                    ph_g1 ^= 1u;
                }
            }
            tc_fence_after();
            if (warp == 2 && !aux->bail) {
                for (int c = 0; c < TC_NB; c += 16) {
                    float v[16];
                    tmem_ld16(tmem + (64u << 16) + slot * TC_NB + c, v);
                    if (lane < TC_DMAX) {
#pragma unroll
                        for (int i = 0; i < 16; ++i) aux->Z[slot][c + i][lane] = lane < D ? v[i] : 0.f;
                    }
                }
            }
            __syncthreads();
            // ---- 5. scan from zero: sub-block aggregates, then the tile aggregate ----
            {
                float S = 0.f;
                for (int i = 0; i < TC_SUB; ++i) {
                    const int j = grp * TC_SUB + i;
                    float acc = aux->Z[slot][j][d];
                    acc = fmaf(phix_row[0], aux->xh[slot][j][0], acc);
                    acc = fmaf(phix_row[1], aux->xh[slot][j][1], acc);
#pragma unroll
                    for (int e = 0; e < TC_DMAX; ++e) acc = fmaf(phi_row[e], __shfl_sync(FULL_MASK, S, e, 16), acc);
                    S = acc;
                }
                aux->Ag[grp][d] = S;
            }
            __syncthreads();
            if (grp == 0) {
                // zero-start incoming state of every sub-block: I_{g+1} = Phi^8 I_g + A_g
                const float* p8 = p.phi_grp + 1 * TC_DMAX * TC_DMAX;  // Phi^8
                float I = 0.f;
                for (int g = 0; g < TC_GROUPS; ++g) {
                    aux->Ig0[slot][g][d] = I;
                    float acc = aux->Ag[g][d];
#pragma unroll
                    for (int e = 0; e < TC_DMAX; ++e)
                        acc = fmaf(__ldg(p8 + d * TC_DMAX + e), __shfl_sync(0x0000ffffu, I, e, 16), acc);
                    I = acc;
                }
                aux->agg[slot][d] = I;
            }
            __syncthreads();
            if (tid == 0 && static_cast<long long>(t) != p.withhold_chunk) {
                float a[KD];
#pragma unroll
                for (int e = 0; e < KD; ++e) a[e] = aux->agg[slot][e];
                publishk<KD>(slots + static_cast<size_t>(t) * 2 * KD, pf, a);
            }
        } else {
            __syncthreads();  // the lookback's X is visible
        }
        // ---- 6. finish the previous tile: states, GEMM 2, output ----
        if (k >= 1) {
            __syncthreads();
            const int ps = slot ^ 1;
            const uint32_t tp = blockIdx.x + (k - 1) * G;
            if (!aux->bail) {
                // true incoming state of the sub-block, then its chunks' states into the operand
                const float* pgm = p.phi_grp + static_cast<size_t>(grp) * TC_DMAX * TC_DMAX;
                float S = aux->Ig0[ps][grp][d];
#pragma unroll
                for (int e = 0; e < TC_DMAX; ++e) S = fmaf(__ldg(pgm + d * TC_DMAX + e), aux->X[e], S);
                for (int i = 0; i < TC_SUB; ++i) {
                    const int j = grp * TC_SUB + i;
                    if (d < D) {
                        const float h = tf32_hi(S);
                        b2h[swz32(j, d)] = h;
                        b2l[swz32(j, d)] = tf32_hi(S - h);
                    }
                    if (d < 2) {  // the chunk's input history in columns D, D + 1
                        const float v = aux->xh[ps][j][d];
                        const float h = tf32_hi(v);
                        b2h[swz32(j, D + d)] = h;
                        b2l[swz32(j, D + d)] = tf32_hi(v - h);
                    }
                    float acc = aux->Z[ps][j][d];
                    acc = fmaf(phix_row[0], aux->xh[ps][j][0], acc);
                    acc = fmaf(phix_row[1], aux->xh[ps][j][1], acc);
#pragma unroll
                    for (int e = 0; e < TC_DMAX; ++e) acc = fmaf(phi_row[e], __shfl_sync(FULL_MASK, S, e, 16), acc);
                    S = acc;
                }
            }
            fence_proxy_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            const bool live2 = !aux->bail;
            if (tid == 0 && live2) {
                const uint32_t dt = tmem + ps * TC_NB;
#pragma unroll
                for (int ks = 0; ks < 4; ++ks) {
                    const uint32_t o = ks * 32;
                    const uint64_t ah = umma_desc(smem_u32(a2) + o);
                    const uint64_t al = umma_desc(smem_u32(a2) + TC_KB * 4 + o);
                    const uint64_t bh = umma_desc(smem_u32(b2h) + o);
                    const uint64_t bl = umma_desc(smem_u32(b2l) + o);
                    umma_tf32(dt, ah, bh, 1u);
                    umma_tf32(dt, ah, bl, 1u);
                    umma_tf32(dt, al, bh, 1u);
                }
                umma_commit(&aux->mb_g2);
            }
            if (live2) {
                if (!wait_mbar_bounded(&aux->mb_g2, ph_g2, p.timeout_ns)) {
                    pend2 = true;
                    if (tid == 0) {
                        aux->bail = 1;
                        raise_error(p.state, epoch, IIR_DEV_ERR_MBARRIER);
                    }
                } else {
                    ph_g2 ^= 1u;
                }
            }
            tc_fence_after();
            if (warp < 2 && !aux->bail) {
                const long long ts = static_cast<long long>(tp) * TC_TILE;
                const int m = warp * 32 + lane;
                for (int c = 0; c < TC_NB; c += 16) {
                    float v[16];
                    tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + ps * TC_NB + c, v);
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const long long g = ts + static_cast<long long>(c + i) * TC_L + m;
                        if (g < p.n) p.y[g] = v[i];
                    }
                }
            }
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
        __syncthreads();
        if (aux->bail) break;
    }
    // an MMA whose completion wait ran out may still run: wait again (bounded) before freeing
    if (pend1) (void)wait_mbar_bounded(&aux->mb_g1, ph_g1, p.timeout_ns);
    if (pend2) (void)wait_mbar_bounded(&aux->mb_g2, ph_g2, p.timeout_ns);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
    if (tid == 0) pipe_finish(p.state, epoch);
}

}  // namespace iirgb

// -------------------------------------------------------------------------------------------
// host: FP64 operators of the cascade over one chunk, operand images, lookback tables, launch
// -------------------------------------------------------------------------------------------
namespace iirhost {

using iirgb::TC_DMAX;
using iirgb::TC_KB;
using iirgb::TC_L;
using iirgb::TC_NB;
using iirgb::TC_TILE;

struct TcPlan {
    int D = 0, KD = 0, sms = 0, grid_max = 0;
    bool input_normal = false;  // carried states in the input-normal basis (else balanced)
    const void* fn = nullptr;
    float* d_tabs = nullptr;  // a1 image, a2 image, phi, phix, phi_grp, pc, pg (one allocation)
    size_t off_a2 = 0, off_phi = 0, off_phix = 0, off_grp = 0, off_pc = 0, off_pg = 0;
    IirLaunchState* d_state = nullptr;
    unsigned long long* d_carry = nullptr;
    size_t carry_cap = 0, carry_bytes = 0;
    unsigned long long launches = 0;
};

namespace {

// Runs the normalised cascade (gain g on the input) over L samples of x from states S0 (D =
// 2K: y_s[-2], y_s[-1]) and input history X0 (x[-2], x[-1]); returns the last section's output
// and every section's output.
void cascade_run(const SectionF32* s, int K, double g, const double* x, int L, const double* S0, const double* X0,
                 std::vector<double>& yK, std::vector<double>& Send, std::vector<std::vector<double>>* all) {
    std::vector<double> u(static_cast<size_t>(L)), v(static_cast<size_t>(L));
    for (int n = 0; n < L; ++n) u[n] = g * x[n];
    double u2 = g * X0[0], u1 = g * X0[1];  // input history of the current section
    Send.assign(static_cast<size_t>(2 * K), 0.0);
    if (all) all->assign(static_cast<size_t>(K), std::vector<double>(static_cast<size_t>(L)));
    for (int k = 0; k < K; ++k) {
        const double b1 = s[k].b1, b2 = s[k].b2, a1 = s[k].a1, a2 = s[k].a2;
        double y2 = S0[2 * k], y1 = S0[2 * k + 1];
        const double ny2 = y2, ny1 = y1;  // this section's output history = next section's input history
        double p2 = u2, p1 = u1;
        for (int n = 0; n < L; ++n) {
            const double w = u[n] + b1 * p1 + b2 * p2;
            const double y = w + a1 * y1 + a2 * y2;
            p2 = p1;
            p1 = u[n];
            y2 = y1;
            y1 = y;
            v[n] = y;
        }
        Send[2 * k] = L >= 2 ? v[L - 2] : ny1;
        Send[2 * k + 1] = v[L - 1];
        if (all) (*all)[k] = v;
        u.swap(v);
        u2 = ny2;
        u1 = ny1;
    }
    yK = u;
}

using Mat = std::vector<double>;  // row-major n x n
Mat matmul(const Mat& A, const Mat& B, int n) {
    Mat C(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
            const double a = A[i * n + k];
            if (a == 0.0) continue;
            for (int j = 0; j < n; ++j) C[i * n + j] += a * B[k * n + j];
        }
    return C;
}
Mat identity(int n) {
    Mat I(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
    return I;
}
Mat matpow(Mat A, unsigned long long e, int n) {
    Mat R = identity(n);
    while (e) {
        if (e & 1ull) R = matmul(R, A, n);
        A = matmul(A, A, n);
        e >>= 1;
    }
    return R;
}

int swz32h(int r, int c) { return (r << 5) + ((((c >> 2) ^ (r & 7))) << 2) + (c & 3); }
float tf32_hi_h(float v) {  // nearest TF32 value (as tf32_hi on the device)
    uint32_t u;
    std::memcpy(&u, &v, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float h;
    std::memcpy(&h, &u, 4);
    return h;
}

// 2D tensor map: x as rows of 64 samples (one chunk per row), box {32, 128}, 128-byte swizzle.
bool encode_chunk_rows_map(CUtensorMap* map, const float* base, long long n);

// Chunk operators of the cascade (FP64): A1 rows 0..63 = T, rows 64..64+D-1 = B; A2 columns
// 0..D-1 = H, D..D+1 = Hx; Phi (TC_DMAX x TC_DMAX), Phix (TC_DMAX x 2).
struct ChunkOps {
    std::vector<double> A1, A2, Phi, Phix;
};

// y of the chunk system over `chunks` chunks of x from zero state (FP64), for the basis check.
std::vector<double> chunk_system_run(const ChunkOps& o, int D, const std::vector<double>& x, int chunks) {
    std::vector<double> y(x.size(), 0.0), S(static_cast<size_t>(D), 0.0), Sn(static_cast<size_t>(D));
    for (int j = 0; j < chunks; ++j) {
        const double* xj = x.data() + static_cast<size_t>(j) * TC_L;
        const double xh[2] = {j ? xj[-2] : 0.0, j ? xj[-1] : 0.0};
        for (int m = 0; m < TC_L; ++m) {
            double a = 0.0;
            for (int c = 0; c < TC_L; ++c) a += o.A1[m * TC_L + c] * xj[c];
            for (int e = 0; e < D; ++e) a += o.A2[m * 32 + e] * S[e];
            a += o.A2[m * 32 + D] * xh[0] + o.A2[m * 32 + D + 1] * xh[1];
            y[static_cast<size_t>(j) * TC_L + m] = a;
        }
        for (int r = 0; r < D; ++r) {
            double a = o.Phix[r * 2] * xh[0] + o.Phix[r * 2 + 1] * xh[1];
            for (int e = 0; e < D; ++e) a += o.Phi[r * TC_DMAX + e] * S[e];
            for (int c = 0; c < TC_L; ++c) a += o.A1[(64 + r) * TC_L + c] * xj[c];
            Sn[r] = a;
        }
        S = Sn;
    }
    return y;
}

// Chooses the carried-state basis S = R S' (Phi' = R^-1 Phi R, Phix' = R^-1 Phix, B' = R^-1 B,
// H' = H R). The cascade's own states (y_s[-2], y_s[-1] of every section) of a low-cutoff filter
// are nearly collinear and differ by decades in size, so the output H S is a small difference
// of large terms and float32 state arithmetic loses digits. The input-normal basis makes the
// state covariance under unit white input the identity (R = Cholesky factor of the
// controllability Gramian P = sum_n s(n) s(n)^T of the impulse's state trajectory): every state
// then has unit variance, no state is a near-copy of another, and |H' S'| terms stay of the
// size of the output. The transformed operators are checked against the plain ones in FP64 on
// a random input; if the check (or the factorization) fails, the diagonal balancing (each
// section's states scaled by its RMS gain) is used instead.
bool state_basis(const SectionF32* secs, int K, double gain, std::vector<double>& A1, std::vector<double>& A2,
                 std::vector<double>& Phi, std::vector<double>& Phix) {
    const int D = 2 * K, L = TC_L;
    const int NL = 1 << 16;
    std::vector<double> imp(static_cast<size_t>(NL), 0.0), yk, se, S0(static_cast<size_t>(D), 0.0);
    const double X0z[2] = {0.0, 0.0};
    std::vector<std::vector<double>> hs;
    imp[0] = 1.0;
    cascade_run(secs, K, gain, imp.data(), NL, S0.data(), X0z, yk, se, &hs);
    // Gramian of the state trajectory s(n) = (y_s[n-2], y_s[n-1])_s
    std::vector<double> P(static_cast<size_t>(D) * D, 0.0), s(static_cast<size_t>(D));
    for (int n = 0; n < NL; ++n) {
        for (int k = 0; k < K; ++k) {
            s[2 * k] = n >= 2 ? hs[k][n - 2] : 0.0;
            s[2 * k + 1] = n >= 1 ? hs[k][n - 1] : 0.0;
        }
        for (int i = 0; i < D; ++i)
            for (int j = 0; j <= i; ++j) P[i * D + j] += s[i] * s[j];
    }
    const ChunkOps plain{A1, A2, Phi, Phix};
    bool ok = true;
    std::vector<double> dsc(static_cast<size_t>(D)), C(static_cast<size_t>(D) * D, 0.0);
    for (int i = 0; i < D && ok; ++i) {
        dsc[i] = std::sqrt(P[i * D + i]);
        ok = dsc[i] > 0.0 && std::isfinite(dsc[i]);
    }
    // Cholesky of the unit-diagonal Gramian P / (dsc dsc^T) = C C^T; R = diag(dsc) C
    for (int j = 0; j < D && ok; ++j) {
        double d = P[j * D + j] / (dsc[j] * dsc[j]);
        for (int k = 0; k < j; ++k) d -= C[j * D + k] * C[j * D + k];
        if (!(d > 0.0)) {
            ok = false;
            break;
        }
        C[j * D + j] = std::sqrt(d);
        for (int i = j + 1; i < D; ++i) {
            double v = P[i * D + j] / (dsc[i] * dsc[j]);
            for (int k = 0; k < j; ++k) v -= C[i * D + k] * C[j * D + k];
            C[i * D + j] = v / C[j * D + j];
        }
    }
    ChunkOps t = plain;
    if (ok) {
        // Rinv_apply: v <- R^-1 v = C^-1 (v / dsc) by forward substitution
        auto rinv = [&](double* v, int stride) {
            for (int i = 0; i < D; ++i) {
                double a = v[i * stride] / dsc[i];
                for (int k = 0; k < i; ++k) a -= C[i * D + k] * v[k * stride];
                v[i * stride] = a / C[i * D + i];
            }
        };
        // R e_c = dsc * C[:, c] (column c of R)
        std::vector<double> R(static_cast<size_t>(D) * D, 0.0);
        for (int i = 0; i < D; ++i)
            for (int c = 0; c <= i; ++c) R[i * D + c] = dsc[i] * C[i * D + c];
        // Phi R, then R^-1 (Phi R) column by column
        std::vector<double> PR(static_cast<size_t>(D) * D, 0.0);
        for (int i = 0; i < D; ++i)
            for (int c = 0; c < D; ++c) {
                double a = 0.0;
                for (int e = c; e < D; ++e) a += plain.Phi[i * TC_DMAX + e] * R[e * D + c];
                PR[i * D + c] = a;
            }
        for (int c = 0; c < D; ++c) rinv(&PR[c], D);
        for (int i = 0; i < D; ++i)
            for (int c = 0; c < D; ++c) t.Phi[i * TC_DMAX + c] = PR[i * D + c];
        for (int c = 0; c < 2; ++c) rinv(&t.Phix[c], 2);
        for (int c = 0; c < L; ++c) rinv(&t.A1[64 * L + c], L);
        for (int m = 0; m < L; ++m)
            for (int c = 0; c < D; ++c) {
                double a = 0.0;
                for (int e = c; e < D; ++e) a += plain.A2[m * 32 + e] * R[e * D + c];
                t.A2[m * 32 + c] = a;
            }
        // FP64 check of the transformed operators on a seeded random input (8 chunks)
        std::vector<double> xr(static_cast<size_t>(8) * L);
        uint64_t st = 0x9E3779B97F4A7C15ull;
        for (double& v : xr) {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            v = static_cast<double>(static_cast<int64_t>(st >> 11) - (1ll << 52)) / static_cast<double>(1ll << 52);
        }
        const std::vector<double> y0 = chunk_system_run(plain, D, xr, 8), y1 = chunk_system_run(t, D, xr, 8);
        double emax = 0.0, ymax = 0.0;
        for (size_t i = 0; i < y0.size(); ++i) {
            emax = std::max(emax, std::fabs(y1[i] - y0[i]));
            ymax = std::max(ymax, std::fabs(y0[i]));
        }
        ok = std::isfinite(emax) && emax <= 1e-10 * std::max(ymax, 1e-300);
    }
    if (!ok) {
        t = plain;
        for (int k = 0; k < K; ++k) {
            double e2 = 0.0;
            for (double v : hs[k]) e2 += v * v;
            const double gk = std::sqrt(e2);
            const double w = (gk > 0.0 && std::isfinite(gk)) ? 1.0 / gk : 1.0;
            for (int r = 2 * k; r < 2 * k + 2; ++r) {
                for (int c = 0; c < D; ++c) t.Phi[r * TC_DMAX + c] *= w;
                for (int c = 0; c < D; ++c) t.Phi[c * TC_DMAX + r] /= w;
                t.Phix[r * 2] *= w;
                t.Phix[r * 2 + 1] *= w;
                for (int c = 0; c < L; ++c) t.A1[(64 + r) * L + c] *= w;
                for (int m = 0; m < L; ++m) t.A2[m * 32 + r] /= w;
            }
        }
    }
    A1.swap(t.A1);
    A2.swap(t.A2);
    Phi.swap(t.Phi);
    Phix.swap(t.Phix);
    return ok;
}

template <int KD>
const void* tc_kernel_fn() {
    return reinterpret_cast<const void*>(iirgb::iir_tc_kernel<KD>);
}

}  // namespace

void tc_plan_destroy(TcPlan* t) {
    if (!t) return;
    cudaDeviceSynchronize();
    if (t->d_tabs) cudaFree(t->d_tabs);
    if (t->d_state) cudaFree(t->d_state);
    if (t->d_carry) cudaFree(t->d_carry);
    delete t;
}

IirLaunchState* tc_plan_state(TcPlan* t) { return t ? t->d_state : nullptr; }
int tc_plan_grid(const TcPlan* t) { return t ? t->grid_max : 0; }

static int tc_alloc_carry(TcPlan* t, size_t tiles) {
    if (t->d_carry) cudaFree(t->d_carry);
    t->d_carry = nullptr;
    tiles = std::max<size_t>(tiles, 1);
    const size_t words = 2 * static_cast<size_t>(t->KD) * (tiles + tiles / 32 + 2);
    int st = cuda_status(cudaMalloc(&t->d_carry, words * 8));
    if (!st) st = cuda_status(cudaMemset(t->d_carry, 0, words * 8));
    if (st) return st;
    t->carry_cap = tiles;
    t->carry_bytes = words * 8;
    return IIR_OK;
}

int tc_plan_create(TcPlan** out, const SectionF32* secs, int K, double gain, size_t max_n) {
    *out = nullptr;
    if (K < 1 || K > IIR_MAX_SECTIONS) return IIR_ERR_INVALID_ARGUMENT;
    TcPlan* t = new TcPlan();
    const int D = 2 * K;
    t->D = D;
    t->KD = D <= 2 ? 2 : D <= 4 ? 4 : D <= 8 ? 8 : 16;
    const int L = TC_L;
    // ---- FP64 operators ----
    std::vector<double> zero(static_cast<size_t>(L), 0.0), imp(static_cast<size_t>(L), 0.0), S0(static_cast<size_t>(D), 0.0);
    const double X0z[2] = {0.0, 0.0};
    imp[0] = 1.0;
    std::vector<double> h, Send;
    std::vector<std::vector<double>> hs;
    cascade_run(secs, K, gain, imp.data(), L, S0.data(), X0z, h, Send, &hs);  // impulse responses
    std::vector<double> A1(static_cast<size_t>(128) * L, 0.0), A2(static_cast<size_t>(128) * 32, 0.0);
    for (int m = 0; m < L; ++m)
        for (int c = 0; c <= m; ++c) A1[m * L + c] = h[m - c];
    for (int k = 0; k < K; ++k)
        for (int c = 0; c < L; ++c) {
            A1[(64 + 2 * k) * L + c] = (L - 2 - c >= 0) ? hs[k][L - 2 - c] : 0.0;
            A1[(64 + 2 * k + 1) * L + c] = hs[k][L - 1 - c];
        }
    Mat Phi(static_cast<size_t>(TC_DMAX) * TC_DMAX, 0.0);
    std::vector<double> Phix(static_cast<size_t>(TC_DMAX) * 2, 0.0);
    for (int dcol = 0; dcol < D + 2; ++dcol) {
        std::vector<double> S(static_cast<size_t>(D), 0.0);
        double X0[2] = {0.0, 0.0};
        if (dcol < D) S[dcol] = 1.0;
        else X0[dcol - D] = 1.0;
        std::vector<double> yk, se;
        cascade_run(secs, K, gain, zero.data(), L, S.data(), X0, yk, se, nullptr);
        for (int m = 0; m < L; ++m) A2[m * 32 + dcol] = yk[m];
        for (int r = 0; r < D; ++r) {
            if (dcol < D) Phi[r * TC_DMAX + dcol] = se[r];
            else Phix[r * 2 + (dcol - D)] = se[r];
        }
    }
    // ---- state basis: input-normal, else per-section balanced (see state_basis) ----
    t->input_normal = state_basis(secs, K, gain, A1, A2, Phi, Phix);
    // ---- host images (float, swizzled, TF32 hi / lo) and tables ----
    std::vector<float> img1(static_cast<size_t>(4) * TC_KB, 0.f), img2(static_cast<size_t>(2) * TC_KB, 0.f);
    for (int m = 0; m < 128; ++m)
        for (int c = 0; c < L; ++c) {
            const float v = static_cast<float>(A1[m * L + c]);
            const float hv = tf32_hi_h(v);
            const size_t idx = static_cast<size_t>(c >> 5) * TC_KB + swz32h(m, c & 31);
            img1[idx] = hv;
            img1[2 * TC_KB + idx] = tf32_hi_h(v - hv);
        }
    for (int m = 0; m < 128; ++m)
        for (int c = 0; c < 32; ++c) {
            const float v = static_cast<float>(A2[m * 32 + c]);
            const float hv = tf32_hi_h(v);
            img2[swz32h(m, c)] = hv;
            img2[TC_KB + swz32h(m, c)] = tf32_hi_h(v - hv);
        }
    const int KD = t->KD;
    std::vector<float> phi(TC_DMAX * TC_DMAX), phix(TC_DMAX * 2), grp(static_cast<size_t>(16) * TC_DMAX * TC_DMAX),
        pc(static_cast<size_t>(33) * KD * KD), pg(static_cast<size_t>(33) * KD * KD);
    for (size_t i = 0; i < phi.size(); ++i) phi[i] = static_cast<float>(Phi[i]);
    for (size_t i = 0; i < phix.size(); ++i) phix[i] = static_cast<float>(Phix[i]);
    const Mat Phi8 = matpow(Phi, 8, TC_DMAX);
    Mat P = identity(TC_DMAX);
    for (int g = 0; g < 16; ++g) {
        for (int i = 0; i < TC_DMAX * TC_DMAX; ++i) grp[static_cast<size_t>(g) * TC_DMAX * TC_DMAX + i] = static_cast<float>(P[i]);
        P = matmul(P, Phi8, TC_DMAX);
    }
    const Mat Q = matpow(Phi, TC_NB, TC_DMAX);        // tile transition
    const Mat Q32 = matpow(Q, 32, TC_DMAX);
    Mat Pq = identity(TC_DMAX), Pq32 = identity(TC_DMAX);
    for (int l = 0; l <= 32; ++l) {
        for (int i = 0; i < KD; ++i)
            for (int j = 0; j < KD; ++j) {
                pc[(static_cast<size_t>(l) * KD + i) * KD + j] = static_cast<float>(Pq[i * TC_DMAX + j]);
                pg[(static_cast<size_t>(l) * KD + i) * KD + j] = static_cast<float>(Pq32[i * TC_DMAX + j]);
            }
        Pq = matmul(Pq, Q, TC_DMAX);
        Pq32 = matmul(Pq32, Q32, TC_DMAX);
    }
    // ---- device ----
    std::vector<float> all;
    auto put = [&](const std::vector<float>& v) {
        const size_t off = all.size();
        all.insert(all.end(), v.begin(), v.end());
        while (all.size() % 4) all.push_back(0.f);  // 16-byte aligned parts
        return off;
    };
    put(img1);
    t->off_a2 = put(img2);
    t->off_phi = put(phi);
    t->off_phix = put(phix);
    t->off_grp = put(grp);
    t->off_pc = put(pc);
    t->off_pg = put(pg);
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev));
    if (!st) st = cuda_status(cudaDeviceGetAttribute(&t->sms, cudaDevAttrMultiProcessorCount, dev));
    if (!st) st = cuda_status(cudaMalloc(&t->d_tabs, all.size() * sizeof(float)));
    if (!st) st = cuda_status(cudaMemcpy(t->d_tabs, all.data(), all.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (!st) st = cuda_status(cudaMalloc(&t->d_state, sizeof(IirLaunchState)));
    if (!st) st = cuda_status(cudaMemset(t->d_state, 0, sizeof(IirLaunchState)));
    if (!st) st = tc_alloc_carry(t, (std::max<size_t>(max_n, 1) + TC_TILE - 1) / TC_TILE);
    if (!st) {
        t->fn = KD == 2 ? tc_kernel_fn<2>() : KD == 4 ? tc_kernel_fn<4>() : KD == 8 ? tc_kernel_fn<8>() : tc_kernel_fn<16>();
        st = cuda_status(cudaFuncSetAttribute(t->fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              static_cast<int>(iirgb::TcSmem::BYTES)));
    }
    if (!st) {
        int nb = 0;
        st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, t->fn, iirgb::TC_THREADS, iirgb::TcSmem::BYTES));
        if (!st && nb < 1) st = IIR_ERR_UNSUPPORTED;
        t->grid_max = std::max(nb, 1) * t->sms;
    }
    if (st) {
        tc_plan_destroy(t);
        return st;
    }
    *out = t;
    return IIR_OK;
}

int tc_plan_execute(TcPlan* t, const float* x, float* y, size_t n, long long timeout_ns, long long withhold,
                    cudaStream_t stream) {
    const size_t tiles = (n + TC_TILE - 1) / TC_TILE;
    if (tiles > 0x7fffffffull) return IIR_ERR_TOO_LARGE;
    if (tiles > t->carry_cap) {
        cudaStreamSynchronize(stream);
        const int st = tc_alloc_carry(t, tiles);
        if (st) return st;
    }
    if (++t->launches >= (1ull << 30)) {
        int st = cuda_status(cudaMemsetAsync(t->d_carry, 0, t->carry_bytes, stream));
        if (!st) st = cuda_status(cudaMemsetAsync(t->d_state, 0, sizeof(IirLaunchState), stream));
        if (st) return st;
        t->launches = 1;
    }
    iirgb::TcParams q;
    std::memset(&q, 0, sizeof(q));
    q.x = x;
    q.y = y;
    q.n = static_cast<long long>(n);
    q.state = t->d_state;
    q.carry = t->d_carry;
    q.a1img = t->d_tabs;
    q.a2img = t->d_tabs + t->off_a2;
    q.phi = t->d_tabs + t->off_phi;
    q.phix = t->d_tabs + t->off_phix;
    q.phi_grp = t->d_tabs + t->off_grp;
    q.pc = t->d_tabs + t->off_pc;
    q.pg = t->d_tabs + t->off_pg;
    q.timeout_ns = timeout_ns;
    q.withhold_chunk = withhold;
    q.ntiles = static_cast<unsigned int>(tiles);
    q.carry_cap = static_cast<unsigned int>(t->carry_cap);
    q.D = t->D;
    q.use_tma = encode_chunk_rows_map(&q.tmap_x, x, static_cast<long long>(n)) ? 1 : 0;
    void* args[] = {&q};
    const int grid = static_cast<int>(std::min<size_t>(tiles, static_cast<size_t>(t->grid_max)));
    return cuda_status(cudaLaunchCooperativeKernel(t->fn, dim3(grid), dim3(iirgb::TC_THREADS), args,
                                                   iirgb::TcSmem::BYTES, stream));
}

namespace {
bool encode_chunk_rows_map(CUtensorMap* map, const float* base, long long n) {
    return encode_rows_map(map, base, n / TC_L, TC_L, 32, TC_NB);
}
}  // namespace

}  // namespace iirhost
