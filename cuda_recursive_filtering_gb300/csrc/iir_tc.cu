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
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/iir_gb300.h"
#include "iir_host_internal.h"
#include "iir_lookk.cuh"
#include "iir_pipe.cuh"

// Largest carried-state count whose tiles the two compute groups split in halves and whose back
// group frees an accumulator before preparing the next tile. The two go together: the shared
// split is validated only with that order (with the other order, preparation first, it gave wrong
// output at 16 states in a trial). Measured at 2^28: faster up to 8 states (order 8: 358 against
// 334 GS/s), slower at 16 (orders 10 / 16: 302 / 336 against 307 / 342 GS/s).
#ifndef IIR_TC_SHARED_MAX_KD
#define IIR_TC_SHARED_MAX_KD 8
#endif

namespace iirgb {

constexpr int TC_L = 64;                  // samples per chunk (GEMM K)
constexpr int TC_NB = 128;                // chunks per tile (GEMM M)
constexpr int TC_TILE = TC_L * TC_NB;     // samples per tile
constexpr int TC_LBW = 1;                 // lookback warps (tiles alternate between them)
constexpr int TC_MW = TC_LBW;             // MMA warp
constexpr int TC_CW0 = TC_LBW + 1;        // first front warp; the back warps follow
constexpr int TC_CW = 8;                  // warps per compute group (front, back)
constexpr int TC_CT = 32 * TC_CW;         // threads per compute group
constexpr int TC_THREADS = 32 * (TC_CW0 + 2 * TC_CW);
constexpr int TC_NACC = 3;                // TMEM accumulators (tiles in flight between GEMM 1 and the outputs)
constexpr int TC_NS = TC_NACC;            // aggregate / X hand-off slots
constexpr int TC_NXH = TC_NACC + 2;       // input-history slots
constexpr int TC_XCOL = 256;              // TMEM columns of the x operand: 2 buffers x [hi 64 | lo 64]
constexpr int TC_DMAX = 16;               // carried states (order <= 16)
constexpr int TC_GROUPS_MAX = 32;         // most scan sub-blocks of a tile
constexpr int TC_LEVELS_MAX = 5;          // most combine levels (log2 of the sub-blocks)

// The scans of a tile's 128 chunks: each compute group splits them into sub-blocks, scanned in
// parallel by LG lanes each (lane = state component), then joined by a Kogge-Stone combine over
// the sub-blocks with Phi^(SUB 2^l). Fewer states need fewer lanes, so a cascade of up to 8 states
// runs twice the sub-blocks at half the length (32 x 4 chunks, 5 combine levels) where 16 states
// take 16 x 8 chunks and 4 levels: the scan and rescan, the kernel's serial CUDA-core phases, take
// half the steps.
template <int KD>
struct TcScan {
    static constexpr int LG_SHIFT = KD <= 8 ? 3 : 4;
    static constexpr int LG = 1 << LG_SHIFT;  // lanes per sub-block
    static constexpr int GROUPS = TC_CW * 32 / LG;
    static constexpr int SUB = TC_NB / GROUPS;   // chunks per sub-block
    static constexpr int LEVELS = GROUPS == 32 ? 5 : 4;
    static_assert(KD <= LG && GROUPS <= TC_GROUPS_MAX && LEVELS <= TC_LEVELS_MAX && (1 << LEVELS) == GROUPS, "scan shape");
    static_assert(2 * SUB <= LG, "one lane per history column of a sub-block's chunks");
};
constexpr int tc_scan_sub(int kd) { return kd <= 8 ? 4 : 8; }  // TcScan<KD>::SUB, for the host
constexpr int TC_N1 = 80;                 // GEMM 1 N: 64 outputs + 16 end states
constexpr int TC_N2 = 64;                 // GEMM 2 N: 64 outputs
constexpr int TC_ACC = 80;                // TMEM columns per accumulator
constexpr int TC_KB = 32 * TC_NB;         // floats of one swizzled [128 rows x 32] block
constexpr int TC_B1KB = 32 * TC_N1;       // floats of one swizzled [80 rows x 32] block
constexpr int TC_H2B = 32 * TC_N2;        // floats of one swizzled [64 rows x 32] block
constexpr int TC_UP = 17;                 // padded row of the end-state transpose
constexpr int TC_LB_MAX = 4;              // deepest truncated lookback (tiles)

struct TcParams {
    CUtensorMap tmap_x;          // x as [n/64 rows][64], box {32, 128}, 128-byte swizzle
    CUtensorMap tmap_y;          // y, the same way (output tiles leave by TMA stores)
    const float* x;
    float* y;
    long long n;
    IirLaunchState* state;
    unsigned long long* carry;   // per tile slot 2*KD words, then per group of 32 tiles
    const float* b1img;          // GEMM 1 B operand [T; B]: [hi kb0, hi kb1, lo kb0, lo kb1] x TC_B1KB
    const float* h2img;          // GEMM 2 B operand [H | Hx]: [hi, lo] x TC_H2B
    const float* phi;            // 16 x 16 (row-major, zero beyond D)
    const float* phix;           // 16 x 2
    const float* phi_pow;        // Phi^(SUB * 2^b), b < TC_LEVELS_MAX: [b][e / 4][d][e % 4] = P[d][e]
    const float* pc;             // Q^l (l <= 32), KD x KD
    const float* pg;             // Q^(32 l) (l <= 32), KD x KD
    long long timeout_ns;
    long long withhold_chunk;
    unsigned int ntiles;
    unsigned int carry_cap;
    int D;
    int use_tma;
    int use_tma_y;               // tmap_y is valid
    int y_vec;                   // y is 16-byte aligned
    int lb_depth;                // truncated lookback depth m (||Q^m|| <= 1e-10), 0: full lookback
    unsigned long long* prof;
};

template <int G>
struct TcAuxG {
    static constexpr int LEVELS = G == 32 ? 5 : 4;
    unsigned long long mb_tma[2], mb_g1[2], mb_g2, mb_split[2], mb_sready, mb_accfree, mb_agg[TC_NS], mb_x[TC_NS];
    uint32_t tmem;
    uint32_t epoch;
    int bail;
    uint32_t g1_issued, g2_issued;   // MMA batches committed (by the MMA warp)
    int pad;
    float agg[TC_NS][TC_DMAX];       // tile aggregate (zero incoming state), for the lookback warp
    float X[TC_NS][TC_DMAX];         // incoming state of the tile, from the lookback warp
    float Ig0[TC_NACC][G][TC_DMAX];  // zero-start incoming state of each sub-block, per tile
    float xh[TC_NXH][TC_NB][2];      // input history of each chunk, per tile
    alignas(16) float phip[LEVELS][TC_DMAX / 4][TC_DMAX][4];  // Phi^(SUB 2^b): [b][e / 4][d][e % 4] = P[d][e]
};

// Shared-memory layout for a scan of G sub-blocks (TcScan<KD>::GROUPS): only the scratch areas of
// the two compute groups depend on it.
template <int G>
struct TcSmemG {
    static constexpr size_t B1 = 0;                             // 4 x TC_B1KB floats
    static constexpr size_t H2 = B1 + 4 * TC_B1KB * 4;          // 2 x TC_H2B
    static constexpr size_t XS = H2 + 2 * TC_H2B * 4;           // 2 stages x 2 k-blocks x TC_KB (TMA target)
    static constexpr size_t A2S = XS + 4 * TC_KB * 4;           // state operand [hi, lo] x TC_KB
    static constexpr size_t SCRF = A2S + 2 * TC_KB * 4;         // front scratch: end-state rows, combine
    static constexpr size_t SCRF_BYTES = (TC_NB * TC_UP + 3 * G * TC_DMAX) * 4;
    static constexpr size_t SCRB = SCRF + SCRF_BYTES;           // back scratch: end-state rows, states, patches
    static constexpr size_t SCRB_BYTES = (TC_NB * TC_UP + G * TC_DMAX + TC_CW * 32 * 8) * 4;
    static constexpr size_t AUX = (SCRB + SCRB_BYTES + 15) / 16 * 16;
    static constexpr size_t BYTES = 1024 + AUX + sizeof(TcAuxG<G>);
    static_assert(H2 % 1024 == 0 && XS % 1024 == 0 && A2S % 1024 == 0, "operand blocks on the 1024-byte swizzle atom");
    static_assert(BYTES <= 232448, "shared memory");
};
template <int KD>
using TcSmem = TcSmemG<TcScan<KD>::GROUPS>;
constexpr size_t tc_smem_bytes(int kd) { return kd <= 8 ? TcSmemG<32>::BYTES : TcSmemG<16>::BYTES; }
static_assert(TC_NACC * TC_ACC <= TC_XCOL && TC_XCOL + 256 <= 512, "TMEM columns");

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
// kind::tf32, D f32, A / B tf32 K-major, M = 128
constexpr uint32_t tc_idesc(int n) { return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((128 >> 4) << 24); }
constexpr uint32_t TC_IDESC1 = tc_idesc(TC_N1);
constexpr uint32_t TC_IDESC2 = tc_idesc(TC_N2);

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
// A from TMEM (M = 128 lanes, K consecutive 32-bit columns), B from shared memory
__device__ __forceinline__ void umma_tf32_ta(uint32_t tmem, uint32_t ta, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem),
        "r"(ta), "l"(db), "r"(idesc), "r"(acc));
}
// BF16 operands (kind::f16): D f32, A / B bf16 K-major, M = 128. A from TMEM packs two bf16 per
// 32-bit column (the lower K index in the low half).
constexpr uint32_t tc_idesc_bf16(int n) { return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128 >> 4) << 24); }
constexpr uint32_t TC_IDESC1_BF16 = tc_idesc_bf16(TC_N1);
__device__ __forceinline__ void umma_bf16_ta(uint32_t tmem, uint32_t ta, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem),
        "r"(ta), "l"(db), "r"(idesc), "r"(acc));
}
// Products of the BF16 split form: BF = 6 takes three parts of each operand (x = b0 + b1 + b2,
// each the nearest bf16 of what the earlier parts left) and the six products whose parts' ranks
// sum to at most 2, which keeps float32 accuracy; BF = 3 takes two parts and b0 c0 + b0 c1 + b1 c0.
template <int BF>
struct TcBf16 {
    static constexpr int PARTS = BF == 6 ? 3 : 2;
    static constexpr int NPROD = BF;
    __device__ static constexpr int a_part(int i) { return i == 0 ? 0 : i == 1 ? 0 : i == 2 ? 1 : i == 3 ? 0 : i == 4 ? 1 : 2; }
    __device__ static constexpr int b_part(int i) { return i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 0 : i == 3 ? 2 : i == 4 ? 1 : 0; }
};
constexpr int TC_BF_PART_BYTES = TC_N1 * 128;  // one bf16 part of the GEMM 1 B image: 80 rows x 64 bf16
static_assert(3 * TC_BF_PART_BYTES <= 4 * TC_B1KB * 4 && TC_BF_PART_BYTES % 1024 == 0, "bf16 image in the B1 area");
__device__ __forceinline__ uint32_t bf16_pair(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half), .y = hi
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ void tmem_st8u(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(v[0]),
                 "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
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
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// barrier of one compute group (named barrier 1: front, 2: back)
__device__ __forceinline__ void bar_group(int id) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(TC_CT) : "memory"); }

// TF32 hi / lo split of 16 samples of the staged tile xt (half `half` of k-block kb of this
// thread's chunk row r, 128-byte swizzled rows of 32 samples) into the x operand columns of TMEM:
// hi at xa + 16 half, lo at xa + 64 + 16 half (xa: the k-block's first column, this warp's lanes).
__device__ __forceinline__ void tc_split16(const float* xt, int kb, int half, int r, uint32_t xa) {
    const float4* row = reinterpret_cast<const float4*>(xt + kb * TC_KB + r * 32);
    float hi[16], lo[16];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float4 v = row[(4 * half + c) ^ (r & 7)];
        const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            hi[4 * c + j] = tf32_hi(e[j]);
            lo[4 * c + j] = tf32_hi(e[j] - hi[4 * c + j]);
        }
    }
    tmem_st16(xa + 16 * half, hi);
    tmem_st16(xa + 64 + 16 * half, lo);
}

// Optional timeline (compiled in with -DIIR_PROFILE): per block, per tile iteration k < 16,
// 16 SM-clock stamps.
#ifdef IIR_PROFILE
#define TC_STAMP(k, slot)                                                                                 \
    do {                                                                                                  \
        if (p.prof && (k) < 16u) p.prof[(static_cast<size_t>(blockIdx.x) * 16 + (k)) * 16 + (slot)] = clock64(); \
    } while (0)
#else
#define TC_STAMP(k, slot) \
    do {                  \
    } while (0)
#endif

// Barrier of one compute group that also returns, to every one of its threads, whether any passed `v`.
__device__ __forceinline__ bool bar_group_any(int id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(v)), "r"(id), "r"(TC_CT)
        : "memory");
    return r != 0u;
}

// Bounded mbarrier wait that also gives up once another thread of the block has given up.
__device__ __forceinline__ bool tc_wait(unsigned long long* bar, uint32_t parity, long long limit_ns, int* bail) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    uint32_t spins = 0;
    while (!mbar_try_wait(bar, parity)) {
        if ((++spins & 63u) == 0u) {
            if (*reinterpret_cast<volatile int*>(bail)) return false;
            if (globaltimer_ns() - t0 > static_cast<uint64_t>(limit_ns)) return false;
        }
    }
    return true;
}
// First give-up of the block reports `code`; later ones only stop.
template <class Aux>
__device__ __forceinline__ void tc_give_up(Aux* aux, const TcParams& p, uint32_t epoch, uint32_t code) {
    if (atomicExch(&aux->bail, 1) == 0) raise_error(p.state, epoch, code);
}

// Truncated lookback (one warp): X = sum_{i < m} Q^i part(t-1-i), tiles before the signal
// contribute nothing. The neglected term Q^m X(t-m) has ||Q^m|| <= 1e-10 (checked on the host
// in FP64), far below float32 resolution, so no chain of inclusive carries is needed: a tile
// waits only for the aggregates of the m tiles before it. Lane i polls tile t-1-i.
template <int KD>
__device__ bool lookback_trunc(const TcParams& p, const unsigned long long* slots, uint32_t t, uint32_t epoch, int m,
                               float (&X)[KD]) {
    const int lane = threadIdx.x & 31;
    const uint32_t pf = 2u * epoch + 1u;
    const bool mine = lane < m && static_cast<uint32_t>(lane) < t;
    float v[KD];
#pragma unroll
    for (int e = 0; e < KD; ++e) v[e] = 0.f;
    const uint64_t t0 = globaltimer_ns();
    uint32_t spin = 32;
    while (true) {
        bool ok = true;
        if (mine) {
            const unsigned long long* s = slots + static_cast<size_t>(t - 1 - lane) * 2 * KD;
#pragma unroll
            for (int i = 0; i < KD; i += 2) {
                unsigned long long a, b;
                ld_relaxed_v2(s + i, a, b);
                ok = ok && word_flag(a) == pf && word_flag(b) == pf;
                v[i] = word_val(a);
                v[i + 1] = word_val(b);
            }
        }
        if (__all_sync(FULL_MASK, ok)) break;
        int give_up = 0;
        if (lane == 0) give_up = lookback_give_up(p, epoch, t0) ? 1 : 0;
        if (__shfl_sync(FULL_MASK, give_up, 0)) return false;
        backoff(spin);
    }
    float u[KD];
    if (mine && lane > 0) {
        matvec<KD>(p.pc + static_cast<size_t>(lane) * KD * KD, v, u);
    } else {
#pragma unroll
        for (int e = 0; e < KD; ++e) u[e] = mine ? v[e] : 0.f;
    }
    if (m > 1) warp_sumk<KD>(u);
#pragma unroll
    for (int e = 0; e < KD; ++e) X[e] = __shfl_sync(FULL_MASK, u[e], 0);
    return true;
}

// Persistent tile pipeline, per block:
//   warps 0 .. TC_LBW-1  lookback of alternate tiles (truncated, or the full two-level one)
//   warp  TC_MW          tcgen05.mma issue: GEMM 1 of a staged tile once its accumulator is
//                        free, GEMM 2 of a solved tile
//   front group (TC_CW warps), per tile k:
//     b. GEMM 1 done -> end-state rows from TMEM -> sub-block scans -> aggregate -> lookback
//     a. tile k+1: TMA data landed -> input history, TF32 split -> MMA warp
//   back group (TC_CW warps), per tile k:
//     c. lookback's X -> states of the tile's chunks -> MMA warp (GEMM 2)
//     d. GEMM 2 done -> outputs from TMEM -> y -> accumulator free
// The groups meet only through mbarriers, so the back group's rescan and stores of one tile run
// beside the front group's scan and split of later tiles. TMEM holds three accumulators; x is
// double-buffered (TMA two tiles ahead); the lookback of tile k runs while the front group
// stages tile k+1 and scans it.
// FULL: the two-level decoupled lookback (tile transitions that have not decayed); otherwise the
// truncated lookback, and the two-level code is not compiled in (it would raise register use).
// BF = 0: GEMM 1 in TF32 with the hi / lo split (three products); BF = 3 or 6: GEMM 1 in BF16
// with the split of TcBf16<BF>. GEMM 2 is TF32 in every form.
template <int KD, bool FULL, int BF>
__global__ void __launch_bounds__(TC_THREADS, 1) iir_tc_kernel(const __grid_constant__ TcParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t a0 = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((a0 + 1023u) & ~1023u) - a0);
    using Sm = TcSmem<KD>;
    float* b1 = reinterpret_cast<float*>(base + Sm::B1);
    float* h2 = reinterpret_cast<float*>(base + Sm::H2);
    float* xs = reinterpret_cast<float*>(base + Sm::XS);
    float* a2s = reinterpret_cast<float*>(base + Sm::A2S);
    using TcAux = TcAuxG<TcScan<KD>::GROUPS>;
    TcAux* aux = reinterpret_cast<TcAux*>(base + Sm::AUX);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int D = p.D;
    const uint32_t G = gridDim.x;
    const uint32_t nk = (p.ntiles > blockIdx.x) ? (p.ntiles - blockIdx.x + G - 1) / G : 0;
    const long long wait_lim = p.timeout_ns < (1ll << 60) ? 4 * p.timeout_ns : p.timeout_ns;

    // ---- setup: operand images, matrix powers, zeroed state operand, TMEM, barriers ----
    {
        const float4* s1 = reinterpret_cast<const float4*>(p.b1img);
        float4* d1 = reinterpret_cast<float4*>(b1);
        for (int i = tid; i < TC_B1KB; i += TC_THREADS) d1[i] = __ldg(s1 + i);  // 4 x TC_B1KB floats
        const float4* s2 = reinterpret_cast<const float4*>(p.h2img);
        float4* d2 = reinterpret_cast<float4*>(h2);
        for (int i = tid; i < TC_H2B / 2; i += TC_THREADS) d2[i] = __ldg(s2 + i);  // 2 x TC_H2B floats
        float4* z = reinterpret_cast<float4*>(a2s);
        for (int i = tid; i < TC_KB / 2; i += TC_THREADS) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // 2 x TC_KB
        float* pp = &aux->phip[0][0][0][0];
        for (int i = tid; i < TcAux::LEVELS * TC_DMAX * TC_DMAX; i += TC_THREADS) pp[i] = __ldg(p.phi_pow + i);
    }
    if (warp == TC_MW) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&aux->tmem)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&aux->mb_tma[0], 1);
        mbar_init(&aux->mb_tma[1], 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(&aux->mb_g1[b], 1);  // per x buffer: tile k uses buffer k & 1
            mbar_init(&aux->mb_split[b], 2);  // one arrival per compute group (their halves of the split)
        }
        mbar_init(&aux->mb_g2, 1);
        mbar_init(&aux->mb_sready, 1);
        mbar_init(&aux->mb_accfree, 1);
        for (int w = 0; w < TC_NS; ++w) {
            mbar_init(&aux->mb_agg[w], 1);
            mbar_init(&aux->mb_x[w], 1);
        }
        fence_mbar_init();
        aux->epoch = static_cast<uint32_t>(*reinterpret_cast<volatile unsigned long long*>(&p.state->ticket) >> 32);
        aux->bail = 0;
        aux->g1_issued = aux->g2_issued = 0;
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = aux->tmem, epoch = aux->epoch;
    unsigned long long* slots = p.carry;
    unsigned long long* gslots = p.carry + static_cast<size_t>(p.carry_cap) * 2 * KD;
    volatile int* vbail = &aux->bail;
    auto tile_of = [&](uint32_t kk) { return blockIdx.x + kk * G; };
    // a whole tile of the signal, staged by TMA (else the front group gathers it)
    auto bulk = [&](uint32_t kk) {
        return p.use_tma && static_cast<long long>(tile_of(kk) + 1) * TC_TILE <= p.n;
    };
    // The compute groups split a TMA-staged tile in halves (front: k-block 0, back: k-block 1) and
    // arrive on mb_split once each; a gathered tile, and every tile of the BF16 forms, is split
    // whole by the front group, which then arrives for both. With 16 states the back group's
    // rescan takes twice the steps and the front's split stays whole, which balances the groups
    // better (order 8: 334 -> 358 GS/s shared; order 16: 275 shared).
    auto shared_split = [&](uint32_t kk) { return BF == 0 && KD <= IIR_TC_SHARED_MAX_KD && bulk(kk); };
    // a whole output tile leaves by TMA stores (else the back group stores it from registers)
    auto bulk_y = [&](uint32_t kk) {
        return p.use_tma_y && static_cast<long long>(tile_of(kk) + 1) * TC_TILE <= p.n;
    };

    if (warp < TC_LBW) {
        // ================= lookback warps: tiles k = warp, warp + TC_LBW, ... =================
        const uint32_t ff = 2u * epoch + 2u;
        for (uint32_t k = warp; k < nk; k += TC_LBW) {
            const int sl = k % TC_NS;
            int got = 0;
            if (lane == 0) {
                got = tc_wait(&aux->mb_agg[sl], (k / TC_NS) & 1u, wait_lim, &aux->bail) ? 1 : 0;
                if (!got) tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
                else if (*vbail) got = 0;
            }
            __syncwarp();
            if (!__shfl_sync(FULL_MASK, got, 0)) break;
            const uint32_t t = tile_of(k);
            if (lane == 0) TC_STAMP(k, 13);
            float own[KD], X[KD];
#pragma unroll
            for (int e = 0; e < KD; ++e) {
                own[e] = aux->agg[sl][e];
                X[e] = 0.f;
            }
            const bool withhold = static_cast<long long>(t) == p.withhold_chunk;
            bool ok = true;
            if constexpr (!FULL) {
                if (t > 0) ok = lookback_trunc<KD>(p, slots, t, epoch, p.lb_depth, X);
            } else if (t > 0) {
                ok = lookback_hier_k<KD>(p, slots, gslots, p.pc, p.pg, t, epoch, own, withhold, X);
            }
            if (lane == 0) {
                if (FULL && ok && !withhold) {
                    float f[KD];
                    matvec<KD>(p.pc + KD * KD, X, f);  // Q X
#pragma unroll
                    for (int e = 0; e < KD; ++e) f[e] += own[e];
                    publishk<KD>(slots + static_cast<size_t>(t) * 2 * KD + KD, ff, f);
                    if ((t & 31u) == 31u) publishk<KD>(gslots + static_cast<size_t>(t >> 5) * 2 * KD + KD, ff, f);
                }
                if (!ok) atomicExch(&aux->bail, 1);  // the lookback has reported its timeout
#pragma unroll
                for (int e = 0; e < TC_DMAX; ++e) aux->X[sl][e] = e < KD ? X[e] : 0.f;
                mbar_arrive(&aux->mb_x[sl]);
                TC_STAMP(k, 14);
            }
            __syncwarp();
            if (!ok) break;
        }
    } else if (warp == TC_MW) {
        // ===== MMA warp: GEMM 2 of a solved tile first (the back group waits on it), GEMM 1 of
        // a staged tile in four pieces of six MMAs so a ready GEMM 2 never queues behind a whole
        // GEMM 1. GEMM 1 of tile k also needs accumulator k % TC_NACC back from tile k - TC_NACC. =====
        // Every barrier phase is observed in order and at most one completed phase of each is
        // unobserved: split and GEMM 1 barriers are per x buffer (tile k + 2 is staged only after
        // GEMM 1 of tile k completed), sready(k + 1) and accfree(k + 1) need GEMM 2 of tile k,
        // which is issued only after accfree(k - 1) was observed.
        // It also issues the x tiles' TMA loads: tiles 0 and 1 at once, tile k + 2 into the buffer of
        // tile k once both groups have split tile k (seen as its split barrier completing), so at
        // most one load per buffer is in flight.
        if (lane == 0) {
            uint32_t k1 = 0, k2 = 0, piece = 0, n_free = 0;
            uint32_t tma_n[2] = {0u, 0u};  // loads issued per buffer
            auto issue_tma = [&](uint32_t kk) {
                const int sb = kk & 1;
                float* dst = xs + sb * 2 * TC_KB;
                mbar_arrive_expect_tx(&aux->mb_tma[sb], 2u * TC_KB * 4u);
                tma_load_2d(dst, &p.tmap_x, 0, static_cast<int>(tile_of(kk) * TC_NB), &aux->mb_tma[sb]);
                tma_load_2d(dst + TC_KB, &p.tmap_x, 32, static_cast<int>(tile_of(kk) * TC_NB), &aux->mb_tma[sb]);
                ++tma_n[sb];
            };
            for (uint32_t kk = 0; kk < 2 && kk < nk; ++kk)
                if (bulk(kk)) issue_tma(kk);
            bool got_split = false;
            uint64_t t_last = globaltimer_ns();
            uint32_t spins = 0;
            while (k1 < nk || k2 < nk) {
                bool progress = false;
                if (n_free < k2 && mbar_try_wait(&aux->mb_accfree, n_free & 1u)) {
                    ++n_free;
                    progress = true;
                }
                if (k2 < k1 && n_free >= k2 && mbar_try_wait(&aux->mb_sready, k2 & 1u)) {
                    tc_fence_after();
                    const uint32_t dt = tmem + static_cast<uint32_t>((k2 % TC_NACC) * TC_ACC);
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {
                        const uint32_t o = ks * 32;
                        const uint64_t ah = umma_desc(smem_u32(a2s) + o);
                        const uint64_t al = umma_desc(smem_u32(a2s) + TC_KB * 4 + o);
                        const uint64_t bh = umma_desc(smem_u32(h2) + o);
                        const uint64_t bl = umma_desc(smem_u32(h2) + TC_H2B * 4 + o);
                        umma_tf32(dt, ah, bh, TC_IDESC2, 1u);
                        umma_tf32(dt, ah, bl, TC_IDESC2, 1u);
                        umma_tf32(dt, al, bh, TC_IDESC2, 1u);
                    }
                    umma_commit(&aux->mb_g2);
                    ++aux->g2_issued;
                    ++k2;
                    progress = true;
                } else if (k1 < nk && (k1 < TC_NACC || n_free + TC_NACC > k1)) {  // accumulator k1 % TC_NACC is free
                    if (!got_split) {
                        got_split = mbar_try_wait(&aux->mb_split[k1 & 1], (k1 >> 1) & 1u);
                        if (got_split && k1 + 2 < nk && bulk(k1 + 2)) issue_tma(k1 + 2);  // buffer k1 & 1 read out
                    }
                    if (got_split) {
                        if (piece == 0) tc_fence_after();
                        const uint32_t xa = tmem + static_cast<uint32_t>(TC_XCOL + (k1 & 1) * 128);  // x hi; lo at + 64
                        const uint32_t dt = tmem + static_cast<uint32_t>((k1 % TC_NACC) * TC_ACC);
                        if constexpr (BF == 0) {
                            const int kb = piece >> 1;
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const int ks = (piece & 1) * 2 + h;
                                const uint32_t ca = static_cast<uint32_t>(kb * 32 + ks * 8);
                                const uint32_t ob = (kb * TC_B1KB) * 4 + ks * 32;
                                const uint64_t bh = umma_desc(smem_u32(b1) + ob);
                                const uint64_t bl = umma_desc(smem_u32(b1) + 2 * TC_B1KB * 4 + ob);
                                umma_tf32_ta(dt, xa + ca, bh, TC_IDESC1, (piece == 0 && h == 0) ? 0u : 1u);
                                umma_tf32_ta(dt, xa + ca, bl, TC_IDESC1, 1u);
                                umma_tf32_ta(dt, xa + 64 + ca, bh, TC_IDESC1, 1u);
                            }
                        } else {
                            // piece = k-step of 16 samples: x part a at columns 32 a + 8 piece (two bf16
                            // per column), B part b at b * TC_BF_PART_BYTES + 32 piece bytes
                            using Bf = TcBf16<BF>;
#pragma unroll
                            for (int i = 0; i < Bf::NPROD; ++i) {
                                const uint32_t ta = xa + static_cast<uint32_t>(32 * Bf::a_part(i) + 8 * piece);
                                const uint64_t db =
                                    umma_desc(smem_u32(b1) + static_cast<uint32_t>(Bf::b_part(i) * TC_BF_PART_BYTES + 32 * piece));
                                umma_bf16_ta(dt, ta, db, TC_IDESC1_BF16, (piece == 0 && i == 0) ? 0u : 1u);
                            }
                        }
                        if (++piece == 4) {
                            umma_commit(&aux->mb_g1[k1 & 1]);
                            ++aux->g1_issued;
                            TC_STAMP(k1, 15);
                            ++k1;
                            piece = 0;
                            got_split = false;
                        }
                        progress = true;
                    }
                }
                if (progress) {
                    t_last = globaltimer_ns();
                } else if ((++spins & 63u) == 0u) {
                    if (*vbail) break;
                    if (globaltimer_ns() - t_last > static_cast<uint64_t>(wait_lim)) {
                        tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
                        break;
                    }
                }
            }
            // loads still in flight (a stopped launch) land before the block leaves: the last load
            // of each buffer completes its phase (tma_n - 1), and every earlier one had landed
            // before the next was issued
            for (int sb = 0; sb < 2; ++sb)
                if (tma_n[sb] > 0) wait_mbar_bounded(&aux->mb_tma[sb], (tma_n[sb] - 1) & 1u, p.timeout_ns);
        }
        __syncwarp();
    } else if (warp < TC_CW0 + TC_CW) {
        // ================= front group =================
        const int ct = tid - 32 * TC_CW0;
        const int cw = warp - TC_CW0;
        const int q = warp & 3;                 // TMEM lane quadrant of this warp
        const int hh = cw >> 2;                 // which of the two warps on the quadrant
        using Scan = TcScan<KD>;
        const int grp = ct >> Scan::LG_SHIFT, d = ct & (Scan::LG - 1);  // scan: sub-block, state component
        float phi_row[KD], phix0, phix1;
#pragma unroll
        for (int e = 0; e < KD; ++e) phi_row[e] = __ldg(p.phi + d * TC_DMAX + e);
        phix0 = __ldg(p.phix + d * 2);
        phix1 = __ldg(p.phix + d * 2 + 1);
        float* U = reinterpret_cast<float*>(base + Sm::SCRF);      // [128][TC_UP] end-state rows
        float* V0 = U + TC_NB * TC_UP;                             // [groups][16] x 2 combine ping-pong
        float* V1 = V0 + Scan::GROUPS * TC_DMAX;
        float* SB = V1 + Scan::GROUPS * TC_DMAX;                   // [groups][16] scan state broadcast
        uint32_t tma_par[2] = {0u, 0u}, g1_par = 0;
        // one recurrence step of the half-warp's state, Phi S + Z_j + Phix xh_j; the state goes
        // through the group's 16-float buffer sb (one store, four broadcast vector loads)
        auto step = [&](float S, int j, const float* xhj, float* sb) {
            __syncwarp();
            sb[d] = S;
            __syncwarp();
            const float4* s4 = reinterpret_cast<const float4*>(sb);
            float s0 = U[j * TC_UP + d], s1 = phix0 * xhj[0], s2 = phix1 * xhj[1], s3 = 0.f;
#pragma unroll
            for (int e = 0; e < KD; e += 4) {
                const float4 v = s4[e >> 2];
                s0 = fmaf(phi_row[e], v.x, s0);
                if (e + 1 < KD) s1 = fmaf(phi_row[e + 1], v.y, s1);
                if (e + 2 < KD) s2 = fmaf(phi_row[e + 2], v.z, s2);
                if (e + 3 < KD) s3 = fmaf(phi_row[e + 3], v.w, s3);
            }
            return (s0 + s1) + (s2 + s3);
        };
        auto mv_smem = [&](int b, const float* v) {  // (Phi^(SUB * 2^b) v)_d, v a 16-byte aligned smem vector
            const float4* m4 = reinterpret_cast<const float4*>(&aux->phip[b][0][d][0]);
            const float4* v4 = reinterpret_cast<const float4*>(v);
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
            for (int e = 0; e < KD; e += 4) {
                const float4 mm = m4[(e >> 2) * TC_DMAX], vv = v4[e >> 2];
                s0 = fmaf(mm.x, vv.x, s0);
                if (e + 1 < KD) s1 = fmaf(mm.y, vv.y, s1);
                if (e + 2 < KD) s2 = fmaf(mm.z, vv.z, s2);
                if (e + 3 < KD) s3 = fmaf(mm.w, vv.w, s3);
            }
            return (s0 + s1) + (s2 + s3);
        };
        // stage tile kk: data landed (TMA) or gathered, input history, TF32 split, then hand it
        // to the MMA warp. Returns the group's stop decision (the same in all of its threads).
        auto stage_tile = [&](uint32_t kk, float hx2, float hx1) {
            const int s = kk & 1;
            float* xt = xs + s * 2 * TC_KB;
            const long long ts = static_cast<long long>(tile_of(kk)) * TC_TILE;
            if (bulk(kk)) {
                if (tc_wait(&aux->mb_tma[s], tma_par[s] & 1u, p.timeout_ns, &aux->bail))
                    ++tma_par[s];
                else
                    tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
                if (ct == 0 && kk > 0) TC_STAMP(kk - 1, 6);
            } else {
                for (int i = ct; i < TC_TILE; i += TC_CT) {
                    const int j = i / TC_L, c = i % TC_L;
                    const long long g = ts + i;
                    xt[(c >> 5) * TC_KB + swz32(j, c & 31)] = (g < p.n) ? p.x[g] : 0.f;
                }
                bar_group(1);
            }
            if (ct < TC_NB) {  // the two samples before each chunk
                float x2, x1;
                if (ct > 0) {
                    x2 = xt[TC_KB + swz32(ct - 1, 30)];
                    x1 = xt[TC_KB + swz32(ct - 1, 31)];
                } else {
                    x2 = hx2;  // the two samples before the tile, loaded ahead by the caller
                    x1 = hx1;
                }
                aux->xh[kk % TC_NXH][ct][0] = x2;
                aux->xh[kk % TC_NXH][ct][1] = x1;
            }
            {  // (the split only reads the staged tile, so it needs no barrier after the capture)
                // this thread's chunk row (TMEM lane 32 q + lane): 32 samples from the swizzled tile,
                // split hi / lo, stored to the x operand columns of buffer kk & 1 -- k-block hh (both
                // halves) when this group splits the tile whole, else half hh of k-block 0 (the back
                // group splits k-block 1)
                const int r = 32 * q + lane;
                const uint32_t xq = tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>(TC_XCOL + (kk & 1) * 128);
                __syncwarp();
                if constexpr (BF == 0) {
                    if (shared_split(kk)) {
                        tc_split16(xt, 0, hh, r, xq);
                    } else {
                        tc_split16(xt, hh, 0, r, xq + 32 * hh);
                        tc_split16(xt, hh, 1, r, xq + 32 * hh);
                    }
                } else {
                    // bf16 parts of the 32 samples, two per column: part a of k-block hh at columns
                    // 32 a + 16 hh of the buffer
                    const float4* row = reinterpret_cast<const float4*>(xt + hh * TC_KB + r * 32);
                    const uint32_t xb = xq + static_cast<uint32_t>(16 * hh);
#pragma unroll
                    for (int half = 0; half < 2; ++half) {
                        uint32_t w[TcBf16<BF>::PARTS][8];
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const float4 v = row[(4 * half + c) ^ (r & 7)];
                            float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                            for (int a = 0; a < TcBf16<BF>::PARTS; ++a) {
                                float part[4];
#pragma unroll
                                for (int j = 0; j < 4; ++j) {
                                    part[j] = __bfloat162float(__float2bfloat16_rn(e[j]));
                                    e[j] -= part[j];
                                }
                                w[a][2 * c] = bf16_pair(part[0], part[1]);
                                w[a][2 * c + 1] = bf16_pair(part[2], part[3]);
                            }
                        }
#pragma unroll
                        for (int a = 0; a < TcBf16<BF>::PARTS; ++a) tmem_st8u(xb + 32 * a + 8 * half, w[a]);
                    }
                }
                tmem_wait_st();
            }
            fence_proxy_async_smem();  // the tile's stage is refilled by TMA next
            tc_fence_before();
            const bool stop = bar_group_any(1, *vbail);
            if (!stop && ct == 0) {
                mbar_arrive(&aux->mb_split[kk & 1]);
                if (!shared_split(kk)) mbar_arrive(&aux->mb_split[kk & 1]);  // the back group's share too
            }
            return stop;
        };

        // the two input samples before tile kk (zero before the signal); loaded one iteration
        // ahead so the load's latency is not on the staging path
        auto hist = [&](uint32_t kk, float& h2v, float& h1v) {
            const long long ts = static_cast<long long>(tile_of(kk)) * TC_TILE;
            h2v = (ct == 0 && ts > 0 && ts - 2 < p.n) ? p.x[ts - 2] : 0.f;
            h1v = (ct == 0 && ts > 0 && ts - 1 < p.n) ? p.x[ts - 1] : 0.f;
        };
        float hx2 = 0.f, hx1 = 0.f;
        if (nk > 0) hist(0, hx2, hx1);
        bool stop = nk > 0 ? stage_tile(0, hx2, hx1) : false;
        if (nk > 1) hist(1, hx2, hx1);
        for (uint32_t k = 0; k < nk && !stop; ++k) {
            if (ct == 0) TC_STAMP(k, 0);
            // ---- a. tile k+1: staged first (its x buffer was read by GEMM 1 of tile k-1, whose
            // completion this group saw), so GEMM 1 of tile k runs meanwhile ----
            if (k + 1 < nk) {
                if (stage_tile(k + 1, hx2, hx1)) break;
                if (k + 2 < nk) hist(k + 2, hx2, hx1);
            }
            if (ct == 0) TC_STAMP(k, 7);
            // ---- b. tile k: sub-block scans, tile aggregate, hand-off to the lookback warp ----
            if (tc_wait(&aux->mb_g1[g1_par & 1], (g1_par >> 1) & 1u, wait_lim, &aux->bail))
                ++g1_par;
            else
                tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
            tc_fence_after();
            if (ct == 0) TC_STAMP(k, 1);
            {
                float v[8];
                __syncwarp();
                tmem_ld8(tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>((k % TC_NACC) * TC_ACC + 64 + 8 * hh), v);
                float* u = U + (32 * q + lane) * TC_UP + 8 * hh;
#pragma unroll
                for (int i = 0; i < 8; ++i) u[i] = v[i];
            }
            if (bar_group_any(1, *vbail)) break;
            if (ct == 0) TC_STAMP(k, 2);
            const float* xhk = &aux->xh[k % TC_NXH][0][0];
            float S = 0.f;
            for (int i = 0; i < Scan::SUB; ++i)
                S = step(S, grp * Scan::SUB + i, xhk + (grp * Scan::SUB + i) * 2, SB + grp * TC_DMAX);
            V0[grp * TC_DMAX + d] = S;
            if (ct == 0) TC_STAMP(k, 3);
            bar_group(1);
            // inclusive scan over the sub-blocks: V_g += Phi^(SUB s) V_(g-s), s = 1, 2, 4, ...
            float* Vc = V0;
            float* Vn = V1;
#pragma unroll
            for (int l = 0; l < Scan::LEVELS; ++l) {
                const int s = 1 << l;
                float a = Vc[grp * TC_DMAX + d];
                if (grp >= s) a += mv_smem(l, Vc + (grp - s) * TC_DMAX);
                Vn[grp * TC_DMAX + d] = a;
                bar_group(1);
                float* tsw = Vc;
                Vc = Vn;
                Vn = tsw;
            }
            if (ct == 0) TC_STAMP(k, 4);
            aux->Ig0[k % TC_NACC][grp][d] = grp > 0 ? Vc[(grp - 1) * TC_DMAX + d] : 0.f;
            if (grp == Scan::GROUPS - 1) aux->agg[k % TC_NS][d] = Vc[grp * TC_DMAX + d];
            bar_group(1);
            if (ct < KD / 2) {  // the aggregate's part words, one pair per lane
                const uint32_t t = tile_of(k);
                if (static_cast<long long>(t) != p.withhold_chunk) {
                    const uint32_t pf = 2u * epoch + 1u;
                    st_relaxed_v2(slots + static_cast<size_t>(t) * 2 * KD + 2 * ct,
                                  pack_word(pf, aux->agg[k % TC_NS][2 * ct]), pack_word(pf, aux->agg[k % TC_NS][2 * ct + 1]));
                }
            }
            if (ct == 0) {
                mbar_arrive(&aux->mb_agg[k % TC_NS]);
                TC_STAMP(k, 5);
            }
            stop = bar_group_any(1, *vbail);
        }
        __syncthreads();
        if (ct == 0)  // GEMM 1 batches still in flight end before TMEM is freed
            while (g1_par < aux->g1_issued &&
                   wait_mbar_bounded(&aux->mb_g1[g1_par & 1], (g1_par >> 1) & 1u, p.timeout_ns))
                ++g1_par;
    } else {
        // ================= back group =================
        const int ct = tid - 32 * (TC_CW0 + TC_CW);
        const int cw = warp - TC_CW0 - TC_CW;
        const int q = warp & 3;
        const int hh = cw >> 2;
        using Scan = TcScan<KD>;
        const int grp = ct >> Scan::LG_SHIFT, d = ct & (Scan::LG - 1);  // scan: sub-block, state component
        float phi_row[KD], phix0, phix1;
#pragma unroll
        for (int e = 0; e < KD; ++e) phi_row[e] = __ldg(p.phi + d * TC_DMAX + e);
        phix0 = __ldg(p.phix + d * 2);
        phix1 = __ldg(p.phix + d * 2 + 1);
        float* scr = reinterpret_cast<float*>(base + Sm::SCRB);
        float* U = scr;                                   // [128][TC_UP] end-state rows
        float* VX = scr + TC_NB * TC_UP;                  // [16][16] incoming-state products
        uint32_t g2_par = 0;
        // one recurrence step of the half-warp's state, Phi S + Z_j + Phix xh_j; the state goes
        // through the group's 16-float buffer sb (one store, four broadcast vector loads)
        auto step = [&](float S, int j, const float* xhj, float* sb) {
            __syncwarp();
            sb[d] = S;
            __syncwarp();
            const float4* s4 = reinterpret_cast<const float4*>(sb);
            float s0 = U[j * TC_UP + d], s1 = phix0 * xhj[0], s2 = phix1 * xhj[1], s3 = 0.f;
#pragma unroll
            for (int e = 0; e < KD; e += 4) {
                const float4 v = s4[e >> 2];
                s0 = fmaf(phi_row[e], v.x, s0);
                if (e + 1 < KD) s1 = fmaf(phi_row[e + 1], v.y, s1);
                if (e + 2 < KD) s2 = fmaf(phi_row[e + 2], v.z, s2);
                if (e + 3 < KD) s3 = fmaf(phi_row[e + 3], v.w, s3);
            }
            return (s0 + s1) + (s2 + s3);
        };
        auto mv_smem = [&](int b, const float* v) {  // (Phi^(SUB * 2^b) v)_d, v a 16-byte aligned smem vector
            const float4* m4 = reinterpret_cast<const float4*>(&aux->phip[b][0][d][0]);
            const float4* v4 = reinterpret_cast<const float4*>(v);
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
            for (int e = 0; e < KD; e += 4) {
                const float4 mm = m4[(e >> 2) * TC_DMAX], vv = v4[e >> 2];
                s0 = fmaf(mm.x, vv.x, s0);
                if (e + 1 < KD) s1 = fmaf(mm.y, vv.y, s1);
                if (e + 2 < KD) s2 = fmaf(mm.z, vv.z, s2);
                if (e + 3 < KD) s3 = fmaf(mm.w, vv.w, s3);
            }
            return (s0 + s1) + (s2 + s3);
        };
        // The back group's half of a TMA-staged tile's split (k-block 1; the front group splits
        // k-block 0): once the tile has landed and GEMM 1 of tile kk - 2 has read the TMEM x buffer
        // that this tile takes over. Returns the group's stop decision.
        uint32_t tma_par_b[2] = {0u, 0u};
        auto split_half = [&](uint32_t kk) {
            if (!shared_split(kk)) return false;  // the front group splits this tile whole
            bool ok = true;
            if (kk >= 2) ok = tc_wait(&aux->mb_g1[(kk - 2) & 1], ((kk - 2) >> 1) & 1u, wait_lim, &aux->bail);
            if (ok) {
                ok = tc_wait(&aux->mb_tma[kk & 1], tma_par_b[kk & 1] & 1u, p.timeout_ns, &aux->bail);
                if (ok) ++tma_par_b[kk & 1];
            }
            if (!ok) {
                tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
            } else {
                tc_fence_after();
                const float* xt = xs + (kk & 1) * 2 * TC_KB;
                const uint32_t xq = tmem + (static_cast<uint32_t>(32 * q) << 16) +
                                    static_cast<uint32_t>(TC_XCOL + (kk & 1) * 128 + 32);
                __syncwarp();
                tc_split16(xt, 1, hh, 32 * q + lane, xq);
                tmem_wait_st();
            }
            fence_proxy_async_smem();
            tc_fence_before();
            const bool st = bar_group_any(2, *vbail);
            if (!st && ct == 0) mbar_arrive(&aux->mb_split[kk & 1]);
            return st;
        };
        float* vx = VX + grp * TC_DMAX;                  // the group's state buffer
        float4* patch = reinterpret_cast<float4*>(VX + Scan::GROUPS * TC_DMAX) + cw * 64;  // [32 rows][2 float4]
        float xin = 0.f;
        // c1. tile kk: the lookback's X, end-state rows from TMEM, Phi^(SUB grp) X (a product of
        // Phi^(SUB * 2^b) over the bits of grp); runs while GEMM 2 of the tile before is in flight
        auto prepare = [&](uint32_t kk) {
            const int sl = kk % TC_NS;
            if (!tc_wait(&aux->mb_x[sl], (kk / TC_NS) & 1u, wait_lim, &aux->bail))
                tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
            tc_fence_after();
            if (ct == 0) TC_STAMP(kk, 8);
            float v[8];
            __syncwarp();
            tmem_ld8(tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>((kk % TC_NACC) * TC_ACC + 64 + 8 * hh), v);
            float* u = U + (32 * q + lane) * TC_UP + 8 * hh;
#pragma unroll
            for (int i = 0; i < 8; ++i) u[i] = v[i];
            vx[d] = aux->X[sl][d];
            __syncwarp();
#pragma unroll
            for (int b = 0; b < Scan::LEVELS; ++b) {
                const float w = mv_smem(b, vx);
                __syncwarp();
                if ((grp >> b) & 1) vx[d] = w;
                __syncwarp();
            }
            xin = vx[d];
        };
        // c2. tile kk (after a group barrier: its rows are in U, the state operand is free):
        // states of its chunks into the state operand, then GEMM 2 by the MMA warp
        auto rescan = [&](uint32_t kk) {
            if (ct == 0) TC_STAMP(kk, 9);
            const float* xhp = &aux->xh[kk % TC_NXH][0][0];
            float S = aux->Ig0[kk % TC_NACC][grp][d] + xin;
            for (int i = 0; i < Scan::SUB; ++i) {
                const int j = grp * Scan::SUB + i;
                if (d < D) {
                    const float h = tf32_hi(S);
                    a2s[swz32(j, d)] = h;
                    a2s[TC_KB + swz32(j, d)] = tf32_hi(S - h);
                } else if (d < D + 2) {  // the chunk's input history in columns D, D + 1
                    const float v = xhp[j * 2 + (d - D)];
                    const float h = tf32_hi(v);
                    a2s[swz32(j, d)] = h;
                    a2s[TC_KB + swz32(j, d)] = tf32_hi(v - h);
                }
                S = step(S, j, xhp + j * 2, vx);
            }
            if (D + 2 > Scan::LG) {  // D = LG: history columns D, D + 1 of the sub-block's chunks, one per lane
                const int j = grp * Scan::SUB + (d >> 1), e = d & 1;
                const float v = xhp[j * 2 + e];
                const float h = tf32_hi(v);
                a2s[swz32(j, D + e)] = h;
                a2s[TC_KB + swz32(j, D + e)] = tf32_hi(v - h);
            }
            fence_proxy_async_smem();
            tc_fence_before();
            const bool st = bar_group_any(2, *vbail);
            if (!st && ct == 0) {
                mbar_arrive(&aux->mb_sready);
                TC_STAMP(kk, 10);
            }
            return st;
        };
        // d. tile kk: GEMM 2 done -> outputs. This thread's chunk (TMEM lane 32 q + lane) has 32
        // consecutive outputs in its registers; they go out through a per-warp patch of 32
        // chunks x 8 samples in four rounds, so each store instruction writes 64-byte runs of y
        // (32 B per half row, half rows swapped every 4 rows: conflict-free writes and reads)
        auto epilogue = [&](uint32_t kk) {
            const bool ok = tc_wait(&aux->mb_g2, g2_par & 1u, wait_lim, &aux->bail);
            if (ok)
                ++g2_par;
            else
                tc_give_up(aux, p, epoch, IIR_DEV_ERR_MBARRIER);
            tc_fence_after();
            if (ct == 0) TC_STAMP(kk, 11);
            if (__all_sync(0xffffffffu, ok) && bulk_y(kk)) {
                // a whole tile: this thread's 32 outputs (chunk row 32 q + lane, k-block hh) into the
                // state operand's buffer, free from GEMM 2 until the next rescan, in the tensor
                // map's 128-byte swizzled layout; store_tile sends it out after the group barrier
                float v[32];
                __syncwarp();
                tmem_ld32(tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>((kk % TC_NACC) * TC_ACC + 32 * hh), v);
                float4* row = reinterpret_cast<float4*>(a2s + hh * TC_KB + (32 * q + lane) * 32);
#pragma unroll
                for (int g = 0; g < 8; ++g) row[g ^ (lane & 7)] = make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2], v[4 * g + 3]);
                fence_proxy_async_smem();
            } else if (__all_sync(0xffffffffu, ok)) {
                const long long ts = static_cast<long long>(tile_of(kk)) * TC_TILE;
                float v[32];
                __syncwarp();
                tmem_ld32(tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>((kk % TC_NACC) * TC_ACC + 32 * hh), v);
                const int sw = (lane >> 2) & 1;
#pragma unroll
                for (int part = 0; part < 4; ++part) {
                    patch[lane * 2 + sw] = make_float4(v[8 * part], v[8 * part + 1], v[8 * part + 2], v[8 * part + 3]);
                    patch[lane * 2 + (sw ^ 1)] = make_float4(v[8 * part + 4], v[8 * part + 5], v[8 * part + 6], v[8 * part + 7]);
                    __syncwarp();
#pragma unroll
                    for (int it = 0; it < 2; ++it) {
                        const int r = it * 16 + (lane >> 1), c4 = lane & 1;
                        const float4 o = patch[r * 2 + (c4 ^ ((r >> 2) & 1))];
                        const long long g = ts + static_cast<long long>(32 * q + r) * TC_L + 32 * hh + 8 * part + 4 * c4;
                        if (p.y_vec && g + 3 < p.n) {
                            *reinterpret_cast<float4*>(p.y + g) = o;
                        } else {
                            if (g < p.n) p.y[g] = o.x;
                            if (g + 1 < p.n) p.y[g + 1] = o.y;
                            if (g + 2 < p.n) p.y[g + 2] = o.z;
                            if (g + 3 < p.n) p.y[g + 3] = o.w;
                        }
                    }
                    __syncwarp();
                }
            }
            tc_fence_before();
        };

        // After the group barrier that follows epilogue(kk): the staged tile leaves by two TMA
        // stores (one per k-block). The issuing thread waits until they have read the buffer
        // (store_read) before the group barrier after which the next rescan overwrites it.
        auto store_tile = [&](uint32_t kk) {
            if (ct == 0 && bulk_y(kk)) {
                const int row0 = static_cast<int>(tile_of(kk) * TC_NB);
                tma_store_2d(&p.tmap_y, 0, row0, a2s);
                tma_store_2d(&p.tmap_y, 32, row0, a2s + TC_KB);
                bulk_commit();
            }
        };
        auto store_read = [&]() {
            if (ct == 0) bulk_wait_read_all();
        };
        bool stop = false;
        for (uint32_t kk = 0; kk < 3 && kk < nk && !stop; ++kk) stop = split_half(kk);
        if (nk > 0 && !stop) {
            prepare(0);
            stop = bar_group_any(2, *vbail) || rescan(0);
        }
        for (uint32_t k = 0; k < nk && !stop; ++k) {
            // tile k + 3's half of the split, three tiles ahead of its GEMM 1 so that the front
            // group never waits for it. It waits for GEMM 1 of tile k + 1 (which needs only splits
            // made earlier; the front group issues it while this group still works on tile k) and
            // for the tile's TMA load (issued when both groups had split tile k + 1).
            if (k + 3 < nk && split_half(k + 3)) break;
            if constexpr (KD <= IIR_TC_SHARED_MAX_KD) {
                // The accumulator of tile k is freed as soon as its outputs are read: GEMM 1 of tile
                // k + 3 waits for it, so the wait for tile k + 1's incoming state (prepare) comes
                // after. (With 16 states this group is the slower one, and prepare(k + 1) overlapping
                // GEMM 2 of tile k, as below, is worth more: orders 10-16 lose 3-7% this way.)
                epilogue(k);
                // (also: GEMM 2 of tile k has read the state operand)
                stop = bar_group_any(2, *vbail);
                if (stop) break;
                if (ct == 0) {
                    mbar_arrive(&aux->mb_accfree);
                    TC_STAMP(k, 12);
                }
                store_tile(k);  // read out while prepare runs
                if (k + 1 < nk) {
                    prepare(k + 1);
                    store_read();
                    stop = bar_group_any(2, *vbail) || rescan(k + 1);  // (rows of tile k + 1 are in U)
                }
            } else {
                if (k + 1 < nk) prepare(k + 1);  // overlaps GEMM 2 of tile k
                epilogue(k);
                // (also: rows of tile k+1 are in U, and GEMM 2 of tile k has read the state operand)
                stop = bar_group_any(2, *vbail);
                if (stop) break;
                if (ct == 0) {
                    mbar_arrive(&aux->mb_accfree);
                    TC_STAMP(k, 12);
                }
                if (bulk_y(k)) {
                    store_tile(k);
                    store_read();
                    bar_group(2);  // the stores have read the buffer that rescan(k + 1) rewrites
                }
                if (k + 1 < nk) stop = rescan(k + 1);
            }
        }
        if (ct == 0) bulk_wait_all();  // the output tiles' TMA stores have completed
        __syncthreads();
        if (ct == 0)  // GEMM 2 batches still in flight end before TMEM is freed
            while (g2_par < aux->g2_issued && wait_mbar_bounded(&aux->mb_g2, g2_par & 1u, p.timeout_ns)) ++g2_par;
    }
    if (warp < TC_CW0) __syncthreads();  // pairs with the compute groups' barrier above
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == TC_MW) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    if (tid == 0) pipe_finish(p.state, epoch);
}

}  // namespace iirgb

// -------------------------------------------------------------------------------------------
// host: FP64 operators of the cascade over one chunk, operand images, lookback tables, launch
// -------------------------------------------------------------------------------------------
namespace iirhost {

using iirgb::TC_B1KB;
using iirgb::TC_DMAX;
using iirgb::TC_H2B;
using iirgb::TC_KB;
using iirgb::TC_N1;
using iirgb::TC_N2;
using iirgb::TC_L;
using iirgb::TC_NB;
using iirgb::TC_TILE;

struct TcPlan {
    int D = 0, KD = 0, sms = 0, grid_max = 0;
    bool input_normal = false;  // carried states in the input-normal basis (else balanced)
    int lb_depth = 0;           // truncated lookback depth (0: full decoupled lookback)
    int bf = 0;                 // GEMM 1 operands: 0 = TF32 hi / lo, 3 or 6 = BF16 split (TcBf16)
    unsigned long long* prof = nullptr;  // timeline buffer (builds with IIR_PROFILE)
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
// Nearest bf16 of a finite float (ties to even), and back.
uint16_t bf16_rn_h(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}
float bf16_to_f_h(uint16_t h) {
    const uint32_t u = static_cast<uint32_t>(h) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
// GEMM 1 operand form of a plan, chosen at plan creation: the BF16 split is built for 5..8 and
// 9..16 carried states with the truncated lookback; every other plan uses TF32. By default 5..8
// states take the BF16 split with three parts and six products: its GEMM 1 takes half the
// tensor-core time of the TF32 split's, at the same float32 accuracy (order 8 on the precision
// workload: 440 GS/s at 7.1e-6 RMS against 419 GS/s at 6.4e-6); with 16 states TF32 is the faster.
// IIR_GB300_TC_BF16 = 0 (TF32), 3 or 6 sets the form wherever the BF16 split is built.
int tc_bf16_form(int kd, bool full) {
    if (full || kd < 8) return 0;
    const char* e = std::getenv("IIR_GB300_TC_BF16");
    if (!e) return kd == 8 ? 6 : 0;
    const int v = std::atoi(e);
    return (v == 3 || v == 6) ? v : 0;
}
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
const void* tc_kernel_fn(bool full, int bf) {
    if (full) return reinterpret_cast<const void*>(iirgb::iir_tc_kernel<KD, true, 0>);
    if constexpr (KD >= 8) {
        if (bf == 3) return reinterpret_cast<const void*>(iirgb::iir_tc_kernel<KD, false, 3>);
        if (bf == 6) return reinterpret_cast<const void*>(iirgb::iir_tc_kernel<KD, false, 6>);
    }
    return reinterpret_cast<const void*>(iirgb::iir_tc_kernel<KD, false, 0>);
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
void tc_plan_set_profile(TcPlan* t, unsigned long long* buf) {
    if (t) t->prof = buf;
}
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
    std::vector<float> img1(static_cast<size_t>(4) * TC_B1KB, 0.f), img2(static_cast<size_t>(2) * TC_H2B, 0.f);
    for (int m = 0; m < TC_N1; ++m)  // GEMM 1 B operand: rows 0..63 T, 64..79 B (zero beyond D)
        for (int c = 0; c < L; ++c) {
            const float v = static_cast<float>(A1[m * L + c]);
            const float hv = tf32_hi_h(v);
            const size_t idx = static_cast<size_t>(c >> 5) * TC_B1KB + swz32h(m, c & 31);
            img1[idx] = hv;
            img1[2 * TC_B1KB + idx] = tf32_hi_h(v - hv);
        }
    for (int m = 0; m < TC_N2; ++m)  // GEMM 2 B operand: rows = outputs, K = [H | Hx]
        for (int c = 0; c < 32; ++c) {
            const float v = static_cast<float>(A2[m * 32 + c]);
            const float hv = tf32_hi_h(v);
            img2[swz32h(m, c)] = hv;
            img2[TC_H2B + swz32h(m, c)] = tf32_hi_h(v - hv);
        }
    const int KD = t->KD;
    std::vector<float> phi(TC_DMAX * TC_DMAX), phix(TC_DMAX * 2), ppow(static_cast<size_t>(iirgb::TC_LEVELS_MAX) * TC_DMAX * TC_DMAX),
        pc(static_cast<size_t>(33) * KD * KD), pg(static_cast<size_t>(33) * KD * KD);
    for (size_t i = 0; i < phi.size(); ++i) phi[i] = static_cast<float>(Phi[i]);
    for (size_t i = 0; i < phix.size(); ++i) phix[i] = static_cast<float>(Phix[i]);
    {
        // Phi^(SUB * 2^b), stored [b][e / 4][d][e % 4] = P[d][e] (SUB = the kernel's sub-block length)
        Mat P = matpow(Phi, iirgb::tc_scan_sub(KD), TC_DMAX);
        for (int b = 0; b < iirgb::TC_LEVELS_MAX; ++b) {
            for (int dd = 0; dd < TC_DMAX; ++dd)
                for (int e = 0; e < TC_DMAX; ++e)
                    ppow[((static_cast<size_t>(b) * (TC_DMAX / 4) + e / 4) * TC_DMAX + dd) * 4 + e % 4] =
                        static_cast<float>(P[dd * TC_DMAX + e]);
            P = matmul(P, P, TC_DMAX);
        }
    }
    const Mat Q = matpow(Phi, TC_NB, TC_DMAX);        // tile transition
    {
        // truncated lookback depth: the least m <= TC_LB_MAX with ||Q^m||_inf <= 1e-10
        Mat Qm = Q;
        t->lb_depth = 0;
        for (int m = 1; m <= iirgb::TC_LB_MAX; ++m) {
            double nrm = 0.0;
            for (int i = 0; i < TC_DMAX; ++i) {
                double r = 0.0;
                for (int j = 0; j < TC_DMAX; ++j) r += std::fabs(Qm[i * TC_DMAX + j]);
                nrm = std::max(nrm, r);
            }
            if (std::isfinite(nrm) && nrm <= 1e-10) {
                t->lb_depth = m;
                break;
            }
            Qm = matmul(Qm, Q, TC_DMAX);
        }
    }
    // GEMM 1 in BF16 (IIR_GB300_TC_BF16): the B operand image is rebuilt as bf16 parts; part b of
    // row m, sample c sits at bf16 index b * 80 * 64 + m * 64 + ((c / 8) ^ (m % 8)) * 8 + c % 8
    // (rows of 128 bytes, 128-byte swizzle)
    t->bf = tc_bf16_form(t->KD, t->lb_depth == 0);
    if (t->bf != 0) {
        std::vector<uint16_t> bimg(static_cast<size_t>(2) * img1.size(), 0);
        const int parts = t->bf == 6 ? 3 : 2;
        for (int m = 0; m < TC_N1; ++m)
            for (int c = 0; c < L; ++c) {
                float rest = static_cast<float>(A1[m * L + c]);
                for (int b = 0; b < parts; ++b) {
                    const uint16_t h = bf16_rn_h(rest);
                    rest -= bf16_to_f_h(h);
                    bimg[static_cast<size_t>(b) * (iirgb::TC_BF_PART_BYTES / 2) + m * 64 + (((c >> 3) ^ (m & 7)) << 3) +
                         (c & 7)] = h;
                }
            }
        std::memcpy(img1.data(), bimg.data(), img1.size() * sizeof(float));
    }
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
    t->off_grp = put(ppow);
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
        const bool full = t->lb_depth == 0;
        t->fn = KD == 2   ? tc_kernel_fn<2>(full, t->bf)
                : KD == 4 ? tc_kernel_fn<4>(full, t->bf)
                : KD == 8 ? tc_kernel_fn<8>(full, t->bf)
                          : tc_kernel_fn<16>(full, t->bf);
        st = cuda_status(cudaFuncSetAttribute(t->fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              static_cast<int>(iirgb::tc_smem_bytes(KD))));
    }
    if (!st) {
        int nb = 0;
        st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, t->fn, iirgb::TC_THREADS, iirgb::tc_smem_bytes(KD)));
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
        if (!st) st = cuda_status(cudaMemsetAsync(t->d_state, 0, IIR_STATE_RESET_BYTES, stream));
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
    q.b1img = t->d_tabs;
    q.h2img = t->d_tabs + t->off_a2;
    q.phi = t->d_tabs + t->off_phi;
    q.phix = t->d_tabs + t->off_phix;
    q.phi_pow = t->d_tabs + t->off_grp;
    q.lb_depth = t->lb_depth;
    q.pc = t->d_tabs + t->off_pc;
    q.pg = t->d_tabs + t->off_pg;
    q.timeout_ns = timeout_ns;
    q.withhold_chunk = withhold;
    q.ntiles = static_cast<unsigned int>(tiles);
    q.carry_cap = static_cast<unsigned int>(t->carry_cap);
    q.D = t->D;
    q.use_tma = encode_chunk_rows_map(&q.tmap_x, x, static_cast<long long>(n)) ? 1 : 0;
    q.use_tma_y = encode_chunk_rows_map(&q.tmap_y, y, static_cast<long long>(n)) ? 1 : 0;
    q.y_vec = (reinterpret_cast<uintptr_t>(y) & 15u) == 0 ? 1 : 0;
    q.prof = t->prof;
    void* args[] = {&q};
    const int grid = static_cast<int>(std::min<size_t>(tiles, static_cast<size_t>(t->grid_max)));
    return cuda_status(cudaLaunchCooperativeKernel(t->fn, dim3(grid), dim3(iirgb::TC_THREADS), args,
                                                   iirgb::tc_smem_bytes(t->KD), stream));
}

namespace {
bool encode_chunk_rows_map(CUtensorMap* map, const float* base, long long n) {
    return encode_rows_map(map, base, n / TC_L, TC_L, 32, TC_NB);
}
}  // namespace

}  // namespace iirhost
