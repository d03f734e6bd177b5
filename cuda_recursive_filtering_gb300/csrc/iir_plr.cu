// iir_plr.cu — PLR realization: the whole cascade as ONE direct-form recurrence of order
// K = 2 * sections, solved by the hierarchical merge of Maleki & Burtscher (ASPLOS'18).
//
// Reference: include/plr_kernels.cuh:484-3107 (PLR_2/4/8/16). Per chunk of BT * X samples in
// the strided layout (thread t holds samples v*BT + t, plr_kernels.cuh:520,535):
//   1. FIR t[n] = x[n] + sum_j b_j x[n-1-j] through shared memory (plr_kernels.cuh:539-562);
//   2. intra-warp iterative doubling: at width w the upper half of each w-group adds
//      sum_j fac_j[u] * y_lower[w/2 - K + j], fac_j = n-nacci factors (response at offset u to
//      a unit value in history slot j; plr_kernels.cuh:564-632);
//   3. inter-warp doubling with the same factors through shared memory (plr_kernels.cuh:634-785);
//   4. segment chaining over the X values per thread (plr_kernels.cuh:787-811): here one thread
//      chains the segments' end states with the segment transition (fac_j at the last K offsets)
//      and every segment is then corrected at once, instead of one segment after another with two
//      block barriers each;
//   5. K-dimensional decoupled lookback for the chunk's incoming state and the carry correction
//      val += sum_j fac_j[i] X_j (plr_kernels.cuh:813-899). The lookback is truncated to the m
//      preceding chunks' aggregates when the chunk transition has decayed (||Phi^m|| <= 1e-10),
//      else two-level over groups of 32 chunks.
// Everything is float32 with plain products and sums, as in the reference, so order 16 keeps
// its direct-form numerical fragility (reported by the accuracy tests, not hidden).
#include "iir_lookk.cuh"
#include "iir_registry.h"

namespace iirgb {

template <int KO, int BT, int X>
struct PlrBlock {
    static constexpr int THREADS = 32 + BT;  // control warp + row threads
    static constexpr int CHUNK = BT * X;
    static constexpr int NWR = BT / 32;
    static_assert(BT % 32 == 0 && KO <= 16 && KO % 2 == 0, "PLR geometry");

    struct Smem {
        float xs[KO + CHUNK];           // input of the chunk with K samples of history
        float sfac[KO][BT];             // fac_j[i] for i < BT
        float wlast[NWR][X][KO];        // last K values of each warp per segment
        float seglast[X][KO];           // last K values of each segment solved from zero state
        float segin[X][KO];             // each segment's true history (last K values of the one before)
        float part[KO];
        float Xc[KO];
        unsigned int chunk, epoch;
        int bail;
    };
    static constexpr size_t SMEM_BYTES = sizeof(Smem);

    __device__ static void run(const IirPlrParams& p, unsigned char* smem_raw) {
        Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
        const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
        if (tid == 0) {
            uint32_t epoch;
            sm.chunk = take_ticket(p.state, p.nchunks, epoch);
            sm.epoch = epoch;
            sm.bail = 0;
        }
        __syncthreads();
        const uint32_t c = sm.chunk, epoch = sm.epoch;
        const long long cs = static_cast<long long>(c) * CHUNK;
        const bool row = warp > 0;
        const int t = tid - 32;       // row thread index
        const int rw = warp - 1;      // row warp index
        const float gain = p.gain;
        float val[X];
        if (row) {
#pragma unroll
            for (int v = 0; v < X; ++v) {
                const long long gi = cs + v * BT + t;
                const float xv = (gi < p.n) ? __ldg(p.x + gi) * gain : 0.f;
                sm.xs[KO + v * BT + t] = xv;
                val[v] = xv;
            }
            if (t < KO) sm.xs[t] = (c > 0) ? __ldg(p.x + cs - KO + t) * gain : 0.f;
#pragma unroll
            for (int j = 0; j < KO; ++j) sm.sfac[j][t] = __ldg(p.fac + static_cast<size_t>(j) * CHUNK + t);
        }
        __syncthreads();
        if (row) {
            // 1. FIR
#pragma unroll
            for (int v = 0; v < X; ++v) {
                const int i = KO + v * BT + t;
                float acc = val[v];
#pragma unroll
                for (int j = 0; j < KO; ++j) acc = fmaf(p.b[j], sm.xs[i - 1 - j], acc);
                val[v] = acc;
            }
            // 2. intra-warp doubling
#pragma unroll
            for (int half = 1; half < 32; half <<= 1) {
                const int gbase = lane & ~(2 * half - 1);
                const bool upper = (lane & half) != 0;
                const int u = lane & (half - 1);
#pragma unroll
                for (int j = 0; j < KO; ++j) {
                    const int src = half - KO + j;  // position in the group of the lower half's value
                    if (src < 0) continue;
                    const float f = sm.sfac[j][u];
#pragma unroll
                    for (int v = 0; v < X; ++v) {
                        const float y = __shfl_sync(FULL_MASK, val[v], gbase + src);
                        if (upper) val[v] = fmaf(f, y, val[v]);
                    }
                }
            }
            // 3. inter-warp doubling through shared memory (row warps only)
#pragma unroll
            for (int hw = 1; hw < NWR; hw <<= 1) {
                if (lane >= 32 - KO) {
#pragma unroll
                    for (int v = 0; v < X; ++v) sm.wlast[rw][v][lane - (32 - KO)] = val[v];
                }
                named_barrier_rows(NWR);
                if (rw & hw) {
                    const int src = (rw & ~(2 * hw - 1)) + hw - 1;  // last warp of the lower half
                    const int u = (rw & (hw - 1)) * 32 + lane;      // offset in the upper half
#pragma unroll
                    for (int j = 0; j < KO; ++j) {
                        const float f = sm.sfac[j][u];
#pragma unroll
                        for (int v = 0; v < X; ++v) val[v] = fmaf(f, sm.wlast[src][v][j], val[v]);
                    }
                }
                named_barrier_rows(NWR);
            }
            // 4. segment chaining. Segment v (BT samples) was solved from zero history; its true
            // last K values are L_v = local_v + Phi L_(v-1), Phi[i][j] = fac_j[BT - K + i] (the
            // response at the segment's last K offsets to history slot j), L_(-1) = 0 (the chunk's
            // own history enters with the carry, step 5); then segment v adds the response to
            // L_(v-1) at every sample.
            if constexpr (X > 1) {
                if (rw == NWR - 1 && lane >= 32 - KO) {
#pragma unroll
                    for (int v = 0; v < X; ++v) sm.seglast[v][lane - (32 - KO)] = val[v];
                }
                named_barrier_rows(NWR);
                if (t < KO) {  // K threads, one component each, in lockstep within the first warp
                    float L = sm.seglast[0][t];
#pragma unroll
                    for (int v = 1; v < X; ++v) {
                        sm.segin[v][t] = L;
                        __syncwarp(0xffffffffu >> (32 - KO));
                        float nl = sm.seglast[v][t];
#pragma unroll
                        for (int j = 0; j < KO; ++j) nl = fmaf(sm.sfac[j][BT - KO + t], sm.segin[v][j], nl);
                        __syncwarp(0xffffffffu >> (32 - KO));
                        L = nl;
                    }
                    sm.part[t] = L;
                }
                named_barrier_rows(NWR);
#pragma unroll
                for (int v = 1; v < X; ++v) {
#pragma unroll
                    for (int j = 0; j < KO; ++j) val[v] = fmaf(sm.sfac[j][t], sm.segin[v][j], val[v]);
                }
            } else {
                if (rw == NWR - 1 && lane >= 32 - KO) sm.part[lane - (32 - KO)] = val[X - 1];
            }
        }
        __syncthreads();  // (A) chunk aggregate in sm.part
        if (!row) {
            float own[KO], Xc[KO];
#pragma unroll
            for (int j = 0; j < KO; ++j) {
                own[j] = sm.part[j];
                Xc[j] = 0.f;
            }
            const bool withhold = static_cast<long long>(c) == p.withhold_chunk;
            const uint32_t pf = 2u * epoch + 1u, ff = 2u * epoch + 2u;
            unsigned long long* slots = p.carry;
            unsigned long long* gslots = p.carry + static_cast<size_t>(p.carry_cap) * 2 * KO;
            if (lane == 0 && !withhold) publishk<KO>(slots + static_cast<size_t>(c) * 2 * KO, pf, own);
            bool ok = true;
            if (c > 0)
                ok = p.lb_depth > 0 ? lookback_trunc_k<KO>(p, slots, p.pc, c, epoch, p.lb_depth, Xc)
                                    : lookback_hier_k<KO>(p, slots, gslots, p.pc, p.pg, c, epoch, own, withhold, Xc);
            if (lane == 0) {
                if (ok && !withhold) {
                    float f[KO];
                    matvec<KO>(p.pc + KO * KO, Xc, f);  // Phi X
#pragma unroll
                    for (int j = 0; j < KO; ++j) f[j] += own[j];
                    publishk<KO>(slots + static_cast<size_t>(c) * 2 * KO + KO, ff, f);
                    if ((c & 31u) == 31u) publishk<KO>(gslots + static_cast<size_t>(c >> 5) * 2 * KO + KO, ff, f);
                }
#pragma unroll
                for (int j = 0; j < KO; ++j) sm.Xc[j] = Xc[j];
                sm.bail = ok ? 0 : 1;
            }
        }
        __syncthreads();  // (B)
        if (sm.bail || !row) return;
        // 5. carry correction and store
#pragma unroll
        for (int v = 0; v < X; ++v) {
            const int i = v * BT + t;
            float acc = val[v];
#pragma unroll
            for (int j = 0; j < KO; ++j) acc = fmaf(__ldg(p.fac + static_cast<size_t>(j) * CHUNK + i), sm.Xc[j], acc);
            const long long gi = cs + i;
            if (gi < p.n) p.y[gi] = acc;
        }
    }
};

template <int KO, int BT, int X>
__global__ void __launch_bounds__(32 + BT) iir_plr_kernel(const __grid_constant__ IirPlrParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    PlrBlock<KO, BT, X>::run(p, smem);
}

template <int KO, int BT, int X>
static void add_plr(std::vector<KernelEntry>& reg) {
    reg.push_back(KernelEntry{IIR_KIND_PLR, BT, X, (const void*)iir_plr_kernel<KO, BT, X>, 32 + BT,
                              PlrBlock<KO, BT, X>::SMEM_BYTES, KO, 0});
}

// Block sizes per order follow the reference's table (plr_kernels.cuh:57-84): the block
// halves as the order doubles so the per-thread carry footprint fits the register budget.
void register_plr(std::vector<KernelEntry>& reg) {
    add_plr<2, 512, 1>(reg);
    add_plr<2, 512, 4>(reg);
    add_plr<2, 512, 8>(reg);
    add_plr<4, 256, 1>(reg);
    add_plr<4, 256, 4>(reg);
    add_plr<4, 256, 8>(reg);
    add_plr<8, 128, 1>(reg);
    add_plr<8, 128, 4>(reg);
    add_plr<8, 128, 8>(reg);
    add_plr<16, 64, 1>(reg);
    add_plr<16, 64, 4>(reg);
    add_plr<16, 64, 8>(reg);
}

}  // namespace iirgb
