// iir_pipe.cuh — pieces shared by the persistent single-section schedule (iir_twopass.cuh):
// the per-block hand-off state, the shared-memory layout constants, bounded mbarrier waits and
// the launch epoch of a persistent grid.
#pragma once
#include "iir_device.cuh"

namespace iirgb {

// Rows per chunk of the single-section pipelines, per samples per row: chunks of 8192 samples,
// except rows of 32 samples for PH and DTCR (128 rows, 4096 samples). Measured at 2^28, order 2,
// 32x32, 256 -> 128 rows: PH 715 -> 769, DTCR_UNROLL 480 -> 512, STCR_UNROLL 719 -> 706 GS/s, so
// STCR keeps 256.
#ifndef IIR_PIPE_ROWS_N32
#define IIR_PIPE_ROWS_N32 128
#endif
#ifndef IIR_PIPE_ROWS_N32_STCR
#define IIR_PIPE_ROWS_N32_STCR 256
#endif
#ifndef IIR_PIPE_ROWS_N64
#define IIR_PIPE_ROWS_N64 128
#endif
#ifndef IIR_PIPE_ROWS_N128
#define IIR_PIPE_ROWS_N128 64
#endif

// Shared-memory layout of the single-section pipelines' chunk buffers (swz in iir_device.cuh):
// 0 = lines (one tensor copy per chunk, contiguous in memory), 1 = planes of 32-sample columns.
// Measured at 2^28 samples, order 2: rows of 64 samples keep lines (planes cost 5-7%: each
// plane copy reads 128 of every 256 bytes); rows of 128 samples take planes, since lines leave
// them 4-way bank conflicts (32x128: PH 530 -> 688, STCR_UNROLL 477 -> 650, DTCR_UNROLL
// 625 -> 725 GS/s).
#ifndef IIR_TWO_PLANES
#define IIR_TWO_PLANES 0
#endif
#ifndef IIR_TWO_PLANES_N128
#define IIR_TWO_PLANES_N128 1
#endif
// Layout of a single-section pipeline's chunk buffer for rows of N samples.
constexpr bool two_planes(int n) { return n >= 128 ? (IIR_TWO_PLANES_N128 != 0) : (IIR_TWO_PLANES != 0); }

struct PipeAux {
    unsigned long long full[8];
    unsigned long long part[8];
    unsigned long long xrdy[8];
    unsigned long long done[8];
    float partv[8][2];
    float xv[8][2];
    float wtot[16][2][2];
    float xch[2][16][2];    // cyclic-reduction tiles over several warps: per-level row hand-off
    float xscan[16][2][2];  // and the warps' top-level scan totals
    unsigned int epoch;
    int bail;      // lookback gave up: no more stores
    int abandon;   // an mbarrier wait ran out: skip every remaining wait
    int pad;
};

template <int ROWS, int N, int S>
struct PipeGeom {
    static constexpr int CHUNK = ROWS * N;
    static constexpr int LINES = CHUNK / 32;
    static_assert(N == 16 || N == 32 || N == 64 || N == 128, "samples per row");
    static_assert(LINES <= 256, "one TMA box per chunk");
    static_assert(S >= 2 && S <= 8, "stages");
    static constexpr size_t DATA_BYTES = static_cast<size_t>(CHUNK) * sizeof(float);
    static constexpr size_t ZIN_BYTES = static_cast<size_t>(ROWS) * 2 * sizeof(float);
    static constexpr size_t HIST_BYTES = 128;  // the 32 input samples before the chunk
    // table cache: C^(r+1) (r < ROWS), G^(t+1) (t < 32), Q^l and Q^(32 l) (l <= 32), A^(N/2)
    static constexpr int TC_CPOW = 0, TC_GPOW = ROWS, TC_QC = ROWS + 32, TC_QG = ROWS + 65, TC_HALF = ROWS + 98,
                         TC_LEN = ROWS + 100;
    static constexpr size_t TC_BYTES = static_cast<size_t>(TC_LEN) * 16;
};

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded mbarrier wait that gives up at once after any earlier wait of the block ran out.
// Its limit is four lookback limits: a stage wait is downstream of a lookback, so a chunk
// whose predecessor never publishes reports the lookback timeout (the cause), not this.
__device__ __forceinline__ bool pipe_wait(PipeAux* aux, unsigned long long* bar, uint32_t parity,
                                          const IirParams& p, uint32_t epoch) {
    if (*reinterpret_cast<volatile int*>(&aux->abandon)) return false;
    const long long limit = p.timeout_ns < (1ll << 60) ? 4 * p.timeout_ns : p.timeout_ns;
    if (wait_mbar_bounded(bar, parity, limit)) return true;
    *reinterpret_cast<volatile int*>(&aux->abandon) = 1;
    raise_error(p.state, epoch, IIR_DEV_ERR_MBARRIER);
    return false;
}

// Last block out advances the launch epoch (every block of a persistent launch runs to the
// end, so the ticket counter is not used).
__device__ __forceinline__ void pipe_finish(IirLaunchState* st, uint32_t epoch) {
    __threadfence();
    const unsigned prev = atomicAdd(&st->done, 1u);
    if (prev == gridDim.x - 1) {
        atomicExch(&st->done, 0u);
        atomicExch(&st->ticket, static_cast<unsigned long long>(epoch + 1u) << 32);
        __threadfence();
    }
}

}  // namespace iirgb
