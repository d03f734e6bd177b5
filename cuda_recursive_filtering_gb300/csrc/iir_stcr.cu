// iir_stcr.cu — STCR realization for sm_103a (cyclic-reduction row solver in iir_cr.cuh).
//
// Reference: include/stcr_kernels.cuh. STCR: one thread per row runs the double-sided first round and the log-depth elimination / back-substitution of both parity halves (stcr_kernels.cuh:279-605, 2586-2964); loop form STCR_*_LOOP, register form STCR_*_UNROLL_* (stcr_kernels.cuh:608-3605).
#include "iir_cr.cuh"
#include "iir_registry.h"

namespace iirgb {

template <int N, int ROWS, bool UNROLL>
__global__ void __launch_bounds__(CrBlock<false, 32, N, ROWS, UNROLL>::THREADS,
                                  CrBlock<false, 32, N, ROWS, UNROLL>::MIN_BLOCKS)
    iir_stcr_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    CrBlock<false, 32, N, ROWS, UNROLL>::run(p, smem);
}

// A tile of BLOCK_SIZE rows is the reference's chunk; a block filters ROWS rows (several
// tiles), so BLOCK_SIZE = 32 and 64 share one instantiation per N.
template <int N, int ROWS, bool UNROLL>
static void add(std::vector<KernelEntry>& reg) {
    using Blk = CrBlock<false, 32, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_STCR_UNROLL : IIR_KIND_STCR;
    for (int b : {32, 64})
        reg.push_back(KernelEntry{kind, b, N, (const void*)iir_stcr_kernel<N, ROWS, UNROLL>, Blk::THREADS, Blk::SMEM_BYTES,
                                  0, ROWS});
}

template <int N, int ROWS, bool UNROLL, int S, int D>
__global__ void __launch_bounds__(64 + CrTwo<false, N, ROWS, UNROLL>::NW * 32,
                                  TwoPassGeom<ROWS, N, S, D>::min_blocks(64 + CrTwo<false, N, ROWS, UNROLL>::NW * 32))
    iir_stcr_two_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    run_twopass<CrTwo<false, N, ROWS, UNROLL>, S, D>(p, smem);
}

#ifndef IIR_TWO_STAGES
#define IIR_TWO_STAGES 3
#endif
#ifndef IIR_TWO_LAG
#define IIR_TWO_LAG 2
#endif

// Single-section two-pass kernel (chosen for one section when registered for the geometry).
template <int N, int ROWS, bool UNROLL>
static void add_two(std::vector<KernelEntry>& reg) {
    using R = CrTwo<false, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_STCR_UNROLL : IIR_KIND_STCR;
    for (int b : {32, 64}) {
        KernelEntry e{kind, b, N, (const void*)iir_stcr_two_kernel<N, ROWS, UNROLL, IIR_TWO_STAGES, IIR_TWO_LAG>,
                      64 + R::NW * 32, TwoPassGeom<ROWS, N, IIR_TWO_STAGES, IIR_TWO_LAG>::SMEM_BYTES, 0, ROWS};
        e.pipeline = 1;
        e.planes = two_planes(N) ? 1 : 0;
        reg.push_back(e);
    }
}

void register_stcr(std::vector<KernelEntry>& reg) {
    // rows per chunk for 32, 64 and 128 samples per row: iir_pipe.cuh
    add_two<32, IIR_PIPE_ROWS_N32_STCR, true>(reg);
    add_two<32, IIR_PIPE_ROWS_N32_STCR, false>(reg);
    add_two<64, IIR_PIPE_ROWS_N64, true>(reg);
    add_two<64, IIR_PIPE_ROWS_N64, false>(reg);
    add_two<128, IIR_PIPE_ROWS_N128, true>(reg);
    add_two<128, IIR_PIPE_ROWS_N128, false>(reg);
    add<16, 128, false>(reg);
    add<32, 128, false>(reg);
    add<64, 128, false>(reg);
    add<128, 64, false>(reg);
    add<16, 128, true>(reg);
    add<32, 128, true>(reg);
    add<64, 128, true>(reg);
    add<128, 64, true>(reg);
}

}  // namespace iirgb
