// iir_dtcr.cu — DTCR realization for sm_103a (cyclic-reduction row solver in iir_cr.cuh).
//
// Reference: include/dtcr_kernels.cuh. DTCR: the first elimination round is fused into the FIR pass and the even / odd halves run concurrently on the two threads of a row (dtcr_kernels.cuh:291-657, 2500-2904); loop form DTCR_*_LOOP, register form DTCR_*_UNROLL_* (dtcr_kernels.cuh:660-3521).
#include "iir_cr.cuh"
#include "iir_registry.h"

namespace iirgb {

template <int N, int ROWS, bool UNROLL>
__global__ void __launch_bounds__(CrBlock<true, 32, N, ROWS, UNROLL>::THREADS,
                                  CrBlock<true, 32, N, ROWS, UNROLL>::MIN_BLOCKS)
    iir_dtcr_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    CrBlock<true, 32, N, ROWS, UNROLL>::run(p, smem);
}

// A tile of BLOCK_SIZE rows is the reference's chunk; a block filters ROWS rows (several
// tiles), so BLOCK_SIZE = 32 and 64 share one instantiation per N.
template <int N, int ROWS, bool UNROLL>
static void add(std::vector<KernelEntry>& reg) {
    using Blk = CrBlock<true, 32, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_DTCR_UNROLL : IIR_KIND_DTCR;
    for (int b : {32, 64})
        reg.push_back(KernelEntry{kind, b, N, (const void*)iir_dtcr_kernel<N, ROWS, UNROLL>, Blk::THREADS, Blk::SMEM_BYTES,
                                  0, ROWS});
}

template <int N, int ROWS, bool UNROLL, int S, int D>
__global__ void __launch_bounds__(64 + CrTwo<true, N, ROWS, UNROLL>::NW * 32,
                                  TwoPassGeom<ROWS, N, S, D>::min_blocks(64 + CrTwo<true, N, ROWS, UNROLL>::NW * 32))
    iir_dtcr_two_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    run_twopass<CrTwo<true, N, ROWS, UNROLL>, S, D>(p, smem);
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
    using R = CrTwo<true, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_DTCR_UNROLL : IIR_KIND_DTCR;
    for (int b : {32, 64}) {
        KernelEntry e{kind, b, N, (const void*)iir_dtcr_two_kernel<N, ROWS, UNROLL, IIR_TWO_STAGES, IIR_TWO_LAG>,
                      64 + R::NW * 32, TwoPassGeom<ROWS, N, IIR_TWO_STAGES, IIR_TWO_LAG>::SMEM_BYTES, 0, ROWS};
        e.pipeline = 1;
        e.planes = two_planes(N) ? 1 : 0;
        reg.push_back(e);
    }
}

void register_dtcr(std::vector<KernelEntry>& reg) {
    // rows per chunk for 32, 64 and 128 samples per row: iir_pipe.cuh
    add_two<32, IIR_PIPE_ROWS_N32, true>(reg);
    add_two<32, IIR_PIPE_ROWS_N32, false>(reg);
    add_two<64, IIR_PIPE_ROWS_N64, true>(reg);
    add_two<64, IIR_PIPE_ROWS_N64, false>(reg);
    add_two<128, IIR_PIPE_ROWS_N128, true>(reg);
    add_two<128, IIR_PIPE_ROWS_N128, false>(reg);
    add<16, 64, false>(reg);
    add<32, 64, false>(reg);
    add<64, 64, false>(reg);
    add<128, 32, false>(reg);
    add<16, 64, true>(reg);
    add<32, 64, true>(reg);
    add<64, 64, true>(reg);
    add<128, 32, true>(reg);
}

}  // namespace iirgb
