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

void register_stcr(std::vector<KernelEntry>& reg) {
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
