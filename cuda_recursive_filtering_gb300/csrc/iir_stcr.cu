// iir_stcr.cu — STCR realization for sm_103a (cyclic-reduction row solver in iir_cr.cuh).
//
// Reference: include/stcr_kernels.cuh. STCR: one thread per row runs the double-sided first round and the log-depth elimination /
// back-substitution of both parity halves (stcr_kernels.cuh:279-605, 2586-2964); loop form
// STCR_*_LOOP, straight-line form STCR_*_UNROLL_* (stcr_kernels.cuh:608-3605).
// BLOCK_SIZE is the tile height B of the cyclic reduction (the reference's thread block): one warp per tile at B = 32,
// two at B = 64 (STCR_64_*, stcr_kernels.cuh:2586-3605).
#include "iir_cr.cuh"
#include "iir_registry.h"

namespace iirgb {

template <int B, int N, int ROWS, bool UNROLL>
__global__ void __launch_bounds__(CrBlock<false, B, N, ROWS, UNROLL>::THREADS,
                                  CrBlock<false, B, N, ROWS, UNROLL>::MIN_BLOCKS)
    iir_stcr_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    CrBlock<false, B, N, ROWS, UNROLL>::run(p, smem);
}

// Cascade kernel on the tail-aggregate schedule (iir_tail.cuh): one lookback per chunk.
template <int B, int N, int ROWS, bool UNROLL>
__global__ void __launch_bounds__(CrBlock<false, B, N, ROWS, UNROLL, true, true>::THREADS,
                                  CrBlock<false, B, N, ROWS, UNROLL, true, true>::MIN_BLOCKS)
    iir_stcr_tail_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    CrBlock<false, B, N, ROWS, UNROLL, true, true>::run(p, smem);
}

// One block per chunk of ROWS rows (ROWS / B tiles), with the per-section and the
// tail-aggregate lookback.
template <int B, int N, int ROWS, bool UNROLL>
static void add(std::vector<KernelEntry>& reg) {
    using Blk = CrBlock<false, B, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_STCR_UNROLL : IIR_KIND_STCR;
    reg.push_back(KernelEntry{kind, B, N, (const void*)iir_stcr_kernel<B, N, ROWS, UNROLL>, Blk::THREADS,
                              Blk::SMEM_BYTES, 0, ROWS});
    KernelEntry t{kind, B, N, (const void*)iir_stcr_tail_kernel<B, N, ROWS, UNROLL>, Blk::THREADS, Blk::SMEM_BYTES,
                  0, ROWS};
    t.tail = 1;
    reg.push_back(t);
}

// A one-tile (32-row) tail kernel for short single-section signals: more, shorter chunks, so
// a launch ends sooner.
template <int B, int N, int ROWS, bool UNROLL>
static void add_tiny(std::vector<KernelEntry>& reg) {
    using Blk = CrBlock<false, B, N, ROWS, UNROLL, true, true>;
    const int kind = UNROLL ? IIR_KIND_STCR_UNROLL : IIR_KIND_STCR;
    KernelEntry t{kind, B, N, (const void*)iir_stcr_tail_kernel<B, N, ROWS, UNROLL>, Blk::THREADS, Blk::SMEM_BYTES,
                  0, ROWS};
    t.tail = 1;
    t.tiny = 1;
    reg.push_back(t);
}

template <int B, int N, int ROWS, bool UNROLL, int S, int D>
__global__ void __launch_bounds__(64 + CrTwo<false, B, N, ROWS, UNROLL>::NW * 32,
                                  TwoPassGeom<ROWS, N, S, D>::min_blocks(64 + CrTwo<false, B, N, ROWS, UNROLL>::NW * 32))
    iir_stcr_two_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    run_twopass<CrTwo<false, B, N, ROWS, UNROLL>, S, D>(p, smem);
}

#ifndef IIR_TWO_STAGES
#define IIR_TWO_STAGES 3
#endif
#ifndef IIR_TWO_LAG
#define IIR_TWO_LAG 2
#endif

// Single-section two-pass kernel (chosen for one section when registered for the geometry).
template <int B, int N, int ROWS, bool UNROLL>
static void add_two(std::vector<KernelEntry>& reg) {
    using R = CrTwo<false, B, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_STCR_UNROLL : IIR_KIND_STCR;
    KernelEntry e{kind, B, N, (const void*)iir_stcr_two_kernel<B, N, ROWS, UNROLL, IIR_TWO_STAGES, IIR_TWO_LAG>,
                  64 + R::NW * 32, TwoPassGeom<ROWS, N, IIR_TWO_STAGES, IIR_TWO_LAG>::SMEM_BYTES, 0, ROWS};
    e.pipeline = 1;
    e.planes = two_planes(N) ? 1 : 0;
    reg.push_back(e);
}

template <int B, bool UNROLL>
static void add_geometry_set(std::vector<KernelEntry>& reg) {
    // rows per chunk for 32, 64 and 128 samples per row: iir_pipe.cuh
    add_two<B, 32, IIR_PIPE_ROWS_N32_STCR, UNROLL>(reg);
    add_two<B, 64, IIR_PIPE_ROWS_N64, UNROLL>(reg);
    add_two<B, 128, IIR_PIPE_ROWS_N128, UNROLL>(reg);
    add<B, 16, 128, UNROLL>(reg);
    add<B, 32, 128, UNROLL>(reg);
    add<B, 64, 128, UNROLL>(reg);
    add<B, 128, 64, UNROLL>(reg);
}

void register_stcr(std::vector<KernelEntry>& reg) {
    add_geometry_set<32, true>(reg);
    add_geometry_set<32, false>(reg);
    add_tiny<32, 64, 32, true>(reg);
    add_tiny<32, 64, 32, false>(reg);
    add_geometry_set<64, true>(reg);
    add_geometry_set<64, false>(reg);
}

}  // namespace iirgb
