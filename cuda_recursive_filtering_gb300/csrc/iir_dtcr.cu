// iir_dtcr.cu — DTCR realization for sm_103a (cyclic-reduction row solver in iir_cr.cuh).
//
// Reference: include/dtcr_kernels.cuh. DTCR: the first elimination round is fused into the FIR pass and the even / odd halves run
// concurrently on the two threads of a row (dtcr_kernels.cuh:291-657, 2500-2904); loop form
// DTCR_*_LOOP, straight-line form DTCR_*_UNROLL_* (dtcr_kernels.cuh:660-3521).
// BLOCK_SIZE is the tile height B of the cyclic reduction (the reference's thread block): two threads per row, so two warps
// per tile at B = 32 and four at B = 64 (dim3(B, 2), dtcr_kernels.cuh:56; DTCR_64_*,
// dtcr_kernels.cuh:2500-3521).
#include "iir_cr.cuh"
#include "iir_registry.h"

namespace iirgb {

template <int B, int N, int ROWS, bool UNROLL>
__global__ void __launch_bounds__(CrBlock<true, B, N, ROWS, UNROLL>::THREADS,
                                  CrBlock<true, B, N, ROWS, UNROLL>::MIN_BLOCKS)
    iir_dtcr_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    CrBlock<true, B, N, ROWS, UNROLL>::run(p, smem);
}

// Cascade kernel on the tail-aggregate schedule (iir_tail.cuh): one lookback per chunk.
template <int B, int N, int ROWS, bool UNROLL>
__global__ void __launch_bounds__(CrBlock<true, B, N, ROWS, UNROLL, true, true>::THREADS,
                                  CrBlock<true, B, N, ROWS, UNROLL, true, true>::MIN_BLOCKS)
    iir_dtcr_tail_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    CrBlock<true, B, N, ROWS, UNROLL, true, true>::run(p, smem);
}

// One block per chunk of ROWS rows (ROWS / B tiles), with the per-section and the
// tail-aggregate lookback.
template <int B, int N, int ROWS, bool UNROLL>
static void add(std::vector<KernelEntry>& reg) {
    using Blk = CrBlock<true, B, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_DTCR_UNROLL : IIR_KIND_DTCR;
    reg.push_back(KernelEntry{kind, B, N, (const void*)iir_dtcr_kernel<B, N, ROWS, UNROLL>, Blk::THREADS,
                              Blk::SMEM_BYTES, 0, ROWS});
    KernelEntry t{kind, B, N, (const void*)iir_dtcr_tail_kernel<B, N, ROWS, UNROLL>, Blk::THREADS, Blk::SMEM_BYTES,
                  0, ROWS};
    t.tail = 1;
    reg.push_back(t);
}

// A one-tile (32-row) tail kernel for short single-section signals: more, shorter chunks, so
// a launch ends sooner.
template <int B, int N, int ROWS, bool UNROLL>
static void add_tiny(std::vector<KernelEntry>& reg) {
    using Blk = CrBlock<true, B, N, ROWS, UNROLL, true, true>;
    const int kind = UNROLL ? IIR_KIND_DTCR_UNROLL : IIR_KIND_DTCR;
    KernelEntry t{kind, B, N, (const void*)iir_dtcr_tail_kernel<B, N, ROWS, UNROLL>, Blk::THREADS, Blk::SMEM_BYTES,
                  0, ROWS};
    t.tail = 1;
    t.tiny = 1;
    reg.push_back(t);
}

template <int B, int N, int ROWS, bool UNROLL, int S, int D>
__global__ void __launch_bounds__(64 + CrTwo<true, B, N, ROWS, UNROLL>::NW * 32,
                                  TwoPassGeom<ROWS, N, S, D>::min_blocks(64 + CrTwo<true, B, N, ROWS, UNROLL>::NW * 32))
    iir_dtcr_two_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    run_twopass<CrTwo<true, B, N, ROWS, UNROLL>, S, D>(p, smem);
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
    using R = CrTwo<true, B, N, ROWS, UNROLL>;
    const int kind = UNROLL ? IIR_KIND_DTCR_UNROLL : IIR_KIND_DTCR;
    KernelEntry e{kind, B, N, (const void*)iir_dtcr_two_kernel<B, N, ROWS, UNROLL, IIR_TWO_STAGES, IIR_TWO_LAG>,
                  64 + R::NW * 32, TwoPassGeom<ROWS, N, IIR_TWO_STAGES, IIR_TWO_LAG>::SMEM_BYTES, 0, ROWS};
    e.pipeline = 1;
    e.planes = two_planes(N) ? 1 : 0;
    reg.push_back(e);
}

template <int B, bool UNROLL>
static void add_geometry_set(std::vector<KernelEntry>& reg) {
    // rows per chunk for 32, 64 and 128 samples per row: iir_pipe.cuh
    add_two<B, 32, IIR_PIPE_ROWS_N32, UNROLL>(reg);
    add_two<B, 64, IIR_PIPE_ROWS_N64, UNROLL>(reg);
    add_two<B, 128, IIR_PIPE_ROWS_N128, UNROLL>(reg);
    add<B, 16, 64, UNROLL>(reg);
    add<B, 32, 64, UNROLL>(reg);
    add<B, 64, 64, UNROLL>(reg);
    add<B, 128, (B > 32 ? 64 : 32), UNROLL>(reg);
}

void register_dtcr(std::vector<KernelEntry>& reg) {
    add_geometry_set<32, true>(reg);
    add_geometry_set<32, false>(reg);
    add_tiny<32, 64, 32, true>(reg);
    add_tiny<32, 64, 32, false>(reg);
    add_geometry_set<64, true>(reg);
    add_geometry_set<64, false>(reg);
}

}  // namespace iirgb
