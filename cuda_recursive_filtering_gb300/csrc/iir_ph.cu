// iir_ph.cu — PH kernels (row solver templates in iir_ph.cuh) and their registration.
#include "iir_ph.cuh"
#include "iir_registry.h"

namespace iirgb {

template <int N, int ROWS, int S, int D>
__global__ void __launch_bounds__(64 + ROWS, TwoPassGeom<ROWS, N, S, D>::min_blocks(64 + ROWS))
    iir_ph_two_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    run_twopass<PhTwo<N, ROWS>, S, D>(p, smem);
}

template <int B, int N, int ROWS>
__global__ void __launch_bounds__(32 + ROWS, BlockGeom<ROWS, N>::min_blocks(32 + ROWS))
    iir_ph_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    PhBlock<B, N, ROWS>::run(p, smem);
}

// Cascade kernel on the tail-aggregate schedule (iir_tail.cuh): one lookback per chunk.
template <int B, int N, int ROWS>
__global__ void __launch_bounds__(32 + ROWS, BlockGeom<ROWS, N>::min_blocks(32 + ROWS))
    iir_ph_tail_kernel(const __grid_constant__ IirParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    PhBlock<B, N, ROWS, true>::run(p, smem);
}

template <int B, int N, int ROWS>
static void add_ph(std::vector<KernelEntry>& reg) {
    reg.push_back(KernelEntry{IIR_KIND_PH, B, N, (const void*)iir_ph_kernel<B, N, ROWS>, 32 + ROWS,
                              BlockGeom<ROWS, N>::SMEM_BYTES, 0, ROWS});
    KernelEntry t{IIR_KIND_PH, B, N, (const void*)iir_ph_tail_kernel<B, N, ROWS>, 32 + ROWS,
                  BlockGeom<ROWS, N>::SMEM_BYTES, 0, ROWS};
    t.tail = 1;
    reg.push_back(t);
}

// A 32-row tail kernel for short single-section signals: more, shorter chunks (a 2^16-sample
// signal is 32 chunks of 2048 instead of 8 of 8192), so a launch ends sooner.
template <int B, int N, int ROWS>
static void add_ph_tiny(std::vector<KernelEntry>& reg) {
    KernelEntry t{IIR_KIND_PH, B, N, (const void*)iir_ph_tail_kernel<B, N, ROWS>, 32 + ROWS,
                  BlockGeom<ROWS, N>::SMEM_BYTES, 0, ROWS};
    t.tail = 1;
    t.tiny = 1;
    reg.push_back(t);
}

#ifndef IIR_TWO_STAGES
#define IIR_TWO_STAGES 3
#endif
#ifndef IIR_TWO_LAG
#define IIR_TWO_LAG 2
#endif

// Single-section two-pass kernel (chosen for one section when registered for the geometry).
template <int B, int N, int ROWS>
static void add_ph_two(std::vector<KernelEntry>& reg) {
    KernelEntry e{IIR_KIND_PH, B, N, (const void*)iir_ph_two_kernel<N, ROWS, IIR_TWO_STAGES, IIR_TWO_LAG>, 64 + ROWS,
                  TwoPassGeom<ROWS, N, IIR_TWO_STAGES, IIR_TWO_LAG>::SMEM_BYTES, 0, ROWS};
    e.pipeline = 1;
    e.planes = two_planes(N) ? 1 : 0;
    reg.push_back(e);
}

// Rows per chunk of the one-block-per-chunk (cascade) kernel, per samples per row.
#ifndef IIR_TICKET_ROWS_N64
#define IIR_TICKET_ROWS_N64 128
#endif

void register_ph(std::vector<KernelEntry>& reg) {
    // single-section pipeline (chosen for one section when registered for the geometry)
    // (rows per chunk for 32, 64 and 128 samples per row: iir_pipe.cuh)
    add_ph_two<32, 32, IIR_PIPE_ROWS_N32>(reg);
    add_ph_two<64, 32, IIR_PIPE_ROWS_N32>(reg);
    add_ph_two<32, 64, IIR_PIPE_ROWS_N64>(reg);
    add_ph_two<64, 64, IIR_PIPE_ROWS_N64>(reg);
    add_ph_two<32, 128, IIR_PIPE_ROWS_N128>(reg);
    add_ph_two<64, 128, IIR_PIPE_ROWS_N128>(reg);
    add_ph<32, 16, 128>(reg);
    add_ph<32, 32, 128>(reg);
    add_ph<32, 64, IIR_TICKET_ROWS_N64>(reg);
    add_ph<32, 128, 64>(reg);
    add_ph<64, 16, 128>(reg);
    add_ph<64, 32, 128>(reg);
    add_ph<64, 64, IIR_TICKET_ROWS_N64>(reg);
    add_ph<64, 128, 64>(reg);
    add_ph_tiny<32, 64, 32>(reg);
    add_ph_tiny<64, 64, 32>(reg);
}

}  // namespace iirgb
