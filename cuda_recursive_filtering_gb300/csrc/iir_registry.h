// iir_registry.h — table of compiled kernel instantiations, filled by each realization's
// translation unit and looked up by the host planner (iir_host.cu). Replaces the
// reference's compile-time KERNEL_FUNC selection (include/stcr_kernels.cuh:3613-3633,
// include/dtcr_kernels.cuh:3527-3547, include/plr_kernels.cuh:3110-3123).
#pragma once
#include <cstddef>
#include <vector>

namespace iirgb {

enum {
    IIR_KIND_PH = 1,
    IIR_KIND_STCR = 2,
    IIR_KIND_STCR_UNROLL = 3,
    IIR_KIND_DTCR = 4,
    IIR_KIND_DTCR_UNROLL = 5,
    IIR_KIND_PLR = 6,
    IIR_KIND_TC = 7,
};

struct KernelEntry {
    int kind;
    int B;          // rows per chunk (PLR: threads per block)
    int N;          // samples per row (PLR: values per thread)
    const void* fn;
    int threads;    // threads per block
    size_t smem;    // dynamic shared memory bytes
    int order;      // PLR direct-form order (0 for the cascaded realizations)
    int rows;       // rows per block (tiles x B) for the row-major realizations
    int pipeline = 0;  // 1: single-section persistent pipeline, launched cooperatively
    int planes = 1;    // chunk buffer layout: 1 = planes of 32-sample columns, 0 = lines (swz)
    int tail = 0;      // 1: cascade kernel on the tail-aggregate schedule (iir_tail.cuh)
    int tiny = 0;      // 1: a 32-row tail kernel that single-section plans use for short signals
};

void register_ph(std::vector<KernelEntry>& reg);
void register_stcr(std::vector<KernelEntry>& reg);
void register_dtcr(std::vector<KernelEntry>& reg);
void register_plr(std::vector<KernelEntry>& reg);

}  // namespace iirgb
