// iir_host_internal.h — planner helpers defined in iir_host.cu and used by the other host
// translation units of the library (not part of the C ABI).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "iir_params.h"
#include "iir_registry.h"

namespace iirhost {

struct SectionF32 {
    float b1, b2, a1, a2;
};

// Registered kernel for (realization, B, N, order, schedule); nullptr if none.
const iirgb::KernelEntry* find_entry(int kind, int B, int N, int order, int pipeline = 0, int tail = 0,
                                     int tiny = 0);
// Resident blocks per SM for a registered kernel; also sets its dynamic shared memory limit.
int blocks_per_sm(const iirgb::KernelEntry& e, int device);
// scipy SOS rows -> b0 = a0 = 1 sections (FP64 division, float32 result) and the gain.
int normalise_sos(const float* sos, int n_sections, std::vector<SectionF32>& out, double& gain);
int normalise_sos(const float* sos, int n_sections, SectionF32* out, double& gain);  // out[n_sections]
// Tail-aggregate schedule: the least number of IIR_TAIL_PIECE-sample pieces (<= max_pieces) over
// which the cascade's state decays below 1e-10 (0 if none), and the cascade's transition over one
// piece (2K x 2K, row-major, float32) in piece_phi.
int tail_pieces(const SectionF32* secs, int K, int max_pieces, std::vector<float>& piece_phi);
// One section's kernel coefficients and its IIR_TAB_STRIDE lane-table entries.
int precompute_section(const SectionF32& s, int kind, int rows, int N, IirSection& q, float4* tab);
// 2D tensor map over a float32 signal viewed as 128-byte lines, box = lines_per_block lines.
bool encode_lines_map(CUtensorMap* map, const float* base, long long n, int lines_per_block);
// 2D tensor map over rows of row_len floats, box {box_inner, box_rows}, 128-byte swizzle.
bool encode_rows_map(CUtensorMap* map, const float* base, long long rows, int row_len, int box_inner, int box_rows);
// The chunk kernels' view: rows of n_per_row samples (one box per 32-sample plane), or lines.
bool encode_chunk_map(CUtensorMap* map, const float* base, long long n, int n_per_row, int rows_per_chunk,
                      bool planes);
// cudaError_t -> IIR_* status (clears the runtime's sticky last error).
int cuda_status(cudaError_t e);
// A launch state's error word ((epoch << 32) | device code, 0 = none) -> IIR_* status.
int device_error_status(unsigned long long word);

// Precision form (iir_tc.cu): the cascade's chunk solve as tensor-core GEMMs.
struct TcPlan;
int tc_plan_create(TcPlan** out, const SectionF32* secs, int n_sections, double gain, size_t max_n);
int tc_plan_execute(TcPlan* t, const float* x, float* y, size_t n, long long timeout_ns, long long withhold,
                    cudaStream_t stream);
IirLaunchState* tc_plan_state(TcPlan* t);
void tc_plan_set_profile(TcPlan* t, unsigned long long* buf);
int tc_plan_grid(const TcPlan* t);
void tc_plan_destroy(TcPlan* t);

}  // namespace iirhost
