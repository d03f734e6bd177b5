// iir_noalloc.cu — iir_sos_filter_noalloc: cascaded-biquad filtering that allocates no memory.
//
// Who needs it: a caller that must not allocate while it filters. cudaMalloc / cudaFree can
// synchronise the whole device and can fail under memory pressure, so a real-time caller (an
// audio or radio callback with a fixed deadline) or a caller whose device memory is reserved
// by another allocator cannot use the plan API, which allocates its launch state, carry slots
// and tables. This entry point keeps all three in one fixed array of static device memory
// (g_scratch below) and launches the PH realization (32 x 64 geometry) on it.
//
// Limits: n <= IIR_NOALLOC_MAX_SAMPLES samples, 1..IIR_MAX_SECTIONS sections. The scratch
// array is shared by every call on a device: calls must be ordered (one stream, or streams
// ordered by events); calls that overlap in time race on the carry slots and produce wrong
// output or a lookback timeout.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/iir_gb300.h"
#include "iir_host_internal.h"
#include "iir_params.h"
#include "iir_registry.h"

using namespace iirgb;
using namespace iirhost;

namespace {

constexpr int NA_B = 32, NA_N = 64;                  // PH geometry: 128 rows x 64 samples
constexpr size_t NA_CHUNK = 128 * 64;                // samples per chunk (= per carry slot)
constexpr size_t NA_MAX_CHUNKS = IIR_NOALLOC_MAX_SAMPLES / NA_CHUNK;
static_assert(IIR_NOALLOC_MAX_SAMPLES % NA_CHUNK == 0, "whole chunks");
// carry words per section: 4 per chunk slot, 4 per group slot, 2 spare slots
constexpr size_t NA_CARRY_WORDS = 4 * (NA_MAX_CHUNKS + NA_MAX_CHUNKS / IIR_GROUP + 2);
constexpr size_t NA_STATE_BYTES = 256;
constexpr size_t NA_TABLE_BYTES = sizeof(float4) * IIR_TAB_STRIDE * IIR_MAX_SECTIONS;
constexpr size_t NA_CARRY_BYTES = sizeof(unsigned long long) * NA_CARRY_WORDS * IIR_MAX_SECTIONS;
constexpr size_t NA_BYTES = NA_STATE_BYTES + NA_TABLE_BYTES + NA_CARRY_BYTES;  // 2.2 MB
static_assert(sizeof(IirLaunchState) <= NA_STATE_BYTES, "launch state fits its slot");
static_assert(NA_TABLE_BYTES % 256 == 0, "carry slots stay 256-byte aligned");

// Layout: [launch state | lane tables (IIR_MAX_SECTIONS x IIR_TAB_STRIDE float4) |
//          carry slots (IIR_MAX_SECTIONS x NA_CARRY_WORDS words)].
// The launch state and the carry slots must start at zero (flags are launch-versioned; they
// are zeroed once per device at setup and again every 2^30 launches). The tables are
// rewritten by every call.
static __device__ __align__(256) unsigned long long g_scratch[NA_BYTES / sizeof(unsigned long long)];

constexpr int NA_MAX_DEVICES = 64;
struct DeviceScratch {
    bool ready = false;
    unsigned char* base = nullptr;
    unsigned long long launches = 0;  // since the slots were last zeroed
};
std::mutex g_mu;
DeviceScratch g_dev[NA_MAX_DEVICES];

// Once per device, with that device current: resolve the array's address and zero it.
int setup(int device, DeviceScratch& d, const KernelEntry& e) {
    if (d.ready) return IIR_OK;
    void* ptr = nullptr;
    int st = cuda_status(cudaGetSymbolAddress(&ptr, g_scratch));
    if (st) return st;
    if (blocks_per_sm(e, device) <= 0) return IIR_ERR_UNSUPPORTED;
    st = cuda_status(cudaMemset(ptr, 0, NA_BYTES));
    if (st) return st;
    st = cuda_status(cudaDeviceSynchronize());
    if (st) return st;
    d.base = static_cast<unsigned char*>(ptr);
    d.launches = 0;
    d.ready = true;
    return IIR_OK;
}

}  // namespace

extern "C" int iir_sos_filter_noalloc(const float* x, float* y, size_t n, const float* sos, int n_sections,
                                      void* stream_) {
    if (!sos || n_sections < 1 || n_sections > IIR_MAX_SECTIONS) return IIR_ERR_INVALID_ARGUMENT;
    if (n > IIR_NOALLOC_MAX_SAMPLES) return IIR_ERR_TOO_LARGE;
    if (n > 0 && (!x || !y)) return IIR_ERR_INVALID_ARGUMENT;
    const char* xb = reinterpret_cast<const char*>(x);
    const char* yb = reinterpret_cast<const char*>(y);
    if (n > 0 && xb < yb + n * sizeof(float) && yb < xb + n * sizeof(float)) return IIR_ERR_INVALID_ARGUMENT;
    const KernelEntry* e = find_entry(IIR_KIND_PH, NA_B, NA_N, 0);
    if (!e || static_cast<size_t>(e->rows) * NA_N != NA_CHUNK) return IIR_ERR_UNSUPPORTED;

    // coefficients and lane tables live on the host stack
    SectionF32 secs[IIR_MAX_SECTIONS];
    double gain = 1.0;
    int st = normalise_sos(sos, n_sections, secs, gain);
    if (st) return st;
    IirParams q;
    std::memset(&q, 0, sizeof(q));
    float4 tabs[IIR_TAB_STRIDE * IIR_MAX_SECTIONS];
    for (int s = 0; s < n_sections; ++s) {
        st = precompute_section(secs[s], IIR_KIND_PH, e->rows, NA_N, q.sec[s], tabs + s * IIR_TAB_STRIDE);
        if (st) return st;
    }

    int device = 0;
    st = cuda_status(cudaGetDevice(&device));
    if (st) return st;
    if (device < 0 || device >= NA_MAX_DEVICES) return IIR_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceScratch& d = g_dev[device];
    st = setup(device, d, *e);
    if (st) return st;
    if (n == 0) return IIR_OK;

    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    unsigned char* tables = d.base + NA_STATE_BYTES;
    unsigned char* carry = tables + NA_TABLE_BYTES;
    // Pageable source: the call returns once the driver has staged the bytes, so the stack
    // buffer may go out of scope; the copy is ordered before the launch on the stream.
    st = cuda_status(cudaMemcpyAsync(tables, tabs, sizeof(float4) * IIR_TAB_STRIDE * n_sections,
                                     cudaMemcpyHostToDevice, stream));
    if (st) return st;
    if (++d.launches >= (1ull << 30)) {
        st = cuda_status(cudaMemsetAsync(d.base, 0, NA_STATE_BYTES, stream));
        if (!st) st = cuda_status(cudaMemsetAsync(carry, 0, NA_CARRY_BYTES, stream));
        if (st) return st;
        d.launches = 1;
    }

    const size_t nchunks = (n + NA_CHUNK - 1) / NA_CHUNK;
    q.x = x;
    q.y = y;
    q.n = static_cast<long long>(n);
    q.state = reinterpret_cast<IirLaunchState*>(d.base);
    q.tables = reinterpret_cast<const float4*>(tables);
    q.carry = reinterpret_cast<unsigned long long*>(carry);
    q.carry_stride = NA_CARRY_WORDS;
    q.carry_cap = static_cast<unsigned int>(NA_MAX_CHUNKS);
    q.nchunks = static_cast<unsigned int>(nchunks);
    q.n_sections = n_sections;
    q.gain = static_cast<float>(gain);
    q.timeout_ns = 1000000000ll;
    q.withhold_chunk = -1;
    const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15u) == 0;
    q.use_tma = (aligned && encode_chunk_map(&q.tmap_x, x, static_cast<long long>(n), NA_N, e->rows, e->planes != 0) &&
                 encode_chunk_map(&q.tmap_y, y, static_cast<long long>(n), NA_N, e->rows, e->planes != 0))
                    ? 1
                    : 0;
    void* args[] = {&q};
    return cuda_status(
        cudaLaunchKernel(e->fn, dim3(static_cast<unsigned>(nchunks)), dim3(e->threads), args, e->smem, stream));
}
