// iir_noalloc.cu — iir_sos_filter_noalloc: cascaded-biquad filtering that allocates no memory.
//
// Who needs it: a caller that must not allocate while it filters. cudaMalloc / cudaFree can
// synchronise the whole device and can fail under memory pressure, so a real-time caller (an
// audio or radio callback with a fixed deadline) or a caller whose device memory is reserved
// by another allocator cannot use the plan API, which allocates its launch state, carry slots
// and tables. This entry point keeps all three in one fixed array of static device memory
// (g_scratch below) and launches the PH realization (32 x 64 geometry) on it.
//
// Each call launches two kernels on the caller's stream: na_prepare_kernel writes the filter's
// lane tables into the array (the tables travel by value in its parameter block, so no host
// buffer has to outlive the call), then the PH kernel filters.
//
// Limits: n <= IIR_NOALLOC_MAX_SAMPLES samples, 1..IIR_MAX_SECTIONS sections. The scratch
// array is shared by every call on a device: calls must be ordered (one stream, or streams
// ordered by events); calls that overlap in time race on the carry slots and produce wrong
// output or a lookback timeout. Such a device-side failure is returned by a later call.
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
// Error words of the devices' launches, in host memory that the devices write to (page-locked
// and mapped once, at the first setup): a failing launch stores its error word here, so a later
// call sees it without synchronising. Static, so nothing is allocated for it.
alignas(4096) unsigned long long g_host_err[4096 / sizeof(unsigned long long)];
static_assert(NA_MAX_DEVICES <= 4096 / sizeof(unsigned long long), "one word per device");

struct DeviceScratch {
    bool ready = false;
    unsigned char* base = nullptr;  // device address of g_scratch on this device
};
std::mutex g_mu;
DeviceScratch g_dev[NA_MAX_DEVICES];
std::once_flag g_register_once;
int g_register_status = IIR_OK;

// Lane tables of up to NA_UPLOAD_SECTIONS sections, passed by value to na_prepare_kernel
// (kernel parameters are limited to 32764 bytes).
constexpr int NA_UPLOAD_SECTIONS = 4;
struct NaUpload {
    float4 tab[NA_UPLOAD_SECTIONS * IIR_TAB_STRIDE];
    unsigned char* base;  // device address of g_scratch
    int first;            // first section of this upload
    int count;            // sections in it
};
static_assert(sizeof(NaUpload) <= 32000, "fits a kernel parameter block");

constexpr int NA_PREP_THREADS = 512;

// One block. The first upload of a call also restarts the launch-versioned state every 2^30
// launches (the epoch is the launch count since the last restart): it zeroes the carry slots
// and the ticket / error words, leaving the host error address in place. A single block does
// it, so no other thread reads the state meanwhile; the filter launch that follows on the
// stream sees epoch 0 and clean slots.
__global__ void __launch_bounds__(NA_PREP_THREADS) na_prepare_kernel(const __grid_constant__ NaUpload u) {
    IirLaunchState* state = reinterpret_cast<IirLaunchState*>(u.base);
    if (u.first == 0) {
        const unsigned long long t = *reinterpret_cast<volatile unsigned long long*>(&state->ticket);
        if ((t >> 32) >= (1ull << 30)) {  // the same value in every thread: a uniform branch
            unsigned long long* carry = reinterpret_cast<unsigned long long*>(u.base + NA_STATE_BYTES + NA_TABLE_BYTES);
            for (size_t i = threadIdx.x; i < NA_CARRY_BYTES / sizeof(unsigned long long); i += blockDim.x) carry[i] = 0ull;
            __syncthreads();
            if (threadIdx.x == 0) {
                state->ticket = 0ull;
                state->error = 0ull;
                state->done = 0u;
            }
        }
    }
    float4* tables = reinterpret_cast<float4*>(u.base + NA_STATE_BYTES) + static_cast<size_t>(u.first) * IIR_TAB_STRIDE;
    for (int i = threadIdx.x; i < u.count * IIR_TAB_STRIDE; i += blockDim.x) tables[i] = u.tab[i];
}

// Once per device, with that device current: resolve the array's address, zero it and point
// its launch state at the device's host error word.
int setup(int device, DeviceScratch& d, const KernelEntry& e) {
    if (d.ready) return IIR_OK;
    std::call_once(g_register_once, [] {
        const cudaError_t r =
            cudaHostRegister(g_host_err, sizeof(g_host_err), cudaHostRegisterMapped | cudaHostRegisterPortable);
        g_register_status = (r == cudaSuccess || r == cudaErrorHostMemoryAlreadyRegistered) ? IIR_OK : cuda_status(r);
        cudaGetLastError();
    });
    if (g_register_status) return g_register_status;
    void* ptr = nullptr;
    int st = cuda_status(cudaGetSymbolAddress(&ptr, g_scratch));
    if (st) return st;
    if (blocks_per_sm(e, device) <= 0) return IIR_ERR_UNSUPPORTED;
    void* herr = nullptr;
    st = cuda_status(cudaHostGetDevicePointer(&herr, &g_host_err[device], 0));
    if (st) return st;
    st = cuda_status(cudaMemset(ptr, 0, NA_BYTES));
    if (st) return st;
    st = cuda_status(cudaMemcpy(static_cast<char*>(ptr) + offsetof(IirLaunchState, host_error), &herr, sizeof(herr),
                                cudaMemcpyHostToDevice));
    if (st) return st;
    st = cuda_status(cudaDeviceSynchronize());
    if (st) return st;
    g_host_err[device] = 0ull;
    d.base = static_cast<unsigned char*>(ptr);
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

    // coefficients and lane tables, on the host stack; the tables reach the device by value in
    // the parameter blocks of na_prepare_kernel
    SectionF32 secs[IIR_MAX_SECTIONS];
    double gain = 1.0;
    int st = normalise_sos(sos, n_sections, secs, gain);
    if (st) return st;
    IirParams q;
    std::memset(&q, 0, sizeof(q));
    NaUpload up[2];
    for (int s = 0; s < n_sections; ++s) {
        NaUpload& u = up[s / NA_UPLOAD_SECTIONS];
        st = precompute_section(secs[s], IIR_KIND_PH, e->rows, NA_N, q.sec[s],
                                u.tab + (s % NA_UPLOAD_SECTIONS) * IIR_TAB_STRIDE);
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
    // a device-side failure of an earlier call on this device (its output is void)
    volatile unsigned long long* herr = &g_host_err[device];
    const unsigned long long failed = *herr;
    if (failed) {
        *herr = 0ull;
        return device_error_status(failed);
    }
    if (n == 0) return IIR_OK;

    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const int uploads = (n_sections + NA_UPLOAD_SECTIONS - 1) / NA_UPLOAD_SECTIONS;
    for (int k = 0; k < uploads; ++k) {
        up[k].base = d.base;
        up[k].first = k * NA_UPLOAD_SECTIONS;
        up[k].count = (n_sections - up[k].first < NA_UPLOAD_SECTIONS) ? n_sections - up[k].first : NA_UPLOAD_SECTIONS;
        void* pargs[] = {&up[k]};
        st = cuda_status(cudaLaunchKernel(reinterpret_cast<const void*>(na_prepare_kernel), dim3(1),
                                          dim3(NA_PREP_THREADS), pargs, 0, stream));
        if (st) return st;
    }

    unsigned char* tables = d.base + NA_STATE_BYTES;
    unsigned char* carry = tables + NA_TABLE_BYTES;
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
