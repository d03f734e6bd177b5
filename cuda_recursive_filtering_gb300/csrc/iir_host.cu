// iir_host.cu — host planner and C ABI (include/iir_gb300.h).
//
// Replaces the reference's per-header setup_kernel_coefficients (ph_kernels.cuh:151-200,
// stcr_kernels.cuh:191-272, dtcr_kernels.cuh:203-289, plr_kernels.cuh:416-476) and the
// buffers its drivers allocate (src/test_accuracy.cu:136-147):
//   * SOS rows are normalised in FP64 (b0 = a0 = 1) and rounded to float32 once; the
//     removed gain multiplies the input in the kernel (FILTER_GAIN, src/test_accuracy.cu:120-124);
//   * every derived table (state-transition powers C^k, chunk transition powers Q^l, cyclic-
//     reduction factors, PLR n-nacci factors) is computed in FP64 from those float32
//     coefficients, then rounded (the reference computes them in float32, T = float,
//     include/iir_utils.hpp:22);
//   * a plan owns the launch state (epoch = launch index, ticket counter), the flag|value
//     carry slots zeroed once at allocation, and the lane tables.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/iir_gb300.h"
#include "iir_host_internal.h"
#include "iir_params.h"
#include "iir_registry.h"

using namespace iirgb;

// Planner helpers, shared with iir_noalloc.cu through iir_host_internal.h.
namespace iirhost {

// ---------------------------------------------------------------------------------------
// kernel registry
// ---------------------------------------------------------------------------------------
std::vector<KernelEntry>& registry() {
    static std::vector<KernelEntry> reg;
    static std::once_flag once;
    std::call_once(once, [] {
        register_ph(reg);
        register_stcr(reg);
        register_dtcr(reg);
        register_plr(reg);
    });
    return reg;
}

const KernelEntry* find_entry(int kind, int B, int N, int order, int pipeline, int tail, int tiny) {
    for (const KernelEntry& e : registry())
        if (e.kind == kind && e.B == B && e.N == N && e.order == order && e.pipeline == pipeline && e.tail == tail &&
            e.tiny == tiny)
            return &e;
    return nullptr;
}

// Schedule of single-section filters: the persistent pipeline where one is registered for
// the realization and geometry, unless IIR_GB300_SCHEDULE=ticket asks for the one-block-per-
// chunk kernel (kept for comparison).
// Tail-aggregate schedule for cascades: at most this many IIR_TAIL_PIECE-sample pieces in a
// chunk's tail (IIR_GB300_TAIL=<pieces>; 0 keeps the per-section lookback everywhere). The
// planner also keeps it within one piece per warp of the block and half of the chunk.
int tail_max_pieces() {  // read when a plan is created
    if (std::getenv("IIR_GB300_FULL_LOOKBACK")) return 0;  // the exact per-section lookback everywhere
    const char* e = std::getenv("IIR_GB300_TAIL");
    return e ? std::max(0, std::atoi(e)) : IIR_TAIL_MAX_PIECES;
}

bool pipeline_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("IIR_GB300_SCHEDULE");
        return !(v && std::strcmp(v, "ticket") == 0);
    }();
    return on;
}

struct OccKey {
    int device;
    const void* fn;
    bool operator<(const OccKey& o) const { return std::tie(device, fn) < std::tie(o.device, o.fn); }
};

// Resident blocks per SM (all blocks of a persistent launch are co-resident).
int blocks_per_sm(const KernelEntry& e, int device) {
    static std::mutex mu;
    static std::map<OccKey, int> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(OccKey{device, e.fn});
    if (it != cache.end()) return it->second;
    cudaFuncSetAttribute(e.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(e.smem));
    cudaFuncSetAttribute(e.fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, e.fn, e.threads, e.smem) != cudaSuccess) {
        cudaGetLastError();
        nb = 0;
    }
    cache[OccKey{device, e.fn}] = nb;
    return nb;
}

// ---------------------------------------------------------------------------------------
// FP64 2x2 algebra (row-major; acts on column vectors (y[n-2], y[n-1]))
// ---------------------------------------------------------------------------------------
struct M2 {
    double a, b, c, d;
};
M2 mmul(const M2& x, const M2& y) {
    return {x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
M2 mpow(M2 x, unsigned long long e) {
    M2 r{1, 0, 0, 1};
    while (e) {
        if (e & 1ull) r = mmul(r, x);
        x = mmul(x, x);
        e >>= 1;
    }
    return r;
}
float4 to_f4(const M2& m) {
    return make_float4(static_cast<float>(m.a), static_cast<float>(m.b), static_cast<float>(m.c),
                       static_cast<float>(m.d));
}
int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

// Normalises scipy SOS rows {b0,b1,b2,a0,a1,a2} to b0 = a0 = 1 (FP64), returns the removed
// gain prod(b0/a0). Reference convention: ph_kernels.cuh:157-161, tools/ref_generate.py:62-67.
int normalise_sos(const float* sos, int n_sections, SectionF32* out, double& gain) {
    gain = 1.0;
    for (int s = 0; s < n_sections; ++s) {
        const double b0 = sos[6 * s + 0], b1 = sos[6 * s + 1], b2 = sos[6 * s + 2];
        const double a0 = sos[6 * s + 3], a1 = sos[6 * s + 4], a2 = sos[6 * s + 5];
        if (!(std::isfinite(b0) && std::isfinite(b1) && std::isfinite(b2) && std::isfinite(a0) &&
              std::isfinite(a1) && std::isfinite(a2)))
            return IIR_ERR_INVALID_ARGUMENT;
        if (a0 == 0.0) return IIR_ERR_INVALID_ARGUMENT;
        if (b0 == 0.0) return IIR_ERR_UNSUPPORTED;  // section gain cannot be factored out
        gain *= b0 / a0;
        out[s] = SectionF32{static_cast<float>(b1 / b0), static_cast<float>(b2 / b0), static_cast<float>(-a1 / a0),
                            static_cast<float>(-a2 / a0)};
    }
    return IIR_OK;
}

int normalise_sos(const float* sos, int n_sections, std::vector<SectionF32>& out, double& gain) {
    out.assign(static_cast<size_t>(n_sections), SectionF32{});
    const int st = normalise_sos(sos, n_sections, out.data(), gain);
    if (st) out.clear();
    return st;
}

// Fills one IirSection and its lane tables for geometry B x N.
int precompute_section(const SectionF32& s, int kind, int rows, int N, IirSection& q, float4* tab) {
    std::memset(&q, 0, sizeof(q));
    q.b1 = s.b1;
    q.b2 = s.b2;
    q.a1 = s.a1;
    q.a2 = s.a2;
    const double a1 = s.a1, a2 = s.a2, b1 = s.b1, b2 = s.b2;
    const M2 A{0.0, 1.0, a2, a1};
    const M2 C = mpow(A, static_cast<unsigned long long>(N));
    const M2 Q = mpow(C, static_cast<unsigned long long>(rows));
    M2 P = C;
    for (int t = 0; t < IIR_MAX_ROWS; ++t) {
        tab[IIR_TAB_CPOW + t] = to_f4(P);
        P = mmul(P, C);
    }
    M2 G = C;
    if (kind != IIR_KIND_PH) {
        // Cyclic reduction: A_{k+1}(z) = A_k(z) A_k(-z) in z^(2^k); e_k, f_k are the stride-2^k
        // recurrence coefficients y[n] + e_k y[n-2^k] + f_k y[n-2^(k+1)] = v_k[n]
        // (stcr_kernels.cuh:93-125 computes the same chain in float32).
        const int L = ilog2(N);
        double e = -a1, f = -a2;
        q.e0 = static_cast<float>(e);
        q.f0 = static_cast<float>(f);
        q.fir5[0] = static_cast<float>(b1 - e);
        q.fir5[1] = static_cast<float>(b2 - e * b1 + f);
        q.fir5[2] = static_cast<float>(f * b1 - e * b2);
        q.fir5[3] = static_cast<float>(f * b2);
        for (int k = 1; k <= L; ++k) {
            const double en = 2.0 * f - e * e, fn = f * f;
            e = en;
            f = fn;
            if (k == 1) {
                q.ha1 = static_cast<float>(-e);
                q.ha2 = static_cast<float>(-f);
            }
            if (k < L) {
                if (!(std::fabs(e) > 1e-30)) return IIR_ERR_UNSUPPORTED;  // singular elimination
                q.cr_r[k] = static_cast<float>(f / e);
                q.cr_e[k] = static_cast<float>(e);
                q.cr_c[k] = static_cast<float>(e - f / e);
                q.cr_d[k] = static_cast<float>(-f * f / e);
            }
        }
        q.top_e = static_cast<float>(e);
        q.top_f = static_cast<float>(f);
        G = M2{0.0, 1.0, -f, -e};
    }
    P = G;
    for (int t = 0; t < 32; ++t) {
        tab[IIR_TAB_GPOW + t] = to_f4(P);
        P = mmul(P, G);
    }
    M2 Gk = G;
    for (int k = 0; k < 6; ++k) {
        const float4 g = to_f4(Gk);
        q.M[k][0] = g.x;
        q.M[k][1] = g.y;
        q.M[k][2] = g.z;
        q.M[k][3] = g.w;
        Gk = mmul(Gk, Gk);
    }
    M2 Pq{1, 0, 0, 1};
    for (int l = 0; l <= 32; ++l) {
        tab[IIR_TAB_QC + l] = to_f4(Pq);
        Pq = mmul(Pq, Q);
    }
    const M2 Qg = mpow(Q, static_cast<unsigned long long>(IIR_GROUP));
    Pq = M2{1, 0, 0, 1};
    for (int l = 0; l <= 32; ++l) {
        tab[IIR_TAB_QG + l] = to_f4(Pq);
        Pq = mmul(Pq, Qg);
    }
    for (int l = IIR_TAB_QG + 33; l < IIR_TAB_STRIDE; ++l) tab[l] = make_float4(0, 0, 0, 0);
    tab[IIR_TAB_HALF] = to_f4(mpow(A, static_cast<unsigned long long>(N / 2)));
    // tail-aggregate schedule: (A^16)^(l+1) for lanes of IIR_TAIL_PIECE / 32 = 16 samples
    {
        const M2 Al = mpow(A, static_cast<unsigned long long>(IIR_TAIL_PIECE / 32));
        M2 Pt = Al;
        for (int l = 0; l < 32; ++l) {
            tab[IIR_TAB_TAIL + l] = to_f4(Pt);
            Pt = mmul(Pt, Al);
        }
    }
    // truncated lookback: the least m <= 4 with ||Q^m||_inf <= 1e-10 (a chunk's incoming state
    // is then the sum of its m predecessors' aggregates to that bound), else 0
    {
        M2 Qm = Q;
        int depth = 0;
        for (int m = 1; m <= 4 && depth == 0; ++m) {
            const double nrm = std::max(std::fabs(Qm.a) + std::fabs(Qm.b), std::fabs(Qm.c) + std::fabs(Qm.d));
            if (std::isfinite(nrm) && nrm <= 1e-10) depth = m;
            Qm = mmul(Qm, Q);
        }
        if (std::getenv("IIR_GB300_FULL_LOOKBACK")) depth = 0;
        tab[IIR_TAB_LBD] = make_float4(static_cast<float>(depth), 0.f, 0.f, 0.f);
    }
    return IIR_OK;
}

// Tail-aggregate schedule (iir_tail.cuh): the least number P of IIR_TAIL_PIECE-sample pieces
// with ||Phi^(IIR_TAIL_PIECE P)||_inf <= 1e-10, where Phi is the cascade's one-sample transition
// of the state (y_s[n-2], y_s[n-1]) of every section s with zero input (section s > 0 also sees
// its predecessor's new output and history through its FIR taps); FP64 from the float32
// coefficients. 0 if P would exceed max_pieces (the state does not decay fast enough).
// piece_phi receives Phi^IIR_TAIL_PIECE, rounded to float32 (2K x 2K, row-major).
int tail_pieces(const SectionF32* secs, int K, int max_pieces, std::vector<float>& piece_phi) {
    const int D = 2 * K;
    std::vector<double> phi(static_cast<size_t>(D) * D, 0.0), newrow(static_cast<size_t>(D));
    std::vector<double> prev(static_cast<size_t>(D), 0.0);
    for (int s = 0; s < K; ++s) {
        std::fill(newrow.begin(), newrow.end(), 0.0);
        newrow[2 * s + 1] += secs[s].a1;
        newrow[2 * s] += secs[s].a2;
        if (s > 0) {
            for (int j = 0; j < D; ++j) newrow[j] += prev[j];  // y_{s-1}[n] itself (b0 = 1)
            newrow[2 * (s - 1) + 1] += secs[s].b1;
            newrow[2 * (s - 1)] += secs[s].b2;
        }
        phi[static_cast<size_t>(2 * s) * D + 2 * s + 1] = 1.0;  // y_s[n-1] becomes y_s[n-2]
        for (int j = 0; j < D; ++j) phi[static_cast<size_t>(2 * s + 1) * D + j] = newrow[j];
        prev = newrow;
    }
    auto mul = [D](const std::vector<double>& a, const std::vector<double>& b) {
        std::vector<double> r(static_cast<size_t>(D) * D, 0.0);
        for (int i = 0; i < D; ++i)
            for (int k = 0; k < D; ++k) {
                const double aik = a[static_cast<size_t>(i) * D + k];
                if (aik == 0.0) continue;
                for (int j = 0; j < D; ++j) r[static_cast<size_t>(i) * D + j] += aik * b[static_cast<size_t>(k) * D + j];
            }
        return r;
    };
    std::vector<double> m = phi;
    for (int e = 1; e < IIR_TAIL_PIECE; e *= 2) m = mul(m, m);  // Phi^IIR_TAIL_PIECE
    piece_phi.assign(m.begin(), m.end());
    std::vector<double> mp = m;
    for (int P = 1; P <= max_pieces; ++P) {
        double norm = 0.0;
        for (int i = 0; i < D; ++i) {
            double row = 0.0;
            for (int j = 0; j < D; ++j) row += std::fabs(mp[static_cast<size_t>(i) * D + j]);
            norm = std::max(norm, row);
        }
        if (!std::isfinite(norm)) return 0;
        if (norm <= 1e-10) return P;
        mp = mul(mp, m);
    }
    return 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda needed).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        cudaGetLastError();
    });
    return fn;
}

// 2D tensor map over a float32 signal viewed as 32-float (128-byte) lines, box = one block
// (lines x 32), 128-byte swizzle. Returns false if the map cannot be built.
bool encode_lines_map(CUtensorMap* map, const float* base, long long n, int lines_per_block) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || n < 32 || (reinterpret_cast<uintptr_t>(base) & 15u)) return false;
    const cuuint64_t dims[2] = {32ull, static_cast<cuuint64_t>(n / 32)};
    const cuuint64_t strides[1] = {128ull};
    const cuuint32_t box[2] = {32u, static_cast<cuuint32_t>(lines_per_block)};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// 2D tensor map over rows of row_len floats (rows x row_len), box {box_inner, box_rows},
// 128-byte swizzle (box_inner * 4 must be 128).
bool encode_rows_map(CUtensorMap* map, const float* base, long long rows, int row_len, int box_inner, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || rows < 1 || (reinterpret_cast<uintptr_t>(base) & 15u) || (row_len * 4) % 16) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(row_len), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(row_len) * 4};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_inner), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// The view a chunk kernel's tensor copies use (tma_load_chunk / tma_store_chunk): with planes,
// rows of n_per_row >= 32 samples, box 32 x rows_per_chunk (one copy per 32-sample plane);
// otherwise (and for 16-sample rows) 32-sample lines, box = the chunk's lines.
bool encode_chunk_map(CUtensorMap* map, const float* base, long long n, int n_per_row, int rows_per_chunk,
                      bool planes) {
    if (planes && n_per_row >= 32) {
        if (n < n_per_row) return false;
        return encode_rows_map(map, base, n / n_per_row, n_per_row, 32, rows_per_chunk);
    }
    return encode_lines_map(map, base, n, rows_per_chunk * n_per_row / 32);
}

// Same view with a one-line box and no swizzle: the 32 samples before a chunk.
bool encode_hist_map(CUtensorMap* map, const float* base, long long n) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || n < 32 || (reinterpret_cast<uintptr_t>(base) & 15u)) return false;
    const cuuint64_t dims[2] = {32ull, static_cast<cuuint64_t>(n / 32)};
    const cuuint64_t strides[1] = {128ull};
    const cuuint32_t box[2] = {32u, 1u};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return IIR_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? IIR_ERR_OUT_OF_MEMORY : IIR_ERR_CUDA;
}

int device_error_status(unsigned long long word) {
    if (word == 0ull) return IIR_OK;
    const unsigned code = static_cast<unsigned>(word & 0xffffffffull);
    return code == IIR_DEV_ERR_TIMEOUT ? IIR_ERR_LOOKBACK_TIMEOUT : IIR_ERR_CUDA;
}

}  // namespace iirhost

using namespace iirhost;

// -------------------------------------------------------------------------------------------
// plan
// -------------------------------------------------------------------------------------------
namespace iirhost {

// Resources of iir_plan_execute_host, created on its first call: one or two slots of device input
// and output buffers (a piece of samples each), the carried state, a copy stream per direction
// and the events that order the three streams.
struct HostStaging {
    size_t cap = 0;               // samples per buffer
    int slots = 0;                // 2 (pieces in flight) or 1 (the whole signal in one piece)
    float* dx[2] = {nullptr, nullptr};
    float* dy[2] = {nullptr, nullptr};
    float* dz = nullptr;          // x[-2], x[-1], y[-2], y[-1] before the next piece
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t loaded[2] = {nullptr, nullptr};    // input slot filled
    cudaEvent_t filtered[2] = {nullptr, nullptr};  // input slot read, output slot written
    cudaEvent_t stored[2] = {nullptr, nullptr};    // output slot copied out
    cudaEvent_t start = nullptr;                   // caller's stream at the call
};

void host_staging_free(HostStaging* h) {
    if (!h) return;
    for (int b = 0; b < 2; ++b) {
        if (h->dx[b]) cudaFree(h->dx[b]);
        if (h->dy[b]) cudaFree(h->dy[b]);
        if (h->loaded[b]) cudaEventDestroy(h->loaded[b]);
        if (h->filtered[b]) cudaEventDestroy(h->filtered[b]);
        if (h->stored[b]) cudaEventDestroy(h->stored[b]);
    }
    if (h->dz) cudaFree(h->dz);
    if (h->start) cudaEventDestroy(h->start);
    if (h->h2d) cudaStreamDestroy(h->h2d);
    if (h->d2h) cudaStreamDestroy(h->d2h);
    delete h;
}

}  // namespace iirhost

struct iir_plan {
    int device = 0;
    int kind = 0;
    int B = 0, N = 0;          // PLR: threads per block, values per thread
    int order = 0;             // PLR order
    int n_sections = 0;
    int sms = 0;
    int grid_max = 0;
    const KernelEntry* entry = nullptr;
    IirLaunchState* d_state = nullptr;
    unsigned long long* d_carry = nullptr;
    size_t carry_cap = 0;      // chunks
    float4* d_tables = nullptr;
    float* d_fac = nullptr;    // PLR factor arrays
    TcPlan* tc = nullptr;      // precision form (tensor cores)
    IirParams params{};
    IirPlrParams plr{};
    long long timeout_ns = 1000000000ll;
    long long withhold = -1;
    unsigned long long launches = 0;  // since the carry slots were last zeroed
    size_t carry_bytes = 0;
    HostStaging* host = nullptr;      // iir_plan_execute_host: device buffers, streams, events
    unsigned long long* h_err = nullptr;  // host-mapped copy of the device error word (IirLaunchState::host_error)
    int pieces = 0;                // tail-aggregate pieces of `entry` (0: per-section lookback)
    // Single-section plans on the persistent two-pass schedule also keep a one-block-per-chunk
    // kernel for signals of at most small_max_n samples, where the persistent grid's fill and
    // drain dominate (its own lane tables; tail-aggregate schedule when the filter allows).
    const KernelEntry* small = nullptr;
    float4* d_tables_small = nullptr;
    int small_pieces = 0;
    size_t small_max_n = 0;
    // ... and, where one is registered, a 32-row tail kernel for signals of at most tiny_max_n
    // samples: more and shorter chunks, so that a short signal's launch ends sooner.
    const KernelEntry* tiny = nullptr;
    float4* d_tables_tiny = nullptr;
    int tiny_pieces = 0;
    size_t tiny_max_n = 0;
};

namespace {

int default_geometry(int kind, int n_sections, int& B, int& N) {
    if (kind == IIR_KIND_PLR) {
        const int order = 2 * n_sections;
        if (B <= 0) B = order <= 2 ? 512 : order <= 4 ? 256 : order <= 8 ? 128 : 64;
        if (N <= 0) N = 8;  // values per thread (PLR_X)
        return IIR_OK;
    }
    if (B <= 0) B = 32;
    if (N <= 0) N = 64;
    return IIR_OK;
}

// Fastest realization by order, measured on GB300 at 2^28 samples (butter(order, 0.05), N(0,1)
// noise plus tones): PH up to order 10 (473 / 376 GS/s at orders 8 / 10; the precision form gives
// 438 / 307); the precision form from order 12, its cost nearly flat in the order while PH's grows
// with the sections (orders 12 / 14 / 16: 307 / 311 / 342 against 302 / 266 / 237 GS/s, with a
// quarter of the error).
int resolve_auto(int kernel, int n_sections) {
    if (kernel != IIR_KERNEL_AUTO) return kernel;
    return n_sections >= 6 ? IIR_KERNEL_TC : IIR_KERNEL_PH;
}

// samples per block (= per lookback unit) of the plan's large-signal kernel, or of kernel e
size_t chunk_samples(const iir_plan* p, const KernelEntry* e = nullptr) {
    if (p->kind == IIR_KIND_PLR) return static_cast<size_t>(p->B) * p->N;
    return static_cast<size_t>((e ? e : p->entry)->rows) * p->N;
}

// Largest signal (samples) a single-section plan filters with its one-block-per-chunk kernel
// instead of the persistent two-pass one (IIR_GB300_SMALL_N; read when a plan is created).
// Measured on GB300 (butter(2, 0.1), 32x64): PH's one-block-per-chunk kernel on the tail-aggregate
// schedule is ahead at every size (2^28: 832 against 764 GS/s); for STCR and DTCR it is ahead up to
// 2^23 samples, the persistent one from 2^24 (DTCR_UNROLL 475 against 446 GS/s there).
size_t small_signal_limit(int kind, bool tail) {
    const char* v = std::getenv("IIR_GB300_SMALL_N");
    if (v) return static_cast<size_t>(std::strtoull(v, nullptr, 10));
    return (kind == IIR_KIND_PH && tail) ? ~size_t(0) : (size_t(1) << 23);
}

// Largest signal a single-section plan filters with its 32-row kernel (IIR_GB300_TINY_N; read when
// a plan is created).
size_t tiny_signal_limit() {
    const char* v = std::getenv("IIR_GB300_TINY_N");
    return v ? static_cast<size_t>(std::strtoull(v, nullptr, 10)) : (size_t(1) << 18);
}

// 64-bit words of carry slots per section (chunk slots, then one slot per group of chunks)
size_t carry_words_per_section(const iir_plan* p, size_t cap_chunks) {
    const size_t w = (p->kind == IIR_KIND_PLR) ? 2 * static_cast<size_t>(p->order) : 4;
    return w * (cap_chunks + cap_chunks / IIR_GROUP + 2);
}

int alloc_carry(iir_plan* p, size_t cap_chunks, cudaStream_t stream) {
    if (p->d_carry) {
        cudaStreamSynchronize(stream);
        cudaFree(p->d_carry);
        p->d_carry = nullptr;
    }
    cap_chunks = std::max<size_t>(cap_chunks, 1);
    const size_t per_section = carry_words_per_section(p, cap_chunks);
    const size_t sections = (p->kind == IIR_KIND_PLR) ? 1 : static_cast<size_t>(p->n_sections);
    const size_t bytes = per_section * sections * sizeof(unsigned long long);
    int st = cuda_status(cudaMalloc(&p->d_carry, bytes));
    if (st) return st;
    // Zeroed once at allocation (reference: cudaMemset(status, 0), src/test_accuracy.cu:145).
    st = cuda_status(cudaMemset(p->d_carry, 0, bytes));
    if (st) return st;
    p->carry_cap = cap_chunks;
    p->carry_bytes = bytes;
    return IIR_OK;
}

// A host-mapped word that the plan's failing launches also write their error to
// (IirLaunchState::host_error), so a later call can see the failure without synchronising.
int attach_host_error(iir_plan* p) {
    void* h = nullptr;
    int st = cuda_status(cudaHostAlloc(&h, sizeof(unsigned long long), cudaHostAllocMapped | cudaHostAllocPortable));
    if (st) return st;
    p->h_err = static_cast<unsigned long long*>(h);
    *p->h_err = 0ull;
    void* d = nullptr;
    st = cuda_status(cudaHostGetDevicePointer(&d, h, 0));
    if (!st)
        st = cuda_status(cudaMemcpy(reinterpret_cast<char*>(p->d_state) + offsetof(IirLaunchState, host_error), &d,
                                    sizeof(d), cudaMemcpyHostToDevice));
    return st;
}

// The device error a launch of the plan left in its host-mapped word (IIR_OK if none), cleared.
// The word is written by the device asynchronously: an error shows up here once the failing
// launch has recorded it, with no synchronisation.
int take_host_error(iir_plan* p) {
    if (!p->h_err) return IIR_OK;
    volatile unsigned long long* w = p->h_err;
    const unsigned long long v = *w;
    if (v == 0ull) return IIR_OK;
    *w = 0ull;
    return device_error_status(v);
}

int plan_common_alloc(iir_plan* p, size_t max_n) {
    int st = cuda_status(cudaGetDevice(&p->device));
    if (st) return st;
    st = cuda_status(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device));
    if (st) return st;
    const int nb = blocks_per_sm(*p->entry, p->device);
    if (nb <= 0) return IIR_ERR_UNSUPPORTED;
    p->grid_max = nb * p->sms;
    st = cuda_status(cudaMalloc(&p->d_state, sizeof(IirLaunchState)));
    if (st) return st;
    st = cuda_status(cudaMemset(p->d_state, 0, sizeof(IirLaunchState)));
    if (st) return st;
    st = attach_host_error(p);
    if (st) return st;
    size_t chunk = chunk_samples(p);
    if (p->small) {
        if (blocks_per_sm(*p->small, p->device) <= 0) return IIR_ERR_UNSUPPORTED;
        chunk = std::min(chunk, chunk_samples(p, p->small));
    }
    if (p->tiny) {
        if (blocks_per_sm(*p->tiny, p->device) <= 0) return IIR_ERR_UNSUPPORTED;
        chunk = std::min(chunk, chunk_samples(p, p->tiny));
    }
    return alloc_carry(p, (std::max<size_t>(max_n, 1) + chunk - 1) / chunk, nullptr);
}

void plan_free(iir_plan* p) {
    if (!p) return;
    if (p->tc) {
        p->d_state = nullptr;  // owned by the precision plan
        tc_plan_destroy(p->tc);
    }
    if (p->host) {
        cudaDeviceSynchronize();
        host_staging_free(p->host);
    }
    if (p->d_state) cudaFree(p->d_state);
    if (p->h_err) cudaFreeHost(p->h_err);
    if (p->d_carry) cudaFree(p->d_carry);
    if (p->d_tables) cudaFree(p->d_tables);
    if (p->d_tables_small) cudaFree(p->d_tables_small);
    if (p->d_tables_tiny) cudaFree(p->d_tables_tiny);
    if (p->d_fac) cudaFree(p->d_fac);
    delete p;
}

// FP64 factor arrays (all chunk offsets) and chunk transition Phi[i][j] = fac_j[chunk-k+i].
void plr_factors_f64(const double* a, int order, int chunk, std::vector<double>& fac) {
    fac.assign(static_cast<size_t>(order) * chunk, 0.0);
    std::vector<double> v(static_cast<size_t>(chunk) + order);
    for (int j = 0; j < order; ++j) {
        std::fill(v.begin(), v.end(), 0.0);
        v[j] = 1.0;  // history slot j: y[j - order]
        for (int i = order; i < chunk + order; ++i) {
            double acc = 0.0;
            for (int m = 0; m < order; ++m) acc += a[m] * v[i - 1 - m];
            v[i] = acc;
        }
        for (int i = 0; i < chunk; ++i) fac[static_cast<size_t>(j) * chunk + i] = v[i + order];
    }
}

void matmul_k(const std::vector<double>& A, const std::vector<double>& B, std::vector<double>& C, int k) {
    std::vector<double> R(static_cast<size_t>(k) * k, 0.0);
    for (int i = 0; i < k; ++i)
        for (int m = 0; m < k; ++m) {
            const double aim = A[static_cast<size_t>(i) * k + m];
            for (int j = 0; j < k; ++j) R[static_cast<size_t>(i) * k + j] += aim * B[static_cast<size_t>(m) * k + j];
        }
    C.swap(R);
}

int plan_create_plr(iir_plan** out, const double* b, const double* a, int order, double gain, int B, int X,
                    size_t max_n) {
    if (order != 2 && order != 4 && order != 8 && order != 16) return IIR_ERR_UNSUPPORTED;
    int Bd = B, Xd = X;
    default_geometry(IIR_KIND_PLR, order / 2, Bd, Xd);
    const KernelEntry* e = find_entry(IIR_KIND_PLR, Bd, Xd, order);
    if (!e) return IIR_ERR_UNSUPPORTED;
    iir_plan* p = new iir_plan();
    p->kind = IIR_KIND_PLR;
    p->B = Bd;
    p->N = Xd;
    p->order = order;
    p->n_sections = order / 2;
    p->entry = e;
    int st = plan_common_alloc(p, max_n);
    if (st) {
        plan_free(p);
        return st;
    }
    const int chunk = Bd * Xd;
    const int k = order;
    // The kernel's in-chunk recurrence runs on the float32-rounded taps, so the factor arrays and
    // the chunk transition are computed (in FP64) for that same polynomial; built from the
    // unrounded taps they would describe a different filter, which the ill-conditioned direct
    // form of order >= 8 turns into errors far above its own rounding.
    std::vector<double> a32(static_cast<size_t>(order));
    for (int j = 0; j < order; ++j) a32[j] = static_cast<double>(static_cast<float>(a[j]));
    std::vector<double> fac;
    plr_factors_f64(a32.data(), order, chunk, fac);
    // Phi and its powers (FP64), rounded once
    std::vector<double> phi(static_cast<size_t>(k) * k), P(static_cast<size_t>(k) * k, 0.0), Pg, phig;
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j)
            phi[static_cast<size_t>(i) * k + j] = fac[static_cast<size_t>(j) * chunk + (chunk - k + i)];
    std::vector<float> tables(2 * 33 * static_cast<size_t>(k) * k);
    for (int i = 0; i < k; ++i) P[static_cast<size_t>(i) * k + i] = 1.0;
    int depth = 0;  // least m <= 4 with ||Phi^m||_inf <= 1e-10 (truncated lookback), else 0
    for (int l = 0; l <= 32; ++l) {
        for (size_t q = 0; q < P.size(); ++q) tables[static_cast<size_t>(l) * k * k + q] = static_cast<float>(P[q]);
        if (l >= 1 && l <= 4 && depth == 0) {
            double norm = 0.0;
            for (int i = 0; i < k; ++i) {
                double row = 0.0;
                for (int j = 0; j < k; ++j) row += std::fabs(P[static_cast<size_t>(i) * k + j]);
                norm = std::max(norm, row);
            }
            if (std::isfinite(norm) && norm <= 1e-10) depth = l;
        }
        matmul_k(P, phi, P, k);
    }
    if (std::getenv("IIR_GB300_FULL_LOOKBACK")) depth = 0;
    phig = phi;  // Phi^32
    for (int sq = 0; sq < 5; ++sq) matmul_k(phig, phig, phig, k);
    Pg.assign(static_cast<size_t>(k) * k, 0.0);
    for (int i = 0; i < k; ++i) Pg[static_cast<size_t>(i) * k + i] = 1.0;
    for (int l = 0; l <= 32; ++l) {
        for (size_t q = 0; q < Pg.size(); ++q)
            tables[(33 + static_cast<size_t>(l)) * k * k + q] = static_cast<float>(Pg[q]);
        matmul_k(Pg, phig, Pg, k);
    }
    std::vector<float> facf(fac.size());
    for (size_t i = 0; i < fac.size(); ++i) facf[i] = static_cast<float>(fac[i]);
    const size_t fac_bytes = facf.size() * sizeof(float), tab_bytes = tables.size() * sizeof(float);
    st = cuda_status(cudaMalloc(&p->d_fac, fac_bytes + tab_bytes));
    if (!st) st = cuda_status(cudaMemcpy(p->d_fac, facf.data(), fac_bytes, cudaMemcpyHostToDevice));
    if (!st)
        st = cuda_status(cudaMemcpy(reinterpret_cast<char*>(p->d_fac) + fac_bytes, tables.data(), tab_bytes,
                                    cudaMemcpyHostToDevice));
    if (st) {
        plan_free(p);
        return st;
    }
    IirPlrParams& q = p->plr;
    std::memset(&q, 0, sizeof(q));
    q.state = p->d_state;
    q.fac = p->d_fac;
    q.pc = p->d_fac + facf.size();
    q.pg = q.pc + 33 * static_cast<size_t>(k) * k;
    q.chunk = chunk;
    q.lb_depth = depth;
    q.gain = static_cast<float>(gain);
    for (int j = 0; j < order; ++j) {
        q.b[j] = static_cast<float>(b[j]);
        q.a[j] = static_cast<float>(a[j]);
    }
    *out = p;
    return IIR_OK;
}

// Merges float32 sections into one direct-form polynomial pair (FP64 convolution).
void merge_sections(const std::vector<SectionF32>& secs, std::vector<double>& bt, std::vector<double>& at) {
    std::vector<double> bp{1.0}, ap{1.0};
    for (const SectionF32& s : secs) {
        const double bs[3] = {1.0, s.b1, s.b2};
        const double as[3] = {1.0, -static_cast<double>(s.a1), -static_cast<double>(s.a2)};
        std::vector<double> nb(bp.size() + 2, 0.0), na(ap.size() + 2, 0.0);
        for (size_t i = 0; i < bp.size(); ++i)
            for (int j = 0; j < 3; ++j) nb[i + j] += bp[i] * bs[j];
        for (size_t i = 0; i < ap.size(); ++i)
            for (int j = 0; j < 3; ++j) na[i + j] += ap[i] * as[j];
        bp.swap(nb);
        ap.swap(na);
    }
    bt.assign(bp.begin() + 1, bp.end());
    at.resize(ap.size() - 1);
    for (size_t i = 1; i < ap.size(); ++i) at[i - 1] = -ap[i];
}

}  // namespace

extern "C" {

int iir_version(void) { return 10000; }

const char* iir_status_string(int status) {
    switch (status) {
        case IIR_OK: return "ok";
        case IIR_ERR_INVALID_ARGUMENT: return "invalid argument";
        case IIR_ERR_UNSUPPORTED: return "unsupported realization / geometry / filter";
        case IIR_ERR_CUDA: return "CUDA runtime error";
        case IIR_ERR_LOOKBACK_TIMEOUT: return "lookback wait exceeded the plan's limit";
        case IIR_ERR_OUT_OF_MEMORY: return "out of device memory";
        case IIR_ERR_TOO_LARGE: return "too many samples";
        default: return "unknown status";
    }
}

int iir_plan_create(iir_plan** out, const float* sos, int n_sections, int kernel, int block_size, int n_blocks,
                    size_t max_n) {
    if (!out || !sos) return IIR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_sections < 1 || n_sections > IIR_MAX_SECTIONS) return IIR_ERR_INVALID_ARGUMENT;
    kernel = resolve_auto(kernel, n_sections);
    if (kernel < IIR_KERNEL_PH || kernel > IIR_KERNEL_TC) return IIR_ERR_INVALID_ARGUMENT;
    std::vector<SectionF32> secs;
    double gain = 1.0;
    int st = normalise_sos(sos, n_sections, secs, gain);
    if (st) return st;
    if (kernel == IIR_KERNEL_PLR) {
        std::vector<double> bt, at;
        merge_sections(secs, bt, at);
        return plan_create_plr(out, bt.data(), at.data(), 2 * n_sections, gain, block_size, n_blocks, max_n);
    }
    if (kernel == IIR_KERNEL_TC) {
        iir_plan* p = new iir_plan();
        p->kind = IIR_KIND_TC;
        p->n_sections = n_sections;
        st = cuda_status(cudaGetDevice(&p->device));
        if (!st) st = tc_plan_create(&p->tc, secs.data(), n_sections, gain, max_n);
        if (st) {
            plan_free(p);
            return st;
        }
        p->d_state = tc_plan_state(p->tc);
        p->grid_max = tc_plan_grid(p->tc);
        st = attach_host_error(p);
        if (st) {
            plan_free(p);
            return st;
        }
        *out = p;
        return IIR_OK;
    }
    int B = block_size, N = n_blocks;
    default_geometry(kernel, n_sections, B, N);
    const KernelEntry* e = nullptr;
    // The tail-aggregate kernel (iir_tail.cuh) when the cascade's state decays within half a
    // chunk, in pieces of IIR_TAIL_PIECE samples, one per warp of the block; else nullptr.
    auto pick_tail = [&](int& pc, std::vector<float>& phi, int tiny_kernel = 0) -> const KernelEntry* {
        if (tail_max_pieces() <= 0) return nullptr;
        const KernelEntry* t = find_entry(kernel, B, N, 0, 0, 1, tiny_kernel);
        if (!t) return nullptr;
        const int cap = std::min({tail_max_pieces(), t->threads / 32, IIR_TAIL_MAX_PIECES,
                                  t->rows * N / (2 * IIR_TAIL_PIECE)});
        pc = cap > 0 ? tail_pieces(secs.data(), n_sections, cap, phi) : 0;
        return pc > 0 ? t : nullptr;
    };
    int pieces = 0, small_pieces = 0, tiny_pieces = 0;
    std::vector<float> phi, small_phi, tiny_phi;
    const KernelEntry* small = nullptr;
    const KernelEntry* tiny = nullptr;
    if (n_sections == 1 && pipeline_enabled()) e = find_entry(kernel, B, N, 0, 1);
    if (e) {
        // single section on the persistent schedule: a one-block-per-chunk kernel for small signals
        small = pick_tail(small_pieces, small_phi);
        if (!small) small = find_entry(kernel, B, N, 0, 0);
        tiny = pick_tail(tiny_pieces, tiny_phi, 1);
    } else if (n_sections > 1) {
        // cascades whose state decays within a chunk: one lookback per chunk
        e = pick_tail(pieces, phi);
    }
    if (!e) e = find_entry(kernel, B, N, 0, 0);
    if (!e) return IIR_ERR_UNSUPPORTED;
    iir_plan* p = new iir_plan();
    p->kind = kernel;
    p->B = B;
    p->N = N;
    p->n_sections = n_sections;
    p->entry = e;
    p->pieces = pieces;
    p->small = small;
    p->small_pieces = small_pieces;
    p->small_max_n = small ? small_signal_limit(kernel, small_pieces > 0) : 0;
    p->tiny = tiny;
    p->tiny_pieces = tiny_pieces;
    p->tiny_max_n = tiny ? tiny_signal_limit() : 0;
    IirParams& q = p->params;
    std::memset(&q, 0, sizeof(q));
    // lane tables of every section for kernel k (rows per chunk), then (tail schedule) the
    // cascade's piece transition
    auto build_tables = [&](const KernelEntry* k, const std::vector<float>& ph, std::vector<float4>& tabs) {
        const size_t phi_f4 = (ph.size() + 3) / 4;
        tabs.assign(static_cast<size_t>(n_sections) * IIR_TAB_STRIDE + phi_f4, make_float4(0, 0, 0, 0));
        for (int s = 0; s < n_sections; ++s) {
            IirSection sec;
            const int r = precompute_section(secs[s], kernel, k->rows, N, sec,
                                             tabs.data() + static_cast<size_t>(s) * IIR_TAB_STRIDE);
            if (r) return r;
            if (k == e) q.sec[s] = sec;  // per-section scalars (the same for both kernels)
        }
        if (!ph.empty())
            std::memcpy(tabs.data() + static_cast<size_t>(n_sections) * IIR_TAB_STRIDE, ph.data(),
                        ph.size() * sizeof(float));
        return static_cast<int>(IIR_OK);
    };
    std::vector<float4> tabs, tabs_small, tabs_tiny;
    st = build_tables(e, phi, tabs);
    if (!st && small) st = build_tables(small, small_phi, tabs_small);
    if (!st && tiny) st = build_tables(tiny, tiny_phi, tabs_tiny);
    if (st) {
        delete p;
        return st;
    }
    st = plan_common_alloc(p, max_n);
    if (!st) st = cuda_status(cudaMalloc(&p->d_tables, tabs.size() * sizeof(float4)));
    if (!st)
        st = cuda_status(cudaMemcpy(p->d_tables, tabs.data(), tabs.size() * sizeof(float4), cudaMemcpyHostToDevice));
    if (!st && small) st = cuda_status(cudaMalloc(&p->d_tables_small, tabs_small.size() * sizeof(float4)));
    if (!st && small)
        st = cuda_status(cudaMemcpy(p->d_tables_small, tabs_small.data(), tabs_small.size() * sizeof(float4),
                                    cudaMemcpyHostToDevice));
    if (!st && tiny) st = cuda_status(cudaMalloc(&p->d_tables_tiny, tabs_tiny.size() * sizeof(float4)));
    if (!st && tiny)
        st = cuda_status(cudaMemcpy(p->d_tables_tiny, tabs_tiny.data(), tabs_tiny.size() * sizeof(float4),
                                    cudaMemcpyHostToDevice));
    if (st) {
        plan_free(p);
        return st;
    }
    q.state = p->d_state;
    q.tables = p->d_tables;
    q.n_sections = n_sections;
    q.gain = static_cast<float>(gain);
    q.tail_pieces = pieces;
    *out = p;
    return IIR_OK;
}

int iir_plan_create_plr_ba(iir_plan** out, const double* b, const double* a, int order, double gain, int block_size,
                           int values_per_thread, size_t max_n) {
    if (!out || !b || !a) return IIR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return plan_create_plr(out, b, a, order, gain, block_size, values_per_thread, max_n);
}

}  // extern "C"

namespace {

// One launch of the plan over device buffers (arguments checked by the caller). zi: initial
// state of a single-section pipeline plan (x[-2], x[-1], y[-2], y[-1]), or null for rest.
int plan_launch(iir_plan* p, const float* x, float* y, size_t n, const float* zi, cudaStream_t stream) {
    if (p->kind == IIR_KIND_TC) {
        const int st = tc_plan_execute(p->tc, x, y, n, p->timeout_ns, p->withhold, stream);
        p->withhold = -1;
        return st;
    }
    // the kernel for this signal: a single-section plan's small-signal kernel up to its limit
    // (a piece that starts from a carried state always takes the persistent schedule)
    const bool use_tiny = p->tiny && !zi && n <= p->tiny_max_n;
    const bool use_small = !use_tiny && p->small && !zi && n <= p->small_max_n;
    const KernelEntry* ent = use_tiny ? p->tiny : use_small ? p->small : p->entry;
    const size_t chunk = chunk_samples(p, ent);
    const size_t nchunks = (n + chunk - 1) / chunk;
    if (nchunks > 0xffffffffull) return IIR_ERR_TOO_LARGE;
    if (nchunks > p->carry_cap) {
        const int st = alloc_carry(p, nchunks, stream);
        if (st) return st;
    }
    // one block per chunk (blocks take tickets in start order; no residency assumption)
    if (nchunks > 0x7fffffffull) return IIR_ERR_TOO_LARGE;
    const int grid = static_cast<int>(nchunks);
    // Flags are 32-bit functions of the launch epoch: re-zero the slots and the launch state
    // long before the epoch could wrap (the reference zeroes its status buffer once).
    if (++p->launches >= (1ull << 30)) {
        int st = cuda_status(cudaMemsetAsync(p->d_carry, 0, p->carry_bytes, stream));
        if (!st) st = cuda_status(cudaMemsetAsync(p->d_state, 0, IIR_STATE_RESET_BYTES, stream));
        if (st) return st;
        p->launches = 1;
    }
    const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15u) == 0;
    cudaError_t err;
    if (p->kind == IIR_KIND_PLR) {
        IirPlrParams& q = p->plr;
        q.x = x;
        q.y = y;
        q.n = static_cast<long long>(n);
        q.carry = p->d_carry;
        q.nchunks = static_cast<unsigned int>(nchunks);
        q.carry_cap = static_cast<unsigned int>(p->carry_cap);
        q.timeout_ns = p->timeout_ns;
        q.withhold_chunk = p->withhold;
        void* args[] = {&q};
        err = cudaLaunchKernel(p->entry->fn, dim3(grid), dim3(p->entry->threads), args, p->entry->smem, stream);
    } else {
        IirParams& q = p->params;
        q.x = x;
        q.y = y;
        q.n = static_cast<long long>(n);
        q.carry = p->d_carry;
        q.nchunks = static_cast<unsigned int>(nchunks);
        q.carry_cap = static_cast<unsigned int>(p->carry_cap);
        q.carry_stride = carry_words_per_section(p, p->carry_cap);
        const int npr = ent->N, rows = ent->rows;
        const bool planes = ent->planes != 0;
        q.use_tma = (aligned && encode_chunk_map(&q.tmap_x, x, static_cast<long long>(n), npr, rows, planes) &&
                     encode_chunk_map(&q.tmap_y, y, static_cast<long long>(n), npr, rows, planes) &&
                     (!ent->pipeline || encode_hist_map(&q.tmap_h, x, static_cast<long long>(n))))
                        ? 1
                        : 0;
        q.timeout_ns = p->timeout_ns;
        q.withhold_chunk = p->withhold;
        q.zi = ent->pipeline ? zi : nullptr;
        q.tables = use_tiny ? p->d_tables_tiny : use_small ? p->d_tables_small : p->d_tables;
        q.tail_pieces = use_tiny ? p->tiny_pieces : use_small ? p->small_pieces : p->pieces;
        void* args[] = {&q};
        if (ent->pipeline) {
            // persistent: at most every resident block, all co-resident (cooperative launch)
            const int pgrid = static_cast<int>(std::min<size_t>(nchunks, static_cast<size_t>(p->grid_max)));
            err = cudaLaunchCooperativeKernel(ent->fn, dim3(pgrid), dim3(ent->threads), args, ent->smem, stream);
        } else {
            err = cudaLaunchKernel(ent->fn, dim3(grid), dim3(ent->threads), args, ent->smem, stream);
        }
    }
    p->withhold = -1;  // one launch only
    return cuda_status(err);
}

// Device buffers, streams and events of iir_plan_execute_host: `slots` input and output buffers of
// `cap` samples each.
int host_staging(iir_plan* p, size_t cap, int slots, HostStaging** out) {
    HostStaging* h = p->host;
    if (h && h->cap >= cap && h->slots >= slots) {
        *out = h;
        return IIR_OK;
    }
    if (h) {
        cudaDeviceSynchronize();
        host_staging_free(h);
        p->host = nullptr;
    }
    h = new HostStaging();
    h->cap = cap;
    h->slots = slots;
    int st = IIR_OK;
    for (int b = 0; b < 2 && !st; ++b) {
        if (b < slots) st = cuda_status(cudaMalloc(&h->dx[b], cap * sizeof(float)));
        if (!st && b < slots) st = cuda_status(cudaMalloc(&h->dy[b], cap * sizeof(float)));
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&h->loaded[b], cudaEventDisableTiming));
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&h->filtered[b], cudaEventDisableTiming));
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&h->stored[b], cudaEventDisableTiming));
    }
    if (!st) st = cuda_status(cudaMalloc(&h->dz, 4 * sizeof(float)));
    if (!st) st = cuda_status(cudaEventCreateWithFlags(&h->start, cudaEventDisableTiming));
    if (!st) st = cuda_status(cudaStreamCreateWithFlags(&h->h2d, cudaStreamNonBlocking));
    if (!st) st = cuda_status(cudaStreamCreateWithFlags(&h->d2h, cudaStreamNonBlocking));
    if (st) {
        host_staging_free(h);
        return st;
    }
    p->host = h;
    *out = h;
    return IIR_OK;
}

}  // namespace

extern "C" {

int iir_plan_execute(iir_plan* p, const float* x, float* y, size_t n, void* stream_) {
    if (!p || (n > 0 && (!x || !y))) return IIR_ERR_INVALID_ARGUMENT;
    if (n == 0) return IIR_OK;
    if (n > (1ull << 40)) return IIR_ERR_TOO_LARGE;
    const char* xb = reinterpret_cast<const char*>(x);
    const char* yb = reinterpret_cast<const char*>(y);
    if (xb < yb + n * sizeof(float) && yb < xb + n * sizeof(float)) return IIR_ERR_INVALID_ARGUMENT;  // overlap
    return plan_launch(p, x, y, n, nullptr, static_cast<cudaStream_t>(stream_));
}

int iir_plan_execute_host(iir_plan* p, const float* x, float* y, size_t n, size_t piece, void* stream_) {
    if (!p || (n > 0 && (!x || !y))) return IIR_ERR_INVALID_ARGUMENT;
    if (n == 0) return IIR_OK;
    if (n > (1ull << 40)) return IIR_ERR_TOO_LARGE;
    const char* xb = reinterpret_cast<const char*>(x);
    const char* yb = reinterpret_cast<const char*>(y);
    if (xb < yb + n * sizeof(float) && yb < xb + n * sizeof(float)) return IIR_ERR_INVALID_ARGUMENT;  // overlap
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    // Pieces carry their state only on the single-section pipeline; other plans take one piece.
    const bool carry = p->kind != IIR_KIND_PLR && p->kind != IIR_KIND_TC && p->entry && p->entry->pipeline;
    if (piece == 0) piece = size_t(1) << 24;
    piece = std::max<size_t>(piece, 1024);
    if (!carry) piece = n;
    piece = std::min(piece, n);
    HostStaging* h = nullptr;
    int st = host_staging(p, piece, carry ? 2 : 1, &h);
    if (st) return st;
    // Work issued to the caller's stream before this call precedes the first copy.
    st = cuda_status(cudaEventRecord(h->start, stream));
    if (!st) st = cuda_status(cudaStreamWaitEvent(h->h2d, h->start, 0));
    size_t i = 0;
    for (size_t off = 0; off < n && !st; off += piece, ++i) {
        const int b = static_cast<int>(i & 1);
        const size_t len = std::min(piece, n - off);
        // input slot b is free once the launch of piece i - 2 (and its state copies) has run
        if (i >= 2) st = cuda_status(cudaStreamWaitEvent(h->h2d, h->filtered[b], 0));
        if (!st) st = cuda_status(cudaMemcpyAsync(h->dx[b], x + off, len * sizeof(float), cudaMemcpyHostToDevice, h->h2d));
        if (!st) st = cuda_status(cudaEventRecord(h->loaded[b], h->h2d));
        // filter on the caller's stream once the input is in and the output slot is free
        if (!st) st = cuda_status(cudaStreamWaitEvent(stream, h->loaded[b], 0));
        if (!st && i >= 2) st = cuda_status(cudaStreamWaitEvent(stream, h->stored[b], 0));
        if (!st) st = plan_launch(p, h->dx[b], h->dy[b], len, i > 0 ? h->dz : nullptr, stream);
        if (!st && off + len < n) {
            // state before the next piece: its last two inputs and outputs (len >= 1024 here)
            st = cuda_status(cudaMemcpyAsync(h->dz, h->dx[b] + len - 2, 2 * sizeof(float), cudaMemcpyDeviceToDevice,
                                             stream));
            if (!st)
                st = cuda_status(cudaMemcpyAsync(h->dz + 2, h->dy[b] + len - 2, 2 * sizeof(float),
                                                 cudaMemcpyDeviceToDevice, stream));
        }
        if (!st) st = cuda_status(cudaEventRecord(h->filtered[b], stream));
        if (!st) st = cuda_status(cudaStreamWaitEvent(h->d2h, h->filtered[b], 0));
        if (!st) st = cuda_status(cudaMemcpyAsync(y + off, h->dy[b], len * sizeof(float), cudaMemcpyDeviceToHost, h->d2h));
        if (!st) st = cuda_status(cudaEventRecord(h->stored[b], h->d2h));
    }
    // the caller's stream completes after the last output copy
    for (int b = 0; b < 2 && !st; ++b)
        if (static_cast<size_t>(b) < i) st = cuda_status(cudaStreamWaitEvent(stream, h->stored[b], 0));
    return st;
}

int iir_plan_check(iir_plan* p, void* stream_) {
    if (!p) return IIR_ERR_INVALID_ARGUMENT;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    int st = cuda_status(cudaStreamSynchronize(stream));
    if (st) return st;
    IirLaunchState hs;
    st = cuda_status(cudaMemcpy(&hs, p->d_state, sizeof(hs), cudaMemcpyDeviceToHost));
    if (st) return st;
    take_host_error(p);  // the same failure, already read from the device word
    if (hs.error == 0ull) return IIR_OK;
    const unsigned long long zero = 0ull;
    cudaMemcpy(reinterpret_cast<char*>(p->d_state) + offsetof(IirLaunchState, error), &zero, sizeof(zero),
               cudaMemcpyHostToDevice);
    return device_error_status(hs.error);
}

int iir_plan_set_timeout_ns(iir_plan* p, long long timeout_ns) {
    if (!p || timeout_ns <= 0) return IIR_ERR_INVALID_ARGUMENT;
    p->timeout_ns = timeout_ns;
    return IIR_OK;
}

int iir_plan_debug_withhold(iir_plan* p, long long chunk) {
    if (!p) return IIR_ERR_INVALID_ARGUMENT;
    p->withhold = chunk;
    return IIR_OK;
}

int iir_plan_info(const iir_plan* p, int* kernel, int* block_size, int* n_blocks, int* grid, int* n_sections) {
    if (!p) return IIR_ERR_INVALID_ARGUMENT;
    if (kernel) *kernel = p->kind;
    if (block_size) *block_size = p->B;
    if (n_blocks) *n_blocks = p->N;
    if (grid) *grid = p->grid_max;
    if (n_sections) *n_sections = p->n_sections;
    return IIR_OK;
}

int iir_plan_launches_per_execute(const iir_plan* p) { return p ? 1 : 0; }

#ifdef IIR_PROFILE
int iir_plan_debug_profile(iir_plan* p, void* dev_buffer) {
    if (!p) return IIR_ERR_INVALID_ARGUMENT;
    p->params.prof = static_cast<unsigned long long*>(dev_buffer);
    if (p->tc) iirhost::tc_plan_set_profile(p->tc, static_cast<unsigned long long*>(dev_buffer));
    return IIR_OK;
}
#endif

int iir_plan_destroy(iir_plan* p) {
    if (!p) return IIR_ERR_INVALID_ARGUMENT;
    plan_free(p);
    return IIR_OK;
}

}  // extern "C"

// -------------------------------------------------------------------------------------------
// one-shot API with a plan cache keyed by (device, stream, kernel, geometry, filter bytes)
// -------------------------------------------------------------------------------------------
namespace {
struct CacheKey {
    int device;
    void* stream;
    int kernel, B, N, n_sections;
    std::string sos;
    bool operator<(const CacheKey& o) const {
        return std::tie(device, stream, kernel, B, N, n_sections, sos) <
               std::tie(o.device, o.stream, o.kernel, o.B, o.N, o.n_sections, o.sos);
    }
};
struct CacheEntry {
    iir_plan* plan;
    unsigned long long used;  // call counter at the last use (least recently used is evicted)
};
// At most this many cached plans (each holds its carry slots, tables and launch state).
constexpr size_t ONE_SHOT_CACHE_MAX = 32;
std::mutex& cache_mu() {
    static std::mutex m;
    return m;
}
std::map<CacheKey, CacheEntry>& cache() {
    static std::map<CacheKey, CacheEntry> c;
    return c;
}
unsigned long long g_calls = 0;  // one-shot calls (LRU clock)
int g_pending = IIR_OK;          // device failure of an evicted plan, returned by the next call
long long g_debug_withhold = -1;  // iir_sos_filter_debug_withhold: chunk withheld by the next call
long long g_debug_timeout_ns = 0;

// Frees a cached plan once its device work has finished; a device failure it recorded becomes
// the pending error of the one-shot API.
void cache_drop(const CacheKey& key, iir_plan* p) {
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != key.device) cudaSetDevice(key.device);
    cudaDeviceSynchronize();
    const int e = take_host_error(p);
    if (e && g_pending == IIR_OK) g_pending = e;
    plan_free(p);
    if (cur != key.device) cudaSetDevice(cur);
}
}  // namespace

extern "C" int iir_sos_filter_geom(const float* x, float* y, size_t n, const float* sos, int n_sections, int kernel,
                                   int block_size, int n_blocks, void* stream) {
    if (!sos || n_sections < 1 || n_sections > IIR_MAX_SECTIONS) return IIR_ERR_INVALID_ARGUMENT;
    int device = 0;
    int st = cuda_status(cudaGetDevice(&device));
    if (st) return st;
    CacheKey key{device, stream, kernel, block_size, n_blocks, n_sections,
                 std::string(reinterpret_cast<const char*>(sos), sizeof(float) * 6 * n_sections)};
    std::lock_guard<std::mutex> lk(cache_mu());
    // a device-side failure of an earlier call is returned first (that call's output is void)
    if (g_pending != IIR_OK) {
        st = g_pending;
        g_pending = IIR_OK;
        return st;
    }
    ++g_calls;
    auto it = cache().find(key);
    iir_plan* p = nullptr;
    if (it == cache().end()) {
        if (cache().size() >= ONE_SHOT_CACHE_MAX) {
            auto lru = cache().begin();
            for (auto c = cache().begin(); c != cache().end(); ++c)
                if (c->second.used < lru->second.used) lru = c;
            cache_drop(lru->first, lru->second.plan);
            cache().erase(lru);
            if (g_pending != IIR_OK) {
                st = g_pending;
                g_pending = IIR_OK;
                return st;
            }
        }
        st = iir_plan_create(&p, sos, n_sections, kernel, block_size, n_blocks, n);
        if (st) return st;
        cache()[key] = CacheEntry{p, g_calls};
    } else {
        p = it->second.plan;
        it->second.used = g_calls;
        st = take_host_error(p);
        if (st) return st;
    }
    if (g_debug_withhold >= 0) {
        // fault injection for one launch: a withheld carry and a short wait limit
        const long long keep = p->timeout_ns;
        p->timeout_ns = g_debug_timeout_ns;
        p->withhold = g_debug_withhold;
        g_debug_withhold = -1;
        st = iir_plan_execute(p, x, y, n, stream);
        p->timeout_ns = keep;
        p->withhold = -1;
        return st;
    }
    return iir_plan_execute(p, x, y, n, stream);
}

extern "C" int iir_sos_filter_debug_withhold(long long chunk, long long timeout_ns) {
    if (chunk < 0 || timeout_ns <= 0) return IIR_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(cache_mu());
    g_debug_withhold = chunk;
    g_debug_timeout_ns = timeout_ns;
    return IIR_OK;
}

extern "C" int iir_sos_filter(const float* x, float* y, size_t n, const float* sos, int n_sections, int kernel,
                              void* stream) {
    return iir_sos_filter_geom(x, y, n, sos, n_sections, kernel, 0, 0, stream);
}

extern "C" int iir_cache_clear(void) {
    std::lock_guard<std::mutex> lk(cache_mu());
    for (auto& kv : cache()) cache_drop(kv.first, kv.second.plan);
    cache().clear();
    const int st = g_pending;
    g_pending = IIR_OK;
    return st;
}
