/*
 * iir_gb300.h — C ABI of the GB300 (sm_103a) cascaded-biquad IIR filtering library.
 *
 * The reference library (Haotian-RA/cuda_recursive_filtering) is header-only: a
 * translation unit defines N_SECTIONS / BLOCK_SIZE / N_BLOCKS as macros, calls
 *   setup_kernel_coefficients(const std::vector<std::array<float,6>>& sos)
 * (include/ph_kernels.cuh:151, include/stcr_kernels.cuh:191,
 *  include/dtcr_kernels.cuh:203, include/plr_kernels.cuh:416)
 * and launches
 *   KERNEL_FUNC<<<grid, block>>>(in, out, status, partcarry, fullcarry, launch)
 * (src/test_accuracy.cu:146, src/test_performance.cu:383) on buffers the caller
 * allocated (src/test_accuracy.cu:136-140).
 *
 * This header replaces that surface with run-time arguments:
 *   - the realization (PH / STCR / DTCR / PLR) and the BLOCK_SIZE x N_BLOCKS
 *     geometry are arguments, not macros;
 *   - a plan owns the launch-versioned status/carry buffers (zeroed once at
 *     allocation, never reset between launches), the monotone launch index and
 *     the chunk ticket counter, so callers no longer allocate them;
 *   - every entry point returns an int status code instead of asserting.
 *
 * All pointers passed as x / y are DEVICE pointers to float32 samples. Streams are
 * passed as `void*` holding a cudaStream_t (NULL = legacy default stream).
 * A plan must be driven from one stream at a time (launches that share a plan's
 * status buffer must be serialised, as in include/ph_kernels.cuh:26-29).
 */
#ifndef IIR_GB300_H
#define IIR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define IIR_OK                    0
#define IIR_ERR_INVALID_ARGUMENT (-1)  /* null pointer, bad n_sections, a0 == 0, ...     */
#define IIR_ERR_UNSUPPORTED      (-2)  /* geometry / order combination not built          */
#define IIR_ERR_CUDA             (-3)  /* a CUDA runtime call failed                      */
#define IIR_ERR_LOOKBACK_TIMEOUT (-4)  /* a chunk waited longer than the plan's limit for a
                                          predecessor's carry; output of that launch is void */
#define IIR_ERR_OUT_OF_MEMORY    (-5)
#define IIR_ERR_TOO_LARGE        (-6)  /* n above the plan's capacity / 2^40 samples        */

/* ---- realizations (reference: include/{ph,stcr,dtcr,plr}_kernels.cuh) ----------- */
#define IIR_KERNEL_AUTO         0   /* fastest realization for the order, measured on GB300:
                                       PH to order 10, the precision form (TC) from order 12 */
#define IIR_KERNEL_PH           1   /* PH_32 / PH_64                      ph_kernels.cuh:208,501   */
#define IIR_KERNEL_STCR         2   /* STCR_*_LOOP (loop-form back-sub)   stcr_kernels.cuh:279,2586 */
#define IIR_KERNEL_STCR_UNROLL  3   /* STCR_*_UNROLL_* (register form)    stcr_kernels.cuh:608-3605 */
#define IIR_KERNEL_DTCR         4   /* DTCR_*_LOOP                        dtcr_kernels.cuh:291,2500 */
#define IIR_KERNEL_DTCR_UNROLL  5   /* DTCR_*_UNROLL_*                    dtcr_kernels.cuh:660-3521 */
#define IIR_KERNEL_PLR          6   /* PLR_2/4/8/16 direct form           plr_kernels.cuh:484-3107  */
#define IIR_KERNEL_TC           7   /* precision form: the cascade's chunk solve as tcgen05 TF32 GEMMs
                                       with split (3-term) products; no counterpart in the reference */

typedef struct iir_plan iir_plan;

/*
 * One-shot filtering, the drop-in for "setup_kernel_coefficients(sos) + one launch".
 *   sos        : n_sections rows of {b0, b1, b2, a0, a1, a2} (host memory, scipy layout).
 *                Rows are normalised on the host in FP64 (b0 = a0 = 1); the removed gain
 *                prod(b0/a0) is applied to the input, as the reference's drivers apply
 *                FILTER_GAIN (src/test_accuracy.cu:120-124). Already-normalised rows
 *                (b0 = a0 = 1, the reference's convention, ph_kernels.cuh:157-161) pass through
 *                unchanged.
 *   kernel     : IIR_KERNEL_*; block_size/n_blocks = 0 selects the tuned geometry.
 *   x, y       : device float32 arrays of n samples; they must not overlap.
 *   stream     : cudaStream_t. The call is stream-ordered; plans are cached internally
 *                per (device, stream, filter, kernel, geometry), at most 32 of them (the least
 *                recently used is freed, after a device synchronisation, to make room).
 * Zero initial state, as the reference (xi1/xi2/yi1/yi2 = 0, ph_kernels.cuh:162-165).
 * Device-side failures (a lookback wait that ran out; the reference spins forever instead,
 * ph_kernels.cuh:397-404) happen after the call has returned. They are reported, without a
 * synchronisation, by a later call: the next call on the same cached plan returns
 * IIR_ERR_LOOKBACK_TIMEOUT and launches nothing (the failed call's output is void), as does
 * the next one-shot call after the failed plan was evicted, and iir_cache_clear.
 */
int iir_sos_filter(const float* x, float* y, size_t n, const float* sos, int n_sections,
                   int kernel, void* stream);

/* Same as iir_sos_filter with an explicit BLOCK_SIZE x N_BLOCKS geometry
 * (reference: -DBLOCK_SIZE / -DN_BLOCKS, run_performance.sh:22-60), block_size in {32, 64},
 * n_blocks in {16, 32, 64, 128}; other values give IIR_ERR_UNSUPPORTED.
 *   - n_blocks is the samples per row (one reference thread's samples).
 *   - STCR / DTCR: block_size is the height of a cyclic-reduction tile in rows, as the
 *     reference's thread block is: STCR has one thread per row (one warp per tile at 32, two
 *     at 64), DTCR two (two warps at 32, four at 64); the warps of a tile pass each level's
 *     boundary rows through shared memory (stcr_kernels.cuh:2586-3605,
 *     dtcr_kernels.cuh:2500-3521).
 *   - PH: block_size 32 and 64 run the same kernel, whose row scan already spans all rows of
 *     the chunk (warp scans joined across warps), the reference's PH_32 and PH_64 block scans
 *     alike (ph_kernels.cuh:208, 501).
 *   - A block filters a chunk of whole tiles (32 to 256 rows); the chunk, not one tile, is
 *     the unit of the lookback.
 * For PLR, block_size is the thread-block size and n_blocks the values per thread (PLR_X,
 * plr_kernels.cuh:94-101). */
int iir_sos_filter_geom(const float* x, float* y, size_t n, const float* sos, int n_sections,
                        int kernel, int block_size, int n_blocks, void* stream);

/* Filtering that allocates nothing (no counterpart in the reference, whose callers allocate
 * the status and carry buffers themselves, src/test_accuracy.cu:136-147). For callers that
 * must not allocate while they filter: cudaMalloc / cudaFree may synchronise the device and
 * may fail under memory pressure, which a real-time caller (an audio or radio callback with a
 * deadline) or a caller whose device memory belongs to another allocator cannot accept.
 * Runs the PH realization (32 x 64) on one fixed static device array (about 2.2 MB per
 * device) that holds the launch state, the lane tables and the carry slots. Each call launches
 * two kernels on `stream`: one that writes the filter's tables into the array (they travel in
 * its parameter block) and the filter itself.
 *   - n <= IIR_NOALLOC_MAX_SAMPLES, else IIR_ERR_TOO_LARGE; 1 <= n_sections <= 8.
 *   - The first call on a device sets the array up (resolves its address, zeroes it, page-locks
 *     a static host word that the device reports failures to, synchronises the device); make
 *     it before any stream capture.
 *   - Every call on a device shares the array: calls must be ordered (one stream, or
 *     streams ordered by events). Calls that overlap in time race and give wrong output.
 *   - A device-side failure of a call (a lookback wait that ran out, as overlapping calls can
 *     cause) is returned by a later call on the same device (IIR_ERR_LOOKBACK_TIMEOUT), which
 *     then launches nothing; the failed call's output is void. */
#define IIR_NOALLOC_MAX_SAMPLES (1ull << 26)
int iir_sos_filter_noalloc(const float* x, float* y, size_t n, const float* sos, int n_sections,
                           void* stream);

/* ---- plan API (reference: setup_kernel_coefficients + the caller-owned buffers) ---- */

/* Creates a plan on the current CUDA device. The status/carry buffers are sized for
 * max_n samples and zeroed once here (reference contract, ph_kernels.cuh:16-24). */
int iir_plan_create(iir_plan** plan, const float* sos, int n_sections, int kernel,
                    int block_size, int n_blocks, size_t max_n);

/* PLR from direct-form taps (reference: PLR_FILTER_B / PLR_FILTER_A of filter_taps.hpp,
 * plr_kernels.cuh:416-427). b[order], a[order] are the taps past the implicit b0 = 1 and
 * the recurrence taps with the sign convention y[n] += a[j] * y[n-j-1]; `gain` multiplies
 * the input. order must be 2, 4, 8 or 16. */
int iir_plan_create_plr_ba(iir_plan** plan, const double* b, const double* a, int order,
                           double gain, int block_size, int values_per_thread, size_t max_n);

/* Launches the filter on x[0..n) -> y[0..n) on `stream` (stream-ordered, no sync). */
int iir_plan_execute(iir_plan* plan, const float* x, float* y, size_t n, void* stream);

/* The same filter over HOST buffers x[0..n) -> y[0..n) (pinned memory gives overlapped copies).
 * Single-section plans on the two-pass schedule (order 2; PH, STCR, DTCR) run in pieces of
 * `piece` samples (0 = 2^24): the input copy of the next piece, the filter of this piece and the
 * output copy of the previous piece overlap on three streams, and each piece starts from the
 * state the previous one left (its last two inputs and outputs). Other plans stage the whole
 * signal. Stream-ordered: y is complete when `stream` has reached the end of this call. Device
 * staging buffers, two copy streams and events are created on the first call (two pieces of
 * input and of output); a call is not meant for stream capture. The reference's drivers copy
 * the signal in, launch and copy out (src/test_accuracy.cu:116-159). */
int iir_plan_execute_host(iir_plan* plan, const float* x, float* y, size_t n, size_t piece,
                          void* stream);

/* Synchronises `stream`, returns the first device-side error recorded by a launch of this
 * plan since the previous call (IIR_OK if none) and clears it. */
int iir_plan_check(iir_plan* plan, void* stream);

/* Sets the lookback wait limit in nanoseconds (default 1e9). A chunk that waits longer
 * for a predecessor's carry records IIR_ERR_LOOKBACK_TIMEOUT and every block of that
 * launch returns early. */
int iir_plan_set_timeout_ns(iir_plan* plan, long long timeout_ns);

/* Fault injection for tests of the bounded wait: chunk `chunk` of the NEXT launch skips
 * publishing its carries (so its successors' waits run out). -1 disables. */
int iir_plan_debug_withhold(iir_plan* plan, long long chunk);

/* Resolved realization / geometry of a plan (after IIR_KERNEL_AUTO and defaults). */
int iir_plan_info(const iir_plan* plan, int* kernel, int* block_size, int* n_blocks,
                  int* grid, int* n_sections);

/* Number of kernel launches one iir_plan_execute issues (for launch accounting). */
int iir_plan_launches_per_execute(const iir_plan* plan);

int iir_plan_destroy(iir_plan* plan);

/* ---- batched segments (no reference counterpart: the reference filters one signal with
 * one compile-time filter per launch, ph_kernels.cuh:151-200, src/test_accuracy.cu:146) ------ */

/* One independent signal of a batch: a channel, or the next chunk of a live stream.
 * zi / zf are device arrays of 2 + 2 * n_sections floats: x[-2], x[-1] (raw input before the
 * segment), then for each section its output history y[-2], y[-1] (the filter domain after
 * b0 / a0 normalisation, the gain applied to the input). zi = NULL starts at rest; zf = NULL
 * skips the final state; zi and zf must not overlap, and no segment's y may overlap any
 * segment's x. A segment with n = 0 writes nothing. */
typedef struct {
    const float* x;
    float* y;
    size_t n;
    int filter;            /* index into the batch's filters */
    const float* zi;
    float* zf;
} iir_segment;

typedef struct iir_batch iir_batch;

/* A batch plan over n_filters cascades: sos holds their rows back to back
 * (sum of n_sections[f] rows of 6), n_sections[f] in 1..8. Capacities grow on demand. */
int iir_batch_create(iir_batch** batch, const float* sos, const int* n_sections, int n_filters,
                     size_t max_segments, size_t max_chunks);
/* Filters every segment in one launch on `stream`: a persistent grid draws the segments' chunks
 * from one work queue (PH solve; the decoupled lookback restricted to each segment, one carry
 * per section; with IIR_GB300_BATCH_TAIL_CHUNKS=n, segments of n chunks or more whose filter's
 * state decays within half a chunk publish one aggregate per chunk from its tail instead).
 * Stream-ordered; launches of one batch plan must be ordered on one stream. */
int iir_batch_execute(iir_batch* batch, const iir_segment* segs, int n_segs, void* stream);
int iir_batch_check(iir_batch* batch, void* stream);
/* A fixed segment table uploaded once (synchronously) for repeated launches: each
 * iir_batch_launch_bound is one kernel launch and nothing else, so it can be captured into a
 * CUDA graph and replayed. The segments' buffers must stay valid while the handle is used; an
 * iir_batch_execute that has to grow the batch's carry slots invalidates earlier handles
 * (iir_batch_launch_bound then returns IIR_ERR_INVALID_ARGUMENT). */
typedef struct iir_batch_bound iir_batch_bound;
int iir_batch_bind(iir_batch* batch, const iir_segment* segs, int n_segs, iir_batch_bound** bound);
int iir_batch_launch_bound(iir_batch_bound* bound, void* stream);
int iir_batch_unbind(iir_batch_bound* bound);
int iir_batch_set_timeout_ns(iir_batch* batch, long long timeout_ns);
int iir_batch_debug_withhold(iir_batch* batch, long long chunk);
/* Sections of filter `filter` (the state length is 2 + 2 * sections). */
int iir_batch_filter_sections(const iir_batch* batch, int filter);
/* Chunk shape of the batch's later launches: rows x samples_per_row, one of 128 x 64 (the
 * default), 128 x 32, 128 x 16 and 64 x 16 (chunks of 8192 down to 1024 samples; a segment
 * occupies whole chunks, so short segments want small ones). IIR_ERR_UNSUPPORTED for any other.
 * Handles bound earlier keep their shape. The tuner in autotune.py chooses it per workload. */
int iir_batch_set_shape(iir_batch* batch, int rows, int samples_per_row);
/* The current chunk shape, its kernel's threads per block, registers per thread and shared memory
 * per block, and the resident blocks per SM (the persistent grid is that times the SM count, or
 * the number of chunks if fewer). Any pointer may be NULL. */
int iir_batch_get_shape(const iir_batch* batch, int* rows, int* samples_per_row, int* threads,
                        int* regs_per_thread, int* smem_bytes, int* blocks_per_sm);
int iir_batch_destroy(iir_batch* batch);

/* ---- helpers ------------------------------------------------------------------------- */
const char* iir_status_string(int status);
int iir_version(void);          /* major*10000 + minor*100 + patch */

/* Drops every plan cached by iir_sos_filter (synchronises the device, frees their memory).
 * Returns a device-side failure recorded by a cached plan and not yet reported, else IIR_OK. */
int iir_cache_clear(void);

/* Fault injection for tests of the one-shot error reporting: the next iir_sos_filter /
 * iir_sos_filter_geom call withholds the carries of chunk `chunk` of its launch and waits at
 * most `timeout_ns` for a predecessor (that launch only). No counterpart in the reference. */
int iir_sos_filter_debug_withhold(long long chunk, long long timeout_ns);

#ifdef __cplusplus
}
#endif
#endif /* IIR_GB300_H */
