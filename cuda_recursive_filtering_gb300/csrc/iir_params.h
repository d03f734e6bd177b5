// iir_params.h — launch parameters shared by the host planner and the sm_103a kernels.
//
// The reference keeps every per-filter constant in module-global __constant__ /
// __device__ symbols filled by cudaMemcpyToSymbol (include/ph_kernels.cuh:45-49,186-199),
// so one module holds one filter. Here the warp-uniform constants travel in a
// __grid_constant__ parameter block (constant bank, free FMA operands) and the
// lane-indexed tables live in a plan-owned device buffer, so any number of plans coexist.
#pragma once
#include <cuda.h>
#include <stdint.h>

#define IIR_MAX_SECTIONS 8
#define IIR_MAX_LEVELS 8          // log2(N_BLOCKS) <= 7
#define IIR_MAX_ROWS 256          // rows (threads x 1 row) per block for the row-major realizations
#define IIR_PLR_MAX_ORDER 16

// Lane tables per section, in float4 units (row-major 2x2 matrices {m00, m01, m10, m11}):
//   [TAB_CPOW + r] = C^(r+1),  C = A^N   (pair transition over one row), r < rows per chunk
//   [TAB_GPOW + t] = G^(t+1),  G = row-scan companion (C for PH; top-level cyclic-reduction
//                                 companion for STCR / DTCR), t < 32 rows per warp
//   [TAB_QC + l]   = Q^l,      Q = A^(rows*N) (chunk transition), l <= 32
//   [TAB_QG + l]   = Q^(32 l)  (group transition powers), l <= 32
//   [TAB_HALF]     = A^(N/2)   (half-row transition)
//   [TAB_LBD].x    = truncated lookback depth of the chunk transition (0: two-level lookback)
//   [TAB_TAIL + l] = (A^16)^(l+1), l < 32 (tail-aggregate schedule: lanes of 16 samples)
#define IIR_GROUP 32
#define IIR_TAB_CPOW 0
#define IIR_TAB_GPOW 256
#define IIR_TAB_QC 288
#define IIR_TAB_QG 321
#define IIR_TAB_HALF 354
#define IIR_TAB_LBD 355  // .x: truncated lookback depth m (||Q^m|| <= 1e-10, m <= 4), 0 = full lookback
#define IIR_TAB_TAIL 356
#define IIR_TAB_STRIDE 388
// Tail-aggregate schedule: a chunk's zero-state aggregate is computed from its last
// tail_pieces x IIR_TAIL_PIECE samples (IirParams::tail_pieces; 0 = per-section lookback), one
// piece per warp. The cascade's state transition over one piece, Phi^IIR_TAIL_PIECE
// (2K x 2K floats, row-major), follows the sections' lane tables.
#define IIR_TAIL_PIECE 512
#define IIR_TAIL_MAX_PIECES 8

// Device-side per-plan launch state. `ticket` packs the launch epoch (the reference's
// `launch` index: part_flag = 2*launch+1, full_flag = 2*launch+2; ph_kernels.cuh:16-24) in its
// high 32 bits and the chunk ticket of the current launch in its low 32 bits, so one atomic
// gives a block both. The block that draws the last chunk of a launch resets the ticket and
// advances the epoch for the next launch (no per-block exit atomics; graph replays and
// launches of different sizes stay consistent). Chunk order = ticket order = block start
// order (the forward-progress argument of ph_kernels.cuh:227-229).
// `host_error` is the device address of a word in host-mapped memory (or null): a failing
// launch also stores its error word there, so the host can see a device-side failure of an
// earlier launch without synchronising (the one-shot entry points report it on their next call).
// Periodic re-zeroing covers the first IIR_STATE_RESET_BYTES only, never host_error.
struct IirLaunchState {
    unsigned long long ticket;       // (epoch << 32) | ticket
    unsigned long long error;        // (epoch << 32) | status code of the first failure
    unsigned int done;               // persistent kernels: blocks of the launch that have exited
    unsigned int pad0;
    unsigned long long* host_error;  // host-mapped error word, or null
};
#define IIR_STATE_RESET_BYTES 24  // ticket, error, done, pad0

struct IirSection {
    float b1, b2;           // FIR taps after b0 normalisation (b0 = 1)
    float a1, a2;           // recurrence y[n] = w[n] + a1 y[n-1] + a2 y[n-2]
    float M[6][4];          // row-scan round matrices G^(2^k), k = 0..5
    // cyclic-reduction factors (STCR / DTCR), level k = 1..7 at index k:
    //   r_k = f_k / e_k, e_k, c_k = e_k - f_k/e_k, d_k = -f_k^2 / e_k
    float cr_r[IIR_MAX_LEVELS], cr_e[IIR_MAX_LEVELS], cr_c[IIR_MAX_LEVELS], cr_d[IIR_MAX_LEVELS];
    float e0, f0;           // e_0 = -a1, f_0 = -a2 (first double-sided round)
    float fir5[4];          // fused FIR + first CR round taps D1..D4 (DTCR)
    float top_e, top_f;     // top-level recurrence across rows: Y_t + e_L Y_{t-1} + f_L Y_{t-2}
    float ha1, ha2;         // parity-half recurrence after the first round: -e_1, -f_1
};

struct IirParams {
    CUtensorMap tmap_x;               // 2D view of x as rows of N samples, box 32 x rows, 128B swizzle (bulk path)
    CUtensorMap tmap_y;
    CUtensorMap tmap_h;               // persistent pipeline: one 32-float line, no swizzle (input history)
    const float* x;
    float* y;
    long long n;
    const float* zi;                  // single-section pipeline: initial state x[-2], x[-1], y[-2], y[-1] (or null)
    unsigned long long* carry;        // per section: [carry_cap][4] chunk slots, then group slots
    IirLaunchState* state;
    const float4* tables;             // [n_sections][IIR_TAB_STRIDE]
    unsigned long long carry_stride;  // words per section
    long long timeout_ns;             // lookback wait limit
    long long withhold_chunk;         // fault injection (-1 = off)
    unsigned int nchunks;
    unsigned int carry_cap;
    int n_sections;
    int use_tma;                      // tensor maps valid (x, y 16-byte aligned) -> TMA staging
    float gain;
    int tail_pieces;                  // tail-aggregate kernels: pieces of IIR_TAIL_PIECE samples in the tail
    unsigned long long* prof;         // per-block phase timestamps (IIR_PROFILE builds only)
    IirSection sec[IIR_MAX_SECTIONS];
};

// PLR (direct form, order k = 2K) parameters.
struct IirPlrParams {
    const float* x;
    float* y;
    long long n;
    unsigned long long* carry;        // [carry_cap][2k] chunk slots (part, full), then group slots
    IirLaunchState* state;
    const float* fac;                 // [k][chunk] n-nacci factor arrays (fac[j][i])
    const float* pc;                  // [33][k][k] chunk-transition powers Phi^l
    const float* pg;                  // [33][k][k] group-transition powers Phi^(32 l)
    long long timeout_ns;
    long long withhold_chunk;
    unsigned int nchunks;
    unsigned int carry_cap;
    int chunk;                        // BLOCK * X
    int lb_depth;                     // truncated lookback depth m (0: two-level lookback)
    float gain;
    float b[IIR_PLR_MAX_ORDER];       // FIR taps past b0 = 1
    float a[IIR_PLR_MAX_ORDER];       // recurrence taps: y[n] += a[j] y[n-j-1]
};

// Status codes stored in IirLaunchState::error (same values as the C ABI).
// ------------------------------------------------------------------------------------------
// Batched segments: many independent signals (channels / stream chunks) in one launch, each
// with its own filter and optional state in / state out.
// State layout (zi / zf, 2 + 2 * n_sections floats): x[-2], x[-1] (raw input), then per
// section its output history y[-2], y[-1].
// Compact lane tables per section, for one chunk shape (ROWS rows of N samples, ROWS <= 128):
#define IIR_BATCH_MAX_ROWS 128
#define IIR_BT_CPOW 0      // C^(r+1), r < ROWS          (C = A^N)
#define IIR_BT_GPOW 128    // C^(t+1), t < 32
#define IIR_BT_QC 160      // Q^l, l <= 32               (Q = C^ROWS, the chunk transition)
#define IIR_BT_QG 193      // Q^(32 l), l <= 32
#define IIR_BT_LBD 226     // .x: truncated lookback depth (0: two-level lookback)
#define IIR_BT_TAIL 228    // (A^16)^(l+1), l < 32        (tail-aggregate schedule)
#define IIR_BT_STRIDE 260
// Phi^IIR_TAIL_PIECE of a filter's cascade (2K x 2K floats, row-major), one block of this many
// floats per filter
#define IIR_BT_PHI_FLOATS (4 * IIR_MAX_SECTIONS * IIR_MAX_SECTIONS)

struct IirBatchFilter {
    float gain;
    int n_sections;
    int sec0;               // index of its first section in the section / table arrays
    int tail;               // tail-aggregate pieces for the batch's chunk shape (0: per-section lookback)
};

struct IirBatchSegment {
    const float* x;
    float* y;
    long long n;
    const float* zi;        // state in (device) or null = at rest
    float* zf;              // state out (device) or null
    unsigned int chunk0;    // first chunk of the segment in the launch's chunk space
    unsigned int group0;    // first group slot of the segment
    int filter;
    int tail_ok;            // long enough for its filter's tail-aggregate schedule (host's choice)
    int lead;               // zero samples before the segment in its first chunk (0..3): a segment
                            // at rest whose x is not 16-byte aligned is chunked on x's 16-byte grid
    int pad;
};

struct IirBatchParams {
    const IirBatchSegment* segs;
    const unsigned int* chunk_start;  // [nsegs + 1], chunk_start[i] = segs[i].chunk0
    const unsigned int* chunk_seg;    // [nchunks]: each chunk's segment (bound tables), or null: search chunk_start
    const IirBatchFilter* filters;
    const IirSection* secs;
    const float4* tables;             // [sections][IIR_BT_STRIDE], for the launch's chunk shape
    const float* phi;                 // [filters][IIR_BT_PHI_FLOATS]
    unsigned long long* carry;        // per section level: [carry_cap][4] chunk slots, then [gcap][4] group slots
    IirLaunchState* state;
    unsigned long long carry_stride;  // words per section level
    long long timeout_ns;
    long long withhold_chunk;         // fault injection (-1 = off)
    unsigned int nsegs;
    unsigned int nchunks;
    unsigned int carry_cap;
    int max_sections;
    unsigned long long* prof;         // unused (shared helpers' profiling hook)
};

#define IIR_DEV_ERR_TIMEOUT 4u
#define IIR_DEV_ERR_MBARRIER 7u
