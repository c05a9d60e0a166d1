/*
 * commkit-gb300: C ABI of the GB300 (sm_103a) coded-modulation receiver
 * back end, the soft LLR demapper and the layered QC-LDPC min-sum decoder
 * of commkit, rebuilt as hand-written CUDA.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Array arguments are DEVICE pointers
 *    unless a comment says "host"; they must stay valid until the work
 *    queued on `stream` has run.
 *  - `stream` is a cudaStream_t passed as void* (NULL: the legacy default
 *    stream).  Work is queued asynchronously; nothing here synchronizes
 *    the stream unless its comment says so.
 *  - Every function returns a ck_status.  On error, ck_last_error() gives
 *    a message for the calling host thread.  No function traps or aborts.
 *  - Bit labels are MSB first; a positive LLR means bit 0 is more likely.
 */
#ifndef COMMKIT_GB300_H
#define COMMKIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ck_status {
    CK_OK = 0,
    CK_ERR_INVALID_ARGUMENT = 1, /* bad size, shape or table: Python ValueError */
    CK_ERR_UNSUPPORTED = 2,      /* valid input outside what the kernels handle */
    CK_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    CK_ERR_OUT_OF_MEMORY = 4,    /* a device allocation failed */
    CK_ERR_DEVICE_TIMEOUT = 5    /* a bounded device-side wait gave up */
} ck_status;

/* Message of the last error on this host thread ("" if none). */
const char* ck_last_error(void);
/* Static description of a status code. */
const char* ck_status_string(int status);
/* Library version, e.g. "0.1.0". */
const char* ck_version(void);

/* ---------------------------------------------------------------------- */
/* LLR demapping of separable (Gray square) QAM                            */
/* ---------------------------------------------------------------------- */

/* Largest number of bits per symbol (commkit/_cuda/llr.py:12, LLR_MAX_K). */
#define CK_LLR_MAX_K 16

/*
 * One axis of a separable constellation for the closed-form max-log
 * (commkit/_cuda/llr.py:163-204, the `re`/`im` tuples
 * (levels, labels, lo, hi, positions)).  Device arrays:
 *   levels (L,) float32, ascending and equally spaced, L >= 2
 *   labels (L,) int32, the axis's k bits of each level, MSB first
 *   lo, hi (k, L) int32, per bit and level the nearest level below /
 *          above with the other bit value, -1 for none
 *   pos    (k,) int32, position of each of the axis's bits in the label
 */
typedef struct ck_axis_maxlog {
    const float* levels;
    const int32_t* labels;
    const int32_t* lo;
    const int32_t* hi;
    const int32_t* pos;
    int32_t L;
    int32_t k;
} ck_axis_maxlog;

/*
 * One axis for the level-metric demapper (commkit/_cuda/llr.py:100-145,
 * the tuples (levels, log_prior, labels, positions)).  Device arrays:
 *   levels (L,) float32; logp (L,) float32 log marginal prior (zeros for
 *   uniform); labels (L,) int32; pos (k,) int32.  L <= 256.
 */
typedef struct ck_axis_levels {
    const float* levels;
    const float* logp;
    const int32_t* labels;
    const int32_t* pos;
    int32_t L;
    int32_t k;
} ck_axis_levels;

/*
 * Closed-form max-log LLRs of a uniform separable constellation.
 * Replaces the launcher `llr_separable_maxlog(x, re, im, *, inv_s2)`
 * (commkit/_cuda/llr.py:150-206) and its kernel (commkit/_cuda/src/llr.cu:262-337).
 *   x   (n,) complex64 symbols (interleaved float pairs), 8-byte aligned
 *   out (n, re->k + im->k) float32 LLRs, the bits of a symbol adjacent
 *   inv_s2 = float32(1 / max(noise_var, 1e-20))
 * n < 2^31; 1 <= k <= CK_LLR_MAX_K.  Results are bit-identical to the
 * reference's float32 formula evaluated in IEEE arithmetic.
 */
int ck_llr_separable_maxlog(const void* x, int64_t n, const ck_axis_maxlog* re,
                            const ck_axis_maxlog* im, float inv_s2, float* out,
                            void* stream);

/*
 * Max-log (exact = 0) or log-sum-exp (exact = 1) LLRs from the metrics of
 * each axis's levels.  Replaces `llr_separable(x, re, im, *, inv_s2, exact)`
 * (commkit/_cuda/llr.py:87-147; kernel commkit/_cuda/src/llr.cu:225-259),
 * with the exact sums of commkit/mapping/_numba_llr.py:35-92.
 */
int ck_llr_separable(const void* x, int64_t n, const ck_axis_levels* re,
                     const ck_axis_levels* im, float inv_s2, int32_t exact, float* out,
                     void* stream);

/*
 * Batched forms: `inv_s2` is a DEVICE array with one value per frame of
 * `frame_len` symbols (symbol i uses inv_s2[i / frame_len]), so frames of
 * different noise variance demap in one launch.  Each frame's LLRs equal
 * those of the single-variance call on that frame.  No counterpart in the
 * reference, whose API takes one noise variance per call.
 */
int ck_llr_separable_maxlog_frames(const void* x, int64_t n, int64_t frame_len,
                                   const float* inv_s2, const ck_axis_maxlog* re,
                                   const ck_axis_maxlog* im, float* out, void* stream);
int ck_llr_separable_frames(const void* x, int64_t n, int64_t frame_len, const float* inv_s2,
                            const ck_axis_levels* re, const ck_axis_levels* im,
                            int32_t exact, float* out, void* stream);

/*
 * Max-log (exact = 0) or log-sum-exp (exact = 1) LLRs from the metrics of
 * every point, -|x - s|^2 inv_s2 + log P(s): constellations without
 * per-axis factors (PSK, 8-QAM, cross QAM, PAM as complex symbols with a
 * zero imaginary part, arbitrary points, any prior).  Replaces
 * `llr(x, points, log_pmf, labels, *, k, inv_s2, exact)`
 * (commkit/_cuda/llr.py:37-84; kernel commkit/_cuda/src/llr.cu:200-223).
 *   x       (n,) complex64 symbols (device)
 *   points  (M,) complex64, log_pmf (M,) float32, labels (M,) int32: each
 *           point's coordinates, log prior and k-bit label, MSB first
 *   out     (n, k) float32 LLRs
 * 1 <= k <= CK_LLR_MAX_K, M >= 1, n < 2^31.  Max-log results are
 * bit-identical to the reference's float32 formula evaluated in IEEE
 * arithmetic; exact ones agree within the rounding of exp and log.
 */
int ck_llr_points(const void* x, int64_t n, const void* points, const float* log_pmf,
                  const int32_t* labels, int32_t M, int32_t k, float inv_s2, int32_t exact,
                  float* out, void* stream);
/* The same with one inv_s2 per frame of frame_len symbols (no reference
 * counterpart; as ck_llr_separable_frames). */
int ck_llr_points_frames(const void* x, int64_t n, int64_t frame_len, const float* inv_s2,
                         const void* points, const float* log_pmf, const int32_t* labels,
                         int32_t M, int32_t k, int32_t exact, float* out, void* stream);

/* ---------------------------------------------------------------------- */
/* Coded-link simulation (the Monte-Carlo error-rate loop)                 */
/* ---------------------------------------------------------------------- */

/*
 * `count` random bits (int8 0/1) from Philox-4x32-10 (seed, stream): bit i
 * is bit i % 32 of word (i / 32) % 4 of the generator's output for counter
 * i / 128.  Replaces the host draws of the reference's error-rate loop
 * (commkit/coding/performance.py:307-309) with a device stream.
 */
int ck_random_bits(int8_t* out, int64_t count, uint64_t seed, uint64_t stream_id, void* stream);

/*
 * Systematic LDPC encoding on the device (commkit/coding/ldpc.py:445-536):
 * words (B, n) = [info | parity][:n] with s = H_info u over GF(2)
 * (info_row_ptr (m + 1), info_cols: the CSR of H over the k information
 * columns) and either
 *   stride >= 1, inverse NULL: the accumulator p_j = s_j + p_{j - stride}
 *     (stride 1: the reference's "accumulate" kind, a dual-diagonal parity
 *     part; stride Z: a block dual-diagonal of identity circulants), or
 *   stride 0, inverse (m, ceil(m/32)) uint32: rows of H_p^-1 packed 32 bits
 *     a word, p = H_p^-1 s (the reference's "inverse" kind).
 * scratch: at least B m bytes (+ 4 B ceil(m/32) + 4 with an inverse).
 */
int ck_ldpc_encode(const int8_t* info, int64_t B, int32_t k, int32_t m, int32_t n,
                   const int32_t* info_row_ptr, const int32_t* info_cols, int32_t stride,
                   const uint32_t* inverse, int8_t* scratch, size_t scratch_bytes, int8_t* words,
                   void* stream);

/*
 * Encoding through a systematic generator, for parity-check matrices whose
 * last m columns are not invertible (the reference's "dense" kind,
 * commkit/coding/ldpc.py:476-481 and :511-533): information bit j goes to
 * column info_cols[j] (k of them, increasing) and parity bit i, the GF(2)
 * product of gen row i with the information bits, to column pivot_cols[i]
 * (rank of them).  gen is (rank, ceil(k/32)) uint32, row i bit j = entry
 * (i, info_cols[j]) of the reduced row echelon form of H.  Columns >= n
 * (punctured) are not written.  scratch: 4 B ceil(k/32) bytes, 4-aligned.
 */
int ck_ldpc_encode_generator(const int8_t* info, int64_t B, int32_t k, int32_t rank, int32_t n,
                             const int32_t* info_cols, const int32_t* pivot_cols, const uint32_t* gen,
                             int8_t* scratch, size_t scratch_bytes, int8_t* words, void* stream);

/*
 * Hard decisions at chosen columns: bits (B, k) int8 with
 * bits[f, j] = (llrs[f, cols[j]] < 0), llrs (B, n) float32, every
 * cols[j] < n.  The decoder's bits for codes whose information columns are
 * not the first k (commkit/coding/ldpc.py:582-586).
 */
int ck_ldpc_column_signs(const float* llrs, int64_t B, int32_t n, const int32_t* cols, int32_t k,
                         int8_t* bits, void* stream);

/*
 * Symbols (n_sym,) complex64 of a bit record: symbol i is the point whose
 * label is bits [i b, (i + 1) b) (MSB first), b = bits_per_symbol, plus
 * Gaussian noise of standard deviation std_re / std_im per component
 * (Box-Muller on Philox counter i of (seed, stream_id)).  Replaces
 * Constellation.map and the AWGN of commkit/coding/performance.py:318-331.
 */
int ck_map_awgn(const int8_t* bits, int64_t n_sym, int32_t bits_per_symbol,
                const void* points_by_label, float std_re, float std_im, uint64_t seed,
                uint64_t stream_id, void* out, void* stream);

/*
 * Adds one decoded batch to counts[7] (device int64): blocks, information
 * bit errors, block errors, pre-FEC bit errors (channel LLR < 0 against the
 * sent bit), detected failures (valid 0), undetected errors (a block in
 * error reported valid), iterations (commkit/coding/performance.py:332-342).
 */
int ck_count_errors(const int8_t* info, const int8_t* decoded, const float* llr, const int8_t* sent,
                    int64_t B, int32_t k, int32_t n, const uint8_t* valid, const int32_t* iters,
                    int64_t* counts, void* stream);

/*
 * GMI loss terms log2(1 + exp(-(1 - 2c) L)) in float32, summed in float64
 * over chunks of CK_GMI_CHUNK LLRs of each of `rows` rows of `len`:
 * partial (rows, ceil(len / CK_GMI_CHUNK)) (commkit/metrics/information.py:
 * 40-88).
 */
#define CK_GMI_CHUNK 4096
int ck_gmi_loss(const float* llr, const int8_t* bits, int64_t rows, int64_t len, double* partial,
                void* stream);

/*
 * One copy of a batch assembly: `bytes` from `src` to `dst`.  Both may be
 * device memory or pinned host memory (the same address on host and device
 * under unified addressing).
 */
typedef struct ck_segment {
    const void* src;
    void* dst;
    int64_t bytes;
} ck_segment;

/*
 * Copies n segments in one launch (no reference counterpart: the request
 * server's batch assembly).  `segments` itself may sit in pinned host
 * memory.  Segments must not overlap one another's destinations.
 */
int ck_gather(const ck_segment* segments, int32_t n, void* stream);

/*
 * Host acquire fence: call after reading a value the device published in
 * mapped host memory (the mixed decoder writes each frame's iteration count
 * last, after a system-scope fence) and before reading the data it guards.
 */
void ck_host_acquire(void);

/*
 * Host release store: writes `value` to `*counter` (mapped host memory)
 * after every earlier store of the calling thread, e.g. the descriptors of a
 * continuous feed's ring before the count that publishes them
 * (ck_ldpc_feed_launch).
 */
void ck_host_publish(uint32_t* counter, uint32_t value);

/* ---------------------------------------------------------------------- */
/* Layered LDPC decoding                                                   */
/* ---------------------------------------------------------------------- */

/*
 * First-fit layer schedule of a parity-check matrix, on the host.
 * Restates LDPCCode._schedule / _first_fit (commkit/coding/ldpc.py:283-296,
 * 422-442): rows in natural order take the lowest layer none of whose rows
 * shares a bit; rows are then stably grouped by layer.
 *   checks, variables (E,) host int32: the edges sorted by (row, column)
 *   row_ptr (m + 1,), cols (E,), layer_ptr (m + 1,) host int32 outputs
 *   *num_layers: layers written to layer_ptr (layer_ptr has L + 1 entries)
 */
int ck_ldpc_schedule(const int32_t* checks, const int32_t* variables, int64_t E, int32_t m,
                     int32_t N, int32_t* row_ptr, int32_t* cols, int32_t* layer_ptr,
                     int32_t* num_layers);

typedef struct ck_ldpc_plan ck_ldpc_plan;

/*
 * A decoding plan for one code on the current device: validates the
 * schedule (host arrays row_ptr (m+1), cols (E), layer_ptr (L+1), the
 * output of LDPCCode._schedule, commkit/coding/ldpc.py:283-296), recovers
 * the circulant structure when the code is quasi-cyclic, and uploads the
 * tables.  Synchronous (it copies the tables to the device).  The rows of
 * a layer must share no variable and every row needs >= 2 edges.
 */
int ck_ldpc_plan_create(const int32_t* row_ptr, const int32_t* cols, const int32_t* layer_ptr,
                        int32_t m, int32_t N, int32_t num_layers, ck_ldpc_plan** plan);
int ck_ldpc_plan_destroy(ck_ldpc_plan* plan);

/* What the plan found. */
typedef struct ck_ldpc_plan_info {
    int32_t quasi_cyclic;   /* 1: circulant tables, 0: CSR tables */
    int32_t lifting;        /* Z (QC only) */
    int32_t base_rows;      /* mb (QC only) */
    int32_t base_cols;      /* nb (QC only) */
    int32_t blocks;         /* nonzero circulants (QC only) */
    int32_t num_checks;     /* m */
    int32_t num_variables;  /* N */
    int32_t num_edges;      /* E */
    int32_t num_layers;     /* L */
    int32_t max_row_degree;
    int32_t device;
} ck_ldpc_plan_info;
int ck_ldpc_plan_get_info(const ck_ldpc_plan* plan, ck_ldpc_plan_info* info);

/*
 * Launch shape of the decoder: threads per frame (a multiple of 32, at
 * most 1024), frames per thread block and where the compressed
 * check-to-variable messages live; 0 lets the plan choose.  Every shape
 * gives the same results bit for bit; it only changes speed.  The
 * autotuner sets it per code.  Sum-product decodes use only the threads
 * per frame and choose their own frames per block and placement; mixed
 * launches use the threads per frame and the placement, and fill their
 * block with as many frames as fit.
 */
typedef struct ck_ldpc_launch {
    int32_t threads_per_frame;
    int32_t frames_per_block;
    int32_t placement; /* CK_LDPC_PLACE_*: where the check-message state lives */
} ck_ldpc_launch;

#define CK_LDPC_PLACE_AUTO 0   /* the plan chooses: EDGES where two frames fit, else SHARED where two fit,
                                  else GLOBAL */
#define CK_LDPC_PLACE_SHARED 1 /* shared memory, beside the frame's LLRs */
#define CK_LDPC_PLACE_GLOBAL 2 /* device memory (L2-resident working set) */
/* One uncompressed message per edge in shared memory (min-sum decoders
 * of circulant codes with rows up to 27 edges, code-specialised, with one
 * thread per row slot, whose frames' messages fit; other decodes with it
 * keep the records as SHARED). */
#define CK_LDPC_PLACE_EDGES 3
int ck_ldpc_plan_set_launch(ck_ldpc_plan* plan, const ck_ldpc_launch* launch);
int ck_ldpc_plan_get_launch(const ck_ldpc_plan* plan, ck_ldpc_launch* launch);
/*
 * The shape a plain decode by `rule` (CK_LDPC_MIN_SUM / CK_LDPC_SUM_PRODUCT)
 * runs with under the current setting, resolved (and its code-specialised
 * kernel compiled, when it has one): threads per frame, frames per block
 * and the placement actually used (SHARED, GLOBAL or EDGES, never AUTO).
 * The plan's device must be current.  No reference counterpart.
 */
int ck_ldpc_plan_resolved_launch(const ck_ldpc_plan* plan, int32_t rule, ck_ldpc_launch* launch);

/*
 * Code-specialised min-sum decoding of a circulant code (no reference
 * counterpart; results identical bit for bit).  On first use the plan
 * generates a decoder kernel with the code's layers, degrees, block columns
 * and shifts as constants and compiles it with NVRTC; min-sum decodes whose
 * frame groups have one thread per row slot (threads per frame == Z rounded
 * up to whole warps) then run it.  AUTO (the default) falls back to the
 * table-driven kernel where NVRTC is missing or the environment sets
 * COMMKIT_GB300_SPECIALISE=0 (COMMKIT_GB300_NVRTC names the NVRTC library
 * to load instead of searching for it); ON makes an unavailable specialisation an
 * error; OFF always uses the table-driven kernel.  get_specialise reports
 * the mode and the state: 0 not compiled yet, 1 compiled, -1 unavailable
 * (ck_last_error() then says why).
 */
#define CK_LDPC_SPECIALISE_AUTO 0
#define CK_LDPC_SPECIALISE_OFF 1
#define CK_LDPC_SPECIALISE_ON 2
int ck_ldpc_plan_set_specialise(ck_ldpc_plan* plan, int32_t mode);
int ck_ldpc_plan_get_specialise(const ck_ldpc_plan* plan, int32_t* mode, int32_t* state);
/*
 * The CUDA source a plan of this schedule would compile for its
 * code-specialised kernels (host only, no device needed): form 0 the plain
 * decoder (one kernel per placement), form 1 a mixed decoder of this code
 * alone, form 2 the same with two threads per row slot (threads per frame
 * 2 Zp), form 3 form 1 with one message per edge in shared memory
 * (CK_LDPC_PLACE_EDGES).  *length gets its
 * size, and up to capacity - 1 bytes of it go to `out` (NUL-terminated).
 * CK_ERR_UNSUPPORTED when the schedule is not circulant.
 */
int ck_ldpc_specialised_source(const int32_t* row_ptr, const int32_t* cols, const int32_t* layer_ptr,
                               int32_t m, int32_t N, int32_t L, int32_t form, char* out, size_t capacity,
                               size_t* length);

#define CK_LDPC_MIN_SUM 0
#define CK_LDPC_SUM_PRODUCT 1

/* Device scratch bytes ck_ldpc_decode needs for B frames with `rule`. */
int ck_ldpc_workspace_size(const ck_ldpc_plan* plan, int64_t B, int32_t rule, size_t* bytes);

/*
 * Layered belief-propagation decoding of B frames.  Replaces the launcher
 * `ldpc_layered(app, row_ptr, cols, layer_ptr, *, scale, offset,
 * max_iterations, early_stop) -> (iters, valid)` (commkit/_cuda/coding.py:
 * 27-67; kernel commkit/_cuda/src/ldpc.cu:107-159) and fuses the steps
 * around it in LDPCCode's _decode (commkit/coding/ldpc.py:544-588): the
 * zero-padding of punctured bits and the hard decisions of the info bits.
 *   llr_in  (B, n_in) float32 channel LLRs, n_in <= N (the last N - n_in
 *           variables, punctured, start at LLR 0)
 *   llr_out (B, n_in) float32 a-posteriori LLRs; may equal llr_in (in place,
 *           the reference's `app` with n_in = N)
 *   rule    CK_LDPC_MIN_SUM (`scale`, `offset` as MinSum; scale in (0, 1]
 *           and offset finite and >= 0, as MinSum checks them at
 *           commkit/coding/ldpc.py:345-347, else CK_ERR_INVALID_ARGUMENT)
 *           or CK_LDPC_SUM_PRODUCT (`scale`, `offset` ignored)
 *   iters   (B,) int32 iterations run (-1 if a device wait gave up)
 *   valid   (B,) uint8 1 when every check is satisfied
 *   bits    (B, k_bits) int8 hard decisions of the first k_bits variables,
 *           or NULL
 *   workspace: device scratch of at least ck_ldpc_workspace_size() bytes,
 *           256-byte aligned; NULL makes the call allocate and free it
 *           stream-ordered (cudaMallocAsync / cudaFreeAsync).
 * Min-sum results (LLRs, bits, iterations, valid) are bit-identical to
 * the reference's kernel and its Numba twin.  Sum-product (the reference's
 * ldpc_layered<true>, commkit/_cuda/src/ldpc.cu:74-91) runs the same
 * float32 operations in the same order and calls logf/tanhf for
 * phi(x) = -log tanh(x/2), so it matches up to the rounding of those
 * functions, as the reference's own GPU and CPU paths do.  B < 2^31.
 */
int ck_ldpc_decode(const ck_ldpc_plan* plan, const float* llr_in, float* llr_out, int64_t B,
                   int32_t n_in, int32_t rule, float scale, float offset,
                   int32_t max_iterations, int32_t early_stop, int32_t* iters, uint8_t* valid,
                   int8_t* bits, int32_t k_bits, void* workspace, size_t workspace_bytes,
                   void* stream);

/*
 * Reads the device status word a decode left in `workspace` (synchronizes
 * `stream`): CK_OK, or CK_ERR_DEVICE_TIMEOUT if a bounded wait gave up.
 */
int ck_ldpc_workspace_status(const void* workspace, void* stream);

/* One code's frames in a mixed-code launch (as ck_ldpc_decode's arguments). */
typedef struct ck_ldpc_batch {
    const ck_ldpc_plan* plan;
    const float* llr_in;  /* (B, n_in) */
    float* llr_out;       /* (B, n_in), may equal llr_in */
    int64_t B;
    int32_t n_in;
    int32_t rule;         /* CK_LDPC_MIN_SUM (the only rule of mixed launches) */
    float scale;
    float offset;
    int32_t max_iterations;
    int32_t early_stop;
    int32_t* iters;       /* (B,) */
    uint8_t* valid;       /* (B,) */
    int8_t* bits;         /* (B, k_bits) or NULL */
    int32_t k_bits;
    /* (B,) device int32, a permutation of 0..B-1: the order in which the
     * frames are taken from the queue (heaviest expected first shortens the
     * launch's tail); NULL for 0..B-1.  Results stay at their frame's place. */
    const int32_t* order;
    /* Optional demapping inside the decoder.  When `symbols` is not NULL,
     * llr_in is not read: frame f's channel LLRs are the closed-form
     * max-log LLRs (bit-identical to ck_llr_separable_maxlog_frames) of its
     * n_in / k symbols at symbols + f * n_in / k, with 1/sigma^2 =
     * inv_s2[f] and k = axis_re->k + axis_im->k (equal axes of 1 to 4
     * bits).  symbols (B, n_in / k) complex64, 8-byte aligned, in device or
     * mapped host memory; inv_s2 (B,) float32; the axis structs in host
     * memory, their arrays on the device.  Saves the LLR round trip through
     * device memory and the demapper launch. */
    const void* symbols;
    const float* inv_s2;
    const ck_axis_maxlog* axis_re;
    const ck_axis_maxlog* axis_im;
    /* Frames of this batch decoded at once per thread block: 0 for as many
     * as fit.  1 gives each frame an SM of its own (a launch's blocks are
     * sized for its largest code), so a long frame finishes sooner. */
    int32_t frames_per_block;
    /* Threads per frame for this batch, 0 for the plan's launch shape.  2 Zp
     * (Zp = Z rounded up to whole warps) runs each layer's base rows on two
     * threads per row slot: a frame's layers take about half as long. */
    int32_t threads_per_frame;
} ck_ldpc_batch;

#define CK_LDPC_MAX_MIXED 12

/* Device scratch bytes of a mixed-code launch of these batches. */
int ck_ldpc_mixed_workspace_size(const ck_ldpc_batch* batches, int32_t num_batches,
                                 size_t* bytes);

/*
 * Frames of up to CK_LDPC_MAX_MIXED batches of quasi-cyclic codes (lengths,
 * rates, iteration budgets; a code may appear in several batches, e.g. one
 * per constellation with fused demapping) decoded in ONE launch of a
 * persistent kernel.
 * Every block can host any code's frame groups; it starts on a code chosen
 * in proportion to the work, pulls that code's frames from a device queue
 * (a frame retires as soon as its syndrome passes, and its group takes the
 * next), and when that queue is empty switches to the code with the most
 * frames left.  Each frame's results are bit-identical to ck_ldpc_decode's.
 * No counterpart in the reference, which decodes one code per call.  All
 * plans must be quasi-cyclic and on the current device.
 */
int ck_ldpc_decode_mixed(const ck_ldpc_batch* batches, int32_t num_batches, void* workspace,
                         size_t workspace_bytes, void* stream);

/*
 * Continuous feed: the mixed decoder kept running while the host adds
 * frames (no counterpart in the reference, which decodes one call's batch
 * at a time).  Each queue is one batch entry (a code with its demapping, as
 * for ck_ldpc_decode_mixed, with fused demapping) whose frames come from a
 * ring of descriptors in mapped host memory that the host fills while the
 * kernel runs.
 *
 * One frame of a feed: its symbols (n_in / k complex64, 8-byte aligned),
 * where its results go (device or mapped host memory; bits ignored when the
 * queue's k_bits is 0), its 1/sigma^2, and its place in the order of
 * publication across queues (seq, compared modulo 2^32).  iters is written
 * last, after the other results and a system-scope fence: a host that reads
 * it >= -1 then sees them all (after ck_host_acquire).
 */
typedef struct ck_ldpc_feed_frame {
    const void* symbols;
    float* llr_out;
    int8_t* bits;
    int32_t* iters;
    uint8_t* valid;
    float inv_s2;
    uint32_t seq;
} ck_ldpc_feed_frame;

/*
 * A queue's ring: `capacity` (a power of two, at most 2^30) descriptors and
 * the count of positions published so far, both in mapped host memory.
 * Position q is frames[q % capacity]; the host writes a position's
 * descriptor, then raises *published past it with ck_host_publish.  A slot
 * may be rewritten once the frame it held has finished (its iters written).
 */
typedef struct ck_ldpc_feed_ring {
    const ck_ldpc_feed_frame* frames;
    const uint32_t* published;
    uint32_t capacity;
} ck_ldpc_feed_ring;

/*
 * Device scratch bytes of a feed over these queues.  The queues are
 * ck_ldpc_batch entries as for ck_ldpc_decode_mixed with fused demapping:
 * plan, n_in, min-sum parameters, k_bits, the two axis structs,
 * frames_per_block and threads_per_frame are read; `symbols` must be
 * non-NULL (the frames' own come from the ring); B, llr_in, llr_out, iters,
 * valid, bits, inv_s2 and order are not read.
 */
int ck_ldpc_feed_workspace_size(const ck_ldpc_batch* queues, int32_t num_queues, size_t* bytes);

/*
 * Zeroes a feed workspace's counts of positions taken (its first 256 bytes),
 * on `stream`: once, before the first launch over the workspace.
 */
int ck_ldpc_feed_reset(void* workspace, void* stream);

/*
 * Launches the continuous decoder: persistent blocks take published frames
 * (each queue's in order; queues as `policy` says: CK_LDPC_FEED_OLDEST or
 * CK_LDPC_FEED_SHORT_FIRST), demap and decode them, and write their results.  A
 * block with nothing to take polls for new frames and returns once none has
 * been published for idle_us microseconds (1 to 1,000,000), or at once when
 * *stop (mapped host memory; may be NULL) is non-zero; the launch ends when
 * every block has returned.  The counts of positions taken stay in the
 * workspace, so a later launch over the same workspace and rings continues
 * where this one stopped.  Results are bit-identical to ck_ldpc_decode's.
 */
int ck_ldpc_feed_launch(const ck_ldpc_batch* queues, const ck_ldpc_feed_ring* rings, int32_t num_queues,
                        const uint32_t* stop, uint32_t idle_us, int32_t policy, void* workspace,
                        size_t workspace_bytes, void* stream);

/* ck_ldpc_feed_launch policies: which queue a block takes next. */
#define CK_LDPC_FEED_OLDEST 0   /* the queue whose oldest untaken frame was published first */
#define CK_LDPC_FEED_SHORT_FIRST 1 /* the same among the short codes' queues (under a quarter of the
                                       longest code's edges per frame) while any has a frame */

/*
 * Host side of a feed, one request at a time: writes the descriptors of
 * `frames` consecutive frames at ring positions [first, first + frames)
 * (modulo capacity), then raises *published to first + frames with a
 * release store.  Frame f reads symbols + f * symbol_bytes and writes its
 * LLRs to llr_out + f * n_in, its bits to bits + f * k_bits (bits may be
 * NULL), its flag to valid[f] and its iteration count, last, to
 * iters_ring[(first + f) % capacity], which this call sets to -2 first
 * (the host polls a queue's counts in one array); its seq is seq0 + f.
 */
int ck_ldpc_feed_publish(ck_ldpc_feed_frame* ring, uint32_t capacity, int32_t* iters_ring, uint32_t* published,
                         uint32_t first, int32_t frames, const void* symbols, int64_t symbol_bytes, float* llr_out,
                         int32_t n_in, int8_t* bits, int32_t k_bits, uint8_t* valid, float inv_s2, uint32_t seq0);

/* Capacity of the decoder's static scratch array (64 MiB per GPU). */
#define CK_LDPC_STATIC_SCRATCH_BYTES (64u * 1024u * 1024u)

/*
 * ck_ldpc_decode without any allocation, for callers that may not allocate
 * device memory while they decode (a real-time receive loop that cannot take
 * cudaMalloc's synchronisation and latency mid-burst, an application that
 * fixed its memory budget at start-up, a host runtime that owns all device
 * memory).  No counterpart in the reference, whose launcher allocates its
 * message buffer on every call.
 * Arguments as ck_ldpc_decode, minus the workspace: the scratch is a
 * CK_LDPC_STATIC_SCRATCH_BYTES array in the library's device memory, held
 * on every GPU that loads it until the process exits.  The first call on a
 * device looks up that array's address (cudaGetSymbolAddress, with the
 * device current), so make it before any stream capture.  All calls on a
 * device share the array: calls whose work overlaps on the GPU race, so
 * serialise them on one stream.  The grid is limited to the frames whose
 * state fits (any B works); a code whose one block of frames needs more
 * scratch than the array holds returns CK_ERR_UNSUPPORTED.  Results are
 * identical to ck_ldpc_decode's.  The call never compiles a code-specialised
 * kernel (loading one allocates): it runs one only when an earlier
 * ck_ldpc_decode of the plan compiled it, else the table-driven kernel, with
 * the same results (a plan set to CK_LDPC_SPECIALISE_ON without a compiled
 * kernel is refused).  A frame whose LLR copy timed out reports iters = -1
 * and valid = 0; that is the only timeout signal on this path.  The cached
 * address does not survive cudaDeviceReset: do not use the entry point after
 * resetting the device in the same process.
 */
int ck_ldpc_decode_static(const ck_ldpc_plan* plan, const float* llr_in, float* llr_out,
                          int64_t B, int32_t n_in, int32_t rule, float scale, float offset,
                          int32_t max_iterations, int32_t early_stop, int32_t* iters,
                          uint8_t* valid, int8_t* bits, int32_t k_bits, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* COMMKIT_GB300_H */
