/*
 * msq_cuda.h — C ABI of the GB300 (sm_103a) SPD matrix-square-root pipeline.
 *
 * This is the drop-in boundary a `cuda_backend` beside the reference's
 * `metal_backend` / `accelerate_backend` binds to.  Every entry point takes
 * plain pointers and sizes, returns an int status (MSQ_OK on success) and
 * never throws.  Device buffers are allocated and owned by the caller; all
 * matrices are column-major (element (row, column) at row + column * n),
 * exactly as in the reference (`PreparedMatrix.values`, src/experiment.hpp:18).
 * Work is enqueued on the context's stream (msq_set_stream); calls are
 * stream-ordered, and only the calls that return host values synchronise.
 *
 * Status codes map onto the reference's error convention: a nonzero status is
 * what `fail()` (src/core.cpp:7-9) raises; msq_last_error() gives the text.
 * Numerical outcomes (not converged, rejected basis, ...) are NOT errors; they
 * are reported in msq_solve_result, as the reference reports them in
 * `CaseResult.status` / `termination_reason` (src/experiment.hpp:64-125).
 */
#ifndef MSQ_CUDA_H
#define MSQ_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  MSQ_OK = 0,
  MSQ_ERR_INVALID_ARGUMENT = 1, /* bad size, format, null or misaligned ptr */
  MSQ_ERR_CUDA = 2,             /* a CUDA runtime/driver call failed        */
  MSQ_ERR_DEVICE_STATUS = 3,    /* a kernel reported an error flag (bounded
                                   wait expired, index out of range)         */
  MSQ_ERR_UNSUPPORTED = 4       /* valid request the library does not serve */
};

/* ---- storage formats ----------------------------------------------------
 * Ids 0..7 equal the reference's HostStorageCodec (src/precision.hpp:24-33),
 * so `static_cast<int>(spec.host_storage)` selects the same codec.
 * MSQ_FMT_FP8_E4M3FN_ROWSCALE has no reference counterpart: E4M3FN codes of
 * x / s_row with one FP32 scale s_row = max|row| / 448 per contiguous row.  */
typedef enum {
  MSQ_FMT_FP32 = 0,
  MSQ_FMT_BF16 = 1,
  MSQ_FMT_FP8_E4M3FN = 2,
  MSQ_FMT_FP8_E5M2 = 3,
  MSQ_FMT_MXFP8_E4M3FN = 4,
  MSQ_FMT_MXFP8_E5M2 = 5,
  MSQ_FMT_FP4_E2M1 = 6,
  MSQ_FMT_MXFP4_E2M1 = 7,
  MSQ_FMT_FP8_E4M3FN_ROWSCALE = 8
} msq_format;

typedef struct msq_ctx msq_ctx;

/* ---- context --------------------------------------------------------------
 * Replaces the RAII `MetalRuntime` (src/metal_runtime.hpp:69-76): owns the
 * device binding, the stream and the kernels' small persistent state.      */
int msq_create(msq_ctx **out, int device);
void msq_destroy(msq_ctx *ctx);
const char *msq_last_error(const msq_ctx *ctx);
/* `stream` is a cudaStream_t (NULL = legacy default stream). */
int msq_set_stream(msq_ctx *ctx, void *stream);
/* Concurrency inside a call (default on): the Jacobi forks its size buckets
 * and its V replay onto internal streams that join back into the context's
 * stream before the call's later work.  enable = 0 keeps every launch on the
 * context's stream, in serial order (same results, bit for bit).          */
int msq_set_concurrency(msq_ctx *ctx, int enable);
/* CUDA graphs (default on): the batched Jacobi's launch sequence is captured
 * once per plan, buffers, tolerance and launch shapes, then replayed; and
 * msq_solve_batched captures its whole plan-group sequence (gather, Jacobi,
 * reconstruction, residuals, corrections, scatter, report copies) on its
 * second call with the same layout, plans, buffers and tolerance, then
 * replays it with one graph launch and one synchronisation (the FP32
 * fallback of a miss, decided on the host, runs after it).
 * enable = 0 launches every kernel directly (same results, bit for bit).   */
int msq_set_graphs(msq_ctx *ctx, int enable);
int msq_synchronize(msq_ctx *ctx);
/* Failure injection for tests of the bounded device waits (process-wide,
 * default 0).  mode 1: the batched Jacobi sweep kernels' shared-memory flag
 * waits look for a value no warp writes, and their tile loads between
 * sweeps wait on an mbarrier with no copy behind it; mode 2: every tcgen05
 * GEMM launch first
 * waits on an mbarrier nothing arrives at (before it issues any copy or
 * MMA).  Each such wait gives up after a short limit, the launch unwinds,
 * and the call's status check returns MSQ_ERR_DEVICE_STATUS ("bounded ...
 * wait expired"); the context stays usable.  Results of the affected launches
 * are meaningless.  Launches captured in CUDA graphs before the mode changed
 * keep their setting: turn graphs off (msq_set_graphs) around such a test.
 * No counterpart in the reference (its Metal waits are host-side).        */
int msq_debug_expire_waits(int mode);
/* Number of this library's kernel launches enqueued so far on `ctx` (a
 * replayed graph counts the launches it holds). */
uint64_t msq_launch_count(const msq_ctx *ctx);
/* Number of CUDA graph launches issued so far on `ctx`. */
uint64_t msq_graph_launch_count(const msq_ctx *ctx);
/* Measured FP32 FMA throughput of the device (TFLOP/s, best of three timed
 * launches of independent FMA chains on every SM): the denominator of the
 * FP32 rooflines (the Jacobi kernels).  Synchronises. */
int msq_fma_rate(msq_ctx *ctx, double *tflops);
/* Launch timing for profiling: between begin and end, an event is recorded
 * on the context's stream after every launch (launches on internal streams
 * get a begin and an end event); end synchronises and writes one line per
 * kernel name, "name<TAB>launches<TAB>total_ms", into `out`.  The duration
 * of a launch on the context's stream is the gap to the previous event, so
 * stream-ordered copies issued between launches count toward the next
 * launch; concurrent launches share the GPU, so for per-kernel costs time
 * with concurrency off. */
int msq_timing_begin(msq_ctx *ctx);
int msq_timing_end(msq_ctx *ctx, char *out, size_t capacity);

/* ---- codecs ---------------------------------------------------------------
 * Byte sizes: storageBytes / scaleBytes (src/configuration.cpp:188-213).
 * For MSQ_FMT_FP8_E4M3FN_ROWSCALE the scale plane is 4 bytes per row.      */
size_t msq_storage_bytes(int format, size_t elements);
size_t msq_scale_bytes(int format, size_t elements, size_t row_length);

/* Encode `elements` FP32 values (device pointer) into `values` (+ `scales`
 * for MX / row-scaled formats).  Bit-exact with the reference host codec
 * copyToStorage (src/storage_codecs.cpp:249-321).  `row_length` is used
 * only by the row-scaled format (elements % row_length must be 0).        */
int msq_encode(msq_ctx *ctx, int format, const float *source, size_t elements,
               size_t row_length, uint8_t *values, uint8_t *scales);
/* Decode back to FP32; bit-exact with storageValueAt
 * (src/storage_codecs.cpp:323-374) for every index.                       */
int msq_decode(msq_ctx *ctx, int format, const uint8_t *values,
               const uint8_t *scales, size_t elements, size_t row_length,
               float *output);

/* ---- stochastic rounding (--rounding stochastic) ---------------------------
 * The reference's device quantizers for stochastic rounding
 * (metal_mixed_sqrt.metal:394-405 hash; :462-484, :545-568, :740-763 FP8 /
 * FP4 element rules; :1888-1907 BF16; MX :971-1000, :1113-1140, :1232-1260),
 * which replace the host copyToStorage (src/storage_codecs.cpp:315-321)
 * when the reference runs with --rounding stochastic --rounding-seed S:
 * element i (flat index) between codes lo < |x| < hi rounds up with
 * probability (|x| - lo) / (hi - lo) against a 24-bit sample of
 * hash(i, seed, stream); BF16 adds one ulp when the hash's low 16 bits are
 * below the 16 dropped bits; zero, NaN and magnitudes at or above the
 * largest finite code keep the nearest code; MX scales as msq_encode.
 * Same buffers and sizes as msq_encode; every format of msq_encode.      */
int msq_encode_stochastic(msq_ctx *ctx, int format, const float *source, size_t elements,
                          size_t row_length, uint32_t seed, uint32_t stream,
                          uint8_t *values, uint8_t *scales);

/* ---- log-spectrum storage (fp8_e4m3fn_log_s, fp4_e2m1_log_s) ---------------
 * Replaces copySpectrumToStorage / spectrumValueAt
 * (src/storage_codecs.cpp:387-460) and the device kernels
 * log_spectrum_metadata / quantize_*_log_s / decode_*_log_s_to_f32
 * (metal_mixed_sqrt.metal:1689-1804): root eigenvalues in blocks of
 * MSQ_LOG_SPECTRUM_BLOCK with metadata (min, span) of log2 s per block (two
 * floats, 8-byte aligned), codes of max * (log2 s - min) / span (max = 448
 * for MSQ_FMT_FP8_E4M3FN, 6 for MSQ_FMT_FP4_E2M1), decoded as
 * exp2(min + span * code / max).  Device semantics: the span is lowered by
 * one ulp when min + span rounds above the block's maximum log.  Inputs
 * must be finite and positive; otherwise the device status is set and the
 * next msq_synchronize returns MSQ_ERR_DEVICE_STATUS.                     */
#define MSQ_LOG_SPECTRUM_BLOCK 8
enum { MSQ_ROUND_NEAREST = 0, MSQ_ROUND_STOCHASTIC = 1 };
size_t msq_spectrum_metadata_bytes(size_t elements);
int msq_spectrum_encode(msq_ctx *ctx, int format, const float *spectrum, size_t elements,
                        int rounding, uint32_t seed, uint32_t stream, uint8_t *values,
                        float *metadata);
int msq_spectrum_decode(msq_ctx *ctx, int format, const uint8_t *values, const float *metadata,
                        size_t elements, float *spectrum);

/* ---- batched layout -------------------------------------------------------
 * A batch is `count` square matrices of orders n[i], packed back to back:
 * matrix i starts at element offset[i] (offsets are in elements; each
 * matrix occupies n[i]*n[i] elements, column-major).  `n` and `offset` are
 * HOST arrays; the library uploads them once per distinct batch layout.   */

/* ---- Jacobi eigensolver ----------------------------------------------------
 * Replaces MetalRuntime::symmetricJacobi (src/metal_runtime.cpp:584-646) and
 * makeJacobiSchedule (src/metal_solver.cpp:50-79).  Parallel-order
 * (round-robin) two-sided cyclic Jacobi over 8x8 block pivots, FP32 storage
 * and FP32 rotation angles (each (c, s) renormalised so c^2 + s^2 = 1 to
 * FP32 rounding), FP64 off-norm.  Sweeps stop once
 * off(A) <= tolerance * ||A||_F or after max_sweeps (tolerance 0: exactly
 * max_sweeps sweeps).  In: matrices (FP32).  Out: vectors (FP32, column j =
 * eigenvector j), eigenvalues (FP32, n[i] per matrix at value offset
 * eig_offset[i] = sum of previous n), sweeps_done / off_ratio per matrix
 * (device arrays, may be NULL).  `matrices` is overwritten (the converged,
 * nearly diagonal matrix).  Orders up to 16384: a matrix above 1024 is
 * solved with every SM (the grid kernels; the call then synchronises the
 * context's stream once per sweep to read the off-norm), the others one CTA
 * each, except the few largest above 256 whose one-CTA solves would outlast
 * the rest of the batch (a cost model; in the tensor-core eigenvector modes:
 * any above 256 when at most 8 are in the batch), which also go to the grid
 * kernels.  Results are the same bits either way.                         */
int msq_jacobi_batched(msq_ctx *ctx, float *matrices, float *vectors,
                       float *eigenvalues, const int32_t *n,
                       const int64_t *offset, int count, double tolerance,
                       int max_sweeps, int32_t *sweeps_done, float *off_ratio);

/* ---- eigenvector accumulation (orders 257..512) ----------------------------
 * No counterpart in the reference, whose V <- V J runs after every round on
 * the CUDA-core equivalent of its GPU (metal_mixed_sqrt.metal:1380-1390).
 * For 256 < n <= 512 on the one-CTA-per-matrix kernels the solver can pair
 * blocks in two levels: super-blocks of 8 blocks (32 indices), rounds 0..6
 * inside each super-block, then per outer round-robin round over
 * super-blocks 8 rounds of cross pairs.  The rotations of rounds 0..14 and
 * of each later group of 8 stay inside 64-index super-pairs, so their
 * product is block diagonal (64x64 blocks) and V <- V Z is a GEMM.
 *   MSQ_VECTORS_AUTO    (-1, default) msq_jacobi_batched: REPLAY;
 *                       msq_solve_batched: TENSOR for BF16 / FP8 / MXFP4
 *                       plans, REPLAY for FP32 plans;
 *   MSQ_VECTORS_REPLAY  (0) round-robin pairing, FP32 replay of every round;
 *   MSQ_VECTORS_BLOCKED (1) two-level pairing, FP32 replay (bit-exact with
 *                       the oracle's blocked Jacobi in the same order);
 *   MSQ_VECTORS_TENSOR  (2) two-level pairing; each stage's 64x64 rotations
 *                       applied to V held in TMEM by tcgen05.mma in split
 *                       BF16 (hi*hi + lo*hi + hi*lo, FP32 accumulation): V
 *                       orthonormal to about 1e-4, eigenvalues unchanged;
 *   MSQ_VECTORS_TENSOR_A (3) two-level pairing; a stage's rounds rotate only
 *                       the 64x64 diagonal blocks (CUDA cores) and the rest
 *                       of A is brought up to date once per stage on the
 *                       tensor cores (B = A Z, A = B^T Z, split BF16), V as
 *                       in mode 2.  Eigenvalues to about 1e-4 ||A||; about
 *                       2x slower than mode 2 on GB300 (the per-stage
 *                       passes stream A through HBM twice).
 * The mode applies to later calls on the context.                          */
enum {
  MSQ_VECTORS_AUTO = -1,
  MSQ_VECTORS_REPLAY = 0,
  MSQ_VECTORS_BLOCKED = 1,
  MSQ_VECTORS_TENSOR = 2,
  MSQ_VECTORS_TENSOR_A = 3
};
int msq_set_jacobi_vectors(msq_ctx *ctx, int mode);
/* The two-level pair table for `blocks` 4-index blocks (even, 2..4096),
 * host-only (no GPU, no context): writes *rounds and, when `pairs` is not
 * NULL and capacity >= rounds * blocks, rounds x blocks/2 pairs (I, J) with
 * I < J, J stored as -1 - J for a pair that keeps the identity rotation.   */
int msq_jacobi_schedule(int blocks, int32_t *pairs, size_t capacity, int *rounds);
/* Which eigensolver path each matrix of a batch of orders n[count] takes
 * under eigenvector mode `mode` (MSQ_VECTORS_REPLAY .. MSQ_VECTORS_TENSOR_A;
 * AUTO resolves to REPLAY for msq_jacobi_batched and the FP32 plans, to
 * TENSOR for batches of low-bit plans): grid[i] = 1 when matrix i is solved
 * by the grid kernels with every SM, 0 when by the batched kernels one CTA
 * each.  Host only (no GPU, no context).                                   */
int msq_jacobi_route(const int32_t *n, int count, int mode, int32_t *grid);

/* ---- launch-shape autotuner -------------------------------------------------
 * The Jacobi sweep buckets matrices by size class and picks each class's CTA
 * size online: while a class is untuned, its first sweeps of a call try each
 * candidate (all candidates compute identical bits) under timing events, and
 * a later call keeps the fastest for that device.  Decisions are
 * process-wide.  msq_autotune_report writes one line per class (candidates,
 * measured ms per matrix-sweep, choice) for `device`; msq_autotune_reset
 * forgets all decisions and, with enable = 0, turns tuning off (classes then
 * use their default shapes).                                               */
int msq_autotune_report(int device, char *out, size_t capacity);
int msq_autotune_reset(int enable);

/* ---- Jacobi without allocation ----------------------------------------------
 * No counterpart in the reference.  For callers that must not allocate
 * device memory: latency-critical loops, where cudaMalloc/cudaFree may
 * synchronise the device and take unbounded time, and host applications that
 * own all device memory and hand the library only their own buffers.  Solves
 * ONE matrix of order n <= MSQ_NOALLOC_MAX_ORDER (256) with the same kernels
 * and results as msq_jacobi_batched; every piece of scratch lives in one
 * static device array of about 0.65 MB, which every GPU that loads the
 * library holds until the process exits.  Needs no msq_ctx and calls no
 * cudaMalloc, cudaFree or other allocating function.  Larger (or
 * non-positive) n, a null buffer, tolerance < 0 or max_sweeps outside
 * [0, 64] return MSQ_ERR_INVALID_ARGUMENT before anything is launched.
 * The first call on a device (the current device) looks up the array's
 * device address once; make that first call before capturing any stream.
 * Each call first resets, with a small kernel on `stream`, the parts of the
 * array that must start at zero (the sweep state and a status word);
 * everything else is written before it is read.  All calls on one device share the one array:
 * calls that overlap on the GPU (on two streams, or from two threads) race
 * on it and corrupt each other's results, so issue them on one stream.
 * `stream` is a cudaStream_t (NULL: the default stream); `matrix` is
 * overwritten as in msq_jacobi_batched; sweeps_done / off_ratio are device
 * pointers to one element each, or NULL.  The call is asynchronous and never
 * synchronises, so a bounded device wait that expires (the condition
 * msq_jacobi_batched returns as MSQ_ERR_DEVICE_STATUS) is reported in the
 * outputs instead: every eigenvalue is NaN, *sweeps_done is -1 and
 * *off_ratio NaN.  A CUDA error already pending on the calling thread is
 * left in place and returned as MSQ_ERR_CUDA before anything is launched; a
 * launch error of this call returns MSQ_ERR_CUDA.                           */
#define MSQ_NOALLOC_MAX_ORDER 256
int msq_jacobi_noalloc(float *matrix, float *vectors, float *eigenvalues, int n,
                       double tolerance, int max_sweeps, void *stream,
                       int32_t *sweeps_done, float *off_ratio);

/* ---- reconstruction ---------------------------------------------------------
 * X = V diag(sqrt(lambda)) V^T per matrix, written as the symmetric product
 * X = W W^T with W = V diag(lambda^(1/4)).  Replaces reconstructTiled /
 * reconstructLowFactorTiled (src/metal_runtime.cpp:429-534).
 * msq_make_factor builds W^T in K-major order (row i of W contiguous) from V
 * and lambda, FP32.  msq_reconstruct consumes W^T in `format`:
 *   MSQ_FMT_FP32        SIMT FP32 GEMM (the plain FP32 path)
 *   MSQ_FMT_BF16        tcgen05 kind::f16 MMA, FP32 accumulate in TMEM
 *   MSQ_FMT_FP8_E4M3FN_ROWSCALE  tcgen05 kind::f8f6f4 (E4M3 x E4M3),
 *                       row scales applied in the epilogue
 *   MSQ_FMT_MXFP4_E2M1  tcgen05 kind::mxf4 block-scaled MMA (E2M1 x E2M1,
 *                       UE8M0 per 32 along K) when every order and offset
 *                       is divisible by 32 (the flat scale blocks are then
 *                       row blocks); otherwise decoded exactly to BF16
 *   MSQ_FMT_MXFP8_E4M3FN  tcgen05 kind::mxf8f6f4 block-scaled MMA; orders
 *                       and offsets divisible by 32, else MSQ_ERR_UNSUPPORTED
 * `values`/`scales` hold the encoded W^T (scales: FP32 per row for
 * row-scaled, the codec's scale bytes for MX).  The solver's MXFP4 plan
 * (msq_solve_batched) quantizes W^T per row block and always takes the
 * kind::mxf4 path.
 * Output X (FP32) uses the same batched layout as the input.              */
int msq_make_factor(msq_ctx *ctx, const float *vectors,
                    const float *eigenvalues, const int32_t *n,
                    const int64_t *offset, int count, float *factor_t);
int msq_reconstruct(msq_ctx *ctx, int format, const void *values,
                    const void *scales, const int32_t *n,
                    const int64_t *offset, int count, float *root);
/* The solver's own reconstruction stage: X0 = Q(W) Q(W)^T from the FP32
 * factor W^T (msq_make_factor) quantized to the plan's format
 * (msq_plan_format) on the way into the MMA tiles: FP32 SIMT GEMM, BF16
 * kind::f16, FP8 per-row kind::f8f6f4, or MXFP4 per row block of 32
 * (any order) kind::mxf4.  Same stage as reconstructLowFactorTiled
 * (src/metal_runtime.cpp:500-534).                                        */
int msq_reconstruct_factor(msq_ctx *ctx, int plan_format, const float *factor_t,
                           const int32_t *n, const int64_t *offset, int count,
                           float *root);

/* ---- residual and Sylvester correction -------------------------------------
 * msq_residual: R = A - X*X with A = (a + a_lo) and X = (x_hi + x_lo) in
 * float-float (about 48 bits, the reference's WorkingFloat, which also keeps
 * A as a (high, low) pair: metal_mixed_sqrt.metal:1268-1317,
 * src/metal_solver.cpp:186-196); writes R as FP32 (may be NULL) and
 * per-matrix ||R||_F^2, ||A||_F^2 (FP64, device, 2 per matrix).  a_lo and
 * x_lo may be NULL (treated as zero).
 * msq_sylvester_sweep: one frozen-basis correction of
 * refineUpdateAndMeasure (src/metal_runtime.cpp:847-966):
 *   C = (V^T R V) o H, H_ij = 1/(s_i + s_j) recomputed from s = sqrt(lambda),
 *   E = V C V^T,  X <- X + (E + E^T)/2 (float-float add into x_hi/x_lo).
 * `gemm_format` selects the correction GEMMs: MSQ_FMT_FP32 (SIMT FP32) or
 * MSQ_FMT_BF16 (tcgen05 split-BF16, three products, FP32 accumulate).
 * `workspace` must hold 2 * sum(n^2) floats.                               */
int msq_residual(msq_ctx *ctx, const float *a, const float *a_lo,
                 const float *x_hi, const float *x_lo, const int32_t *n,
                 const int64_t *offset, int count, float *residual,
                 double *norms);
int msq_sylvester_sweep(msq_ctx *ctx, int gemm_format, const float *vectors,
                        const float *eigenvalues, const float *residual,
                        const int32_t *n, const int64_t *offset, int count,
                        float *x_hi, float *x_lo, float *workspace);

/* msq_native_sylvester_sweep: one correction of the reference's
 * native-quantized mode (--correction native_quantized, refineNativeStaged /
 * refineNativePerStage, src/metal_runtime.cpp:292-411, driven at
 * src/metal_solver.cpp:829-848): every operand and intermediate is stored in
 * `format` (any msq_encode format; MSQ_FMT_FP32 keeps FP32):
 *   R_q = Q(R), W1 = Q(Vt R_q), W2 = Q(W1 V), C = Q(W2_ij / (s_i + s_j)),
 *   W1 = Q(V C), E = Q(W1 Vt),   X <- X + (E + E^T)/2 (float-float),
 * where Q quantizes an FP32 matrix to `format` with nearest rounding (per
 * matrix; row length n for the row-scaled format) and decodes it, and the
 * products are FP32 with each element an FMA chain over the inner index in
 * order (the reference's matmul kernels on decoded operands,
 * metal_mixed_sqrt.metal:39-56).  vectors / vectors_t: the decoded stored
 * basis V and transposed basis V^T (stored separately, as the reference
 * stores them); spectrum: the decoded root eigenvalues s (sum(n) floats,
 * matrix i at the prefix sum of n).  workspace: 3 * E floats, E = max over
 * matrices of offset + n^2.  Every step runs over the whole batch in one
 * launch (the quantizer round-trips each matrix in place); codes / scales
 * are not used and may be NULL.                                           */
int msq_native_sylvester_sweep(msq_ctx *ctx, int format, const float *vectors,
                               const float *vectors_t, const float *spectrum,
                               const float *residual, const int32_t *n,
                               const int64_t *offset, int count, float *x_hi, float *x_lo,
                               float *workspace, uint8_t *codes, uint8_t *scales);

/* The reference's CSV schema (writeSummaryHeader / writeIterationsHeader,
 * src/reporting.cpp:124-166, 305-327): the header lines of the summary and
 * per-iteration files that the C++ mirror's writers (cuda_backend.hpp) fill
 * row by row.  Host only (no GPU needed).  Returns MSQ_ERR_INVALID_ARGUMENT
 * when a buffer is too small.                                             */
int msq_csv_headers(char *summary, size_t summary_capacity, char *iterations,
                    size_t iterations_capacity);

/* ---- general products for the stage-3 spectral plans -----------------------
 * The pieces of run_spectral's FP32 products (3_spectral/spectral.cpp:
 * 1145-1230: MPS GEMMs, apply_scale_f32, working_add, residual_and_norm)
 * for operands that are not symmetric (an explicit basis inverse):
 * msq_gemm: C = op(A) op(B) per matrix (FP32 FMA), op = transpose when
 *   trans_* != 0; with `eigenvalues` (device, batched as lambda) each C_ij
 *   is divided by sqrt(lambda_i) + sqrt(lambda_j) (the Sylvester step).
 * msq_working_add: X <- X + E in float-float (x_hi, x_lo), no symmetrisation.
 * msq_residual_general: msq_residual for a general X.                      */
int msq_gemm(msq_ctx *ctx, int trans_a, int trans_b, const float *a, const float *b,
             const int32_t *n, const int64_t *offset, int count,
             const float *eigenvalues, float *c);
int msq_working_add(msq_ctx *ctx, float *x_hi, float *x_lo, const float *e,
                    const int32_t *n, const int64_t *offset, int count);
int msq_residual_general(msq_ctx *ctx, const float *a, const float *a_lo,
                         const float *x_hi, const float *x_lo, const int32_t *n,
                         const int64_t *offset, int count, float *residual,
                         double *norms);

/* ---- whole-pipeline batched solve ------------------------------------------
 * The GPU-resident solve of solveGpuResidentSpd (src/metal_solver.cpp:92-336)
 * over a batch: Jacobi -> (quantize W) -> reconstruct -> Sylvester sweeps ->
 * final float-float residual, per-matrix plan, with FP32 fallback for every
 * matrix whose final residual misses `tolerance`: FP32 Jacobi to 1e-7
 * (continuing the plan's rotations where those are FP32), FP32
 * reconstruction and FP32 correction sweeps until the tolerance is met
 * (one to four; a matrix that still misses it reports its residual).      */
typedef enum {
  MSQ_PLAN_FP32 = 0,   /* Jacobi to 1e-7, FP32 reconstruction, no sweeps    */
  MSQ_PLAN_BF16 = 1,   /* BF16 W, tcgen05 reconstruction                    */
  MSQ_PLAN_FP8 = 2,    /* FP8-E4M3 W with per-row FP32 scale               */
  MSQ_PLAN_MXFP4 = 3   /* MXFP4 W (E2M1 + E8M0 per 32 along K)              */
} msq_plan_format;

typedef struct {
  int32_t format;        /* msq_plan_format                                  */
  int32_t sweeps;        /* Sylvester correction sweeps (0, 1, 2)            */
  double jacobi_tolerance; /* off(A) <= jacobi_tolerance * ||A||_F           */
  int32_t jacobi_max_sweeps;
  int32_t reserved;
} msq_plan;

typedef struct {
  double final_residual;   /* ||A - X^2||_F / ||A||_F, float-float         */
  double initial_residual; /* residual of the reconstruction X0            */
  int32_t jacobi_sweeps;    /* Jacobi sweeps (a continued fallback: both passes) */
  int32_t corrections;     /* Sylvester sweeps applied                     */
  int32_t accepted;        /* 1: the plan met the tolerance; 0: fell back  */
  int32_t fallback;        /* 1: result comes from the FP32 fallback       */
  double plan_residual;    /* the plan's own final residual (before any
                              fallback; equals final_residual when accepted) */
} msq_solve_result;

/* a: FP32 matrices (device, batched layout); root: FP32 output (device).
 * plans: HOST array of `count` plans (NULL = MSQ_PLAN_FP32 for all).
 * results: HOST array of `count` results (may be NULL).                   */
int msq_solve_batched(msq_ctx *ctx, const float *a, const int32_t *n,
                      const int64_t *offset, int count, const msq_plan *plans,
                      double tolerance, float *root, msq_solve_result *results);

/* ---- learned plan selector -------------------------------------------------
 * MLP 16 -> 64 -> 64 -> 8 (ReLU), BF16 weights, FP32 accumulation.  The
 * reference picks plans by fixed rules (runAdaptiveMetalCase,
 * src/metal_solver.cpp:976-1001; the cond < 1000 rule of
 * 3_spectral/spectral.cpp:837-838); this network replaces those rules.
 * msq_features: 16 per-matrix features from A (device) into `features`
 * (device, FP32, 16 per matrix).  Parameters live in one FP32 master array
 * (device) of MSQ_MLP_PARAMS floats; the kernels read its BF16 copy.       */
#define MSQ_MLP_IN 16
#define MSQ_MLP_HIDDEN 64
#define MSQ_MLP_OUT 8
#define MSQ_MLP_PARAMS \
  (MSQ_MLP_IN * MSQ_MLP_HIDDEN + MSQ_MLP_HIDDEN + \
   MSQ_MLP_HIDDEN * MSQ_MLP_HIDDEN + MSQ_MLP_HIDDEN + \
   MSQ_MLP_HIDDEN * MSQ_MLP_OUT + MSQ_MLP_OUT)
int msq_features(msq_ctx *ctx, const float *a, const int32_t *n,
                 const int64_t *offset, int count, float *features);
int msq_mlp_forward(msq_ctx *ctx, const float *params, const float *features,
                    int rows, float *logits);
/* Softmax cross-entropy over masked targets: grad_params += dL/dparams.
 * targets: per row, 8 floats in [0,1] (1 = plan acceptable) weighted by
 * `costs`; see the implementation for the exact loss.  loss: device scalar. */
int msq_mlp_backward(msq_ctx *ctx, const float *params, const float *features,
                     const float *targets, int rows, float *grad_params,
                     float *loss);
int msq_mlp_step(msq_ctx *ctx, float *params, const float *grad_params,
                 float *adam_m, float *adam_v, int step, float learning_rate);

#ifdef __cplusplus
}
#endif

#endif /* MSQ_CUDA_H */
