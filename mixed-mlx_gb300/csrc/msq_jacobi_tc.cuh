// Two-level pairing tables and the tensor-core eigenvector update of the
// batched Jacobi (msq_jacobi_tc.cu).  Internal.
#pragma once

#include "msq_internal.cuh"

#include <cstdint>
#include <vector>

namespace msq {

// Orders whose batched Jacobi may use the two-level pairing (modes 1 and 2
// of msq_set_jacobi_vectors): 66..128 blocks, at most 8 super-pairs, and
// V rows of at most 512 columns, one TMEM allocation.
constexpr int kTwoLevelMinOrder = 257;
constexpr int kTwoLevelMaxOrder = 512;

// Pair table of the two-level schedule for nb blocks (nb even): rounds x
// nb / 2 pairs (I, J), I < J, with J stored as -1 - J for an identity pair.
void twoLevelSchedule(int nb, std::vector<int32_t> &pairs);

// Host tables of the tensor-core eigenvector update for the batch matrices
// `ids` (all of order kTwoLevelMinOrder..kTwoLevelMaxOrder).
struct TcVectorsTables {
  std::vector<int32_t> prog;      // per distinct block count: rounds x super-pairs x 8 entries
  std::vector<int32_t> prog_off;  // per batch matrix: its program in prog (-1: none)
  std::vector<int64_t> image_off; // per batch matrix: its first 16 KB rotation image
  int64_t images = 0;
  std::vector<int32_t> form_work; // (matrix, stage) pairs
  std::vector<int32_t> apply_work;// (matrix, first row) pairs
};
void tcVectorsTables(const int *host_n, int count, const std::vector<int> &ids,
                     TcVectorsTables &out);

// Device view of the tables (inside an allocation owned by the caller).
struct TcVectorsDevice {
  const int2 *form_work = nullptr;
  int form_items = 0;
  const int2 *apply_work = nullptr;
  int apply_items = 0;
  const int32_t *prog = nullptr;
  const int32_t *prog_off = nullptr;
  const int64_t *image_off = nullptr;
};

// One stage rotation Z (64x64) as a tcgen05 B operand: Z^T split into BF16
// hi and lo, each 64 rows x 128 bytes in the SWIZZLE_128B K-major layout
// (term hi at 0, lo at kImageTermBytes).
constexpr int64_t kRotationImageBytes = 16384;
constexpr int kImageTermBytes = 8192;

// Two-level Jacobi on the tensor cores (mode 2) for the batch matrices
// `ids`: host tables and their device view.
struct TwoLevelTables {
  std::vector<int32_t> ids;         // the matrices
  std::vector<int32_t> inner;       // (matrix, super-pair) items, stage by stage
  std::vector<int> stage_first, stage_count;  // per stage: range of inner items
  std::vector<int64_t> diag_off;    // per batch matrix: first 64x64 diagonal block
  int64_t diag_blocks = 0;
};
void twoLevelTables(const int *host_n, int count, const std::vector<int> &ids, TwoLevelTables &out);

struct TwoLevelDevice {
  const int32_t *ids = nullptr;
  int count = 0;
  const int2 *inner = nullptr;
  std::vector<int> stage_first, stage_count;
  const int64_t *diag_off = nullptr;
};

// One launch of the two-level Jacobi on `stream`: the convergence check
// (first: symmetrise and take ||A||^2), then, if sweep is true, every stage
// (inner kernel, B = A Z, A = B^T Z).  b_scratch: one float per matrix
// element of the batch; diag: 4096 floats per diagonal block.
int twoLevelEnqueue(msq_ctx *ctx, cudaStream_t stream, const TwoLevelDevice &t,
                    const TcVectorsDevice &v, float *matrices, float *b_scratch, float *diag,
                    uint8_t *images, const int64_t *a_offset, const int32_t *n,
                    const int64_t *eig_offset, float *eigenvalues, void *state, double tol,
                    const double *tols, int max_sweeps, bool first, bool sweep, int parity);

// Enqueues, on `stream`, the update V <- V Z_1 ... Z_S of one logged sweep
// for the matrices of `d`: the stage rotations Z_s (64x64 blocks, from the
// log) are formed into split-BF16 tcgen05 operand images, then applied to V
// in TMEM.  `state` is the Jacobi state array (JacobiState), `parity` the
// log buffer.
// form = false: the images already exist (written by the two-level inner
// kernel); only the V update runs.
int tcVectorsEnqueue(msq_ctx *ctx, cudaStream_t stream, const TcVectorsDevice &d, float *vectors,
                     const int64_t *a_offset, const int32_t *n, const void *state,
                     const float *log, const int64_t *log_offset, uint8_t *images, int parity,
                     bool form);

}  // namespace msq
