// Stage entry points shared between translation units.
#pragma once

#include "msq_internal.cuh"

namespace msq {

// msq_jacobi.cu
// True when jacobiEnqueue on this batch may run inside a whole-solve graph
// capture (no grid-path matrix, no size class still being tuned).
bool jacobiCapturable(msq_ctx *ctx, const DeviceBatch *b, bool low_bit_basis);
// low_bit_basis: the caller quantizes the basis to BF16 or fewer bits, so the
// automatic eigenvector mode may accumulate V on the tensor cores.
// tols_device / tols_host: optional per-matrix tolerances (device for the
// batched kernels, host for the grid path), replacing `tolerance`.
// keep_vectors: `vectors` already holds the accumulated rotations of an
// earlier solve whose rotated matrix is `matrices` (the solve continues from
// there instead of starting from the identity).
int jacobiEnqueue(msq_ctx *ctx, const DeviceBatch *b, float *matrices, float *vectors,
                  float *eigenvalues, double tolerance, int max_sweeps,
                  int32_t *sweeps_done, float *off_ratio, bool low_bit_basis,
                  const double *tols_device = nullptr, const double *tols_host = nullptr,
                  bool keep_vectors = false);

// msq_tc.cu — tcgen05 reconstruction X = W W^T from the FP32 factor F = W^T
// (quantized to `format` on the fly) or from already encoded flat codes.
int reconstructLowBit(msq_ctx *ctx, const DeviceBatch *b, int format, const float *f,
                      float *x);
int reconstructEncoded(msq_ctx *ctx, const DeviceBatch *b, int format, const void *values,
                       const void *scales, float *x);

// msq_tc.cu — tensor-core Sylvester GEMM chain (the correction is returned in
// *correction, one of ws0/ws1) and the split-BF16 residual.  basis_packed:
// the split operands of V and V^T are still those of the previous chain on
// the same V and batch (no tensor-core call in between), so they are not
// packed again.
int sylvesterTc(msq_ctx *ctx, const DeviceBatch *b, const float *v, const float *lam,
                const float *r, float *ws0, float *ws1, float **correction,
                bool basis_packed = false);
int residualTc(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *x_hi,
               const float *x_lo, float *r, double *norms);

// msq_codecs.cu — x <- decode(encode(x)) for every matrix of the batch in
// one launch (MX blocks and scale rows within each matrix).
int quantizeBatch(msq_ctx *ctx, int format, const DeviceBatch *b, float *x);

// msq_solve.cu
int sylvesterSweep(msq_ctx *ctx, const DeviceBatch *b, int gemm_format, const float *v,
                   const float *lam, const float *r, float *x_hi, float *x_lo, float *ws0,
                   float *ws1, bool basis_packed = false);

}  // namespace msq
