// Host-side entry points of the dense (CUDA-core) kernels in msq_dense.cu.
#pragma once

#include "msq_internal.cuh"

namespace msq {

enum GemmEpilogue : int {
  kEpilogueStore = 0,
  kEpilogueInverseH = 1,  // C_ij / (sqrt(lambda_i) + sqrt(lambda_j))
};

struct GemmArgs {
  const int4 *work;
  int items;
  const float *a, *b;
  float *c;
  const int64_t *a_offset, *b_offset, *c_offset;
  const int32_t *n;
  const float *eigenvalues;
  const int64_t *eig_offset;
  int a_mmajor;  // A(i,k) at i + k*n instead of k + i*n
  int b_nmajor;  // B(k,j) at j + k*n instead of k + j*n
};

struct ResidualArgs {
  const int4 *work;
  int items;
  const float *a, *a_lo, *x_hi, *x_lo;
  float *r;
  double *norms;
  const int64_t *offset;
  const int32_t *n;
};

// Flat (matrix, tile_i, tile_j) work list for square tiles of size `tile`.
int gemmWork(msq_ctx *ctx, const DeviceBatch *b, int tile, const int4 **work, int *items);
// C = A B per matrix, FP32 FMA; by default A(i,k) = a[k + i*n] and
// B(k,j) = bm[k + j*n] (C = a^T bm).
int gemmTN(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *bm, float *c,
           int epilogue, const float *eigenvalues, bool a_mmajor = false,
           bool b_nmajor = false);
// R = (a + a_lo) - (x_hi + x_lo)^2 in float-float; a_lo and x_lo may be null.
int residualFF(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *x_hi,
               const float *x_lo, float *r, double *norms, const float *a_lo = nullptr);
int makeFactor(msq_ctx *ctx, const DeviceBatch *b, const float *v, const float *lam, float *f);
int transpose(msq_ctx *ctx, const DeviceBatch *b, const float *src, float *dst);
int symmetricAdd(msq_ctx *ctx, const DeviceBatch *b, float *x_hi, float *x_lo, const float *e);
// The same residual for a general (not necessarily symmetric) X.
int residualFFGeneral(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *x_hi,
                      const float *x_lo, float *r, double *norms, const float *a_lo = nullptr);
// X <- X + E in float-float, no symmetrisation.
int workingAdd(msq_ctx *ctx, const DeviceBatch *b, float *x_hi, float *x_lo, const float *e);
// One n x n matrix: C = A B with in-order FMA chains; C_ij = W_ij / (s_i + s_j).
int matmulFma(msq_ctx *ctx, const float *a, const float *b, float *c, int n);
int diagonalSylvester(msq_ctx *ctx, const float *w, const float *s, float *c, int n);
// The same for every matrix of a batch in one launch (s at eig_offset).
int matmulFmaBatch(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *bm, float *c);
int diagonalSylvesterBatch(msq_ctx *ctx, const DeviceBatch *b, const float *w, const float *s,
                           float *c);

}  // namespace msq
