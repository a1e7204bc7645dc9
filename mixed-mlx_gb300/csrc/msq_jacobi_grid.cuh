// Grid-parallel Jacobi for one large matrix (msq_jacobi_grid.cu).  Internal.
#pragma once

#include "msq_internal.cuh"

namespace msq {

// Solves one matrix on the context's stream with every SM: `matrix`
// (column-major n x n, overwritten with the rotated matrix), `vectors`
// (column-major eigenvectors), `eigenvalues` (n).  Synchronises the context's
// stream once per sweep to read the off-norm.  Reports the sweeps applied,
// the final off(A)/||A||_F and ||A||_F^2.  keep_vectors: `vectors` holds
// the rotations of an earlier solve of this matrix (continued, not reset).
int gridJacobiSolve(msq_ctx *ctx, float *matrix, float *vectors, float *eigenvalues, int n,
                    double tolerance, int max_sweeps, int *sweeps_out, double *off_ratio_out,
                    double *norm2_out, bool keep_vectors = false);

}  // namespace msq
