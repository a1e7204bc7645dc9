/* Shim: BLAS prototypes the reference calls, bound to scipy's OpenBLAS.
 * Test infrastructure only (oracle/_ref). */
#pragma once
#include <vecLib/lapack_types.h>

#define dgemm_ scipy_dgemm_
#define sgemm_ scipy_sgemm_
#define dsyrk_ scipy_dsyrk_
#define ssymm_ scipy_ssymm_

#ifdef __cplusplus
extern "C" {
#endif
void scipy_dgemm_(const char *ta, const char *tb, const __LAPACK_int *m,
                  const __LAPACK_int *n, const __LAPACK_int *k,
                  const double *alpha, const double *a, const __LAPACK_int *lda,
                  const double *b, const __LAPACK_int *ldb, const double *beta,
                  double *c, const __LAPACK_int *ldc);
void scipy_sgemm_(const char *ta, const char *tb, const __LAPACK_int *m,
                  const __LAPACK_int *n, const __LAPACK_int *k,
                  const float *alpha, const float *a, const __LAPACK_int *lda,
                  const float *b, const __LAPACK_int *ldb, const float *beta,
                  float *c, const __LAPACK_int *ldc);
void scipy_dsyrk_(const char *uplo, const char *trans, const __LAPACK_int *n,
                  const __LAPACK_int *k, const double *alpha, const double *a,
                  const __LAPACK_int *lda, const double *beta, double *c,
                  const __LAPACK_int *ldc);
void scipy_ssymm_(const char *side, const char *uplo, const __LAPACK_int *m,
                  const __LAPACK_int *n, const float *alpha, const float *a,
                  const __LAPACK_int *lda, const float *b,
                  const __LAPACK_int *ldb, const float *beta, float *c,
                  const __LAPACK_int *ldc);
#ifdef __cplusplus
}
#endif
