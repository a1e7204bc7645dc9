/* Shim: LAPACK prototypes the reference calls (src/numerics.cpp,
 * src/accelerate_backend.cpp), bound to scipy's OpenBLAS exported names.
 * Test infrastructure only (oracle/_ref). */
#pragma once
#include <vecLib/lapack_types.h>

#define dsyevd_ scipy_dsyevd_
#define ssyevd_ scipy_ssyevd_
#define dgees_ scipy_dgees_
#define sgees_ scipy_sgees_
#define strsyl_ scipy_strsyl_
#define dtrsyl_ scipy_dtrsyl_

#ifdef __cplusplus
extern "C" {
#endif
typedef __LAPACK_bool (*msq_shim_select_d)(double *, double *);
typedef __LAPACK_bool (*msq_shim_select_s)(float *, float *);
void scipy_dsyevd_(const char *jobz, const char *uplo, const __LAPACK_int *n,
                   double *a, const __LAPACK_int *lda, double *w, double *work,
                   const __LAPACK_int *lwork, __LAPACK_int *iwork,
                   const __LAPACK_int *liwork, __LAPACK_int *info);
void scipy_ssyevd_(const char *jobz, const char *uplo, const __LAPACK_int *n,
                   float *a, const __LAPACK_int *lda, float *w, float *work,
                   const __LAPACK_int *lwork, __LAPACK_int *iwork,
                   const __LAPACK_int *liwork, __LAPACK_int *info);
void scipy_dgees_(const char *jobvs, const char *sort, msq_shim_select_d select,
                  const __LAPACK_int *n, double *a, const __LAPACK_int *lda,
                  __LAPACK_int *sdim, double *wr, double *wi, double *vs,
                  const __LAPACK_int *ldvs, double *work,
                  const __LAPACK_int *lwork, __LAPACK_bool *bwork,
                  __LAPACK_int *info);
void scipy_sgees_(const char *jobvs, const char *sort, msq_shim_select_s select,
                  const __LAPACK_int *n, float *a, const __LAPACK_int *lda,
                  __LAPACK_int *sdim, float *wr, float *wi, float *vs,
                  const __LAPACK_int *ldvs, float *work,
                  const __LAPACK_int *lwork, __LAPACK_bool *bwork,
                  __LAPACK_int *info);
void scipy_strsyl_(const char *trana, const char *tranb,
                   const __LAPACK_int *isgn, const __LAPACK_int *m,
                   const __LAPACK_int *n, const float *a,
                   const __LAPACK_int *lda, const float *b,
                   const __LAPACK_int *ldb, float *c, const __LAPACK_int *ldc,
                   float *scale, __LAPACK_int *info);
void scipy_dtrsyl_(const char *trana, const char *tranb,
                   const __LAPACK_int *isgn, const __LAPACK_int *m,
                   const __LAPACK_int *n, const double *a,
                   const __LAPACK_int *lda, const double *b,
                   const __LAPACK_int *ldb, double *c, const __LAPACK_int *ldc,
                   double *scale, __LAPACK_int *info);
#ifdef __cplusplus
}
#endif
