/*
 * LP64 Fortran BLAS entry points (dgemm_, daxpy_, dcopy_, dscal_) forwarded to
 * the ILP64 OpenBLAS that numpy bundles (symbols scipy_*_64_).  Used only to
 * link the unmodified CAPS sources for the oracle build (oracle/build_ref.sh).
 */
#include <stdint.h>
extern void scipy_dgemm_64_(const char *, const char *, const int64_t *, const int64_t *,
                            const int64_t *, const double *, const double *, const int64_t *,
                            const double *, const int64_t *, const double *, double *,
                            const int64_t *);
extern void scipy_daxpy_64_(const int64_t *, const double *, const double *, const int64_t *,
                            double *, const int64_t *);
extern void scipy_dcopy_64_(const int64_t *, const double *, const int64_t *, double *,
                            const int64_t *);
extern void scipy_dscal_64_(const int64_t *, const double *, double *, const int64_t *);

void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha, double *a, int *lda,
            double *b, int *ldb, double *beta, double *c, int *ldc)
{
    int64_t M = *m, N = *n, K = *k, LA = *lda, LB = *ldb, LC = *ldc;
    scipy_dgemm_64_(ta, tb, &M, &N, &K, alpha, a, &LA, b, &LB, beta, c, &LC);
}
void daxpy_(int *n, double *alpha, double *x, int *incx, double *y, int *incy)
{
    int64_t N = *n, IX = *incx, IY = *incy;
    scipy_daxpy_64_(&N, alpha, x, &IX, y, &IY);
}
void dcopy_(int *n, double *x, int *incx, double *y, int *incy)
{
    int64_t N = *n, IX = *incx, IY = *incy;
    scipy_dcopy_64_(&N, x, &IX, y, &IY);
}
void dscal_(int *n, double *alpha, double *x, int *incx)
{
    int64_t N = *n, IX = *incx;
    scipy_dscal_64_(&N, alpha, x, &IX);
}
