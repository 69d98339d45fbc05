/* Project-written declarations of the CBLAS entry points that the
 * reference's Native/Native.Matrix/*.c files call. The definitions live in
 * oracle/ref_blas_shim.c (plain reference-BLAS loops). Test infrastructure. */
#ifndef EGX_ORACLE_CBLAS_H
#define EGX_ORACLE_CBLAS_H
#include <stddef.h>
typedef int blasint;
typedef struct { double real; double imag; } openblas_complex_double;
#define OPENBLAS_NEEDBUNDERSCORE 1
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
void cblas_zaxpy(blasint n, const void *alpha, const void *x, blasint incx, void *y, blasint incy);
void cblas_zcopy(blasint n, const void *x, blasint incx, void *y, blasint incy);
void cblas_zscal(blasint n, const void *alpha, void *x, blasint incx);
void cblas_zdotc_sub(blasint n, const void *x, blasint incx, const void *y, blasint incy, void *ret);
void cblas_zdotu_sub(blasint n, const void *x, blasint incx, const void *y, blasint incy, void *ret);
void cblas_zgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, blasint m, blasint n,
                 const void *alpha, const void *a, blasint lda, const void *x, blasint incx,
                 const void *beta, void *y, blasint incy);
void cblas_ztrsv(enum CBLAS_ORDER order, enum CBLAS_UPLO uplo, enum CBLAS_TRANSPOSE trans,
                 enum CBLAS_DIAG diag, blasint n, const void *a, blasint lda, void *x, blasint incx);
double cblas_dznrm2(blasint n, const void *x, blasint incx);
void cblas_zimatcopy(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, blasint rows, blasint cols,
                     const double *alpha, double *a, blasint lda, blasint ldb);
#endif
