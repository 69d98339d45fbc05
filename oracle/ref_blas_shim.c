/* Reference-BLAS shim for compiling the reference's native math files
 * (Native/Native.Matrix/{green_scalar,full_zgemv,green_conv,green_tensor}.c)
 * into the oracle's known-answer library oracle/_ref/libntv_math_ref.so.
 *
 * TEST INFRASTRUCTURE ONLY: the reference links OpenBLAS or MKL
 * (Native/make.inc:12,28), which are not vendored and not installed here.
 * These are straightforward loops following the published reference-BLAS
 * algorithms (netlib BLAS: zaxpy, zcopy, zscal, zdotc, zdotu, zgemv, zspmv,
 * ztrsv, dznrm2, zrot, zrotg), written for this project. */
#include <complex.h>
#include <math.h>
#include <string.h>
#include "cblas.h"

typedef double _Complex zc;

static zc ld(const void *p, long i) { return ((const zc *)p)[i]; }

void cblas_zaxpy(blasint n, const void *alpha, const void *x, blasint incx, void *y, blasint incy)
{
    zc a = *(const zc *)alpha;
    zc *yy = (zc *)y;
    for (long i = 0; i < n; i++) yy[i * incy] += a * ld(x, i * incx);
}

void cblas_zcopy(blasint n, const void *x, blasint incx, void *y, blasint incy)
{
    zc *yy = (zc *)y;
    for (long i = 0; i < n; i++) yy[i * incy] = ld(x, i * incx);
}

void cblas_zscal(blasint n, const void *alpha, void *x, blasint incx)
{
    zc a = *(const zc *)alpha;
    zc *xx = (zc *)x;
    for (long i = 0; i < n; i++) xx[i * incx] *= a;
}

void cblas_zdotc_sub(blasint n, const void *x, blasint incx, const void *y, blasint incy, void *ret)
{
    zc s = 0;
    for (long i = 0; i < n; i++) s += conj(ld(x, i * incx)) * ld(y, i * incy);
    *(zc *)ret = s;
}

void cblas_zdotu_sub(blasint n, const void *x, blasint incx, const void *y, blasint incy, void *ret)
{
    zc s = 0;
    for (long i = 0; i < n; i++) s += ld(x, i * incx) * ld(y, i * incy);
    *(zc *)ret = s;
}

/* y = alpha*op(A)*x + beta*y for an m x n matrix A in the given storage. */
void cblas_zgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, blasint m, blasint n,
                 const void *alpha, const void *a, blasint lda, const void *x, blasint incx,
                 const void *beta, void *y, blasint incy)
{
    zc al = *(const zc *)alpha, be = *(const zc *)beta;
    zc *yy = (zc *)y;
    long rows = (trans == CblasNoTrans) ? m : n;
    long cols = (trans == CblasNoTrans) ? n : m;
    for (long i = 0; i < rows; i++) {
        zc s = 0;
        for (long j = 0; j < cols; j++) {
            /* element op(A)[i][j] */
            long r = (trans == CblasNoTrans) ? i : j;
            long c = (trans == CblasNoTrans) ? j : i;
            zc aij = (order == CblasRowMajor) ? ld(a, r * lda + c) : ld(a, c * lda + r);
            if (trans == CblasConjTrans) aij = conj(aij);
            s += aij * ld(x, j * incx);
        }
        zc prev = (be == 0) ? 0 : be * yy[i * incy];
        yy[i * incy] = prev + al * s;
    }
}

/* Upper, non-unit, column-major triangular solve (the only form used). */
void cblas_ztrsv(enum CBLAS_ORDER order, enum CBLAS_UPLO uplo, enum CBLAS_TRANSPOSE trans,
                 enum CBLAS_DIAG diag, blasint n, const void *a, blasint lda, void *x, blasint incx)
{
    (void)order; (void)uplo; (void)trans; (void)diag;
    zc *xx = (zc *)x;
    for (long j = n - 1; j >= 0; j--) {
        if (xx[j * incx] != 0) {
            xx[j * incx] /= ld(a, j * lda + j);
            zc t = xx[j * incx];
            for (long i = j - 1; i >= 0; i--) xx[i * incx] -= t * ld(a, j * lda + i);
        }
    }
}

double cblas_dznrm2(blasint n, const void *x, blasint incx)
{
    double scale = 0.0, ssq = 1.0;
    for (long i = 0; i < n; i++) {
        zc v = ld(x, i * incx);
        double parts[2] = {creal(v), cimag(v)};
        for (int k = 0; k < 2; k++) {
            if (parts[k] != 0.0) {
                double t = fabs(parts[k]);
                if (scale < t) { ssq = 1.0 + ssq * (scale / t) * (scale / t); scale = t; }
                else ssq += (t / scale) * (t / scale);
            }
        }
    }
    return scale * sqrt(ssq);
}

void cblas_zimatcopy(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, blasint rows, blasint cols,
                     const double *alpha, double *a, blasint lda, blasint ldb)
{
    (void)order; (void)trans; (void)rows; (void)cols; (void)alpha; (void)a; (void)lda; (void)ldb;
}

/* Symmetric packed (upper) matrix-vector product. */
void zspmv_(char *uplo, blasint *n_, double *alpha, double *ap, double *x, blasint *incx,
            double *beta, double *y, blasint *incy)
{
    (void)uplo;
    long n = *n_;
    zc al = *(zc *)alpha, be = *(zc *)beta;
    zc *yy = (zc *)y;
    const zc *A = (const zc *)ap;
    const zc *xx = (const zc *)x;
    for (long i = 0; i < n; i++) yy[i * *incy] = (be == 0) ? 0 : be * yy[i * *incy];
    long kk = 0;
    for (long j = 0; j < n; j++) {
        zc t1 = al * xx[j * *incx], t2 = 0;
        for (long i = 0; i < j; i++) {
            yy[i * *incy] += t1 * A[kk + i];
            t2 += A[kk + i] * xx[i * *incx];
        }
        yy[j * *incy] += t1 * A[kk + j] + al * t2;
        kk += j + 1;
    }
}

/* Plane rotation with a real cosine and a complex sine. */
void zrot_(blasint *n, double *cx, blasint *incx, double *cy, blasint *incy, double *c, double *s)
{
    zc *x = (zc *)cx, *y = (zc *)cy;
    zc ss = *(zc *)s;
    for (long i = 0; i < *n; i++) {
        zc t = *c * x[i * *incx] + ss * y[i * *incy];
        y[i * *incy] = *c * y[i * *incy] - conj(ss) * x[i * *incx];
        x[i * *incx] = t;
    }
}

/* Classic reference ZROTG: c = |a|/norm, s = (a/|a|) conj(b)/norm. */
void zrotg_(double *ca_, double *cb_, double *c, double *s)
{
    zc ca = *(zc *)ca_, cb = *(zc *)cb_;
    if (cabs(ca) == 0.0) {
        *c = 0.0;
        *(zc *)s = 1.0;
        *(zc *)ca_ = cb;
    } else {
        double scale = cabs(ca) + cabs(cb);
        double a1 = cabs(ca / scale), b1 = cabs(cb / scale);
        double norm = scale * sqrt(a1 * a1 + b1 * b1);
        zc alpha = ca / cabs(ca);
        *c = cabs(ca) / norm;
        *(zc *)s = alpha * conj(cb) / norm;
        *(zc *)ca_ = alpha * norm;
    }
}
