/* Project-written declarations of the Fortran-77 BLAS entry points used by
 * the reference's Native/Native.Matrix/*.c files. Test infrastructure. */
#ifndef EGX_ORACLE_F77BLAS_H
#define EGX_ORACLE_F77BLAS_H
void zspmv_(char *uplo, blasint *n, double *alpha, double *ap, double *x, blasint *incx,
            double *beta, double *y, blasint *incy);
void zrotg_(double *ca, double *cb, double *c, double *s);
#endif
