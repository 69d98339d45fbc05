/* CPU restatement of the per-point Green block contraction of the CIE
 * operator apply, multi-threaded: the CPU baseline of the benchmark and a
 * second check of the numpy oracle (oracle/operator.py: contract).
 *
 * TEST INFRASTRUCTURE ONLY (oracle): not part of the product.
 *
 * Follows Extreme.Cartesian/Forward/AtoA/ConvolutionOperator.cs:274-327
 * (ApplyGreenTensorAlongZ): for every spectral point, with the packed
 * symmetric blocks applied like BLAS zspmv 'U' (packed index rc + tr(tr+1)/2,
 * rc <= tr) and the asymmetric blocks like zgemv (index rc*nz + tr):
 *   out_x =  Sxx x + Sxy y + Axz z
 *   out_y =  Sxy x + Syy y + Ayz z
 *   out_z = -Axz^T x - Ayz^T y + Szz z
 * Component blocks are [npts][block]; in/out are [npts][3][nz]. Points are
 * split over `nthreads` OpenMP threads (0: the runtime default).
 */
#include <complex.h>
#include <omp.h>

typedef double _Complex zc;

static void spmv_acc(int nz, const zc *p, const zc *x, zc *y)
{
    long idx = 0;
    for (int tr = 0; tr < nz; tr++) {
        zc acc = 0;
        zc xt = x[tr];
        for (int rc = 0; rc < tr; rc++, idx++) {
            zc a = p[idx];
            y[rc] += a * xt;
            acc += a * x[rc];
        }
        y[tr] += acc + p[idx] * xt;
        idx++;
    }
}

void oracle_contract(long npts, int nz, const zc *xx, const zc *xy, const zc *yy, const zc *zz, const zc *xz,
                     const zc *yz, const zc *in, zc *out, int nthreads)
{
    long s = (long)nz * (nz + 1) / 2;
    long a = (long)nz * nz;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (long p = 0; p < npts; p++) {
        const zc *x = in + p * 3 * nz;
        const zc *y = x + nz;
        const zc *z = y + nz;
        zc *ox = out + p * 3 * nz;
        zc *oy = ox + nz;
        zc *oz = oy + nz;
        for (int k = 0; k < 3 * nz; k++) ox[k] = 0;
        spmv_acc(nz, xx + p * s, x, ox);
        spmv_acc(nz, xy + p * s, y, ox);
        spmv_acc(nz, xy + p * s, x, oy);
        spmv_acc(nz, yy + p * s, y, oy);
        spmv_acc(nz, zz + p * s, z, oz);
        const zc *bxz = xz + p * a;
        const zc *byz = yz + p * a;
        for (int rc = 0; rc < nz; rc++) {
            zc accx = 0, accy = 0;
            zc xr = x[rc], yr = y[rc];
            for (int tr = 0; tr < nz; tr++) {
                zc gxz = bxz[rc * nz + tr];
                zc gyz = byz[rc * nz + tr];
                accx += gxz * z[tr];
                accy += gyz * z[tr];
                oz[tr] -= gxz * xr + gyz * yr;
            }
            ox[rc] += accx;
            oy[rc] += accy;
        }
    }
}

int oracle_max_threads(void) { return omp_get_max_threads(); }
