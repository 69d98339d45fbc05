// CIE convolution operator kernels.
//
// One apply (ConvolutionOperator.CalculateOperatorAorKr, ConvolutionOperator.cs:162-171)
// is five kernels over the spectral buffer buf[2nx][2ny][B], B = nrhs*3*nz:
//   k_fwd_y     : rx = r*x, scale by the forward factors, zero-pad, DFT along y
//                 (ApplyOperatorR + PrepareForForwardFft + half of the forward FFT);
//                 only the nx rows that hold data are transformed;
//   k_lines     : DFT along x over all 2ny columns, reading only the nx non-zero rows;
//   k_contract  : per spectral point, the 3x3 block product with the Green tensor
//                 (ApplyGreenTensorAlongZ, :274-327), one CTA per stored quadrant point
//                 serving the up to four points that share its block;
//   k_lines     : inverse DFT along x, writing only the nx rows that are extracted;
//   k_bwd_y     : inverse DFT along y, extraction with the backward factors and the
//                 last step (ExtractData + PerformLastStep, :187-231).
#include <algorithm>
#include <type_traits>

#include "egx_ds.cuh"
#include "egx_fft_reg.cuh"
#include "egx_operator.cuh"

namespace egx {

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ int sym_index(int i, int j) {
    return (i <= j) ? i + j * (j + 1) / 2 : j + i * (i + 1) / 2;
}

template <typename T>
__global__ void k_fwd_y(const C<T> *__restrict__ x, const OperatorData<T> op, C<T> *__restrict__ buf, const OpDims d,
                        const FftPlan plan, const C<T> *__restrict__ tw, int bt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C<T> *sa = reinterpret_cast<C<T> *>(smem_raw);
    C<T> *sb = sa + plan.n * bt;
    const int i = blockIdx.x;
    const int b0 = blockIdx.y * bt;
    const int n1 = plan.n;
    const int per = 3 * d.nz;
    for (int item = threadIdx.x; item < n1 * bt; item += blockDim.x) {
        int j = item / bt, col = item - j * bt;
        int b = b0 + col;
        C<T> v = mk<T>(0, 0);
        if (j < d.ny && b < d.B) {
            int rhs = b / per, rem = b - rhs * per;
            int k = rem % d.nz, c = rem / d.nz;
            long cell = (long)i * d.ny + j;
            C<T> xv = x[rhs * d.nvec + (cell * 3 + c) * d.nz + k];
            C<T> rx = cmul<T>(op.r[cell * d.nz + k], xv);
            v = cmul<T>(op.fwd[k], rx);
        }
        sa[item] = v;
    }
    __syncthreads();
    C<T> *res = fft_smem<T>(sa, sb, plan, bt, tw, -1);
    for (int item = threadIdx.x; item < n1 * bt; item += blockDim.x) {
        int j = item / bt, col = item - j * bt;
        int b = b0 + col;
        if (b < d.B) buf[((long)i * n1 + j) * d.B + b] = res[item];
    }
}

// DFT of `lines` interleaved sequences: element e of line L, column b at
// base + L*lstride + e*estride + b. Elements e >= nload read as zero, only
// e < nstore are written back.
template <typename T>
__global__ void k_lines(C<T> *buf, long lstride, long estride, int B, int nload, int nstore, const FftPlan plan,
                        const C<T> *__restrict__ tw, int bt, int sign) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C<T> *sa = reinterpret_cast<C<T> *>(smem_raw);
    C<T> *sb = sa + plan.n * bt;
    const long base = (long)blockIdx.x * lstride;
    const int b0 = blockIdx.y * bt;
    const int n = plan.n;
    for (int item = threadIdx.x; item < n * bt; item += blockDim.x) {
        int e = item / bt, col = item - e * bt;
        int b = b0 + col;
        C<T> v = mk<T>(0, 0);
        if (e < nload && b < B) v = buf[base + e * estride + b];
        sa[item] = v;
    }
    __syncthreads();
    C<T> *res = fft_smem<T>(sa, sb, plan, bt, tw, sign);
    for (int item = threadIdx.x; item < n * bt; item += blockDim.x) {
        int e = item / bt, col = item - e * bt;
        int b = b0 + col;
        if (e < nstore && b < B) buf[base + e * estride + b] = res[item];
    }
}

template <typename T>
__global__ void k_bwd_y(const C<T> *__restrict__ buf, const C<T> *__restrict__ x, const OperatorData<T> op,
                        C<T> *__restrict__ y, const OpDims d, const FftPlan plan, const C<T> *__restrict__ tw, int bt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C<T> *sa = reinterpret_cast<C<T> *>(smem_raw);
    C<T> *sb = sa + plan.n * bt;
    const int i = blockIdx.x;
    const int b0 = blockIdx.y * bt;
    const int n1 = plan.n;
    const int per = 3 * d.nz;
    for (int item = threadIdx.x; item < n1 * bt; item += blockDim.x) {
        int j = item / bt, col = item - j * bt;
        int b = b0 + col;
        sa[item] = (b < d.B) ? buf[((long)i * n1 + j) * d.B + b] : mk<T>(0, 0);
    }
    __syncthreads();
    C<T> *res = fft_smem<T>(sa, sb, plan, bt, tw, +1);
    for (int item = threadIdx.x; item < d.ny * bt; item += blockDim.x) {
        int j = item / bt, col = item - j * bt;
        int b = b0 + col;
        if (b >= d.B) continue;
        int rhs = b / per, rem = b - rhs * per;
        int k = rem % d.nz, c = rem / d.nz;
        long cell = (long)i * d.ny + j;
        long idx = rhs * d.nvec + (cell * 3 + c) * d.nz + k;
        C<T> yv = cmul<T>(op.bwd[k], res[item]);
        C<T> xv = x[idx];
        C<T> rx = cmul<T>(op.r[cell * d.nz + k], xv);
        C<T> out;
        if (op.type == EGX_OP_A) out = csub<T>(csub<T>(xv, yv), rx);
        else out = cadd<T>(yv, rx);
        y[idx] = out;
    }
}

// ------------------------------------------------------------------
// The same three steps on the register-resident DFT (egx_fft_reg.cuh) for
// lengths in {64, 128, 256, 512}: one CTA per line and 128-byte tile of
// columns, every global access a whole row segment of BT columns. The y
// passes and the forward x pass run 64-byte tiles (512 threads per CTA for
// complex64, four CTAs per SM at 32 registers), whose CTAs overlap their
// load, exchange and store phases better than two 1,024-thread CTAs of
// 128-byte tiles (fwd y 0.174 -> 0.146 ms, fwd x 0.240 -> 0.227 ms at
// 256x256x48, two sources); the backward x pass keeps 128-byte tiles
// (0.211 ms, 0.248 with 64-byte tiles).
template <typename T, int N, int BT>
__global__ void __launch_bounds__(reg_threads<N, T, BT>(), reg_min_blocks<N, T, BT>())
    k_fwd_y_r(const C<T> *__restrict__ x, const OperatorData<T> op, C<T> *__restrict__ buf, const OpDims d,
              const C<T> *__restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.y;
    const int b = blockIdx.x * BT + (int)(threadIdx.x % BT);
    const bool bok = b < d.B;
    const int per = 3 * d.nz;
    const int rhs = bok ? b / per : 0, rem = b - rhs * per, k = rem % d.nz;
    const C<T> f = bok ? op.fwd[k] : mk<T>(0, 0);
    const C<T> *xr = x + rhs * d.nvec + rem;
    auto load = [&](int j) -> C<T> {
        if (!bok || j >= d.ny) return mk<T>(0, 0);
        const long cell = (long)i * d.ny + j;
        return cmul<T>(f, cmul<T>(op.r[cell * d.nz + k], xr[cell * per]));
    };
    auto store = [&](int j, C<T> v) {
        if (bok) buf[((long)i * N + j) * d.B + b] = v;
    };
    fft_reg<T, N, BT>(reinterpret_cast<C<T> *>(smem_raw), tw, -1, load, store);
}

template <typename T, int N, int BT>
__global__ void __launch_bounds__(reg_threads<N, T, BT>())
    k_lines_r(C<T> *buf, long lstride, long estride, int B, int nload, int nstore, const C<T> *__restrict__ tw,
              int sign) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = blockIdx.x * BT + (int)(threadIdx.x % BT);
    const bool bok = b < B;
    C<T> *line = buf + (long)blockIdx.y * lstride + b;
    auto load = [&](int e) -> C<T> { return (bok && e < nload) ? line[e * estride] : mk<T>(0, 0); };
    auto store = [&](int e, C<T> v) {
        if (bok && e < nstore) line[e * estride] = v;
    };
    fft_reg<T, N, BT>(reinterpret_cast<C<T> *>(smem_raw), tw, sign, load, store);
}

template <typename T, int N, int BT>
__global__ void __launch_bounds__(reg_threads<N, T, BT>(), reg_min_blocks<N, T, BT>())
    k_bwd_y_r(const C<T> *__restrict__ buf, const C<T> *__restrict__ x, const OperatorData<T> op,
              C<T> *__restrict__ y, const OpDims d, const C<T> *__restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.y;
    const int b = blockIdx.x * BT + (int)(threadIdx.x % BT);
    const bool bok = b < d.B;
    const int per = 3 * d.nz;
    const int rhs = bok ? b / per : 0, rem = b - rhs * per, k = rem % d.nz;
    const C<T> bw = bok ? op.bwd[k] : mk<T>(0, 0);
    const C<T> *row = buf + (long)i * N * d.B + b;
    auto load = [&](int j) -> C<T> { return bok ? row[(long)j * d.B] : mk<T>(0, 0); };
    auto store = [&](int j, C<T> v) {
        if (!bok || j >= d.ny) return;
        const long cell = (long)i * d.ny + j;
        const long idx = rhs * d.nvec + cell * per + rem;
        const C<T> yv = cmul<T>(bw, v);
        const C<T> xv = x[idx];
        const C<T> rx = cmul<T>(op.r[cell * d.nz + k], xv);
        y[idx] = (op.type == EGX_OP_A) ? csub<T>(csub<T>(xv, yv), rx) : cadd<T>(yv, rx);
    };
    fft_reg<T, N, BT>(reinterpret_cast<C<T> *>(smem_raw), tw, +1, load, store);
}

// Lines whose second half is the parity image of the first: element e of a
// line is v[e] for e < N/2, 0 at e = N/2 and par * v[N - e] beyond, with only
// v[0 .. N/2) stored; outputs e < nstore are written back in place.
template <typename T, int N>
__global__ void __launch_bounds__(reg_threads<N, T>())
    k_lines_sym_r(C<T> *buf, long lstride, long estride, int B, T par, int nstore, const C<T> *__restrict__ tw,
                  int sign) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int BT = RegCols<T>::BT, NH = N / 2;
    const int b = blockIdx.y * BT + (int)(threadIdx.x % BT);
    const bool bok = b < B;
    C<T> *line = buf + (long)blockIdx.x * lstride + b;
    auto load = [&](int e) -> C<T> {
        if (!bok || e == NH) return mk<T>(0, 0);
        if (e < NH) return line[e * estride];
        const C<T> v = line[(N - e) * estride];
        return mk<T>(par * v.x, par * v.y);
    };
    auto store = [&](int e, C<T> v) {
        if (bok && e < nstore) line[e * estride] = v;
    };
    fft_reg<T, N>(reinterpret_cast<C<T> *>(smem_raw), tw, sign, load, store);
}

template <typename T, int N, int BT = RegCols<T>::BT>
static void reg_attr(const void *fn) {
    constexpr size_t sm = reg_smem<N, T, BT>();
    raise_smem_limit(fn, sm);
}

// which: 0 fwd_y, 1 lines, 2 bwd_y
template <typename T, int N, int BT>
static void launch_reg(int which, cudaStream_t s, int nlines, const C<T> *x, const OperatorData<T> *op, C<T> *buf,
                       C<T> *y, const OpDims *d, long lstride, long estride, int B, int nload, int nstore,
                       const C<T> *tw, int sign) {
    constexpr size_t sm = reg_smem<N, T, BT>();
    constexpr int thr = reg_threads<N, T, BT>();
    // column tiles on x: the CTAs in flight together cover whole rows of a
    // line (every column of an (x, y) point's 3 nz values, per source),
    // rather than one tile of many lines, so DRAM sees long runs
    const dim3 grid((B + BT - 1) / BT, nlines);
    if (which == 0) {
        reg_attr<T, N, BT>((const void *)k_fwd_y_r<T, N, BT>);
        k_fwd_y_r<T, N, BT><<<grid, thr, sm, s>>>(x, *op, buf, *d, tw);
    } else if (which == 1) {
        reg_attr<T, N, BT>((const void *)k_lines_r<T, N, BT>);
        k_lines_r<T, N, BT><<<grid, thr, sm, s>>>(buf, lstride, estride, B, nload, nstore, tw, sign);
    } else {
        reg_attr<T, N, BT>((const void *)k_bwd_y_r<T, N, BT>);
        k_bwd_y_r<T, N, BT><<<grid, thr, sm, s>>>(buf, x, *op, y, *d, tw);
    }
}

template <typename T, int N>
static void launch_reg_tile(int which, cudaStream_t s, int nlines, const C<T> *x, const OperatorData<T> *op,
                            C<T> *buf, C<T> *y, const OpDims *d, long lstride, long estride, int B, int nload,
                            int nstore, const C<T> *tw, int sign, int tile) {
    // 64-byte tiles for the y passes and for x passes that write more rows
    // than they read; 128-byte tiles otherwise (unless the tuner chose)
    if (tile == 1 || (tile == 0 && (which != 1 || nload < nstore)))
        launch_reg<T, N, RegCols<T>::BTN>(which, s, nlines, x, op, buf, y, d, lstride, estride, B, nload, nstore, tw,
                                           sign);
    else
        launch_reg<T, N, RegCols<T>::BT>(which, s, nlines, x, op, buf, y, d, lstride, estride, B, nload, nstore, tw,
                                          sign);
}

// returns false when n has no register plan
template <typename T>
static bool run_reg(int n, int which, int nlines, int B, cudaStream_t s, const C<T> *x, const OperatorData<T> *op,
                    C<T> *buf, C<T> *y, const OpDims *d, long lstride, long estride, int nload, int nstore,
                    const C<T> *tw, int sign, int tile = 0) {
    if (!reg_fft_ok(n)) return false;
    switch (n) {
        case 64: launch_reg_tile<T, 64>(which, s, nlines, x, op, buf, y, d, lstride, estride, B, nload, nstore, tw, sign, tile); break;
        case 128: launch_reg_tile<T, 128>(which, s, nlines, x, op, buf, y, d, lstride, estride, B, nload, nstore, tw, sign, tile); break;
        case 256: launch_reg_tile<T, 256>(which, s, nlines, x, op, buf, y, d, lstride, estride, B, nload, nstore, tw, sign, tile); break;
        default: launch_reg_tile<T, 512>(which, s, nlines, x, op, buf, y, d, lstride, estride, B, nload, nstore, tw, sign, tile); break;
    }
    return true;
}

// Block contraction, one CTA per stored quadrant point (a, b). The block is
// staged in shared memory when it fits (G_IN_SMEM), else read through L1.
template <typename T, bool G_IN_SMEM>
__global__ void k_contract(C<T> *buf, const C<T> *__restrict__ G, const OpDims d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nz = d.nz;
    const int S = nz * (nz + 1) / 2, lda = nz + 1, A = nz * lda, Bs = 4 * S + 2 * A;
    const int q = blockIdx.x;
    const int a = q / (d.ny + 1), bq = q - a * (d.ny + 1);
    const int n1 = 2 * d.ny;
    const int kx[2] = {a, 2 * d.nx - a};
    const int ky[2] = {bq, 2 * d.ny - bq};
    const int nkx = (a == 0 || a == d.nx) ? 1 : 2;
    const int nky = (bq == 0 || bq == d.ny) ? 1 : 2;
    const int npts = nkx * nky;
    const int per = 3 * nz;
    const int nv = npts * d.nrhs;

    C<T> *sX = reinterpret_cast<C<T> *>(smem_raw);
    C<T> *sG = sX + 4 * d.nrhs * per;
    const C<T> *gq = G + (long)q * Bs;
    const C<T> *g;
    if (G_IN_SMEM) {
        for (int t = threadIdx.x; t < Bs; t += blockDim.x) sG[t] = gq[t];
        g = sG;
    } else {
        g = gq;
    }
    for (int t = threadIdx.x; t < nv * per; t += blockDim.x) {
        int v = t / per, e = t - v * per;
        int p = v / d.nrhs, rhs = v - p * d.nrhs;
        long pt = (long)kx[p / nky] * n1 + ky[p % nky];
        sX[t] = buf[pt * d.B + rhs * per + e];
    }
    __syncthreads();
    const C<T> *gxx = g, *gxy = g + S, *gyy = g + 2 * S, *gzz = g + 3 * S;
    const C<T> *gxz = g + 4 * S, *gyz = g + 4 * S + A;
    for (int o = threadIdx.x; o < per * nv; o += blockDim.x) {
        int v = o % nv;
        int ci = o / nv;
        int cout = ci / nz, i = ci - cout * nz;
        int p = v / d.nrhs, rhs = v - p * d.nrhs;
        int mx = (p / nky) == 1, my = (p % nky) == 1;
        const C<T> *X = sX + v * per;
        C<T> a1 = mk<T>(0, 0), a2 = mk<T>(0, 0), a3 = mk<T>(0, 0);
        if (cout == 0) {
            for (int j = 0; j < nz; j++) {
                int s = sym_index(i, j);
                cfma<T>(a1, gxx[s], X[j]);
                cfma<T>(a2, gxy[s], X[nz + j]);
                cfma<T>(a3, gxz[i * lda + j], X[2 * nz + j]);
            }
            // Sxy odd/odd, Axz odd in x
            if (mx != my) a2 = mk<T>(-a2.x, -a2.y);
            if (mx) a3 = mk<T>(-a3.x, -a3.y);
        } else if (cout == 1) {
            for (int j = 0; j < nz; j++) {
                int s = sym_index(i, j);
                cfma<T>(a1, gxy[s], X[j]);
                cfma<T>(a2, gyy[s], X[nz + j]);
                cfma<T>(a3, gyz[i * lda + j], X[2 * nz + j]);
            }
            if (mx != my) a1 = mk<T>(-a1.x, -a1.y);
            if (my) a3 = mk<T>(-a3.x, -a3.y);
        } else {
            for (int j = 0; j < nz; j++) {
                cfma<T>(a1, gxz[j * lda + i], X[j]);
                cfma<T>(a2, gyz[j * lda + i], X[nz + j]);
                cfma<T>(a3, gzz[sym_index(i, j)], X[2 * nz + j]);
            }
            // -Axz^T x - Ayz^T y
            if (!mx) a1 = mk<T>(-a1.x, -a1.y);
            if (!my) a2 = mk<T>(-a2.x, -a2.y);
        }
        C<T> acc = cadd<T>(cadd<T>(a1, a2), a3);
        long pt = (long)kx[p / nky] * n1 + ky[p % nky];
        buf[pt * d.B + rhs * per + cout * nz + i] = acc;
    }
}

// ---------------------------------------------------------------------------
// The complex128 contraction in double-FP32 arithmetic (the mixed form's
// refinement residual). GB300 runs complex128 FMAs at 1/64 of the FP32 rate,
// which makes the FP64 block product above compute-bound; here every
// operand is a pair of floats hi + lo (47 significant bits) and every dot
// product runs as Dot2 (Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26 (2005), Algorithm 5.3): each product
// made error-free with one FMA (TwoProduct), each sum with Knuth's TwoSum,
// the errors added in a second float. The result is as accurate as if it
// had been computed in ~47-bit arithmetic and then rounded to complex128.

constexpr int kDsV = 8;  // right-hand-side points per pass of a thread

// One CTA per stored quadrant point, one thread per output row (component,
// layer) for all its points and right-hand sides; the point's vectors are
// staged as float pairs {re h, re l, im h, im l} in shared memory, the Green
// block is read from global memory and split in registers. Sign flips of the
// D_p symmetries negate the running sums around a block (exact).
__global__ void __launch_bounds__(160) k_contract_ds(double2 *buf, const double2 *__restrict__ G, const OpDims d) {
    extern __shared__ __align__(16) float4 sXd[];
    const int nz = d.nz;
    const int S = nz * (nz + 1) / 2, lda = nz + 1, A = nz * lda, Bs = 4 * S + 2 * A;
    const int q = blockIdx.x;
    const int a = q / (d.ny + 1), bq = q - a * (d.ny + 1);
    const int n1 = 2 * d.ny;
    const int kx[2] = {a, 2 * d.nx - a};
    const int ky[2] = {bq, 2 * d.ny - bq};
    const int nky = (bq == 0 || bq == d.ny) ? 1 : 2;
    const int npts = ((a == 0 || a == d.nx) ? 1 : 2) * nky;
    const int per = 3 * nz;
    const int nv = npts * d.nrhs;
    for (int t = threadIdx.x; t < nv * per; t += blockDim.x) {
        const int v = t / per, e = t - v * per;
        const int p = v / d.nrhs, rhs = v - p * d.nrhs;
        const long pt = (long)kx[p / nky] * n1 + ky[p % nky];
        const double2 x = buf[pt * d.B + rhs * per + e];
        float4 o;
        ds_split(x.x, o.x, o.y);
        ds_split(x.y, o.z, o.w);
        sXd[t] = o;
    }
    __syncthreads();
    const int row = threadIdx.x;
    if (row >= per) return;
    const int cout = row / nz, i = row - cout * nz;
    const double2 *gq = G + (long)q * Bs;
    // per block: base of its Green component and the index kind
    // (0 symmetric packed (i, j), 1 row i of a full nz x lda block, 2 column i)
    const double2 *base[3];
    int kind[3];
    if (cout == 0) {
        base[0] = gq, kind[0] = 0;               // Sxx
        base[1] = gq + S, kind[1] = 0;           // Sxy
        base[2] = gq + 4 * S, kind[2] = 1;       // Axz
    } else if (cout == 1) {
        base[0] = gq + S, kind[0] = 0;           // Sxy
        base[1] = gq + 2 * S, kind[1] = 0;       // Syy
        base[2] = gq + 4 * S + A, kind[2] = 1;   // Ayz
    } else {
        base[0] = gq + 4 * S, kind[0] = 2;       // Axz^T
        base[1] = gq + 4 * S + A, kind[1] = 2;   // Ayz^T
        base[2] = gq + 3 * S, kind[2] = 0;       // Szz
    }
    for (int v0 = 0; v0 < nv; v0 += kDsV) {
        const int cnt = min(kDsV, nv - v0);
        float sr[kDsV], cr[kDsV], si[kDsV], ci[kDsV];
#pragma unroll
        for (int u = 0; u < kDsV; u++) sr[u] = cr[u] = si[u] = ci[u] = 0.f;
        for (int blk = 0; blk < 3; blk++) {
            // the block's sign per point: cout 0: Sxy odd/odd, Axz odd in x;
            // cout 1: Sxy odd/odd, Ayz odd in y; cout 2: -Axz^T, -Ayz^T even
            float sg[kDsV];
#pragma unroll
            for (int u = 0; u < kDsV; u++) {
                const int p = (v0 + u) / d.nrhs;
                const bool mx = (p / nky) == 1, my = (p % nky) == 1;
                bool flip = false;
                if (cout == 0) flip = blk == 1 ? mx != my : (blk == 2 ? mx : false);
                else if (cout == 1) flip = blk == 0 ? mx != my : (blk == 2 ? my : false);
                else flip = blk == 0 ? !mx : (blk == 1 ? !my : false);
                sg[u] = flip ? -1.f : 1.f;
                sr[u] *= sg[u], cr[u] *= sg[u], si[u] *= sg[u], ci[u] *= sg[u];
            }
            const double2 *gb = base[blk];
            const int kd = kind[blk];
            const float4 *X = sXd + (long)v0 * per + blk * nz;
            for (int j = 0; j < nz; j++) {
                const int idx = kd == 0 ? sym_index(i, j) : (kd == 1 ? i * lda + j : j * lda + i);
                const double2 g = __ldg(gb + idx);
                float grh, grl, gih, gil;
                ds_split(g.x, grh, grl);
                ds_split(g.y, gih, gil);
#pragma unroll
                for (int u = 0; u < kDsV; u++) {
                    if (u < cnt) {
                        const float4 x = X[(long)u * per + j];
                        ds_dot2(sr[u], cr[u], grh, grl, x.x, x.y);
                        ds_dot2(sr[u], cr[u], -gih, -gil, x.z, x.w);
                        ds_dot2(si[u], ci[u], grh, grl, x.z, x.w);
                        ds_dot2(si[u], ci[u], gih, gil, x.x, x.y);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kDsV; u++) sr[u] *= sg[u], cr[u] *= sg[u], si[u] *= sg[u], ci[u] *= sg[u];
        }
#pragma unroll
        for (int u = 0; u < kDsV; u++) {
            if (u < cnt) {
                const int v = v0 + u;
                const int p = v / d.nrhs, rhs = v - p * d.nrhs;
                const long pt = (long)kx[p / nky] * n1 + ky[p % nky];
                buf[pt * d.B + rhs * per + row] =
                    make_double2((double)sr[u] + (double)cr[u], (double)si[u] + (double)ci[u]);
            }
        }
    }
}

bool contract_ds_fits(int nz, int nrhs) {
    return 3 * nz <= 160 && (size_t)4 * nrhs * 3 * nz * sizeof(float4) <= 96 * 1024;
}

static int threads_for(int items) { return items >= 256 ? 256 : (items >= 128 ? 128 : 64); }

template <typename T>
static void set_smem(const void *fn, size_t bytes) {
    raise_smem_limit(fn, bytes);
}

template <typename T>
void operator_apply(const OpDims &d, const OperatorData<T> &op, const C<T> *G, const C<T> *x, C<T> *y, C<T> *buf,
                    const C<T> *tw0, const C<T> *tw1, const FftPlan &p0, const FftPlan &p1, cudaStream_t s,
                    long *launches, Timers *tm, int *err) {
    const int n0 = 2 * d.nx, n1 = 2 * d.ny;
    const int koff = sizeof(T) == sizeof(double) ? 0 : EGX_K_C64;
    int ev;
    // 1. r*x, forward factors, zero padding, DFT along y (rows i < nx)
    {
        ev = tm ? tm->begin(EGX_K_FWD_Y + koff, s) : -1;
        if (!run_reg<T>(n1, 0, d.nx, d.B, s, x, &op, buf, nullptr, &d, 0, 0, 0, 0, tw1, -1, d.fft_tile)) {
            int bt = fft_cols(n1, sizeof(C<T>));
            size_t sm = 2 * (size_t)n1 * bt * sizeof(C<T>);
            set_smem<T>((const void *)k_fwd_y<T>, sm);
            dim3 grid(d.nx, (d.B + bt - 1) / bt);
            k_fwd_y<T><<<grid, threads_for(n1 * bt / 2), sm, s>>>(x, op, buf, d, p1, tw1, bt);
        }
        if (tm) tm->end(ev, s);
    }
    // 2. DFT along x over all columns; rows >= nx are zero
    {
        ev = tm ? tm->begin(EGX_K_FWD_X + koff, s) : -1;
        if (!run_reg<T>(n0, 1, n1, d.B, s, nullptr, nullptr, buf, nullptr, nullptr, d.B, (long)n1 * d.B, d.nx, n0,
                        tw0, -1, d.fft_tile)) {
            int bt = fft_cols(n0, sizeof(C<T>));
            size_t sm = 2 * (size_t)n0 * bt * sizeof(C<T>);
            set_smem<T>((const void *)k_lines<T>, sm);
            dim3 grid(n1, (d.B + bt - 1) / bt);
            k_lines<T><<<grid, threads_for(n0 * bt / 2), sm, s>>>(buf, d.B, (long)n1 * d.B, d.B, d.nx, n0, p0, tw0,
                                                                  bt, -1);
        }
        if (tm) tm->end(ev, s);
    }
    // 3. block contraction
    {
        GreenDims gd{d.nx, d.ny, d.nz};
        size_t sx = (size_t)4 * d.nrhs * 3 * d.nz * sizeof(C<T>);
        size_t sg = (size_t)gd.Bs() * sizeof(C<T>);
        int thr = 256;
        ev = tm ? tm->begin(EGX_K_CONTRACT + koff, s) : -1;
        if (std::is_same<T, float>::value && sb_layout(d.nz)) {
            // the complex64 copy is in the sub-block layout for these nz
            EGX_CHECK(err, EGX_ERR_INVALID, "complex64 contraction needs the device error flag");
            long extra = 0;
            launch_contract_sb(reinterpret_cast<float2 *>(buf), reinterpret_cast<const float2 *>(G), d, err, s,
                               &extra);
            if (launches) *launches += extra - 1;
        } else if (std::is_same<T, float>::value && err && d.contract_variant == 0 && contract_mma_fits(d.nz, d.nrhs)) {
            launch_contract_mma(reinterpret_cast<float2 *>(buf), reinterpret_cast<const float2 *>(G), d, err, s);
        } else if (std::is_same<T, float>::value && err && d.contract_variant != 2 && contract_c64_fits(d.nz, d.nrhs)) {
            launch_contract_c64(reinterpret_cast<float2 *>(buf), reinterpret_cast<const float2 *>(G), d, err, s);
        } else if (std::is_same<T, double>::value && d.ds && contract_ds_fits(d.nz, d.nrhs)) {
            const int per = 3 * d.nz;
            const size_t sm = (size_t)4 * d.nrhs * per * sizeof(float4);
            set_smem<T>((const void *)k_contract_ds, sm);
            k_contract_ds<<<(unsigned)gd.Q(), (per + 31) / 32 * 32, sm, s>>>(reinterpret_cast<double2 *>(buf),
                                                                             reinterpret_cast<const double2 *>(G), d);
        } else if (sx + sg <= 200 * 1024) {
            set_smem<T>((const void *)k_contract<T, true>, sx + sg);
            k_contract<T, true><<<(unsigned)gd.Q(), thr, sx + sg, s>>>(buf, G, d);
        } else {
            set_smem<T>((const void *)k_contract<T, false>, sx);
            k_contract<T, false><<<(unsigned)gd.Q(), thr, sx, s>>>(buf, G, d);
        }
        if (tm) tm->end(ev, s);
    }
    // 4. inverse DFT along x; only rows < nx are needed afterwards
    {
        ev = tm ? tm->begin(EGX_K_BWD_X + koff, s) : -1;
        if (!run_reg<T>(n0, 1, n1, d.B, s, nullptr, nullptr, buf, nullptr, nullptr, d.B, (long)n1 * d.B, n0, d.nx,
                        tw0, +1, d.fft_tile)) {
            int bt = fft_cols(n0, sizeof(C<T>));
            size_t sm = 2 * (size_t)n0 * bt * sizeof(C<T>);
            set_smem<T>((const void *)k_lines<T>, sm);
            dim3 grid(n1, (d.B + bt - 1) / bt);
            k_lines<T><<<grid, threads_for(n0 * bt / 2), sm, s>>>(buf, d.B, (long)n1 * d.B, d.B, n0, d.nx, p0, tw0,
                                                                  bt, +1);
        }
        if (tm) tm->end(ev, s);
    }
    // 5. inverse DFT along y, extraction, last step
    {
        ev = tm ? tm->begin(EGX_K_BWD_Y + koff, s) : -1;
        if (!run_reg<T>(n1, 2, d.nx, d.B, s, x, &op, buf, y, &d, 0, 0, 0, 0, tw1, +1, d.fft_tile)) {
            int bt = fft_cols(n1, sizeof(C<T>));
            size_t sm = 2 * (size_t)n1 * bt * sizeof(C<T>);
            set_smem<T>((const void *)k_bwd_y<T>, sm);
            dim3 grid(d.nx, (d.B + bt - 1) / bt);
            k_bwd_y<T><<<grid, threads_for(n1 * bt / 2), sm, s>>>(buf, x, op, y, d, p1, tw1, bt);
        }
        if (tm) tm->end(ev, s);
    }
    EGX_CUDA(cudaGetLastError());
    if (launches) *launches += 5;
}

template <typename T>
void fft2d(C<T> *buf, int n0, int n1, int howmany, int sign, const C<T> *tw0, const C<T> *tw1, const FftPlan &p0,
           const FftPlan &p1, cudaStream_t s, long *launches) {
    if (!run_reg<T>(n1, 1, n0, howmany, s, nullptr, nullptr, buf, nullptr, nullptr, (long)n1 * howmany, howmany, n1,
                    n1, tw1, sign)) {
        int bt = fft_cols(n1, sizeof(C<T>));
        size_t sm = 2 * (size_t)n1 * bt * sizeof(C<T>);
        set_smem<T>((const void *)k_lines<T>, sm);
        dim3 grid(n0, (howmany + bt - 1) / bt);
        k_lines<T><<<grid, threads_for(n1 * bt / 2), sm, s>>>(buf, (long)n1 * howmany, howmany, howmany, n1, n1, p1,
                                                              tw1, bt, sign);
    }
    if (!run_reg<T>(n0, 1, n1, howmany, s, nullptr, nullptr, buf, nullptr, nullptr, howmany, (long)n1 * howmany, n0,
                    n0, tw0, sign)) {
        int bt = fft_cols(n0, sizeof(C<T>));
        size_t sm = 2 * (size_t)n0 * bt * sizeof(C<T>);
        set_smem<T>((const void *)k_lines<T>, sm);
        dim3 grid(n1, (howmany + bt - 1) / bt);
        k_lines<T><<<grid, threads_for(n0 * bt / 2), sm, s>>>(buf, howmany, (long)n1 * howmany, howmany, n0, n0, p0,
                                                              tw0, bt, sign);
    }
    EGX_CUDA(cudaGetLastError());
    if (launches) *launches += 2;
}

template <typename T>
void fft_lines(C<T> *buf, int nlines, long lstride, long estride, int B, int nload, int nstore, const FftPlan &p,
               const C<T> *tw, int sign, cudaStream_t s, long *launches) {
    if (run_reg<T>(p.n, 1, nlines, B, s, nullptr, nullptr, buf, nullptr, nullptr, lstride, estride, nload, nstore, tw,
                   sign)) {
        EGX_CUDA(cudaGetLastError());
        if (launches) *launches += 1;
        return;
    }
    int bt = fft_cols(p.n, sizeof(C<T>));
    size_t sm = 2 * (size_t)p.n * bt * sizeof(C<T>);
    set_smem<T>((const void *)k_lines<T>, sm);
    dim3 grid(nlines, (B + bt - 1) / bt);
    k_lines<T><<<grid, threads_for(p.n * bt / 2), sm, s>>>(buf, lstride, estride, B, nload, nstore, p, tw, bt, sign);
    EGX_CUDA(cudaGetLastError());
    if (launches) *launches += 1;
}

template <typename T, int N>
static void launch_sym(dim3 grid, cudaStream_t s, C<T> *buf, long lstride, long estride, int B, T par, int nstore,
                       const C<T> *tw, int sign) {
    reg_attr<T, N>((const void *)k_lines_sym_r<T, N>);
    k_lines_sym_r<T, N><<<grid, reg_threads<N, T>(), reg_smem<N, T>(), s>>>(buf, lstride, estride, B, par, nstore, tw,
                                                                            sign);
}

bool fft_lines_sym_ok(int n) { return reg_fft_ok(n); }

template <typename T>
void fft_lines_sym(C<T> *buf, int nlines, long lstride, long estride, int B, int parity, int nstore, int n,
                   const C<T> *tw, int sign, cudaStream_t s, long *launches) {
    EGX_CHECK(reg_fft_ok(n), EGX_ERR_INVALID, "mirrored FFT lines need a length in {64, 128, 256, 512}");
    dim3 grid(nlines, (B + RegCols<T>::BT - 1) / RegCols<T>::BT);
    const T par = (T)parity;
    switch (n) {
        case 64: launch_sym<T, 64>(grid, s, buf, lstride, estride, B, par, nstore, tw, sign); break;
        case 128: launch_sym<T, 128>(grid, s, buf, lstride, estride, B, par, nstore, tw, sign); break;
        case 256: launch_sym<T, 256>(grid, s, buf, lstride, estride, B, par, nstore, tw, sign); break;
        default: launch_sym<T, 512>(grid, s, buf, lstride, estride, B, par, nstore, tw, sign); break;
    }
    EGX_CUDA(cudaGetLastError());
    if (launches) *launches += 1;
}

template void fft_lines_sym<double>(C<double> *, int, long, long, int, int, int, int, const C<double> *, int,
                                    cudaStream_t, long *);
template void fft_lines_sym<float>(C<float> *, int, long, long, int, int, int, int, const C<float> *, int,
                                   cudaStream_t, long *);

template void fft_lines<double>(C<double> *, int, long, long, int, int, int, const FftPlan &, const C<double> *, int,
                                cudaStream_t, long *);
template void fft_lines<float>(C<float> *, int, long, long, int, int, int, const FftPlan &, const C<float> *, int,
                               cudaStream_t, long *);

std::vector<double> twiddles(int n) {
    std::vector<double> t(2 * (size_t)n);
    for (int m = 0; m < n; m++) {
        // reduce to the first octant for accuracy
        double ang = 2.0 * M_PI * (double)m / (double)n;
        t[2 * m] = cos(ang);
        t[2 * m + 1] = -sin(ang);
        if (4 * m == n) { t[2 * m] = 0.0; t[2 * m + 1] = -1.0; }
        if (2 * m == n) { t[2 * m] = -1.0; t[2 * m + 1] = 0.0; }
        if (4 * m == 3 * n) { t[2 * m] = 0.0; t[2 * m + 1] = 1.0; }
    }
    return t;
}

template void operator_apply<double>(const OpDims &, const OperatorData<double> &, const C<double> *,
                                     const C<double> *, C<double> *, C<double> *, const C<double> *,
                                     const C<double> *, const FftPlan &, const FftPlan &, cudaStream_t, long *,
                                     Timers *, int *);
template void operator_apply<float>(const OpDims &, const OperatorData<float> &, const C<float> *, const C<float> *,
                                    C<float> *, C<float> *, const C<float> *, const C<float> *, const FftPlan &,
                                    const FftPlan &, cudaStream_t, long *, Timers *, int *);
template void fft2d<double>(C<double> *, int, int, int, int, const C<double> *, const C<double> *, const FftPlan &,
                            const FftPlan &, cudaStream_t, long *);
template void fft2d<float>(C<float> *, int, int, int, int, const C<float> *, const C<float> *, const FftPlan &,
                           const FftPlan &, cudaStream_t, long *);

}  // namespace egx
