// The CIE convolution operator on the device
// (Extreme.Cartesian/Forward/AtoA/ConvolutionOperator.cs:45-327).
#pragma once

#include "egx_fft.cuh"

namespace egx {

// Device-side spectral Green tensor: only the (nx+1) x (ny+1) quadrant of
// spectral points is stored; the other three quadrants follow from the
// parity of each component in real space (GreenTensorFftPopulator.cs:170-185):
// xx, yy, zz even/even, xy odd/odd, xz odd in x, yz odd in y.
// Per point, one contiguous block of Bs entries:
//   xx | xy | yy | zz  (packed rc + tr*(tr+1)/2, S = nz(nz+1)/2 each)
//   xz | yz            (rc*(nz+1) + tr, A = nz*(nz+1) each: rows padded by one
//                       entry so that reading a row or a column with one lane
//                       per index is free of shared-memory bank conflicts)
struct GreenDims {
    int nx, ny, nz;
    int S() const { return nz * (nz + 1) / 2; }
    int lda() const { return nz + 1; }
    int A() const { return nz * (nz + 1); }
    int Bs() const { return 4 * S() + 2 * A(); }
    long Q() const { return (long)(nx + 1) * (ny + 1); }
};

struct OpDims {
    int nx, ny, nz, nrhs;
    int B;       // batch of the spectral buffer: nrhs * 3 * nz
    long nvec;   // elements of one anomaly vector: nx*ny*3*nz
    int ds = 0;  // complex128 apply: contraction in double-FP32 arithmetic
    // kernel variants chosen by the apply tuner (egx_tune_apply): FFT
    // column tile of the register passes (0 the built-in choice per pass,
    // 1 64-byte tiles, 2 128-byte tiles) and the complex64 contraction of
    // the packed Green layout (0 the built-in order, 1 the TMA-staged
    // CUDA-core kernel, 2 the generic kernel)
    int fft_tile = 0;
    int contract_variant = 0;
};

template <typename T>
struct OperatorData {
    const C<T> *r;    // [nx*ny*nz]
    const C<T> *fwd;  // [nz]
    const C<T> *bwd;  // [nz]
    int type;         // EGX_OP_A / EGX_OP_CHI0
};

// Launch the full apply y = K x (nrhs vectors) on `stream`.
template <typename T>
void operator_apply(const OpDims &d, const OperatorData<T> &op, const C<T> *G, const C<T> *x, C<T> *y, C<T> *buf,
                    const C<T> *tw0, const C<T> *tw1, const FftPlan &p0, const FftPlan &p1, cudaStream_t s,
                    long *launches, Timers *timers = nullptr, int *err = nullptr);

// the double-FP32 complex128 contraction covers 3 nz <= 160 and its staged
// vectors fit in 96 KiB
bool contract_ds_fits(int nz, int nrhs);

// complex64 contraction with TMA-staged blocks (egx_contract.cu); `err`
// receives EGX_ERR_TIMEOUT if a bounded wait expires.
bool contract_c64_fits(int nz, int nrhs);
size_t contract_c64_smem(int nz, int nrhs);
void launch_contract_c64(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s);
// complex64 Green copy and contraction in the 4x4 sub-block layout
// (egx_contract_sb.cu), used for every complex64 apply when sb_layout(nz);
// other nz keep the packed layout of GreenDims.
bool sb_layout(int nz);
long sb_block(int nz);                      // complex entries per stored point
long green_c64_entries(const GreenDims &gd);  // size of the complex64 copy
void green_to_c64(const double2 *g64, float2 *g32, const GreenDims &gd, cudaStream_t s, long *launches);
void launch_contract_sb(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s, long *launches);
// complex64 contraction on the tensor cores (egx_contract_mma.cu)
bool contract_mma_fits(int nz, int nrhs);
size_t contract_mma_smem(int nz, int nrhs);
void launch_contract_mma(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s);

// DFTs of `nlines` interleaved sequences: element e of line L, column b at
// L*lstride + e*estride + b (b < B); elements e >= nload read as zero and
// only e < nstore are written back.
template <typename T>
void fft_lines(C<T> *buf, int nlines, long lstride, long estride, int B, int nload, int nstore, const FftPlan &p,
               const C<T> *tw, int sign, cudaStream_t s, long *launches);

// DFTs of length n of lines stored by their first half: element e is
// v[e] for e < n/2, 0 at n/2 and parity * v[n - e] beyond (a real-space
// Green component and its mirror image); outputs e < nstore are written back
// in place. Lengths with a register plan only (fft_lines_sym_ok).
bool fft_lines_sym_ok(int n);
template <typename T>
void fft_lines_sym(C<T> *buf, int nlines, long lstride, long estride, int B, int parity, int nstore, int n,
                   const C<T> *tw, int sign, cudaStream_t s, long *launches);

// In-place batched 2-D DFT (egx_fft2d).
template <typename T>
void fft2d(C<T> *buf, int n0, int n1, int howmany, int sign, const C<T> *tw0, const C<T> *tw1, const FftPlan &p0,
           const FftPlan &p1, cudaStream_t s, long *launches);

}  // namespace egx
