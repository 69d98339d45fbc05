// Index maps of the complex64 Green copy's 4x4 sub-block layout (nz in
// {16, 32, 48}), shared by the repack, the contraction kernels and the host
// tests: plain inline functions, compiled for the host and the device.
//
// One stored spectral point holds, for nb = nz / 4:
//   xx | xy | yy | zz : the nb(nb+1)/2 upper-triangle 4x4 sub-blocks (I <= J)
//                       of each symmetric block, sub-block I + J(J+1)/2;
//   xz | yz           : all nb*nb sub-blocks, sub-block I*nb + J;
// entry (a, b) of sub-block (I, J) at 16 * sub-block + ((a*4 + b) ^ sb_swz(I, J)).
#pragma once

#if defined(__CUDACC__)
#define EGX_HD __host__ __device__
#else
#define EGX_HD
#endif

namespace egx {

EGX_HD inline int sb_sym(int nz) { return (nz / 4) * (nz / 4 + 1) / 2 * 16; }
EGX_HD inline int sb_asy(int nz) { return (nz / 4) * (nz / 4) * 16; }

// Entry (a, b) of the stored 4x4 sub-block (I, J) of a component block sits
// at a * 4 + b XOR sb_swz(I, J): a checkerboard over the sub-blocks that
// sends the FP16 kernels' A-fragment loads of two horizontally adjacent
// sub-blocks (read in place) to the even and the odd entries, and those of
// two vertically adjacent ones (read transposed) to entries 0-3, 8-11 and
// 4-7, 12-15 -- different banks, where the plain order put both on the
// same ones. The neighbour (a, b + 1) of an entry with b even is then at
// index ^ 1, the neighbour (a + 1, b) of one with a even at index ^ 4.
EGX_HD inline int sb_swz(int I, int J) { return (J & 1) | ((I & 1) << 2); }

// index in the sub-block layout of the entry G(row, col) of the 3nz x 3nz
// point operator, up to the sign of the -A^T blocks
EGX_HD inline int sb_index(int nz, int row, int col) {
    const int co = row / nz, i = row - co * nz, ci = col / nz, j = col - ci * nz;
    const int S = sb_sym(nz), A = sb_asy(nz), nb = nz / 4;
    if ((co < 2 && ci < 2) || (co == 2 && ci == 2)) {
        const int c = (co == 2) ? 3 : ((co == 0 && ci == 0) ? 0 : ((co == 1 && ci == 1) ? 2 : 1));
        int I = i >> 2, J = j >> 2, a = i & 3, b = j & 3;
        if (I > J) {
            int s = I;
            I = J;
            J = s;
            s = a;
            a = b;
            b = s;
        }
        return c * S + (I + J * (J + 1) / 2) * 16 + ((a * 4 + b) ^ sb_swz(I, J));
    }
    if (ci == 2)
        return 4 * S + co * A + ((i >> 2) * nb + (j >> 2)) * 16 + (((i & 3) * 4 + (j & 3)) ^ sb_swz(i >> 2, j >> 2));
    return 4 * S + ci * A + ((j >> 2) * nb + (i >> 2)) * 16 + (((j & 3) * 4 + (i & 3)) ^ sb_swz(j >> 2, i >> 2));
}

// the inverse for the repack: index d of the sub-block layout -> index of
// its entry in the packed complex128 quadrant (GreenDims: a packed triangle
// S0 per symmetric component, rows of xz and yz padded to nz + 1)
EGX_HD inline int sb_packed_source(int nz, int d) {
    const int S = sb_sym(nz), A = sb_asy(nz), nb = nz / 4;
    const int S0 = nz * (nz + 1) / 2, lda = nz + 1, A0 = nz * lda;
    if (d < 4 * S) {
        const int c = d / S, r = d - c * S, sbi = r >> 4;
        int J = 0;
        while ((J + 1) * (J + 2) / 2 <= sbi) J++;
        const int I = sbi - J * (J + 1) / 2, e = (r & 15) ^ sb_swz(I, J);
        const int i = 4 * I + (e >> 2), j = 4 * J + (e & 3);
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        return c * S0 + lo + hi * (hi + 1) / 2;
    }
    const int d2 = d - 4 * S, co = d2 / A, r = d2 - co * A, sbi = r >> 4;
    const int I = sbi / nb, J = sbi - I * nb, e = (r & 15) ^ sb_swz(I, J);
    return 4 * S0 + co * A0 + (4 * I + (e >> 2)) * lda + 4 * J + (e & 3);
}

}  // namespace egx
