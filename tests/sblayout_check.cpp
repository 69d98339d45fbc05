// Host check of the complex64 Green copy's sub-block layout
// (extreme_gb300/csrc/egx_sblayout.cuh), built with the host compiler by
// tests/test_sblayout.py. For nz in {16, 32, 48} it prints one line:
//   nz <nz> entries <BS> errors <n> wavefronts <w> ideal <i>
// errors counts violations of: every stored index reached; the repack's
// inverse (sb_packed_source) naming the packed complex128 entry of the
// same (row, col), written here from the packed layout's definition; the
// FP16 kernels' pair rule (the neighbour of an entry in an even column at
// index ^ 1, or ^ 4 in a transposed sub-block). wavefronts counts the
// shared-memory wavefronts of those kernels' A-fragment loads over every
// 16 x 16 tile (two 8-byte loads per lane and entry, half-warps of 16
// lanes, 32 four-byte banks); ideal is the conflict-free count.
#include <cstdio>
#include <vector>

#include "egx_sblayout.cuh"

using namespace egx;

// packed quadrant: xx|xy|yy|zz as rc + tr(tr+1)/2 triangles of S0 entries,
// then xz|yz row-major with rows of nz + 1; zx, zy are the transposes
static int packed_index(int nz, int row, int col) {
    const int co = row / nz, i = row % nz, ci = col / nz, j = col % nz;
    const int S0 = nz * (nz + 1) / 2, lda = nz + 1, A0 = nz * lda;
    if ((co < 2 && ci < 2) || (co == 2 && ci == 2)) {
        const int c = (co == 2) ? 3 : ((co == 0 && ci == 0) ? 0 : ((co == 1 && ci == 1) ? 2 : 1));
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        return c * S0 + lo + hi * (hi + 1) / 2;
    }
    if (ci == 2) return 4 * S0 + co * A0 + i * lda + j;
    return 4 * S0 + ci * A0 + j * lda + i;
}

static int half_warp_wavefronts(const int *entry) {
    int worst = 0;
    for (int pair = 0; pair < 16; pair++) {  // an 8-byte entry covers banks 2p, 2p + 1
        int distinct[16], n = 0;
        for (int l = 0; l < 16; l++) {
            if ((entry[l] & 15) != pair) continue;
            bool seen = false;
            for (int k = 0; k < n; k++) seen |= distinct[k] == entry[l];
            if (!seen) distinct[n++] = entry[l];
        }
        if (n > worst) worst = n;
    }
    return worst;
}

static void check(int nz) {
    const int R = 3 * nz, BS = 4 * sb_sym(nz) + 2 * sb_asy(nz);
    std::vector<int> hit(BS, 0);
    long errors = 0;
    for (int r = 0; r < R; r++)
        for (int c = 0; c < R; c++) {
            const int d = sb_index(nz, r, c);
            if (d < 0 || d >= BS) {
                errors++;
                continue;
            }
            hit[d] = 1;
            if (sb_packed_source(nz, d) != packed_index(nz, r, c)) errors++;
            if ((c & 1) == 0) {
                const int x = d ^ sb_index(nz, r, c + 1);
                if (x != 1 && x != 4) errors++;
            }
        }
    for (int d = 0; d < BS; d++) errors += hit[d] ? 0 : 1;
    long wavefronts = 0, ideal = 0;
    for (int mt = 0; mt < R / 16; mt++)
        for (int kt = 0; kt < R / 16; kt++)
            for (int e = 0; e < 4; e++)
                for (int second = 0; second < 2; second++) {
                    int entry[32];
                    for (int lane = 0; lane < 32; lane++) {
                        const int g = lane >> 2, t = lane & 3;
                        const int r0 = 16 * mt + g + 8 * (e & 1), c0 = 16 * kt + 2 * t + 8 * (e >> 1);
                        const int off = sb_index(nz, r0, c0);
                        entry[lane] = second ? (off ^ (off ^ sb_index(nz, r0, c0 + 1))) : off;
                    }
                    wavefronts += half_warp_wavefronts(entry) + half_warp_wavefronts(entry + 16);
                    ideal += 2;
                }
    std::printf("nz %d entries %d errors %ld wavefronts %ld ideal %ld\n", nz, BS, errors, wavefronts, ideal);
}

int main() {
    check(16);
    check(32);
    check(48);
    return 0;
}
