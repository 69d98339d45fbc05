// Block contraction of the CIE operator in complex64 on the tensor cores
// (ConvolutionOperator.ApplyGreenTensorAlongZ, ConvolutionOperator.cs:274-327)
// for nz in {16, 32, 48}, one or two right-hand sides per pass, reading the
// mixed form's Green copy in a 4x4 sub-block layout.
//
// Sub-block layout of one stored spectral point (nb = nz/4):
//   xx | xy | yy | zz : the nb(nb+1)/2 upper-triangle 4x4 sub-blocks (I <= J)
//                       of the symmetric block, sub-block I + J(J+1)/2,
//                       element (i%4)*4 + (j%4) ^ sb_swz(I, J); diagonal
//                       sub-blocks whole;
//   xz | yz           : all nb*nb sub-blocks, sub-block I*nb + J, element
//                       (rc%4)*4 + (tr%4) ^ sb_swz(I, J).
// A TF32 fragment load of a half-warp (4 rows x 4 columns of G, either
// orientation) falls in one 128-byte sub-block; the FP16 kernels' loads of
// entry pairs span two adjacent sub-blocks, which the sb_swz checkerboard
// sends to different banks: both conflict-free.
//
// Each 8-byte entry holds the Green value scaled by one power of two for
// the whole tensor and split into FP16 high parts and remainders of Re and
// Im (split_entry: 22 significant bits, the precision of a TF32 split); the
// trailing entry of the copy holds the largest magnitude and 1/scale.
//
// Algebra: the four spectral points sharing a stored block are right-hand
// sides of one (3nz x 3nz) complex matrix after D_p sign flips; each product
// of split operands takes three MMAs (hi.hi + hi.lo + lo.hi), which keeps
// complex64 accuracy.
//
// Four kernels, one CTA per SM looping over stored points, the offsets of
// each warp's A fragments held in registers (built once). The -A^T blocks
// (z rows, x|y columns) take their sign on the B values.
//  * k_contract_ws<NZ> (two right-hand sides, the stacked solve of both
//    polarisations; built in): FP16 m16n8k16 with A fragments straight from
//    the split entries, work split by role -- one warp per 16-row tile over
//    all column tiles, two warps splitting the next point's right-hand
//    sides, one producer lane (see the kernel).
//  * k_contract_sh<NZ> (two; the tuner's variant 2): the same products with
//    12 warps in lockstep, 3 row groups x 4 column groups, partial sums per
//    row tile met in shared memory and added by the warps with the fewest
//    column tiles.
//  * k_contract_sb3<NZ> (two; variant 1) on the TF32 m16n8k8 path, the
//    entries recombined to complex64 first, and k_contract_sb<NZ, 1> for one
//    right-hand side.
//
// Per stored point: one TMA bulk copy of the block (and, in the lockstep
// and TF32 kernels, one per present right-hand-side segment) into one of
// two stages, issued two points ahead and completing on the stage's
// mbarrier (waits bounded to 2 s; on expiry EGX_ERR_TIMEOUT is recorded in
// *err and the kernel returns).
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "egx_krylov.cuh"
#include "egx_operator.cuh"
#include "egx_wait.cuh"
#include "egx_sblayout.cuh"

namespace egx {

namespace {

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    return mbar_wait_ns(bar, parity, limit_ns);
}

__device__ __forceinline__ void bar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ float2 lds64(uint32_t a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}

__device__ __forceinline__ void sts128(uint32_t a, uint4 v) {
    asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}

// TF32 high part rounded to nearest (ties away from zero) on the magnitude
__device__ __forceinline__ uint32_t tf32_hi(uint32_t bits) { return (bits + 0x1000u) & 0xffffe000u; }

// a = hi + lo, hi TF32; the tensor core reads the top 19 bits of lo
__device__ __forceinline__ void split(float a, uint32_t &hi, uint32_t &lo) {
    hi = tf32_hi(__float_as_uint(a));
    lo = __float_as_uint(a - __uint_as_float(hi));
}

// both parts rounded (right-hand sides: split once per point)
__device__ __forceinline__ void split_rn(float a, uint32_t &hi, uint32_t &lo) {
    hi = tf32_hi(__float_as_uint(a));
    lo = tf32_hi(__float_as_uint(a - __uint_as_float(hi)));
}

// 2^(top - e) with 2^(e-1) <= m < 2^e for a normal m > 0, the exponent
// read from the bit pattern; 1 for zero, subnormal or non-finite m
__host__ __device__ inline float pow2_scale(float m, int top) {
    uint32_t u;
    memcpy(&u, &m, 4);
    const int ef = (int)((u >> 23) & 0xffu);
    if (ef == 0 || ef == 255) return 1.f;
    int k = top - (ef - 126);
    k = k > 127 ? 127 : (k < -126 ? -126 : k);
    const uint32_t r = (uint32_t)(127 + k) << 23;
    float f;
    memcpy(&f, &r, 4);
    return f;
}

// One entry of the split Green copy: the scaled Re and Im as FP16 high
// parts (rounded to 11 significant bits) and FP16 remainders,
// x = Re hi | Im hi << 16, y = Re lo | Im lo << 16; hi + lo keeps 22 bits.
__device__ __forceinline__ uint2 split_entry(float re, float im) {
    const float rh = __uint_as_float(tf32_hi(__float_as_uint(re)));
    const float ih = __uint_as_float(tf32_hi(__float_as_uint(im)));
    const __half2 h = __floats2half2_rn(rh, ih), l = __floats2half2_rn(re - rh, im - ih);
    return make_uint2(*reinterpret_cast<const uint32_t *>(&h), *reinterpret_cast<const uint32_t *>(&l));
}

// the complex64 value of a split entry (inv undoes the copy's scale)
__device__ __forceinline__ float2 unsplit_entry(uint2 u, float inv) {
    const float2 h = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
    const float2 l = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
    return make_float2((h.x + l.x) * inv, (h.y + l.y) * inv);
}

__device__ __forceinline__ void mma_tf32(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr uint64_t kWait = 2000000000ull;

// complex128 packed quadrant (GreenDims layout) -> the split sub-block copy.
// Two passes over the same index map: the first (WRITE false) takes the
// largest |Re|, |Im| into tail[0] (as its bit pattern, which orders like the
// value for non-negative floats; zeroed by the caller); the second scales by
// s = 2^(14 - e), 2^e above that largest magnitude (so |Re| + |Im| < 2^15
// fits FP16), writes the split entries and 1/s into tail[1]. tail is the
// copy's trailing entry, g32[Q BS].
template <bool WRITE>
__global__ void k_repack_sb(const double2 *__restrict__ g64, uint2 *__restrict__ g32, long Q, int nz) {
    const int S = sb_sym(nz), A = sb_asy(nz), BS = 4 * S + 2 * A;
    // packed layout (GreenDims): S0 per symmetric block, rows of xz/yz padded to nz + 1
    const int S0 = nz * (nz + 1) / 2, lda = nz + 1, A0 = nz * lda, BS0 = 4 * S0 + 2 * A0;
    const long total = Q * BS;
    uint32_t *tail = reinterpret_cast<uint32_t *>(g32 + total);
    float scale = 1.f;
    if (WRITE) {
        scale = pow2_scale(__uint_as_float(tail[0]), 14);
        if (blockIdx.x == 0 && threadIdx.x == 0) tail[1] = __float_as_uint(1.f / scale);
    }
    float vmax = 0.f;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const long q = idx / BS;
        const int d = (int)(idx - q * BS);
        const double2 v = g64[q * BS0 + sb_packed_source(nz, d)];
        if (WRITE)
            g32[idx] = split_entry((float)(v.x * scale), (float)(v.y * scale));
        else
            vmax = fmaxf(vmax, fmaxf(fabsf((float)v.x), fabsf((float)v.y)));
    }
    if (!WRITE) {
        const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(vmax));
        if ((threadIdx.x & 31) == 0 && m) atomicMax(tail, m);
    }
}

template <int NZ, int NRHS>
struct Sb {
    static constexpr int R = 3 * NZ, MT = R / 16, KT = R / 8, NB = NZ / 4;
    static constexpr int SYM = NB * (NB + 1) / 2 * 16, ASY = NB * NB * 16, BS = 4 * SYM + 2 * ASY;
    // 3 row groups x 4 column groups: 12 warps, 3 per SM sub-partition;
    // column group kg owns column tiles [kt0(kg), kt0(kg + 1))
    static constexpr int MG = 3, KG = 4, MPW = MT / MG, KMAX = (KT + KG - 1) / KG;
    static constexpr int THREADS = 32 * MG * KG;
    static constexpr int XB = NRHS * R;  // complex per spectral point and pass
    static constexpr uint32_t G_BYTES = BS * 8u;
    static constexpr uint32_t X_BYTES = 4u * XB * 8u;
    static constexpr uint32_t BF_BYTES = KT * NRHS * 2u * 32u * 16u;
    static constexpr uint32_t PART_BYTES = KG * MT * 4u * NRHS * 32u * 4u;
    // partial sums get their own region when it fits, else they reuse the
    // B fragments (one more barrier per point)
    static constexpr bool PART_ALIAS = 2 * G_BYTES + 2 * X_BYTES + BF_BYTES + PART_BYTES > 227u * 1024u;
    static constexpr uint32_t OFF_X = 2 * G_BYTES, OFF_BF = OFF_X + 2 * X_BYTES;
    static constexpr uint32_t OFF_PART = PART_ALIAS ? OFF_BF : OFF_BF + BF_BYTES;
    static constexpr uint32_t SMEM = PART_ALIAS ? OFF_BF + BF_BYTES : OFF_PART + PART_BYTES;
    static_assert(MT % MG == 0, "row tiles must split over the row groups");
    static_assert(!PART_ALIAS || PART_BYTES <= BF_BYTES, "partials must fit in the B-fragment region");
    static_assert(MT <= MG * KG, "one warp per row tile in the epilogue");
    static_assert(G_BYTES % 128 == 0 && X_BYTES % 128 == 0, "stage alignment");
    __host__ __device__ static constexpr int kt0(int kg) { return kg * KT / KG; }
};

template <int NZ, int NRHS>
__global__ void __launch_bounds__(Sb<NZ, NRHS>::THREADS, 1)
    k_contract_sb(float2 *buf, const float2 *__restrict__ G, const int nx, const int ny, const int B, const int rhs0,
                  int *err) {
    using P = Sb<NZ, NRHS>;
    constexpr int R = P::R, MPW = P::MPW, KMAX = P::KMAX;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int status;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int mg = warp % P::MG, kg = warp / P::MG;
    const int ktb = P::kt0(kg), kcnt = P::kt0(kg + 1) - ktb;
    const uint32_t sG = saddr(smem), sX = sG + P::OFF_X, sBF = sG + P::OFF_BF;
    const uint32_t bar0 = saddr(&bars[0]);
    const long Q = (long)(nx + 1) * (ny + 1);
    const int n1 = 2 * ny;
    // 1 / the split copy's scale, in its trailing entry
    const float ginv = __uint_as_float(reinterpret_cast<const uint2 *>(G)[Q * P::BS].y);

    // offsets (complex units) of this lane's A-fragment entries: pair
    // (row tile mg*MPW + im, column tile ktb + ik), entries e = 0..3, two
    // 16-bit offsets per word; computed through the (still unused) stage-0
    // block buffer and then held in registers
    constexpr int TABN = MPW * KMAX * 2;
    static_assert(P::MG * P::KG * TABN * 32 * 4 <= P::G_BYTES, "offset scratch must fit in one stage");
    uint32_t tab[TABN];
    {
        uint32_t *scratch = reinterpret_cast<uint32_t *>(smem) + (size_t)warp * TABN * 32 + lane;
#pragma unroll 1
        for (int p = 0; p < MPW * KMAX; p++) {
            const int im = p / KMAX, ik = p - im * KMAX;
            uint32_t w0 = 0, w1 = 0;
            if (ik < kcnt) {
                const int r0 = 16 * (mg * MPW + im) + g, c0 = 8 * (ktb + ik) + t;
                w0 = (uint32_t)sb_index(NZ, r0, c0) | ((uint32_t)sb_index(NZ, r0 + 8, c0) << 16);
                w1 = (uint32_t)sb_index(NZ, r0, c0 + 4) | ((uint32_t)sb_index(NZ, r0 + 8, c0 + 4) << 16);
            }
            scratch[(2 * p) * 32] = w0;
            scratch[(2 * p + 1) * 32] = w1;
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < TABN; j++) tab[j] = scratch[j * 32];
    }

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        status = 0;
    }
    __syncthreads();

    auto issue = [&](long qq, int stage) {
        const int a = (int)(qq / (ny + 1)), bq = (int)(qq - (long)a * (ny + 1));
        const int nkx = (a == 0 || a == nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == ny) ? 1 : 2;
        const uint32_t bar = bar0 + 8 * stage;
        bar_expect(bar, P::G_BYTES + (uint32_t)(nkx * nky) * (P::XB * 8u));
        bulk_g2s(sG + stage * P::G_BYTES, G + qq * P::BS, P::G_BYTES, bar);
        for (int p = 0; p < 4; p++) {
            const int mx = p >> 1, my = p & 1;
            if (mx < nkx && my < nky) {
                const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
                bulk_g2s(sX + stage * P::X_BYTES + p * (P::XB * 8u), buf + pt * B + (long)rhs0 * R, P::XB * 8u, bar);
            }
        }
    };
    long q = blockIdx.x;
    if (tid == 0) {
        if (q < Q) issue(q, 0);
        if (q + gridDim.x < Q) issue(q + gridDim.x, 1);
    }

    for (int it = 0; q < Q; q += gridDim.x, it++) {
        const int stage = it & 1;
        const uint32_t parity = (it >> 1) & 1;
        const uint32_t bar = bar0 + 8 * stage;
        if (tid == 0 && !bar_wait(bar, parity, kWait)) status = 1;
        __syncthreads();
        if (status) {
            if (tid == 0) {
                atomicExch(err, EGX_ERR_TIMEOUT);
                bar_wait(bar0 + 8 * (stage ^ 1), ((it + 1) >> 1) & 1, kWait);
            }
            return;
        }
        bar_wait(bar, parity, kWait);  // acquire the stage for every thread
        const int a = (int)(q / (ny + 1)), bq = (int)(q - (long)a * (ny + 1));
        const int nkx = (a == 0 || a == nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == ny) ? 1 : 2;

        // B fragments, split once: entry (kt, rhs, part, lane), part 0 = [Xr | Xi], 1 = [-Xi | Xr]
        const uint32_t sXq = sX + stage * P::X_BYTES;
        for (int e = tid; e < P::KT * NRHS * 32; e += P::THREADS) {
            const int ln = e & 31, rest = e >> 5, r = rest % NRHS, kt = rest / NRHS;
            const int gg = ln >> 2, tt = ln & 3;
            const int v = gg & 3, mx = v >> 1, my = v & 1;
            const bool im = gg >= 4, present = mx < nkx && my < nky;
            uint32_t w[8];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int k = 8 * kt + tt + 4 * h;
                float2 x = make_float2(0.f, 0.f);
                if (present) {
                    x = lds64(sXq + (uint32_t)(v * P::XB + r * R + k) * 8u);
                    const int comp = k / NZ;
                    if ((comp == 0 && mx) || (comp == 1 && my)) x = make_float2(-x.x, -x.y);
                }
                split_rn(im ? x.y : x.x, w[h], w[2 + h]);
                split_rn(im ? x.x : -x.y, w[4 + h], w[6 + h]);
            }
            const uint32_t base = sBF + (uint32_t)((kt * NRHS + r) * 2) * 512u + ln * 16u;
            sts128(base, make_uint4(w[0], w[1], w[2], w[3]));
            sts128(base + 512u, make_uint4(w[4], w[5], w[6], w[7]));
        }
        __syncthreads();

        float acc[MPW][NRHS][4];
#pragma unroll
        for (int im = 0; im < MPW; im++)
#pragma unroll
            for (int r = 0; r < NRHS; r++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[im][r][c] = 0.f;
        // plain shared-memory reads: the compiler may schedule them freely
        // between the barriers that order them against the stage's TMA and
        // the B-fragment pass
        const uint2 *Gq = reinterpret_cast<const uint2 *>(smem + stage * P::G_BYTES);
        const uint4 *BFq = reinterpret_cast<const uint4 *>(smem + P::OFF_BF) + lane;
#pragma unroll
        for (int ik = 0; ik < KMAX; ik++) {
            if (ik >= kcnt) break;
            const int kt = ktb + ik;
            // the -A^T tiles: z rows (row group 2) x x|y columns
            const uint32_t bsign = (mg == 2 && kt < 2 * NZ / 8) ? 0x80000000u : 0u;
            uint4 b1[NRHS], b2[NRHS];
#pragma unroll
            for (int r = 0; r < NRHS; r++) {
                b1[r] = BFq[((kt * NRHS + r) * 2) * 32];
                b2[r] = BFq[((kt * NRHS + r) * 2 + 1) * 32];
                b1[r].x ^= bsign;
                b1[r].y ^= bsign;
                b1[r].z ^= bsign;
                b1[r].w ^= bsign;
                b2[r].x ^= bsign;
                b2[r].y ^= bsign;
                b2[r].z ^= bsign;
                b2[r].w ^= bsign;
            }
            // A fragments of all row tiles of this column tile: [im][re hi, re lo, im hi, im lo][e]
            uint32_t af[MPW][4][4];
#pragma unroll
            for (int im = 0; im < MPW; im++) {
                const uint32_t t0 = tab[(im * KMAX + ik) * 2], t1 = tab[(im * KMAX + ik) * 2 + 1];
                const uint32_t off[4] = {t0 & 0xffffu, t0 >> 16, t1 & 0xffffu, t1 >> 16};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float2 gv = unsplit_entry(Gq[off[e]], ginv);
                    split(gv.x, af[im][0][e], af[im][1][e]);
                    split(gv.y, af[im][2][e], af[im][3][e]);
                }
            }
            // six products per right-hand side; consecutive MMAs go to
            // different row tiles, so their accumulator chains overlap
#pragma unroll
            for (int r = 0; r < NRHS; r++) {
#pragma unroll
                for (int im = 0; im < MPW; im++) mma_tf32(acc[im][r], af[im][0], b1[r].x, b1[r].y);
#pragma unroll
                for (int im = 0; im < MPW; im++) mma_tf32(acc[im][r], af[im][2], b2[r].x, b2[r].y);
#pragma unroll
                for (int im = 0; im < MPW; im++) mma_tf32(acc[im][r], af[im][0], b1[r].z, b1[r].w);
#pragma unroll
                for (int im = 0; im < MPW; im++) mma_tf32(acc[im][r], af[im][2], b2[r].z, b2[r].w);
#pragma unroll
                for (int im = 0; im < MPW; im++) mma_tf32(acc[im][r], af[im][1], b1[r].x, b1[r].y);
#pragma unroll
                for (int im = 0; im < MPW; im++) mma_tf32(acc[im][r], af[im][3], b2[r].x, b2[r].y);
            }
        }
        // partial sums [kg][mt][r][c][lane]; when they reuse the B-fragment
        // region every warp must be done with its fragments first
        float *PART = reinterpret_cast<float *>(smem + P::OFF_PART) + lane;
        if (P::PART_ALIAS) __syncthreads();
#pragma unroll
        for (int im = 0; im < MPW; im++)
#pragma unroll
            for (int r = 0; r < NRHS; r++)
#pragma unroll
                for (int c = 0; c < 4; c++)
                    PART[(((kg * P::MT + mg * MPW + im) * NRHS + r) * 4 + c) * 32] = acc[im][r][c];
        __syncthreads();  // the stage is free; all partials are written
        if (tid == 0 && q + 2L * gridDim.x < Q) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q + 2L * gridDim.x, stage);
        }
        // warp w < MT adds the column groups' partials of row tile w and stores
        if (warp < P::MT) {
            const int mt = warp;
            {
#pragma unroll
                for (int r = 0; r < NRHS; r++) {
                    float y[4];
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        float s = 0.f;
#pragma unroll
                        for (int k = 0; k < P::KG; k++) s += PART[(((k * P::MT + mt) * NRHS + r) * 4 + c) * 32];
                        y[c] = s;
                    }
                    // C: rows g, g+8; columns 2t, 2t+1 (t < 2: Re of v = 2t, 2t+1; t >= 2: Im of v = 2t-4, 2t-3)
                    float o[4];
#pragma unroll
                    for (int c = 0; c < 4; c++) o[c] = __shfl_xor_sync(0xffffffffu, y[c], 2);
                    if (t < 2) {
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const int row = 16 * mt + g + 8 * (c >> 1);
                            const int v = 2 * t + (c & 1);
                            const int mx = v >> 1, my = v & 1;
                            if (mx < nkx && my < nky) {
                                float2 val = make_float2(y[c], o[c]);
                                const int comp = row / NZ;
                                if ((comp == 0 && mx) || (comp == 1 && my)) val = make_float2(-val.x, -val.y);
                                const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
                                buf[pt * B + (long)(rhs0 + r) * R + row] = val;
                            }
                        }
                    }
                }
            }
        }
    }
}

// Two right-hand sides with three real products per complex product
// (Gauss): T1 = Gr Xr, T2 = Gi Xi, T3 = (Gr + Gi)(Xr + Xi), Yr = T1 - T2,
// Yi = T3 - T1 - T2. The eight columns of one n8 tile are the four points
// sharing the stored block times the two right-hand sides (column 4 rhs + v),
// so a (row tile, column tile) pair takes 3 products x 3 TF32 passes = 9 MMAs
// where the embedded form takes 12.
//
// Each lane reads the two B values of its column straight from the staged
// right-hand sides and splits them in registers (no separate B-fragment pass
// and barrier). The eight (point, source) segments of a stage are copied
// 32 bytes apart modulo 128, so one fragment load of a warp takes the
// minimum two shared-memory wavefronts. Two block barriers per point: before
// the partial sums are written (the previous reduction has read them) and
// after (with the stage-wait status); then the stage is refilled and warps
// w < MT reduce and store.
template <int NZ>
struct Sb3 {
    static constexpr int R = 3 * NZ, MT = R / 16, KT = R / 8, NB = NZ / 4;
    static constexpr int SYM = NB * (NB + 1) / 2 * 16, ASY = NB * NB * 16, BS = 4 * SYM + 2 * ASY;
    static constexpr int MG = 3, KG = 4, MPW = MT / MG, KMAX = (KT + KG - 1) / KG;
    static constexpr int THREADS = 32 * MG * KG;
    static constexpr uint32_t SEG = R * 8u;        // bytes of one (point, source) segment
    static constexpr uint32_t XS = SEG + 32u;      // its stride in a stage
    static constexpr uint32_t G_BYTES = BS * 8u;
    static constexpr uint32_t X_BYTES = 8u * XS;   // 4 points x 2 sources
    static constexpr uint32_t PART_BYTES = KG * MT * 2u * 4u * 32u * 4u;
    static constexpr uint32_t OFF_X = 2 * G_BYTES, OFF_PART = OFF_X + 2 * X_BYTES;
    static constexpr uint32_t SMEM = OFF_PART + PART_BYTES;
    static_assert(MT % MG == 0, "row tiles must split over the row groups");
    static_assert(SMEM + 256 <= 227u * 1024u, "shared memory per block");
    static_assert(MT <= MG * KG, "one warp per row tile in the epilogue");
    static_assert(G_BYTES % 128 == 0 && SEG % 16 == 0 && XS % 128 == 32, "stage alignment and bank skew");
    __host__ __device__ static constexpr int kt0(int kg) { return kg * KT / KG; }
};

template <int NZ, bool BAL>
__global__ void __launch_bounds__(Sb3<NZ>::THREADS, 1)
    k_contract_sb3(float2 *buf, const float2 *__restrict__ G, const int nx, const int ny, const int B, const int rhs0,
                   int *err) {
    using P = Sb3<NZ>;
    constexpr int R = P::R, MPW = P::MPW, KMAX = P::KMAX;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int mg = warp % P::MG, kg = warp / P::MG;
    const int ktb = P::kt0(kg), kcnt = P::kt0(kg + 1) - ktb;
    // warps of the column groups with the fewest column tiles, numbered
    // 0 .. nlight-1 (light = -1 for the others)
    int light = -1, nlight = 0;
    {
        int mincnt = P::KT;
        for (int k = 0; k < P::KG; k++) mincnt = min(mincnt, P::kt0(k + 1) - P::kt0(k));
        for (int w = 0; w < P::MG * P::KG; w++) {
            const int wk = w / P::MG;
            if (P::kt0(wk + 1) - P::kt0(wk) == mincnt) {
                if (w == warp) light = nlight;
                nlight++;
            }
        }
    }
    const uint32_t sG = saddr(smem), sX = sG + P::OFF_X;
    const uint32_t bar0 = saddr(&bars[0]);
    const long Q = (long)(nx + 1) * (ny + 1);
    const int n1 = 2 * ny;
    // 1 / the split copy's scale, in its trailing entry
    const float ginv = __uint_as_float(reinterpret_cast<const uint2 *>(G)[Q * P::BS].y);
    // this lane's B column: point v, source rb
    const int bv = g & 3, brs = g >> 2, bmx = bv >> 1, bmy = bv & 1;

    // A-fragment offsets in registers, built through the stage-0 block buffer
    constexpr int TABN = MPW * KMAX * 2;
    static_assert(P::MG * P::KG * TABN * 32 * 4 <= P::G_BYTES, "offset scratch must fit in one stage");
    uint32_t tab[TABN];
    {
        uint32_t *scratch = reinterpret_cast<uint32_t *>(smem) + (size_t)warp * TABN * 32 + lane;
#pragma unroll 1
        for (int p = 0; p < MPW * KMAX; p++) {
            const int im = p / KMAX, ik = p - im * KMAX;
            uint32_t w0 = 0, w1 = 0;
            if (ik < kcnt) {
                const int r0 = 16 * (mg * MPW + im) + g, c0 = 8 * (ktb + ik) + t;
                w0 = (uint32_t)sb_index(NZ, r0, c0) | ((uint32_t)sb_index(NZ, r0 + 8, c0) << 16);
                w1 = (uint32_t)sb_index(NZ, r0, c0 + 4) | ((uint32_t)sb_index(NZ, r0 + 8, c0 + 4) << 16);
            }
            scratch[(2 * p) * 32] = w0;
            scratch[(2 * p + 1) * 32] = w1;
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < TABN; j++) tab[j] = scratch[j * 32];
    }

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](long qq, int stage) {
        const int a = (int)(qq / (ny + 1)), bq = (int)(qq - (long)a * (ny + 1));
        const int nkx = (a == 0 || a == nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == ny) ? 1 : 2;
        const uint32_t bar = bar0 + 8 * stage;
        bar_expect(bar, P::G_BYTES + (uint32_t)(nkx * nky) * (2u * P::SEG));
        bulk_g2s(sG + stage * P::G_BYTES, G + qq * P::BS, P::G_BYTES, bar);
        for (int p = 0; p < 4; p++) {
            const int mx = p >> 1, my = p & 1;
            if (mx < nkx && my < nky) {
                const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
#pragma unroll
                for (int r = 0; r < 2; r++)
                    bulk_g2s(sX + stage * P::X_BYTES + (uint32_t)(p * 2 + r) * P::XS, buf + pt * B + (long)(rhs0 + r) * R,
                             P::SEG, bar);
            }
        }
    };
    long q = blockIdx.x;
    if (tid == 0) {
        if (q < Q) issue(q, 0);
        if (q + gridDim.x < Q) issue(q + gridDim.x, 1);
    }

    float *PART = reinterpret_cast<float *>(smem + P::OFF_PART) + lane;
    for (int it = 0; q < Q; q += gridDim.x, it++) {
        const int stage = it & 1;
        const uint32_t parity = (it >> 1) & 1;
        const uint32_t bar = bar0 + 8 * stage;
        // every thread acquires the stage itself (bounded); the barrier after
        // the partial sums shares the outcome
        const bool late = !bar_wait(bar, parity, kWait);
        const int a = (int)(q / (ny + 1)), bq = (int)(q - (long)a * (ny + 1));
        const int nkx = (a == 0 || a == nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == ny) ? 1 : 2;
        const bool bpresent = bmx < nkx && bmy < nky;
        const float2 *xcol = reinterpret_cast<const float2 *>(smem + P::OFF_X + stage * P::X_BYTES +
                                                              (uint32_t)(bv * 2 + brs) * P::XS);

        float acc[MPW][3][4];
#pragma unroll
        for (int im = 0; im < MPW; im++)
#pragma unroll
            for (int j = 0; j < 3; j++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[im][j][c] = 0.f;
        const uint2 *Gq = reinterpret_cast<const uint2 *>(smem + stage * P::G_BYTES);
#pragma unroll
        for (int ik = 0; ik < KMAX; ik++) {
            if (ik >= kcnt) break;
            const int kt = ktb + ik;
            // B values of rows 8kt + t and 8kt + t + 4 of this lane's column,
            // with the D_p sign of their component and the sign of the -A^T
            // tiles (z rows of row group 2 x x|y columns)
            float2 x0 = make_float2(0.f, 0.f), x1 = make_float2(0.f, 0.f);
            if (bpresent) {
                x0 = xcol[8 * kt + t];
                x1 = xcol[8 * kt + t + 4];
            }
            const int comp = (8 * kt) / NZ;
            const bool flip = ((comp == 0 && bmx) || (comp == 1 && bmy)) != (mg == 2 && comp < 2);
            if (flip) {
                x0 = make_float2(-x0.x, -x0.y);
                x1 = make_float2(-x1.x, -x1.y);
            }
            // [Xr, Xi, Xr + Xi] x (hi b0, hi b1, lo b0, lo b1)
            uint32_t b[3][4];
            split_rn(x0.x, b[0][0], b[0][2]);
            split_rn(x1.x, b[0][1], b[0][3]);
            split_rn(x0.y, b[1][0], b[1][2]);
            split_rn(x1.y, b[1][1], b[1][3]);
            split_rn(x0.x + x0.y, b[2][0], b[2][2]);
            split_rn(x1.x + x1.y, b[2][1], b[2][3]);
#pragma unroll
            for (int im = 0; im < MPW; im++) {
                // [Gr hi, Gr lo, Gi hi, Gi lo, Gs hi, Gs lo][e]
                uint32_t af[6][4];
                const uint32_t t0 = tab[(im * KMAX + ik) * 2], t1 = tab[(im * KMAX + ik) * 2 + 1];
                const uint32_t off[4] = {t0 & 0xffffu, t0 >> 16, t1 & 0xffffu, t1 >> 16};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float2 gv = unsplit_entry(Gq[off[e]], ginv);
                    split(gv.x, af[0][e], af[1][e]);
                    split(gv.y, af[2][e], af[3][e]);
                    split(gv.x + gv.y, af[4][e], af[5][e]);
                }
                // three independent accumulator chains per row tile
#pragma unroll
                for (int j = 0; j < 3; j++) mma_tf32(acc[im][j], af[2 * j], b[j][0], b[j][1]);
#pragma unroll
                for (int j = 0; j < 3; j++) mma_tf32(acc[im][j], af[2 * j], b[j][2], b[j][3]);
#pragma unroll
                for (int j = 0; j < 3; j++) mma_tf32(acc[im][j], af[2 * j + 1], b[j][0], b[j][1]);
            }
        }
        __syncthreads();  // the previous point's reduction has read the partial sums
        // partial sums [kg][mt][re|im][c][lane]
#pragma unroll
        for (int im = 0; im < MPW; im++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float t1 = acc[im][0][c], t2 = acc[im][1][c], t3 = acc[im][2][c];
                const int base = ((kg * P::MT + mg * MPW + im) * 2) * 4 + c;
                PART[base * 32] = t1 - t2;
                PART[(base + 4) * 32] = t3 - t1 - t2;
            }
        if (__syncthreads_or(late)) {  // partials written; the stage is free
            if (tid == 0) {
                atomicExch(err, EGX_ERR_TIMEOUT);
                bar_wait(bar0 + 8 * (stage ^ 1), ((it + 1) >> 1) & 1, kWait);
            }
            return;
        }
        if (tid == 0 && q + 2L * gridDim.x < Q) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q + 2L * gridDim.x, stage);
        }
        // reduction units: with BAL, the 2 MT half row tiles (rows g or g + 8)
        // over the warps of the column groups with the fewest column tiles;
        // else row tile w by warp w < MT
        const int ubeg = BAL ? (light >= 0 ? light : 2 * P::MT) : (warp < P::MT ? warp : P::MT);
        const int uend = BAL ? 2 * P::MT : (warp < P::MT ? warp + 1 : P::MT);
        const int ustep = BAL ? nlight : 1;
        for (int u = ubeg; u < uend; u += ustep) {
            const int mt = BAL ? u >> 1 : u;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                if (BAL && (c >> 1) != (u & 1)) continue;
                float yr = 0.f, yi = 0.f;
#pragma unroll
                for (int k = 0; k < P::KG; k++) {
                    const int base = ((k * P::MT + mt) * 2) * 4 + c;
                    yr += PART[base * 32];
                    yi += PART[(base + 4) * 32];
                }
                // C: rows g, g+8; column 2t + (c & 1) = 4 rhs + point
                const int row = 16 * mt + g + 8 * (c >> 1);
                const int col = 2 * t + (c & 1), v = col & 3, r = col >> 2;
                const int mx = v >> 1, my = v & 1;
                if (mx < nkx && my < nky) {
                    float2 val = make_float2(yr, yi);
                    const int comp = row / NZ;
                    if ((comp == 0 && mx) || (comp == 1 && my)) val = make_float2(-val.x, -val.y);
                    const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
                    buf[pt * B + (long)(rhs0 + r) * R + row] = val;
                }
            }
        }
    }
}

// Two right-hand sides on the FP16 tensor-core path. The split copy holds
// every Green entry as FP16 high parts and remainders of its scaled Re and
// Im (split_entry), so the A fragments of mma.sync m16n8k16 come straight
// from shared memory, two entries and four byte permutes per register
// quartet, with no conversion. The right-hand sides are scaled per column
// by a power of two (2^(13 - e) over the rows this warp multiplies; the four
// lanes of a column agree by shuffle) and split the same way in registers.
// Four real products per complex product, three FP16 passes each
// (hi.hi + hi.lo + lo.hi, 22 bits per operand as the TF32 split):
//   T1 = Gr Xr, T2 = Gi Xi, T3 = Gr Xi, T4 = Gi Xr, Yr = T1 - T2, Yi = T3 + T4,
// 12 MMAs of K = 16 per (row tile, column tile) pair where the TF32 form
// takes 18 of K = 8 for the same K. Each warp divides its partial sums by
// its scales before they meet.
//
// Work split as k_contract_sb3 (12 warps, 3 row groups x 4 column groups,
// column tiles of 16, two TMA stages, two block barriers per point, the
// reduction on the warps with the fewest column tiles).
template <int NZ>
struct Sh {
    static constexpr int R = 3 * NZ, MT = R / 16, KT = R / 16, NB = NZ / 4;
    static constexpr int SYM = NB * (NB + 1) / 2 * 16, ASY = NB * NB * 16, BS = 4 * SYM + 2 * ASY;
    // 3 row groups (one component each) x 4 column groups; for nz = 32,
    // whose 6 column tiles do not split in four, 6 x 2 (3 tiles each)
    static constexpr int MG = NZ == 32 ? 6 : 3, KG = NZ == 32 ? 2 : 4;
    static constexpr int MPW = MT / MG, KMAX = (KT + KG - 1) / KG;
    static constexpr int THREADS = 32 * MG * KG;
    static constexpr uint32_t SEG = R * 8u, XS = SEG + 32u;
    static constexpr uint32_t G_BYTES = BS * 8u;
    static constexpr uint32_t X_BYTES = 8u * XS;
    static constexpr uint32_t PART_BYTES = KG * MT * 2u * 4u * 32u * 4u;
    static constexpr uint32_t OFF_X = 2 * G_BYTES, OFF_PART = OFF_X + 2 * X_BYTES;
    static constexpr uint32_t SMEM = OFF_PART + PART_BYTES;
    static_assert(MT % MG == 0, "row tiles must split over the row groups");
    static_assert(SMEM + 256 <= 227u * 1024u, "shared memory per block");
    static_assert(MT <= MG * KG, "reduction units");
    static_assert(NZ % (16 * MPW) == 0, "a row group within one component");
    static_assert(BS < 0x8000, "16-bit offsets with a stride flag");
    static_assert(G_BYTES % 128 == 0 && SEG % 16 == 0 && XS % 128 == 32, "stage alignment and bank skew");
    __host__ __device__ static constexpr int kt0(int kg) { return kg * KT / KG; }
};

// (a, b) -> FP16 pairs hi, lo with a = hi + lo (hi rounded to 11 significant
// bits in FP32, which FP16 holds exactly in its normal range); the low half
// holds a (the smaller row index of the fragment)
__device__ __forceinline__ void split_h2(float a, float b, uint32_t &hi, uint32_t &lo) {
    const float ha = __uint_as_float(tf32_hi(__float_as_uint(a)));
    const float hb = __uint_as_float(tf32_hi(__float_as_uint(b)));
    const __half2 h = __floats2half2_rn(ha, hb);
    const __half2 l = __floats2half2_rn(a - ha, b - hb);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

// d = a b (zero accumulator)
__device__ __forceinline__ void mma_f16_zero(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%10,%10,%10,%10};"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(0.f));
}

__device__ __forceinline__ void mma_f16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// offset of entry (row, col), col even, and whether (row, col + 1) sits at
// offset ^ 1 or, in the transposed sub-blocks, at offset ^ 4 (bit 15)
template <int NZ>
__host__ __device__ inline uint32_t sh_entry(int row, int col) {
    const int a = sb_index(NZ, row, col), b = sb_index(NZ, row, col + 1);
    return (uint32_t)a | ((a ^ b) == 4 ? 0x8000u : 0u);
}

template <int NZ>
__global__ void __launch_bounds__(Sh<NZ>::THREADS, 1)
    k_contract_sh(float2 *buf, const float2 *__restrict__ G, const int nx, const int ny, const int B, const int rhs0,
                  int *err) {
    using P = Sh<NZ>;
    constexpr int R = P::R, MPW = P::MPW, KMAX = P::KMAX;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int mg = warp % P::MG, kg = warp / P::MG;
    const int ktb = P::kt0(kg), kcnt = P::kt0(kg + 1) - ktb;
    int light = -1, nlight = 0;
    {
        int mincnt = P::KT;
        for (int k = 0; k < P::KG; k++) mincnt = min(mincnt, P::kt0(k + 1) - P::kt0(k));
        for (int w = 0; w < P::MG * P::KG; w++) {
            const int wk = w / P::MG;
            if (P::kt0(wk + 1) - P::kt0(wk) == mincnt) {
                if (w == warp) light = nlight;
                nlight++;
            }
        }
    }
    const uint32_t sG = saddr(smem), sX = sG + P::OFF_X;
    const uint32_t bar0 = saddr(&bars[0]);
    const long Q = (long)(nx + 1) * (ny + 1);
    const int n1 = 2 * ny;
    const int bv = g & 3, brs = g >> 2, bmx = bv >> 1, bmy = bv & 1;
    // 1 / the split copy's scale, in its trailing entry
    const float ginv = __uint_as_float(reinterpret_cast<const uint2 *>(G)[Q * P::BS].y);
    // this row group's rows are z rows (its -A^T tiles take the sign)
    const bool zrows = (16 * MPW * mg) / NZ == 2;

    // A-fragment entries (g, 2t), (g + 8, 2t), (g, 2t + 8), (g + 8, 2t + 8)
    // of each (row tile, column tile) pair, two 16-bit entries per word
    constexpr int TABN = MPW * KMAX * 2;
    static_assert(P::MG * P::KG * TABN * 32 * 4 <= P::G_BYTES, "offset scratch must fit in one stage");
    uint32_t tab[TABN];
    {
        uint32_t *scratch = reinterpret_cast<uint32_t *>(smem) + (size_t)warp * TABN * 32 + lane;
#pragma unroll 1
        for (int p = 0; p < MPW * KMAX; p++) {
            const int im = p / KMAX, ik = p - im * KMAX;
            uint32_t w0 = 0, w1 = 0;
            if (ik < kcnt) {
                const int r0 = 16 * (mg * MPW + im) + g, c0 = 16 * (ktb + ik) + 2 * t;
                w0 = sh_entry<NZ>(r0, c0) | (sh_entry<NZ>(r0 + 8, c0) << 16);
                w1 = sh_entry<NZ>(r0, c0 + 8) | (sh_entry<NZ>(r0 + 8, c0 + 8) << 16);
            }
            scratch[(2 * p) * 32] = w0;
            scratch[(2 * p + 1) * 32] = w1;
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < TABN; j++) tab[j] = scratch[j * 32];
    }

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](long qq, int stage) {
        const int a = (int)((unsigned)qq / (unsigned)(ny + 1)), bq = (int)qq - a * (ny + 1);
        const int nkx = (a == 0 || a == nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == ny) ? 1 : 2;
        const uint32_t bar = bar0 + 8 * stage;
        bar_expect(bar, P::G_BYTES + (uint32_t)(nkx * nky) * (2u * P::SEG));
        bulk_g2s(sG + stage * P::G_BYTES, G + qq * P::BS, P::G_BYTES, bar);
        for (int p = 0; p < 4; p++) {
            const int mx = p >> 1, my = p & 1;
            if (mx < nkx && my < nky) {
                const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
#pragma unroll
                for (int r = 0; r < 2; r++)
                    bulk_g2s(sX + stage * P::X_BYTES + (uint32_t)(p * 2 + r) * P::XS, buf + pt * B + (long)(rhs0 + r) * R,
                             P::SEG, bar);
            }
        }
    };
    long q = blockIdx.x;
    if (tid == 0) {
        // the offset scratch in stage 0 was read through the generic proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (q < Q) issue(q, 0);
        if (q + gridDim.x < Q) issue(q + gridDim.x, 1);
    }

    float *PART = reinterpret_cast<float *>(smem + P::OFF_PART) + lane;
    for (int it = 0; q < Q; q += gridDim.x, it++) {
        const int stage = it & 1;
        const uint32_t parity = (it >> 1) & 1;
        const uint32_t bar = bar0 + 8 * stage;
        const bool late = !bar_wait(bar, parity, kWait);
        // Q < 2^31 (checked at launch): 32-bit point decoding
        const int a = (int)((unsigned)q / (unsigned)(ny + 1)), bq = (int)q - a * (ny + 1);
        const int nkx = (a == 0 || a == nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == ny) ? 1 : 2;
        const bool bpresent = bmx < nkx && bmy < nky;
        const float4 *xcol = reinterpret_cast<const float4 *>(smem + P::OFF_X + stage * P::X_BYTES +
                                                              (uint32_t)(bv * 2 + brs) * P::XS);

        // this lane's right-hand-side values: rows 16 kt + 2t, +1 and
        // 16 kt + 2t + 8, +9 of its column, with the D_p sign of their
        // component and the sign of the -A^T tiles
        float4 xv[KMAX][2];
        float m = 0.f;
#pragma unroll
        for (int ik = 0; ik < KMAX; ik++) {
            xv[ik][0] = xv[ik][1] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ik < kcnt && bpresent) {
                const int kt = ktb + ik;
                xv[ik][0] = xcol[8 * kt + t];
                xv[ik][1] = xcol[8 * kt + 4 + t];
                const int comp = (16 * kt) / NZ;
                if (((comp == 0 && bmx) || (comp == 1 && bmy)) != (zrows && comp < 2)) {
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        xv[ik][h] = make_float4(-xv[ik][h].x, -xv[ik][h].y, -xv[ik][h].z, -xv[ik][h].w);
                }
#pragma unroll
                for (int h = 0; h < 2; h++)
                    m = fmaxf(m, fmaxf(fmaxf(fabsf(xv[ik][h].x), fabsf(xv[ik][h].y)),
                                       fmaxf(fabsf(xv[ik][h].z), fabsf(xv[ik][h].w))));
            }
        }
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
        const float scB = pow2_scale(m, 13);
        // B fragments [ik][Xr, Xi][hi b0, hi b1, lo b0, lo b1]
        uint32_t bf[KMAX][2][4];
#pragma unroll
        for (int ik = 0; ik < KMAX; ik++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float4 v = xv[ik][h];  // (re, im) of two consecutive rows
                split_h2(v.x * scB, v.z * scB, bf[ik][0][h], bf[ik][0][2 + h]);
                split_h2(v.y * scB, v.w * scB, bf[ik][1][h], bf[ik][1][2 + h]);
            }

        // T1 = Gr Xr, T2 = Gi Xi, T3 = Gr Xi, T4 = Gi Xr per row tile
        // (the first k tile's first products start from zero accumulators)
        float acc[MPW][4][4];
        if (kcnt <= 0) {
#pragma unroll
            for (int im = 0; im < MPW; im++)
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[im][j][c] = 0.f;
        }
        const uint2 *Gq = reinterpret_cast<const uint2 *>(smem + stage * P::G_BYTES);
#pragma unroll
        for (int ik = 0; ik < KMAX; ik++) {
            if (ik >= kcnt) break;
#pragma unroll
            for (int im = 0; im < MPW; im++) {
                // [Gr hi, Gr lo, Gi hi, Gi lo][a0..a3]
                uint32_t af[4][4];
                const uint32_t t0 = tab[(im * KMAX + ik) * 2], t1 = tab[(im * KMAX + ik) * 2 + 1];
                const uint32_t ent[4] = {t0 & 0xffffu, t0 >> 16, t1 & 0xffffu, t1 >> 16};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const uint32_t off = ent[e] & 0x7fffu, nb = (ent[e] & 0x8000u) ? 4u : 1u;
                    const uint2 u = Gq[off], w = Gq[off ^ nb];
                    af[0][e] = __byte_perm(u.x, w.x, 0x5410);
                    af[2][e] = __byte_perm(u.x, w.x, 0x7632);
                    af[1][e] = __byte_perm(u.y, w.y, 0x5410);
                    af[3][e] = __byte_perm(u.y, w.y, 0x7632);
                }
                // product j: A = Gr (j even) or Gi, B = Xr (j = 0, 3) or Xi
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int ai = (j == 0 || j == 2) ? 0 : 2, bi = (j == 0 || j == 3) ? 0 : 1;
                    if (ik == 0) mma_f16_zero(acc[im][j], af[ai], bf[ik][bi][0], bf[ik][bi][1]);
                    else mma_f16(acc[im][j], af[ai], bf[ik][bi][0], bf[ik][bi][1]);
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int ai = (j == 0 || j == 2) ? 0 : 2, bi = (j == 0 || j == 3) ? 0 : 1;
                    mma_f16(acc[im][j], af[ai], bf[ik][bi][2], bf[ik][bi][3]);
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int ai = (j == 0 || j == 2) ? 1 : 3, bi = (j == 0 || j == 3) ? 0 : 1;
                    mma_f16(acc[im][j], af[ai], bf[ik][bi][0], bf[ik][bi][1]);
                }
            }
        }
        // undo the scales: accumulator columns 2t and 2t + 1 carry the
        // scales of the lanes that hold those B columns
        const float inv = ginv / scB;
        const float inv0 = __shfl_sync(0xffffffffu, inv, (2 * t) * 4);
        const float inv1 = __shfl_sync(0xffffffffu, inv, (2 * t + 1) * 4);
        __syncthreads();  // the previous point's reduction has read the partial sums
#pragma unroll
        for (int im = 0; im < MPW; im++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float f = (c & 1) ? inv1 : inv0;
                const int base = ((kg * P::MT + mg * MPW + im) * 2) * 4 + c;
                PART[base * 32] = (acc[im][0][c] - acc[im][1][c]) * f;
                PART[(base + 4) * 32] = (acc[im][2][c] + acc[im][3][c]) * f;
            }
        if (__syncthreads_or(late)) {  // partials written; the stage is free
            if (tid == 0) {
                atomicExch(err, EGX_ERR_TIMEOUT);
                bar_wait(bar0 + 8 * (stage ^ 1), ((it + 1) >> 1) & 1, kWait);
            }
            return;
        }
        if (tid == 0 && q + 2L * gridDim.x < Q) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q + 2L * gridDim.x, stage);
        }
        // half row tiles (rows g or g + 8) over the warps with the fewest
        // column tiles
        const int ubeg = light >= 0 ? light : 2 * P::MT;
        for (int u = ubeg; u < 2 * P::MT; u += nlight) {
            const int mt = u >> 1;
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const int c = 2 * (u & 1) + cc;
                float yr = 0.f, yi = 0.f;
#pragma unroll
                for (int k = 0; k < P::KG; k++) {
                    const int base = ((k * P::MT + mt) * 2) * 4 + c;
                    yr += PART[base * 32];
                    yi += PART[(base + 4) * 32];
                }
                const int row = 16 * mt + g + 8 * (c >> 1);
                const int col = 2 * t + (c & 1), v = col & 3, r = col >> 2;
                const int mx = v >> 1, my = v & 1;
                if (mx < nkx && my < nky) {
                    float2 val = make_float2(yr, yi);
                    const int comp = row / NZ;
                    if ((comp == 0 && mx) || (comp == 1 && my)) val = make_float2(-val.x, -val.y);
                    const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
                    buf[pt * B + (long)(rhs0 + r) * R + row] = val;
                }
            }
        }
    }
}

// k_contract_ws<NZ>: the two-source FP16 split contraction with its work
// split by role, so that the phases of one point overlap the products of
// another instead of running in lockstep behind block barriers.
//  * MMA warps, one per row tile (MT of them): every k tile of their tile,
//    12 products per k tile as in k_contract_sh, accumulators alternating
//    by k tile; the output leaves from the accumulators (no partial sums).
//  * two split warps: load the right-hand sides of a point from global
//    memory (the Green stage carries no right-hand sides), take one scale
//    per column over all its rows, split into FP16 fragments in a double
//    buffer, while the MMA warps work on the point before.
//  * one producer lane: a TMA bulk copy of the next Green block into the
//    stage the MMA warps released.
// Hand-offs are mbarriers; every wait is bounded, and a wait that gives up
// records EGX_ERR_TIMEOUT and raises a block-wide abort flag that ends every
// role's loop within one poll.
template <int NZ>
struct Ws {
    static constexpr int R = 3 * NZ, MT = R / 16, KT = R / 16, BS = Sh<NZ>::BS;
    static constexpr int NSPLIT = 2, PRODUCER = MT + NSPLIT, THREADS = 32 * (MT + NSPLIT + 1);
    static constexpr int KPS = (KT + NSPLIT - 1) / NSPLIT;  // k tiles per split warp
    static constexpr uint32_t G_BYTES = BS * 8u;
    static constexpr uint32_t BF_BYTES = KT * 2u * 32u * 16u;  // [KT][Xr, Xi][32 lanes] uint4
    static constexpr uint32_t OFF_BF = 2 * G_BYTES, OFF_INV = OFF_BF + 2 * BF_BYTES;
    static constexpr uint32_t OFF_MAX = OFF_INV + 2u * 8u * 4u;
    static constexpr uint32_t SMEM = OFF_MAX + 2u * NSPLIT * 8u * 4u;
    static_assert(SMEM + 256 <= 227u * 1024u, "shared memory per block");
    static_assert(MT * KT * 2 * 32 * 4 <= G_BYTES, "offset scratch must fit in one stage");
    static_assert(G_BYTES % 128 == 0 && OFF_BF % 16 == 0, "stage alignment");
};

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// bounded wait that also ends once another thread of the block gave up
__device__ __forceinline__ bool ws_wait(uint32_t bar, uint32_t parity, volatile int *abort, int *err) {
    const uint64_t t0 = wait_clock_ns();
    while (!mbar_try_parity(bar, parity)) {
        if (*abort) return false;
        if (wait_clock_ns() - t0 > kWait) {
            *abort = 1;
            atomicExch(err, EGX_ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

// the same for all 32 lanes of a warp, which leave or go on together (the
// MMA and shuffle code after it needs the whole warp)
__device__ __forceinline__ bool ws_wait_warp(uint32_t bar, uint32_t parity, volatile int *abort, int *err) {
    const bool ok = ws_wait(bar, parity, abort, err);
    return __all_sync(0xffffffffu, ok);
}

template <int NZ>
__global__ void __launch_bounds__(Ws<NZ>::THREADS, 1)
    k_contract_ws(float2 *buf, const float2 *__restrict__ G, const int nx, const int ny, const int B, const int rhs0,
                  int *err) {
    using P = Ws<NZ>;
    constexpr int R = P::R, KT = P::KT;
    extern __shared__ __align__(128) unsigned char smem[];
    // [full, sempty, bfull, bempty, cmax] x 2: Green block landed, stage
    // read, fragments split, fragments read, split warps' column maxima
    __shared__ __align__(8) uint64_t bars[10];
    __shared__ int abort_flag;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const uint32_t sG = saddr(smem);
    const uint32_t b_full = saddr(&bars[0]), b_sempty = b_full + 16, b_bfull = b_full + 32;
    const uint32_t b_bempty = b_full + 48, b_max = b_full + 64;
    volatile int *abort = &abort_flag;
    const int Q = (nx + 1) * (ny + 1);  // below 2^31, checked at launch
    const int n1 = 2 * ny;
    // 1 / the split copy's scale, in its trailing entry
    const float ginv = __uint_as_float(reinterpret_cast<const uint2 *>(G)[(long)Q * P::BS].y);
    uint4 *BFRAG = reinterpret_cast<uint4 *>(smem + P::OFF_BF);
    float *INV = reinterpret_cast<float *>(smem + P::OFF_INV);
    float *CMAX = reinterpret_cast<float *>(smem + P::OFF_MAX);

    // MMA warps: A-fragment entries (g, 2t), (g + 8, 2t), (g, 2t + 8),
    // (g + 8, 2t + 8) of each k tile of the warp's row tile
    uint32_t tab[2 * KT];
    if (warp < P::MT) {
        uint32_t *scratch = reinterpret_cast<uint32_t *>(smem) + (size_t)warp * 2 * KT * 32 + lane;
#pragma unroll 1
        for (int kt = 0; kt < KT; kt++) {
            const int r0 = 16 * warp + g, c0 = 16 * kt + 2 * t;
            scratch[(2 * kt) * 32] = sh_entry<NZ>(r0, c0) | (sh_entry<NZ>(r0 + 8, c0) << 16);
            scratch[(2 * kt + 1) * 32] = sh_entry<NZ>(r0, c0 + 8) | (sh_entry<NZ>(r0 + 8, c0 + 8) << 16);
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 2 * KT; j++) tab[j] = scratch[j * 32];
    }
    if (tid == 0) {
        abort_flag = 0;
        for (int i = 0; i < 2; i++) {
            mbar_init(b_full + 8 * i, 1);
            mbar_init(b_sempty + 8 * i, 32 * P::MT);
            mbar_init(b_bfull + 8 * i, 32 * P::NSPLIT);
            mbar_init(b_bempty + 8 * i, 32 * P::MT);
            mbar_init(b_max + 8 * i, 32 * P::NSPLIT);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp < P::MT) {
        // ---- MMA warp: row tile mt
        const int mt = warp;
        // z rows: the -A^T tiles of the x and y columns take the sign
        const bool zrows = (16 * mt) / NZ == 2;
        for (int it = 0, q = blockIdx.x; q < Q; q += gridDim.x, it++) {
            const int s = it & 1;
            const uint32_t par = (it >> 1) & 1;
            if (!ws_wait_warp(b_full + 8 * s, par, abort, err) || !ws_wait_warp(b_bfull + 8 * s, par, abort, err))
                break;
            const uint2 *Gq = reinterpret_cast<const uint2 *>(smem + s * P::G_BYTES);
            const uint4 *bfr = BFRAG + (size_t)s * (P::BF_BYTES / 16) + lane;
            // T1 = Gr Xr, T2 = Gi Xi, T3 = Gr Xi, T4 = Gi Xr, even and odd k tiles
            float acc[2][4][4];
#pragma unroll
            for (int kt = 0; kt < KT; kt++) {
                const uint32_t flip = (zrows && (16 * kt) / NZ < 2) ? 0x80008000u : 0u;
                // B fragments [Xr, Xi][hi b0, hi b1, lo b0, lo b1]; the sign
                // flips both FP16 halves (the split commutes with it)
                uint32_t bf[2][4];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint4 f = bfr[(kt * 2 + h) * 32];
                    bf[h][0] = f.x ^ flip;
                    bf[h][1] = f.y ^ flip;
                    bf[h][2] = f.z ^ flip;
                    bf[h][3] = f.w ^ flip;
                }
                // [Gr hi, Gr lo, Gi hi, Gi lo][a0..a3]
                uint32_t af[4][4];
                const uint32_t t0 = tab[2 * kt], t1 = tab[2 * kt + 1];
                const uint32_t ent[4] = {t0 & 0xffffu, t0 >> 16, t1 & 0xffffu, t1 >> 16};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const uint32_t off = ent[e] & 0x7fffu, nb = (ent[e] & 0x8000u) ? 4u : 1u;
                    const uint2 u = Gq[off], w = Gq[off ^ nb];
                    af[0][e] = __byte_perm(u.x, w.x, 0x5410);
                    af[2][e] = __byte_perm(u.x, w.x, 0x7632);
                    af[1][e] = __byte_perm(u.y, w.y, 0x5410);
                    af[3][e] = __byte_perm(u.y, w.y, 0x7632);
                }
                float (*ac)[4] = acc[kt & 1];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int ai = (j == 0 || j == 2) ? 0 : 2, bi = (j == 0 || j == 3) ? 0 : 1;
                    if (kt < 2) mma_f16_zero(ac[j], af[ai], bf[bi][0], bf[bi][1]);
                    else mma_f16(ac[j], af[ai], bf[bi][0], bf[bi][1]);
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int ai = (j == 0 || j == 2) ? 0 : 2, bi = (j == 0 || j == 3) ? 0 : 1;
                    mma_f16(ac[j], af[ai], bf[bi][2], bf[bi][3]);
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int ai = (j == 0 || j == 2) ? 1 : 3, bi = (j == 0 || j == 3) ? 0 : 1;
                    mma_f16(ac[j], af[ai], bf[bi][0], bf[bi][1]);
                }
            }
            // undo the scales of accumulator columns 2t and 2t + 1
            const float inv0 = INV[s * 8 + 2 * t], inv1 = INV[s * 8 + 2 * t + 1];
            mbar_arrive(b_sempty + 8 * s);
            mbar_arrive(b_bempty + 8 * s);
            const int a = (int)((unsigned)q / (unsigned)(ny + 1)), bq = q - a * (ny + 1);
            const int nkx = (a == 0 || a == nx) ? 1 : 2;
            const int nky = (bq == 0 || bq == ny) ? 1 : 2;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                // rows g (c < 2) and g + 8 of the tile, column 2t + (c & 1):
                // mirror point col & 3, source col >> 2
                const int row = 16 * mt + g + 8 * (c >> 1);
                const int col = 2 * t + (c & 1), v = col & 3, r = col >> 2;
                const int mx = v >> 1, my = v & 1;
                if (mx < nkx && my < nky) {
                    const float f = (c & 1) ? inv1 : inv0;
                    const float t1 = acc[0][0][c] + acc[1][0][c], t2 = acc[0][1][c] + acc[1][1][c];
                    const float t3 = acc[0][2][c] + acc[1][2][c], t4 = acc[0][3][c] + acc[1][3][c];
                    float2 val = make_float2((t1 - t2) * f, (t3 + t4) * f);
                    const int comp = row / NZ;
                    if ((comp == 0 && mx) || (comp == 1 && my)) val = make_float2(-val.x, -val.y);
                    const long pt = (long)(mx ? 2 * nx - a : a) * n1 + (my ? 2 * ny - bq : bq);
                    buf[pt * B + (long)(rhs0 + r) * R + row] = val;
                }
            }
        }
    } else if (warp < P::PRODUCER) {
        // ---- split warp hh: k tiles hh, hh + NSPLIT, ... of every column
        const int hh = warp - P::MT;
        const int bv = g & 3, brs = g >> 2, bmx = bv >> 1, bmy = bv & 1;
        for (int it = 0, q = blockIdx.x; q < Q; q += gridDim.x, it++) {
            const int s = it & 1;
            const uint32_t par = (it >> 1) & 1;
            const int a = (int)((unsigned)q / (unsigned)(ny + 1)), bq = q - a * (ny + 1);
            const int nkx = (a == 0 || a == nx) ? 1 : 2;
            const int nky = (bq == 0 || bq == ny) ? 1 : 2;
            const bool bpresent = bmx < nkx && bmy < nky;
            // this lane's column: mirror point bv, source brs; rows
            // 16 kt + 2t, +1 and 16 kt + 2t + 8, +9 with the D_p sign of
            // their component (loads issued before the buffer wait)
            float4 xv[P::KPS][2];
            if (bpresent) {
                const long pt = (long)(bmx ? 2 * nx - a : a) * n1 + (bmy ? 2 * ny - bq : bq);
                const float4 *xcol = reinterpret_cast<const float4 *>(buf + pt * B + (long)(rhs0 + brs) * R);
#pragma unroll
                for (int i = 0; i < P::KPS; i++) {
                    const int kt = hh + P::NSPLIT * i;
                    if (kt < KT) {
                        xv[i][0] = xcol[8 * kt + t];
                        xv[i][1] = xcol[8 * kt + 4 + t];
                    }
                }
            }
            if (it >= 2 && !ws_wait_warp(b_bempty + 8 * s, par ^ 1u, abort, err)) break;
            float m = 0.f;
#pragma unroll
            for (int i = 0; i < P::KPS; i++) {
                const int kt = hh + P::NSPLIT * i;
                if (kt >= KT) continue;
                if (!bpresent) {
                    xv[i][0] = xv[i][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    continue;
                }
                const int comp = (16 * kt) / NZ;
                if ((comp == 0 && bmx) || (comp == 1 && bmy)) {
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        xv[i][h] = make_float4(-xv[i][h].x, -xv[i][h].y, -xv[i][h].z, -xv[i][h].w);
                }
#pragma unroll
                for (int h = 0; h < 2; h++)
                    m = fmaxf(m, fmaxf(fmaxf(fabsf(xv[i][h].x), fabsf(xv[i][h].y)),
                                       fmaxf(fabsf(xv[i][h].z), fabsf(xv[i][h].w))));
            }
            // one scale per column over all its rows: the split warps'
            // maxima meet in shared memory
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
            if (t == 0) CMAX[(s * P::NSPLIT + hh) * 8 + g] = m;
            mbar_arrive(b_max + 8 * s);
            if (!ws_wait_warp(b_max + 8 * s, par, abort, err)) break;
            float mc = 0.f;
#pragma unroll
            for (int h = 0; h < P::NSPLIT; h++) mc = fmaxf(mc, CMAX[(s * P::NSPLIT + h) * 8 + g]);
            const float scB = pow2_scale(mc, 13);
            uint4 *bfw = BFRAG + (size_t)s * (P::BF_BYTES / 16) + lane;
#pragma unroll
            for (int i = 0; i < P::KPS; i++) {
                const int kt = hh + P::NSPLIT * i;
                if (kt >= KT) continue;
                // [Xr, Xi] x [hi b0, hi b1, lo b0, lo b1]
                uint4 fr, fi;
                split_h2(xv[i][0].x * scB, xv[i][0].z * scB, fr.x, fr.z);
                split_h2(xv[i][1].x * scB, xv[i][1].z * scB, fr.y, fr.w);
                split_h2(xv[i][0].y * scB, xv[i][0].w * scB, fi.x, fi.z);
                split_h2(xv[i][1].y * scB, xv[i][1].w * scB, fi.y, fi.w);
                bfw[(kt * 2) * 32] = fr;
                bfw[(kt * 2 + 1) * 32] = fi;
            }
            if (hh == 0 && t == 0) INV[s * 8 + g] = ginv / scB;
            mbar_arrive(b_bfull + 8 * s);
        }
    } else if (lane == 0) {
        // ---- producer: the Green block of each point into a free stage
        int issued = 0;
        for (int it = 0, q = blockIdx.x; q < Q; q += gridDim.x, it++) {
            const int s = it & 1;
            if (it >= 2 && !ws_wait(b_sempty + 8 * s, ((it >> 1) + 1) & 1, abort, err)) break;
            // the stage was read through the generic proxy (and stage 0
            // held the offset scratch)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bar_expect(b_full + 8 * s, P::G_BYTES);
            bulk_g2s(sG + s * P::G_BYTES, G + (long)q * P::BS, P::G_BYTES, b_full + 8 * s);
            issued = it + 1;
        }
        // no copy in flight when the block exits (bounded)
        for (int j = issued > 2 ? issued - 2 : 0; j < issued; j++)
            mbar_wait_ns(b_full + 8 * (j & 1), (j >> 1) & 1, kWait);
    }
}

template <int NZ>
void launch_sh(float2 *buf, const float2 *G, const OpDims &d, int rhs0, int *err, cudaStream_t s, int nsm) {
    using P = Sh<NZ>;
    raise_smem_limit((const void *)k_contract_sh<NZ>, P::SMEM);
    const long Q = (long)(d.nx + 1) * (d.ny + 1);
    EGX_CHECK(Q < (1L << 31), EGX_ERR_INVALID, "sub-block contraction: (nx + 1)(ny + 1) must be below 2^31");
    const unsigned grid = (unsigned)std::min<long>(Q, nsm);
    k_contract_sh<NZ><<<grid, P::THREADS, P::SMEM, s>>>(buf, G, d.nx, d.ny, d.B, rhs0, err);
    EGX_CUDA(cudaGetLastError());
}

template <int NZ>
void launch_ws(float2 *buf, const float2 *G, const OpDims &d, int rhs0, int *err, cudaStream_t s, int nsm) {
    using P = Ws<NZ>;
    raise_smem_limit((const void *)k_contract_ws<NZ>, P::SMEM);
    const long Q = (long)(d.nx + 1) * (d.ny + 1);
    EGX_CHECK(Q < (1L << 31), EGX_ERR_INVALID, "sub-block contraction: (nx + 1)(ny + 1) must be below 2^31");
    const unsigned grid = (unsigned)std::min<long>(Q, nsm);
    k_contract_ws<NZ><<<grid, P::THREADS, P::SMEM, s>>>(buf, G, d.nx, d.ny, d.B, rhs0, err);
    EGX_CUDA(cudaGetLastError());
}

template <int NZ, bool BAL>
void launch_sb3(float2 *buf, const float2 *G, const OpDims &d, int rhs0, int *err, cudaStream_t s, int nsm) {
    using P = Sb3<NZ>;
    raise_smem_limit((const void *)k_contract_sb3<NZ, BAL>, P::SMEM);
    const long Q = (long)(d.nx + 1) * (d.ny + 1);
    const unsigned grid = (unsigned)std::min<long>(Q, nsm);
    k_contract_sb3<NZ, BAL><<<grid, P::THREADS, P::SMEM, s>>>(buf, G, d.nx, d.ny, d.B, rhs0, err);
    EGX_CUDA(cudaGetLastError());
}

template <int NZ, int NRHS>
void launch_sb(float2 *buf, const float2 *G, const OpDims &d, int rhs0, int *err, cudaStream_t s, int nsm) {
    using P = Sb<NZ, NRHS>;
    raise_smem_limit((const void *)k_contract_sb<NZ, NRHS>, P::SMEM);
    const long Q = (long)(d.nx + 1) * (d.ny + 1);
    const unsigned grid = (unsigned)std::min<long>(Q, nsm);
    k_contract_sb<NZ, NRHS><<<grid, P::THREADS, P::SMEM, s>>>(buf, G, d.nx, d.ny, d.B, rhs0, err);
    EGX_CUDA(cudaGetLastError());
}

template <int NZ>
void launch_nz(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s, int nsm, long *launches) {
    // contract_variant: 1 k_contract_sb3 (TF32 split), 2 k_contract_sh
    // (FP16 split, all warps in lockstep), 0 the built-in choice:
    // k_contract_ws (FP16 split by role: 1.110 against 1.293 ms per
    // two-source launch at 256x256x48)
    const int v = d.contract_variant;
    for (int r0 = 0; r0 < d.nrhs;) {
        if (d.nrhs - r0 >= 2) {
            if (v == 1)
                launch_sb3<NZ, true>(buf, G, d, r0, err, s, nsm);
            else if (v == 2)
                launch_sh<NZ>(buf, G, d, r0, err, s, nsm);
            else
                launch_ws<NZ>(buf, G, d, r0, err, s, nsm);
            r0 += 2;
        } else {
            launch_sb<NZ, 1>(buf, G, d, r0, err, s, nsm);
            r0 += 1;
        }
        if (launches) ++*launches;
    }
}

}  // namespace

bool sb_layout(int nz) { return nz == 16 || nz == 32 || nz == 48; }

long sb_block(int nz) { return 4L * sb_sym(nz) + 2L * sb_asy(nz); }

// the sub-block layout carries two trailing entries: the largest component
// magnitude (and padding that keeps 16-byte multiples)
long green_c64_entries(const GreenDims &gd) {
    return sb_layout(gd.nz) ? gd.Q() * sb_block(gd.nz) + 2 : gd.Q() * (long)gd.Bs();
}

void green_to_c64(const double2 *g64, float2 *g32, const GreenDims &gd, cudaStream_t s, long *launches) {
    if (sb_layout(gd.nz)) {
        const long total = gd.Q() * sb_block(gd.nz);
        const unsigned blocks = (unsigned)std::min<long>((total + 255) / 256, 152L * 64);
        uint2 *g = reinterpret_cast<uint2 *>(g32);
        EGX_CUDA(cudaMemsetAsync(g + total, 0, 2 * sizeof(uint2), s));
        k_repack_sb<false><<<blocks, 256, 0, s>>>(g64, g, gd.Q(), gd.nz);
        k_repack_sb<true><<<blocks, 256, 0, s>>>(g64, g, gd.Q(), gd.nz);
        EGX_CUDA(cudaGetLastError());
        if (launches) ++*launches;
    } else {
        convert_d2f(g64, g32, gd.Q() * gd.Bs(), 1.0, s);
    }
    if (launches) ++*launches;
}

void launch_contract_sb(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s, long *launches) {
    static int nsm = 0;
    if (!nsm) EGX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
    switch (d.nz) {
        case 16: launch_nz<16>(buf, G, d, err, s, nsm, launches); break;
        case 32: launch_nz<32>(buf, G, d, err, s, nsm, launches); break;
        case 48: launch_nz<48>(buf, G, d, err, s, nsm, launches); break;
        default: throw Error(EGX_ERR_INVALID, "sub-block contraction needs nz in {16, 32, 48}");
    }
}

}  // namespace egx
