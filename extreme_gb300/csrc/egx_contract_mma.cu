// Block contraction of the CIE operator in complex64 on the tensor cores
// (ConvolutionOperator.ApplyGreenTensorAlongZ, ConvolutionOperator.cs:274-327),
// one right-hand side per apply.
//
// Same algebra as egx_contract.cu: the four spectral points p sharing a stored
// quadrant block are right-hand sides of one (3nz x 3nz) complex matrix G
// after X'_v = D_p X_v; Y_v = D_p (G X'_v). The complex product is embedded
// in real arithmetic,
//     [Yr | Yi] = Gr [Xr | Xi] + Gi [-Xi | Xr],
// and computed with mma.sync m16n8k8 TF32 tiles: rows of G in 16-row tiles
// (one warp each), complex columns in 8-column tiles, the 4 vectors' real
// and imaginary parts as the 8 columns of the n dimension. Each operand is
// split into a TF32 high part and a TF32 remainder and three products are
// accumulated (Ahi Bhi + Ahi Blo + Alo Bhi), which keeps complex64 accuracy.
//
// Per stored point (one CTA per SM, loop over points):
//   one TMA bulk copy of the packed block and up to four of the right-hand
//   sides into one of two shared-memory stages, issued two points ahead and
//   completing on one mbarrier per stage (waits bounded to 2 s; on expiry
//   EGX_ERR_TIMEOUT is recorded in *err and the kernel returns);
//   a cooperative pass turns the right-hand sides into split B fragments in
//   shared memory (shared by all row tiles);
//   each warp gathers its A fragments through an offset table built once per
//   CTA -- entry (row, column) holds the index of G(row, column) in the
//   stored block (packed symmetric rc + tr(tr+1)/2 or row-padded
//   rc*(nz+1) + tr), the sign of the transposed xz/yz blocks in bit 15 and a
//   zero slot for the padding of the last tiles -- and runs the MMAs;
//   real and imaginary parts meet through a warp shuffle and are stored.
#include <cstdint>

#include "egx_operator.cuh"
#include "egx_wait.cuh"

namespace egx {

namespace {

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns) {
    return mbar_wait_ns(saddr(bar), parity, limit_ns);
}

__device__ __forceinline__ void bar_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
        "l"(src), "r"(bytes), "r"(saddr(bar))
        : "memory");
}

__device__ __forceinline__ uint32_t tf32_rna(float a) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(a));
    return r;
}

// a = hi + lo with both parts TF32
__device__ __forceinline__ void split_tf32(float a, uint32_t &hi, uint32_t &lo) {
    hi = tf32_rna(a);
    lo = tf32_rna(a - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr uint64_t kWait = 2000000000ull;

struct MmaGeom {
    int nz, R, MT, KT, S, lda, A, Bs, Bpad;
};

__host__ __device__ inline MmaGeom mma_geom(int nz) {
    MmaGeom g;
    g.nz = nz;
    g.R = 3 * nz;
    g.MT = (g.R + 15) / 16;
    g.KT = (g.R + 7) / 8;
    g.S = nz * (nz + 1) / 2;
    g.lda = nz + 1;
    g.A = nz * g.lda;
    g.Bs = 4 * g.S + 2 * g.A;
    g.Bpad = g.Bs + 2;  // + a zero slot, keeps 16-byte alignment
    return g;
}

// index of G(row, col) in the stored block (bit 15: negate), or the zero slot
__device__ uint32_t g_index(const MmaGeom &m, int row, int col) {
    if (row >= m.R || col >= m.R) return (uint32_t)m.Bs;
    const int nz = m.nz;
    const int co = row / nz, i = row - co * nz, ci = col / nz, j = col - ci * nz;
    if ((co < 2 && ci < 2) || (co == 2 && ci == 2)) {
        const int base = (co == 2) ? 3 * m.S : ((co == 0 && ci == 0) ? 0 : ((co == 1 && ci == 1) ? 2 * m.S : m.S));
        const int off = i <= j ? i + j * (j + 1) / 2 : j + i * (i + 1) / 2;
        return (uint32_t)(base + off);
    }
    if (ci == 2) return (uint32_t)(4 * m.S + co * m.A + i * m.lda + j);   // (x|y row i, z col j): A[i][j]
    return (uint32_t)(4 * m.S + ci * m.A + j * m.lda + i) | 0x8000u;      // (z row i, x|y col j): -A[j][i]
}

__global__ void __launch_bounds__(320, 1)
    k_contract_mma(float2 *buf, const float2 *__restrict__ G, const OpDims d, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int status;
    const MmaGeom m = mma_geom(d.nz);
    const int R = m.R, B = d.B;  // B = R (one right-hand side)
    const int MT = m.MT, KT = m.KT;
    float2 *Gs[2];
    Gs[0] = reinterpret_cast<float2 *>(smem_raw);
    Gs[1] = Gs[0] + m.Bpad;
    float2 *Xs[2];
    Xs[0] = Gs[1] + m.Bpad;           // [4 points][R]
    Xs[1] = Xs[0] + 4 * (size_t)B;
    uint2 *TAB = reinterpret_cast<uint2 *>(Xs[1] + 4 * (size_t)B);       // [MT][KT][32]
    uint4 *BF = reinterpret_cast<uint4 *>(TAB + (size_t)MT * KT * 32);    // [KT][2][32]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const long Q = (long)(d.nx + 1) * (d.ny + 1);
    const int n1 = 2 * d.ny;
    const uint32_t gbytes = (uint32_t)m.Bs * sizeof(float2);
    const uint32_t xbytes = (uint32_t)B * sizeof(float2);

    for (int e = tid; e < MT * KT * 32; e += blockDim.x) {
        const int ln = e & 31, tile = e >> 5;
        const int mt = tile / KT, kt = tile - mt * KT;
        const int r0 = 16 * mt + (ln >> 2), c0 = 8 * kt + (ln & 3);
        const uint32_t a0 = g_index(m, r0, c0), a1 = g_index(m, r0 + 8, c0);
        const uint32_t a2 = g_index(m, r0, c0 + 4), a3 = g_index(m, r0 + 8, c0 + 4);
        TAB[e] = make_uint2(a0 | (a1 << 16), a2 | (a3 << 16));
    }
    if (tid == 0) {
        Gs[0][m.Bs] = make_float2(0.f, 0.f);
        Gs[1][m.Bs] = make_float2(0.f, 0.f);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&bars[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&bars[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        status = 0;
    }
    __syncthreads();

    auto issue = [&](long qq, int stage) {
        const int a = (int)(qq / (d.ny + 1)), bq = (int)(qq - (long)a * (d.ny + 1));
        const int nkx = (a == 0 || a == d.nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == d.ny) ? 1 : 2;
        bar_expect(&bars[stage], gbytes + (uint32_t)(nkx * nky) * xbytes);
        bulk_g2s(Gs[stage], G + qq * m.Bs, gbytes, &bars[stage]);
        for (int p = 0; p < 4; p++) {
            const int mx = p >> 1, my = p & 1;
            if (mx < nkx && my < nky) {
                const long pt = (long)(mx ? 2 * d.nx - a : a) * n1 + (my ? 2 * d.ny - bq : bq);
                bulk_g2s(Xs[stage] + (size_t)p * B, buf + pt * B, xbytes, &bars[stage]);
            }
        }
    };
    long q = blockIdx.x;
    if (tid == 0) {
        if (q < Q) issue(q, 0);
        if (q + gridDim.x < Q) issue(q + gridDim.x, 1);
    }

    const bool active = warp < MT;
    const int mt = warp;

    for (int it = 0; q < Q; q += gridDim.x, it++) {
        const int stage = it & 1;
        const uint32_t parity = (it >> 1) & 1;
        if (tid == 0 && !bar_wait(&bars[stage], parity, kWait)) status = 1;
        __syncthreads();
        if (status) {
            if (tid == 0) {
                atomicExch(err, EGX_ERR_TIMEOUT);
                bar_wait(&bars[stage ^ 1], ((it + 1) >> 1) & 1, kWait);
            }
            return;
        }
        bar_wait(&bars[stage], parity, kWait);  // acquire the stage for every thread
        const int a = (int)(q / (d.ny + 1)), bq = (int)(q - (long)a * (d.ny + 1));
        const int nkx = (a == 0 || a == d.nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == d.ny) ? 1 : 2;
        // split B fragments: entry (kt, lane) = {b1h, b1l} rows k, k+4 | {b2h, b2l}
        {
            const float2 *Xq = Xs[stage];
            for (int e = tid; e < KT * 32; e += blockDim.x) {
                const int kt = e >> 5, ln = e & 31;
                const int gg = ln >> 2, tt = ln & 3;
                const int v = gg & 3, mx = v >> 1, my = v & 1;   // column gg: Re (gg < 4) / Im of vector v
                const bool im = gg >= 4;
                const bool present = mx < nkx && my < nky;
                uint32_t w[8];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int k = 8 * kt + tt + 4 * h;
                    float2 x = make_float2(0.f, 0.f);
                    if (k < R && present) {
                        x = Xq[(size_t)v * B + k];
                        const int comp = k / d.nz;
                        if ((comp == 0 && mx) || (comp == 1 && my)) x = make_float2(-x.x, -x.y);
                    }
                    const float b1 = im ? x.y : x.x;    // [Xr | Xi]
                    const float b2 = im ? x.x : -x.y;   // [-Xi | Xr]
                    split_tf32(b1, w[h], w[2 + h]);
                    split_tf32(b2, w[4 + h], w[6 + h]);
                }
                BF[(size_t)e * 2] = make_uint4(w[0], w[1], w[2], w[3]);
                BF[(size_t)e * 2 + 1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
        }
        __syncthreads();
        if (active) {
            const float2 *Gq = Gs[stage];
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            const uint2 *tab = TAB + (size_t)mt * KT * 32 + lane;
#pragma unroll 2
            for (int kt = 0; kt < KT; kt++) {
                const uint2 te = tab[(size_t)kt * 32];
                const uint32_t ix[4] = {te.x & 0xffffu, te.x >> 16, te.y & 0xffffu, te.y >> 16};
                uint32_t arh[4], arl[4], aih[4], ail[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    float2 gv = Gq[ix[e] & 0x7fffu];
                    const float sg = (ix[e] & 0x8000u) ? -1.f : 1.f;
                    split_tf32(sg * gv.x, arh[e], arl[e]);
                    split_tf32(sg * gv.y, aih[e], ail[e]);
                }
                const uint4 p1 = BF[((size_t)kt * 32 + lane) * 2], p2 = BF[((size_t)kt * 32 + lane) * 2 + 1];
                mma_tf32(acc, arh, p1.x, p1.y);
                mma_tf32(acc, arh, p1.z, p1.w);
                mma_tf32(acc, arl, p1.x, p1.y);
                mma_tf32(acc, aih, p2.x, p2.y);
                mma_tf32(acc, aih, p2.z, p2.w);
                mma_tf32(acc, ail, p2.x, p2.y);
            }
            // C: rows g, g+8; columns 2t, 2t+1 (t < 2: Re of v = 2t, 2t+1; t >= 2: Im of v = 2t-4, 2t-3)
            float o[4];
#pragma unroll
            for (int c = 0; c < 4; c++) o[c] = __shfl_xor_sync(0xffffffffu, acc[c], 2);
            if (t < 2) {
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const int row = 16 * mt + g + 8 * (c >> 1);
                    const int v = 2 * t + (c & 1);
                    const int mx = v >> 1, my = v & 1;
                    if (row < R && mx < nkx && my < nky) {
                        float2 y = make_float2(acc[c], o[c]);
                        const int comp = row / d.nz;
                        if ((comp == 0 && mx) || (comp == 1 && my)) y = make_float2(-y.x, -y.y);
                        const long pt = (long)(mx ? 2 * d.nx - a : a) * n1 + (my ? 2 * d.ny - bq : bq);
                        buf[pt * B + row] = y;
                    }
                }
            }
        }
        __syncthreads();
        // the stage is free: fetch the point two steps ahead into it
        if (tid == 0 && q + 2L * gridDim.x < Q) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q + 2L * gridDim.x, stage);
        }
    }
}

}  // namespace

size_t contract_mma_smem(int nz, int nrhs) {
    (void)nrhs;
    const MmaGeom m = mma_geom(nz);
    const size_t B = (size_t)m.R;
    return 2 * (size_t)m.Bpad * 8 + 2 * 4 * B * 8 + (size_t)m.MT * m.KT * 32 * 8 + (size_t)m.KT * 32 * 32;
}

bool contract_mma_fits(int nz, int nrhs) {
    if (nrhs != 1) return false;
    const MmaGeom m = mma_geom(nz);
    if (nz % 2 != 0) return false;       // 16-byte bulk copies of the right-hand sides
    if (m.Bs >= 0x7fff) return false;     // 15-bit offsets
    if (m.MT * 32 > 320) return false;
    return contract_mma_smem(nz, nrhs) <= 226 * 1024;
}

void launch_contract_mma(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s) {
    static int nsm = 0;
    if (!nsm) EGX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
    const MmaGeom m = mma_geom(d.nz);
    GreenDims gd{d.nx, d.ny, d.nz};
    const size_t sm = contract_mma_smem(d.nz, d.nrhs);
    const unsigned grid = (unsigned)std::min<long>(gd.Q(), nsm);
    const int thr = std::max(64, m.MT * 32);
    raise_smem_limit((const void *)k_contract_mma, sm);
    k_contract_mma<<<grid, thr, sm, s>>>(buf, G, d, err);
    EGX_CUDA(cudaGetLastError());
}

}  // namespace egx
