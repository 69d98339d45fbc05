// Block contraction of the CIE operator in complex64
// (ConvolutionOperator.ApplyGreenTensorAlongZ, ConvolutionOperator.cs:274-327),
// persistent CTAs with TMA-staged Green blocks.
//
// Algebra: the four spectral points p sharing a stored quadrant block have the
// operators D_p G D_p, D_p = diag(dx, dy, 1) per component (dx = -1 on the
// mirrored-x point, dy likewise), since xy, xz, yz carry exactly these
// parities. With X'_v = D_p X_v, all 4*NRHS vectors are right-hand sides of
// one (3nz x 3nz) complex matrix G: Y'_v = G X'_v and Y_v = D_p Y'_v.
//
// Data path per stored point (one CTA per SM, loop over points):
//   TMA bulk copy (cp.async.bulk, mbarrier complete_tx) of the packed block
//   into one of two shared-memory stages, issued two points ahead;
//   the right-hand sides are read one point ahead into registers and stored
//   pre-signed (X' = D_p X) together with a rotated copy (-Im, Re);
//   each thread owns two rows r = (component, i) and four vectors and walks a
//   quarter of the columns k = (component, j) (NRHS = 1; with NRHS = 2 the
//   four groups are two vector halves x two column halves), reading G in its
//   stored form -- packed symmetric (rc + tr(tr+1)/2) or row-padded
//   (rc*(nz+1) + tr) -- with one lane per row, which is bank-conflict free for
//   both layouts; a complex multiply-add is two packed fma.rn.f32x2;
//   the groups meet through shared memory.
// Waits on the mbarriers are bounded (2 s); on expiry the kernel records
// EGX_ERR_TIMEOUT in *err and returns.
#include <cstdint>

#include "egx_operator.cuh"
#include "egx_wait.cuh"

namespace egx {

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Bounded wait: true when the phase completed within the limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns) {
    return mbar_wait_ns(smem_addr(bar), parity, limit_ns);
}

// One bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
// from global memory into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// acc += (a, a) * (b0, b1), packed
__device__ __forceinline__ void fma2(unsigned long long &acc, unsigned long long aa, unsigned long long b) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(aa), "l"(b));
}
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    return ((unsigned long long)__float_as_uint(hi) << 32) | (unsigned long long)__float_as_uint(lo);
}
__device__ __forceinline__ float2 unpack2(unsigned long long v) {
    return make_float2(__uint_as_float((unsigned)(v & 0xffffffffull)), __uint_as_float((unsigned)(v >> 32)));
}

constexpr uint64_t kWaitNs = 2000000000ull;

// offset of G(row (co, i), column (ci, j)) in the stored block and its sign
struct RowBlock {
    int form;   // 0 packed symmetric, 1 row-padded A[i][j], 2 transposed -A[j][i]
    int base;
};

__device__ __forceinline__ RowBlock row_block(int co, int ci, int S, int A) {
    RowBlock rb;
    if (co < 2 && ci < 2) {
        rb.form = 0;
        rb.base = (co == 0 && ci == 0) ? 0 : ((co == 1 && ci == 1) ? 2 * S : S);
    } else if (co == 2 && ci == 2) {
        rb.form = 0;
        rb.base = 3 * S;
    } else if (ci == 2) {
        rb.form = 1;
        rb.base = 4 * S + co * A;
    } else {
        rb.form = 2;
        rb.base = 4 * S + ci * A;
    }
    return rb;
}

template <int NRHS>
__global__ void __launch_bounds__(384, 1)
    k_contract_c64(float2 *buf, const float2 *__restrict__ G, const OpDims d, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int status;
    constexpr int V = 4 * NRHS;          // vectors per point
    constexpr int JP = NRHS == 1 ? 4 : 2;  // column parts
    const int nz = d.nz;
    const int R = 3 * nz;
    const int H = (R + 1) / 2;           // row pairs
    const int S = nz * (nz + 1) / 2, lda = nz + 1, A = nz * lda, Bs = 4 * S + 2 * A;
    float2 *Gs0 = reinterpret_cast<float2 *>(smem_raw);
    float2 *Gs1 = Gs0 + Bs;
    float2 *X = Gs1 + Bs;               // [R][V]  D_p X
    float2 *X2 = X + (size_t)R * V;     // [R][V]  (-Im, Re) of D_p X
    float2 *P = X2 + (size_t)R * V;     // [JP][R][V] partial sums
    const int tid = threadIdx.x, nthr = blockDim.x;
    const long Q = (long)(d.nx + 1) * (d.ny + 1);
    const int n1 = 2 * d.ny;
    const uint32_t bytes = (uint32_t)Bs * sizeof(float2);

    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        status = 0;
    }
    __syncthreads();
    long q = blockIdx.x;
    if (tid == 0) {
        if (q < Q) tma_load_1d(Gs0, G + q * Bs, bytes, &bars[0]);
        if (q + gridDim.x < Q) tma_load_1d(Gs1, G + (q + gridDim.x) * Bs, bytes, &bars[1]);
    }
    // right-hand sides of one point, t = k*V + v, already multiplied by D_p
    const int nxv = (R * V + nthr - 1) / nthr;  // <= 4 by construction
    float2 xr[4];
    auto load_x = [&](long qq) {
        const int a = (int)(qq / (d.ny + 1)), bq = (int)(qq - (long)a * (d.ny + 1));
        const int nkx = (a == 0 || a == d.nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == d.ny) ? 1 : 2;
#pragma unroll
        for (int m = 0; m < 4; m++) {
            int t = tid + m * nthr;
            float2 val = make_float2(0.f, 0.f);
            if (m < nxv && t < R * V && qq < Q) {
                int k = t / V, v = t - (t / V) * V;
                int p = v / NRHS, rhs = v - p * NRHS;
                int mx = p >> 1, my = p & 1;
                if (mx < nkx && my < nky) {
                    long pt = (long)(mx ? 2 * d.nx - a : a) * n1 + (my ? 2 * d.ny - bq : bq);
                    val = buf[pt * d.B + rhs * R + k];
                    int comp = k / nz;
                    if ((comp == 0 && mx) || (comp == 1 && my)) val = make_float2(-val.x, -val.y);
                }
            }
            xr[m] = val;
        }
    };
    load_x(q);

    // this thread: rows r0 = pr, r1 = pr + H (if < R); group g. Groups are
    // whole warps so that every warp walks one column range.
    const int GT = ((H + 31) / 32) * 32;
    const int g = tid / GT;
    const int pr = tid - g * GT;
    const bool active = g < 4 && pr < H;
    const int vg = NRHS == 1 ? 0 : (g >> 1);       // vector half
    const int jpart = NRHS == 1 ? g : (g & 1);     // column part
    const int v0 = 4 * vg;
    const int jq = (nz + JP - 1) / JP;
    const int j0 = min(jpart * jq, nz), j1 = min(j0 + jq, nz);
    int rows[2] = {active ? pr : 0, pr + H};
    const bool has1 = active && rows[1] < R;
    if (!has1) rows[1] = rows[0];
    int co[2], ii[2], Ti[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        co[h] = rows[h] / nz;
        ii[h] = rows[h] - co[h] * nz;
        Ti[h] = ii[h] * (ii[h] + 1) / 2;
    }

    for (int it = 0; q < Q; q += gridDim.x, it++) {
        const int stage = it & 1;
        const uint32_t parity = (it >> 1) & 1;
        // stash the right-hand sides of this point, fetch the next ones
#pragma unroll
        for (int m = 0; m < 4; m++) {
            int t = tid + m * nthr;
            if (m < nxv && t < R * V) {
                X[t] = xr[m];
                X2[t] = make_float2(-xr[m].y, xr[m].x);
            }
        }
        load_x(q + gridDim.x);
        if (tid == 0) {
            if (!mbar_wait_bounded(&bars[stage], parity, kWaitNs)) status = 1;
        }
        __syncthreads();
        if (status) {
            if (tid == 0) {
                atomicExch(err, EGX_ERR_TIMEOUT);
                mbar_wait_bounded(&bars[stage ^ 1], ((it + 1) >> 1) & 1, kWaitNs);
            }
            return;
        }
        mbar_wait_bounded(&bars[stage], parity, kWaitNs);  // acquire for every thread (already complete)
        const float2 *Gs = stage ? Gs1 : Gs0;
        const int a = (int)(q / (d.ny + 1)), bq = (int)(q - (long)a * (d.ny + 1));
        const int nkx = (a == 0 || a == d.nx) ? 1 : 2;
        const int nky = (bq == 0 || bq == d.ny) ? 1 : 2;
        if (active) {
            unsigned long long acc[2][4];
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int u = 0; u < 4; u++) acc[h][u] = 0ull;
#pragma unroll 1
            for (int ci = 0; ci < 3; ci++) {
                const RowBlock b0 = row_block(co[0], ci, S, A), b1 = row_block(co[1], ci, S, A);
                const float s0 = b0.form == 2 ? -1.f : 1.f, s1 = b1.form == 2 ? -1.f : 1.f;
                const float4 *Xc = reinterpret_cast<const float4 *>(X + (size_t)(ci * nz) * V + v0);
                const float4 *X2c = reinterpret_cast<const float4 *>(X2 + (size_t)(ci * nz) * V + v0);
                int tj = j0 * (j0 + 1) / 2;
#pragma unroll 2
                for (int j = j0; j < j1; j++) {
                    int o0, o1;
                    o0 = b0.form == 0 ? b0.base + (ii[0] <= j ? ii[0] + tj : j + Ti[0])
                                      : (b0.form == 1 ? b0.base + ii[0] * lda + j : b0.base + j * lda + ii[0]);
                    o1 = b1.form == 0 ? b1.base + (ii[1] <= j ? ii[1] + tj : j + Ti[1])
                                      : (b1.form == 1 ? b1.base + ii[1] * lda + j : b1.base + j * lda + ii[1]);
                    tj += j + 1;
                    const float2 g0 = Gs[o0], g1 = Gs[o1];
                    const unsigned long long g0r = pack2(s0 * g0.x, s0 * g0.x), g0i = pack2(s0 * g0.y, s0 * g0.y);
                    const unsigned long long g1r = pack2(s1 * g1.x, s1 * g1.x), g1i = pack2(s1 * g1.y, s1 * g1.y);
                    const float4 xa = Xc[(size_t)j * (V / 2)], xb = Xc[(size_t)j * (V / 2) + 1];
                    const float4 ya = X2c[(size_t)j * (V / 2)], yb = X2c[(size_t)j * (V / 2) + 1];
                    const unsigned long long xv[4] = {pack2(xa.x, xa.y), pack2(xa.z, xa.w), pack2(xb.x, xb.y),
                                                      pack2(xb.z, xb.w)};
                    const unsigned long long yv[4] = {pack2(ya.x, ya.y), pack2(ya.z, ya.w), pack2(yb.x, yb.y),
                                                      pack2(yb.z, yb.w)};
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        fma2(acc[0][u], g0r, xv[u]);
                        fma2(acc[0][u], g0i, yv[u]);
                        fma2(acc[1][u], g1r, xv[u]);
                        fma2(acc[1][u], g1i, yv[u]);
                    }
                }
            }
            // partial sums of this column part
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (h == 1 && !has1) break;
#pragma unroll
                for (int u = 0; u < 4; u++) P[((size_t)jpart * R + rows[h]) * V + v0 + u] = unpack2(acc[h][u]);
            }
        }
        __syncthreads();
        // this stage is free again: fetch the point two steps ahead into it
        if (tid == 0 && q + 2L * gridDim.x < Q) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tma_load_1d(stage ? Gs1 : Gs0, G + (q + 2L * gridDim.x) * Bs, bytes, &bars[stage]);
        }
        for (int t = tid; t < R * V; t += nthr) {
            const int rr = t / V, v = t - (t / V) * V;
            const int p = v / NRHS, rhs = v - p * NRHS;
            const int mx = p >> 1, my = p & 1;
            if (mx < nkx && my < nky) {
                float2 y = P[t];
#pragma unroll
                for (int jp = 1; jp < JP; jp++) {
                    const float2 o = P[(size_t)jp * R * V + t];
                    y.x += o.x;
                    y.y += o.y;
                }
                const int c = rr / nz;
                if ((c == 0 && mx) || (c == 1 && my)) y = make_float2(-y.x, -y.y);
                long pt = (long)(mx ? 2 * d.nx - a : a) * n1 + (my ? 2 * d.ny - bq : bq);
                buf[pt * d.B + rhs * R + rr] = y;
            }
        }
    }
}

}  // namespace

size_t contract_c64_smem(int nz, int nrhs) {
    GreenDims gd{1, 1, nz};
    const size_t R = 3 * (size_t)nz, V = 4 * (size_t)nrhs, JP = nrhs == 1 ? 4 : 2;
    return 2 * (size_t)gd.Bs() * sizeof(float2) + 2 * R * V * sizeof(float2) + JP * R * V * sizeof(float2);
}

static int contract_threads(int nz) {
    const int H = (3 * nz + 1) / 2;
    return 4 * (((H + 31) / 32) * 32);
}

bool contract_c64_fits(int nz, int nrhs) {
    const int R = 3 * nz;
    const int thr = contract_threads(nz);
    if (nrhs != 1 && nrhs != 2) return false;
    if (thr > 384) return false;
    if ((R * 4 * nrhs + thr - 1) / thr > 4) return false;
    return contract_c64_smem(nz, nrhs) <= 225 * 1024;
}

void launch_contract_c64(float2 *buf, const float2 *G, const OpDims &d, int *err, cudaStream_t s) {
    static int nsm = 0;
    if (!nsm) EGX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
    GreenDims gd{d.nx, d.ny, d.nz};
    const int thr = contract_threads(d.nz);
    const size_t sm = contract_c64_smem(d.nz, d.nrhs);
    const unsigned grid = (unsigned)std::min<long>(gd.Q(), nsm);
    if (d.nrhs == 1) {
        raise_smem_limit((const void *)k_contract_c64<1>, sm);
        k_contract_c64<1><<<grid, thr, sm, s>>>(buf, G, d, err);
    } else {
        raise_smem_limit((const void *)k_contract_c64<2>, sm);
        k_contract_c64<2><<<grid, thr, sm, s>>>(buf, G, d, err);
    }
    EGX_CUDA(cudaGetLastError());
}

}  // namespace egx
