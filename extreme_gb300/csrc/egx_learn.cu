// Learned flexible preconditioner: a spectral network z = N(v) used as the
// right preconditioner of the complex64 inner FGMRES of the mixed form (the
// RightPreconditionerRequest plug point, Extreme.Fgmres/FlexibleGmresSolver.cs:24-36),
// trained on (residual v, GMRES-preconditioner output) pairs that the solver
// generates, with the forward and backward passes on BF16 tensor-core GEMMs
// (mma.sync m16n8k16, FP32 accumulation) and Adam, all in this file.
//
// Network, per sample on the nx x ny x nz anomaly mesh (depth is a spatial
// axis), channels last; on the device sample b is stored as nz slices, row
// ((b nz + z) nx + x) ny + y of every activation:
//   input  X0[z][x][y][7]: Re of the 3 components of v / rms(v), Im of the
//          3 components, log10(omega mu0 sigma dx dy) of the cell
//   lift   H0 = X0 P + bP                                  (7 -> width)
//   L layers  H_{l+1} = act(S_l(H_l) + H_l Wp_l + Dz_l H_l + b_l),
//          act = GELU (tanh form) on all but the last,
//          S_l = Bx (Wm_l . (Bx^T H[z] By)) By^T per depth slice: 16 x 16
//          retained lateral modes in a real Fourier basis (cos 0..7, sin 1..8
//          per direction, unit columns), a width x width channel mixing per
//          mode shared by all depths; Dz_l: an nz x nz depth mixing per layer
//   output Out = H_L Q + bQ                                (width -> 6)
//   z = v + rms(v) (Out_Re + i Out_Im); Q starts at zero, so an untrained
//   network is the identity preconditioner.
// Loss per batch: mean over samples of |Out - T|^2 / |T|^2 with T = (z* - v)
// / rms(v) the target correction.
//
// Weights and activations are FP32 in memory; every GEMM converts its
// operands to BF16 on the way into shared memory and accumulates in FP32.
#include <cuda_bf16.h>

#include <cmath>
#include <random>
#include <vector>

#include "egx_ctx.cuh"
#include "egx_learn.cuh"

namespace egx {

namespace {

constexpr int KM = 16;  // retained modes per lateral direction

// ------------------------------------------------------------------ GEMM
// C[m, n] = alpha sum_k A[m, k] B[k, n] + beta C[m, n], batched over z with
// arbitrary strides (transposes are strides): element (m, k) of batch b at
// A[b a_b + m a_m + k a_k], likewise B (k, n) and C (m, n). With ksplit > 1
// (batch 1) the z index splits K instead and the partial products are added
// to C atomically (C zeroed by the caller): the weight gradients, whose K is
// every row of the batch.
struct GemmArgs {
    int M, N, K, batch, ksplit;
    const float *A;
    long a_m, a_k, a_b;
    const float *B;
    long b_k, b_n, b_b;
    float *C;
    long c_m, c_n, c_b;
    float alpha, beta;
};

constexpr int GBM = 64, GBN = 64, GBK = 32, GPAD = 8;

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// 128 threads: 2 x 2 warps, each a 32 x 32 sub-tile (2 m16 x 4 n8)
__global__ void __launch_bounds__(128) k_gemm_bf16(const GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[GBM][GBK + GPAD];  // (m, k)
    __shared__ __align__(16) __nv_bfloat16 Bs[GBN][GBK + GPAD];  // (n, k)
    const int b = g.ksplit > 1 ? 0 : blockIdx.z;
    int kbeg = 0, kend = g.K;
    if (g.ksplit > 1) {
        const int kc = ((g.K + g.ksplit - 1) / g.ksplit + GBK - 1) / GBK * GBK;
        kbeg = blockIdx.z * kc;
        kend = min(g.K, kbeg + kc);
    }
    const float *A = g.A + (long)b * g.a_b;
    const float *B = g.B + (long)b * g.b_b;
    float *C = g.C + (long)b * g.c_b;
    // one CTA per (m, n) tile on grid x (rows of the pointwise GEMMs run to
    // millions, past grid y's limit)
    const int ntn = (g.N + GBN - 1) / GBN;
    const int m0 = (int)(blockIdx.x / ntn) * GBM, n0 = (int)(blockIdx.x % ntn) * GBN;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int gq = lane >> 2, tq = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[i][j][c] = 0.f;
    // loads run along whichever index is contiguous in memory
    const bool a_kfast = g.a_k == 1 || g.a_m != 1, b_kfast = g.b_k == 1 && g.b_n != 1;
    for (int k0 = kbeg; k0 < kend; k0 += GBK) {
        for (int e = tid; e < GBM * GBK; e += 128) {
            const int m = a_kfast ? e / GBK : e % GBM, k = a_kfast ? e % GBK : e / GBM;
            const int gm = m0 + m, gk = k0 + k;
            As[m][k] = __float2bfloat16_rn((gm < g.M && gk < kend) ? A[gm * g.a_m + gk * g.a_k] : 0.f);
        }
        for (int e = tid; e < GBN * GBK; e += 128) {
            const int n = b_kfast ? e / GBK : e % GBN, k = b_kfast ? e % GBK : e / GBN;
            const int gn = n0 + n, gk = k0 + k;
            Bs[n][k] = __float2bfloat16_rn((gn < g.N && gk < kend) ? B[gk * g.b_k + gn * g.b_n] : 0.f);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GBK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int r = wm + 16 * i + gq;
                af[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 2 * tq]);
                af[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 2 * tq]);
                af[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 2 * tq + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 2 * tq + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = wn + 8 * j + gq;
                bfr[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + 2 * tq]);
                bfr[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + 2 * tq + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j][0], bfr[j][1]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int m = m0 + wm + 16 * i + gq + 8 * (c >> 1), n = n0 + wn + 8 * j + 2 * tq + (c & 1);
                if (m < g.M && n < g.N) {
                    float *p = C + m * g.c_m + n * g.c_n;
                    const float v = g.alpha * acc[i][j][c];
                    if (g.ksplit > 1)
                        atomicAdd(p, v);
                    else
                        *p = g.beta != 0.f ? v + g.beta * *p : v;
                }
            }
}

void gemm(const GemmArgs &g, cudaStream_t s, long *launches) {
    const long tiles = (long)((g.M + GBM - 1) / GBM) * ((g.N + GBN - 1) / GBN);
    EGX_CHECK(g.M >= 1 && g.N >= 1 && tiles <= 0x7fffffffL && g.batch <= 65535 && (g.ksplit <= 1 || g.batch == 1),
              EGX_ERR_INVALID, "bad GEMM shape");
    dim3 grid((unsigned)tiles, 1, g.ksplit > 1 ? g.ksplit : g.batch);
    k_gemm_bf16<<<grid, 128, 0, s>>>(g);
    EGX_CUDA(cudaGetLastError());
    if (launches) ++*launches;
}

// -------------------------------------------------------------- elementwise
__device__ __forceinline__ float gelu(float x) {
    const float c = 0.7978845608028654f;  // sqrt(2/pi)
    return 0.5f * x * (1.f + tanhf(c * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_d(float x) {
    const float c = 0.7978845608028654f;
    const float u = c * (x + 0.044715f * x * x * x), th = tanhf(u);
    return 0.5f * (1.f + th) + 0.5f * x * (1.f - th * th) * c * (1.f + 3.f * 0.044715f * x * x);
}

// pre[r][c] += bias[c]; out = act ? gelu(pre) : pre
__global__ void k_bias_act(float *pre, const float *__restrict__ bias, long rows, int cols, int act, float *out) {
    const long n = rows * cols;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float v = pre[i] + bias[i % cols];
        pre[i] = v;
        out[i] = act ? gelu(v) : v;
    }
}

__global__ void k_gelu_bwd(float *d, const float *__restrict__ pre, long n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        d[i] *= gelu_d(pre[i]);
}

// out[c] = sum_r x[r][c] (out zeroed by the caller)
__global__ void k_colsum(const float *__restrict__ x, long rows, int cols, float *out) {
    const int c = blockIdx.y * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float acc = 0.f;
    for (long r = blockIdx.x; r < rows; r += gridDim.x) acc += x[r * cols + c];
    atomicAdd(out + c, acc);
}

// per-sample sum of |v|^2 over n complex entries (out zeroed by the caller)
__global__ void k_sample_norm2(const float2 *__restrict__ v, long n, double *out) {
    const int b = blockIdx.y;
    double acc = 0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 x = v[(long)b * n + i];
        acc += (double)x.x * x.x + (double)x.y * x.y;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out + b, acc);
}

// scale[b] = 1/rms, rms[b] = sqrt(sum / n) (0 and 0 for a zero vector)
__global__ void k_rms(const double *sum, long n, int batch, float *inv, float *rms) {
    const int b = threadIdx.x;
    if (b >= batch) return;
    const double r = sqrt(sum[b] / (double)n);
    rms[b] = (float)r;
    inv[b] = r > 0 ? (float)(1.0 / r) : 0.f;
}

// X0[row][ch], row = (b nz + z) ncell + cell: Re of the 3 components, Im of
// the 3 components (scaled by inv[b]), the log-conductivity of model
// b % nmodels
__global__ void k_encode(const float2 *__restrict__ v, const float *__restrict__ inv, const float *__restrict__ logsig,
                         int nmodels, long ncell, int nz, int batch, float *X) {
    const long N = ncell * 3 * nz, total = (long)batch * nz * ncell * 7;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % 7);
        const long row = i / 7, cell = row % ncell, s = row / ncell;
        const int z = (int)(s % nz), b = (int)(s / nz);
        float val;
        if (ch < 6) {
            const int c = ch % 3;
            const float2 x = v[(long)b * N + (cell * 3 + c) * nz + z];
            val = (ch < 3 ? x.x : x.y) * inv[b];
        } else {
            val = logsig[((long)(b % nmodels) * ncell + cell) * nz + z];
        }
        X[i] = val;
    }
}

// the target in the output layout T[row][6]: Re | Im of t / rms(v)
__global__ void k_encode_target(const float2 *__restrict__ t, const float *__restrict__ inv, long ncell, int nz,
                                int batch, float *T) {
    const long N = ncell * 3 * nz, total = (long)batch * nz * ncell * 6;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % 6), c = ch % 3;
        const long row = i / 6, cell = row % ncell, s = row / ncell;
        const int z = (int)(s % nz), b = (int)(s / nz);
        const float2 x = t[(long)b * N + (cell * 3 + c) * nz + z];
        T[i] = (ch < 3 ? x.x : x.y) * inv[b];
    }
}

// z = v + rms (Out_Re + i Out_Im), back in the anomaly layout
__global__ void k_decode(const float2 *__restrict__ v, const float *__restrict__ rms, const float *__restrict__ out,
                         long ncell, int nz, int batch, float2 *z) {
    const long N = ncell * 3 * nz, total = (long)batch * N;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / N);
        const long e = i - (long)b * N, cell = e / (3 * nz);
        const int c = (int)((e / nz) % 3), zz = (int)(e % nz);
        const long row = ((long)b * nz + zz) * ncell + cell;
        const float r = rms[b];
        const float2 x = v[i];
        z[i] = make_float2(x.x + r * out[row * 6 + c], x.y + r * out[row * 6 + 3 + c]);
    }
}

// per-sample |Out - T|^2 and |T|^2 (zeroed by the caller): e2[b], t2[b]
__global__ void k_loss_sums(const float *__restrict__ out, const float *__restrict__ T, long per_sample, double *e2,
                            double *t2) {
    const int b = blockIdx.y;
    double ae = 0, at = 0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < per_sample; i += (long)gridDim.x * blockDim.x) {
        const long j = (long)b * per_sample + i;
        const double d = (double)out[j] - T[j];
        ae += d * d;
        at += (double)T[j] * T[j];
    }
    for (int o = 16; o > 0; o >>= 1) {
        ae += __shfl_xor_sync(0xffffffffu, ae, o);
        at += __shfl_xor_sync(0xffffffffu, at, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(e2 + b, ae);
        atomicAdd(t2 + b, at);
    }
}

// dOut = 2 (Out - T) / (batch |T_b|^2)
__global__ void k_loss_grad(const float *__restrict__ out, const float *__restrict__ T, const double *t2,
                            long per_sample, int batch, float *dout) {
    const long total = per_sample * batch;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / per_sample);
        const double den = t2[b] > 0 ? (double)batch * t2[b] : 1.0;
        dout[i] = (float)(2.0 * ((double)out[i] - T[i]) / den);
    }
}

__global__ void k_adam(float *p, const float *__restrict__ g, float *m, float *v, long n, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

unsigned blocks_for(long n) { return (unsigned)std::min<long>((n + 255) / 256, 152L * 32); }

}  // namespace

}  // namespace egx

// -------------------------------------------------------------------- network
struct egx_net {
    int nx = 0, ny = 0, nz = 0, W = 0, L = 0, cin = 0, cout = 0;
    long ncell = 0, n_params = 0;
    int nmodels = 0;  // conductivity models set (sample b uses model b % nmodels)
    int tc = 1;       // pointwise GEMMs on the tcgen05 kernel (egx_net_use_tcgen05)
    int *err = nullptr;  // the context's device error flag
    long off_P = 0, off_bP = 0, off_Q = 0, off_bQ = 0;
    std::vector<long> off_Wm, off_Wp, off_Dz, off_b;
    egx::DevBuf params, grads, adam_m, adam_v, bx, by, logsig;
    int step = 0, cap = 0;
    // activations of the last forward pass (batch <= cap)
    egx::DevBuf X0, Out, T, dOut, U1, V, S1, dH, dH2, dS1, dV, dU, dU1, sums, scal;
    egx::DevBuf H[9], Pre[8], U[8];  // layers <= 8
    float *p(long off) { return params.as<float>() + off; }
    float *gr(long off) { return grads.as<float>() + off; }
};

namespace egx {

namespace {

void ensure_batch(egx_net *n, int batch) {
    if (batch <= n->cap) return;
    const long S = (long)batch * n->nz;  // depth slices of the batch
    const long rows = S * n->ncell, W = n->W;
    n->X0.ensure(rows * n->cin * sizeof(float));
    n->Out.ensure(rows * n->cout * sizeof(float));
    n->T.ensure(rows * n->cout * sizeof(float));
    n->dOut.ensure(rows * n->cout * sizeof(float));
    for (int l = 0; l <= n->L; l++) n->H[l].ensure(rows * W * sizeof(float));
    for (int l = 0; l < n->L; l++) {
        n->Pre[l].ensure(rows * W * sizeof(float));
        n->U[l].ensure((size_t)S * KM * KM * W * sizeof(float));
    }
    n->U1.ensure((size_t)S * KM * n->ny * W * sizeof(float));
    n->V.ensure((size_t)S * KM * KM * W * sizeof(float));
    n->S1.ensure((size_t)S * n->nx * KM * W * sizeof(float));
    n->dH.ensure(rows * W * sizeof(float));
    n->dH2.ensure(rows * W * sizeof(float));
    n->dS1.ensure((size_t)S * n->nx * KM * W * sizeof(float));
    n->dV.ensure((size_t)S * KM * KM * W * sizeof(float));
    n->dU.ensure((size_t)S * KM * KM * W * sizeof(float));
    n->dU1.ensure((size_t)S * KM * n->ny * W * sizeof(float));
    n->sums.ensure(3 * (size_t)batch * sizeof(double));
    n->scal.ensure(2 * (size_t)batch * sizeof(float));
    n->cap = batch;
}

GemmArgs ga(int M, int N, int K, int batch, const float *A, long a_m, long a_k, long a_b, const float *B, long b_k,
            long b_n, long b_b, float *C, long c_m, long c_n, long c_b, float beta = 0.f) {
    GemmArgs g;
    g.M = M, g.N = N, g.K = K, g.batch = batch;
    g.A = A, g.a_m = a_m, g.a_k = a_k, g.a_b = a_b;
    g.B = B, g.b_k = b_k, g.b_n = b_n, g.b_b = b_b;
    g.C = C, g.c_m = c_m, g.c_n = c_n, g.c_b = c_b;
    g.alpha = 1.f, g.beta = beta, g.ksplit = 1;
    return g;
}

// a weight gradient: K = all rows, split over CTAs, added atomically
GemmArgs wgrad(GemmArgs g) {
    g.ksplit = (int)std::min<long>(256, std::max<long>(1, (long)g.K / 512));
    return g;
}

// a pointwise GEMM C[M x N] (+)= A[M x K] B (B by strides; K, N <= 32) on
// the tcgen05 kernel (egx_learn_tc.cu), or on the warp-level kernel when the
// network's tcgen05 path is off or the width exceeds 32
void pw(egx_net *n, int M, int K, const float *A, const float *B, long b_k, long b_n, int N, float *C, bool acc,
        cudaStream_t s, long *launches) {
    if (n->tc && pw_gemm_tc_fits(K, N)) {
        pw_gemm_tc(A, M, K, B, b_k, b_n, N, C, acc, n->err, s);
        if (launches) ++*launches;
    } else {
        gemm(ga(M, N, K, 1, A, K, 1, 0, B, b_k, b_n, 0, C, N, 1, 0, acc ? 1.f : 0.f), s, launches);
    }
}

// X0 (encoded) -> Out; keeps the activations for backward. The B samples
// are B nz depth slices for the lateral operations.
void forward(egx_net *n, int B, cudaStream_t s, long *launches) {
    const int nx = n->nx, ny = n->ny, W = n->W, nz = n->nz;
    const int S = B * nz;
    const long rows = (long)S * n->ncell, slab = n->ncell * W;
    const float *bx = n->bx.as<float>(), *by = n->by.as<float>();
    pw(n, (int)rows, n->cin, n->X0.as<float>(), n->p(n->off_P), W, 1, W, n->H[0].as<float>(), false, s, launches);
    k_bias_act<<<blocks_for(rows * W), 256, 0, s>>>(n->H[0].as<float>(), n->p(n->off_bP), rows, W, 0,
                                                     n->H[0].as<float>());
    for (int l = 0; l < n->L; l++) {
        const float *Hl = n->H[l].as<float>();
        float *U1 = n->U1.as<float>(), *Ul = n->U[l].as<float>(), *V = n->V.as<float>(), *S1 = n->S1.as<float>();
        float *Pre = n->Pre[l].as<float>();
        // U1[s] = Bx^T H[s]                     (KM x ny W) per depth slice s
        gemm(ga(KM, ny * W, nx, S, bx, 1, KM, 0, Hl, (long)ny * W, 1, (long)nx * ny * W, U1, (long)ny * W, 1,
                (long)KM * ny * W),
             s, launches);
        // U[s, i] = By^T U1[s, i]              (KM x W)
        gemm(ga(KM, W, ny, S * KM, by, 1, KM, 0, U1, W, 1, (long)ny * W, Ul, W, 1, (long)KM * W), s, launches);
        // V[:, mode] = U[:, mode] Wm[mode]      (S x W) per mode
        gemm(ga(S, W, W, KM * KM, Ul, (long)KM * KM * W, 1, W, n->p(n->off_Wm[l]), W, 1, (long)W * W, V,
                (long)KM * KM * W, 1, W),
             s, launches);
        // S1[s] = Bx V[s]                       (nx x KM W)
        gemm(ga(nx, KM * W, KM, S, bx, KM, 1, 0, V, (long)KM * W, 1, (long)KM * KM * W, S1, (long)KM * W, 1,
                (long)nx * KM * W),
             s, launches);
        // Pre[s, x] = By S1[s, x]               (ny x W)
        gemm(ga(ny, W, KM, S * nx, by, KM, 1, 0, S1, W, 1, (long)KM * W, Pre, W, 1, (long)ny * W), s, launches);
        // Pre += H Wp
        pw(n, (int)rows, W, Hl, n->p(n->off_Wp[l]), W, 1, W, Pre, true, s, launches);
        // Pre[b, z] += sum_z' Dz[z, z'] H[b, z']   (nz x ncell W) per sample
        gemm(ga(nz, (int)slab, nz, B, n->p(n->off_Dz[l]), nz, 1, 0, Hl, slab, 1, (long)nz * slab, Pre, slab, 1,
                (long)nz * slab, 1.f),
             s, launches);
        k_bias_act<<<blocks_for(rows * W), 256, 0, s>>>(Pre, n->p(n->off_b[l]), rows, W, l < n->L - 1 ? 1 : 0,
                                                         n->H[l + 1].as<float>());
        if (launches) ++*launches;
    }
    pw(n, (int)rows, W, n->H[n->L].as<float>(), n->p(n->off_Q), n->cout, 1, n->cout, n->Out.as<float>(), false, s,
       launches);
    k_bias_act<<<blocks_for(rows * n->cout), 256, 0, s>>>(n->Out.as<float>(), n->p(n->off_bQ), rows, n->cout, 0,
                                                           n->Out.as<float>());
    if (launches) *launches += 2;
    EGX_CUDA(cudaGetLastError());
}

void colsum(const float *x, long rows, int cols, float *out, cudaStream_t s, long *launches) {
    dim3 grid((unsigned)std::min<long>(rows, 1024), (cols + 127) / 128);
    k_colsum<<<grid, 128, 0, s>>>(x, rows, cols, out);
    if (launches) ++*launches;
}

// dOut -> grads (zeroed here)
void backward(egx_net *n, int B, cudaStream_t s, long *launches) {
    const int nx = n->nx, ny = n->ny, W = n->W, nz = n->nz;
    const int S = B * nz;
    const long rows = (long)S * n->ncell, slab = n->ncell * W;
    const float *bx = n->bx.as<float>(), *by = n->by.as<float>();
    EGX_CUDA(cudaMemsetAsync(n->grads.p, 0, n->n_params * sizeof(float), s));
    float *dOut = n->dOut.as<float>();
    // dQ = H_L^T dOut, dbQ, dH = dOut Q^T
    gemm(wgrad(ga(W, n->cout, (int)rows, 1, n->H[n->L].as<float>(), 1, W, 0, dOut, n->cout, 1, 0, n->gr(n->off_Q),
                  n->cout, 1, 0)),
         s, launches);
    colsum(dOut, rows, n->cout, n->gr(n->off_bQ), s, launches);
    pw(n, (int)rows, n->cout, dOut, n->p(n->off_Q), 1, n->cout, W, n->dH.as<float>(), false, s, launches);
    for (int l = n->L - 1; l >= 0; l--) {
        float *dPre = n->dH.as<float>(), *dH2 = n->dH2.as<float>();
        const float *Hl = n->H[l].as<float>(), *Ul = n->U[l].as<float>();
        if (l < n->L - 1) {
            k_gelu_bwd<<<blocks_for(rows * W), 256, 0, s>>>(dPre, n->Pre[l].as<float>(), rows * W);
            if (launches) ++*launches;
        }
        colsum(dPre, rows, W, n->gr(n->off_b[l]), s, launches);
        // dWp = H^T dPre; dH2 = dPre Wp^T
        gemm(wgrad(ga(W, W, (int)rows, 1, Hl, 1, W, 0, dPre, W, 1, 0, n->gr(n->off_Wp[l]), W, 1, 0)), s, launches);
        pw(n, (int)rows, W, dPre, n->p(n->off_Wp[l]), 1, W, W, dH2, false, s, launches);
        // spectral branch
        float *dS1 = n->dS1.as<float>(), *dV = n->dV.as<float>(), *dU = n->dU.as<float>(), *dU1 = n->dU1.as<float>();
        gemm(ga(KM, W, ny, S * nx, by, 1, KM, 0, dPre, W, 1, (long)ny * W, dS1, W, 1, (long)KM * W), s, launches);
        gemm(ga(KM, KM * W, nx, S, bx, 1, KM, 0, dS1, (long)KM * W, 1, (long)nx * KM * W, dV, (long)KM * W, 1,
                (long)KM * KM * W),
             s, launches);
        gemm(ga(W, W, S, KM * KM, Ul, 1, (long)KM * KM * W, W, dV, (long)KM * KM * W, 1, W, n->gr(n->off_Wm[l]), W,
                1, (long)W * W),
             s, launches);
        gemm(ga(S, W, W, KM * KM, dV, (long)KM * KM * W, 1, W, n->p(n->off_Wm[l]), 1, W, (long)W * W, dU,
                (long)KM * KM * W, 1, W),
             s, launches);
        gemm(ga(ny, W, KM, S * KM, by, KM, 1, 0, dU, W, 1, (long)KM * W, dU1, W, 1, (long)ny * W), s, launches);
        gemm(ga(nx, ny * W, KM, S, bx, KM, 1, 0, dU1, (long)ny * W, 1, (long)KM * ny * W, dH2, (long)ny * W, 1,
                (long)nx * ny * W, 1.f),
             s, launches);
        // depth mixing: dH2[b, z'] += sum_z Dz[z, z'] dPre[b, z]; dDz[z, z'] =
        // sum over samples and (cell, channel) of dPre[b, z] H[b, z'] (each
        // sample's product added into the gradient)
        gemm(ga(nz, (int)slab, nz, B, n->p(n->off_Dz[l]), 1, nz, 0, dPre, slab, 1, (long)nz * slab, dH2, slab, 1,
                (long)nz * slab, 1.f),
             s, launches);
        for (int b = 0; b < B; b++)
            gemm(wgrad(ga(nz, nz, (int)slab, 1, dPre + (long)b * nz * slab, slab, 1, 0, Hl + (long)b * nz * slab, 1,
                          slab, 0, n->gr(n->off_Dz[l]), nz, 1, 0, 1.f)),
                 s, launches);
        n->dH.swap(n->dH2);
    }
    // dP = X0^T dH0, dbP
    gemm(wgrad(ga(n->cin, W, (int)rows, 1, n->X0.as<float>(), 1, n->cin, 0, n->dH.as<float>(), W, 1, 0,
                  n->gr(n->off_P), W, 1, 0)),
         s, launches);
    colsum(n->dH.as<float>(), rows, W, n->gr(n->off_bP), s, launches);
    EGX_CUDA(cudaGetLastError());
}

// inv/rms of v per sample into n->scal; X0 from v
void encode(egx_net *n, const float2 *v, int B, cudaStream_t s, long *launches) {
    const long N = n->ncell * 3 * n->nz;
    double *sums = n->sums.as<double>();
    float *inv = n->scal.as<float>(), *rms = inv + B;
    EGX_CUDA(cudaMemsetAsync(sums, 0, B * sizeof(double), s));
    k_sample_norm2<<<dim3((unsigned)std::min<long>((N + 255) / 256, 512), B), 256, 0, s>>>(v, N, sums);
    k_rms<<<1, 64, 0, s>>>(sums, N, B, inv, rms);
    k_encode<<<blocks_for((long)B * n->nz * n->ncell * n->cin), 256, 0, s>>>(
        v, inv, n->logsig.as<float>(), n->nmodels, n->ncell, n->nz, B, n->X0.as<float>());
    if (launches) *launches += 3;
}

void check_batch(int batch) { EGX_CHECK(batch >= 1 && batch <= 64, EGX_ERR_INVALID, "batch must be in [1, 64]"); }

}  // namespace

void net_apply(egx_net *n, const float2 *v, float2 *z, int batch, cudaStream_t s, long *launches) {
    check_batch(batch);
    EGX_CHECK(n->logsig.p, EGX_ERR_STATE, "learned preconditioner has no model (egx_net_set_model)");
    ensure_batch(n, batch);
    encode(n, v, batch, s, launches);
    forward(n, batch, s, launches);
    const float *rms = n->scal.as<float>() + batch;
    k_decode<<<blocks_for((long)batch * n->ncell * 3 * n->nz), 256, 0, s>>>(v, rms, n->Out.as<float>(), n->ncell,
                                                                            n->nz, batch, z);
    EGX_CUDA(cudaGetLastError());
    if (launches) ++*launches;
}

long net_length(const egx_net *n) { return n->ncell * 3 * n->nz; }

}  // namespace egx

using namespace egx;

extern "C" {

int egx_net_create(egx_ctx *ctx, int nx, int ny, int nz, int width, int layers, unsigned seed, egx_net **out) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(out && nx >= 2 && ny >= 2 && nz >= 1 && width >= 8 && width <= 256 && layers >= 1 && layers <= 8,
                  EGX_ERR_INVALID, "bad network dimensions");
        set_device(ctx);
        auto n = std::unique_ptr<egx_net>(new egx_net());
        n->nx = nx, n->ny = ny, n->nz = nz, n->W = width, n->L = layers;
        n->err = ctx->errflag.as<int>();
        n->cin = 7, n->cout = 6, n->ncell = (long)nx * ny;
        long off = 0;
        auto take = [&](long k) {
            const long o = off;
            off += (k + 3) / 4 * 4;
            return o;
        };
        n->off_P = take((long)n->cin * width);
        n->off_bP = take(width);
        for (int l = 0; l < layers; l++) {
            n->off_Wm.push_back(take((long)KM * KM * width * width));
            n->off_Wp.push_back(take((long)width * width));
            n->off_Dz.push_back(take((long)nz * nz));
            n->off_b.push_back(take(width));
        }
        n->off_Q = take((long)width * n->cout);
        n->off_bQ = take(n->cout);
        n->n_params = off;
        std::vector<float> p(off, 0.f);
        std::mt19937 rng(seed);
        std::normal_distribution<float> nd(0.f, 1.f);
        auto fill = [&](long o, long k, float sd) {
            for (long i = 0; i < k; i++) p[o + i] = sd * nd(rng);
        };
        fill(n->off_P, (long)n->cin * width, 1.f / std::sqrt((float)n->cin));
        for (int l = 0; l < layers; l++) {
            fill(n->off_Wm[l], (long)KM * KM * width * width, 1.f / (float)width);
            fill(n->off_Wp[l], (long)width * width, 1.f / std::sqrt((float)width));
            fill(n->off_Dz[l], (long)nz * nz, 0.5f / std::sqrt((float)nz));
        }
        // Q = 0: the untrained network is the identity preconditioner
        n->params.ensure(off * sizeof(float));
        n->grads.ensure(off * sizeof(float));
        n->adam_m.ensure(off * sizeof(float));
        n->adam_v.ensure(off * sizeof(float));
        EGX_CUDA(cudaMemcpy(n->params.p, p.data(), off * sizeof(float), cudaMemcpyHostToDevice));
        EGX_CUDA(cudaMemset(n->adam_m.p, 0, off * sizeof(float)));
        EGX_CUDA(cudaMemset(n->adam_v.p, 0, off * sizeof(float)));
        // real Fourier bases: cos 0..7, sin 1..8, unit columns
        auto basis = [](int len, DevBuf &dst) {
            std::vector<float> b((size_t)len * KM);
            for (int i = 0; i < KM; i++) {
                double nrm = 0;
                std::vector<double> col(len);
                for (int x = 0; x < len; x++) {
                    const double a = 2.0 * M_PI * x / len;
                    col[x] = i < 8 ? std::cos(i * a) : std::sin((i - 7) * a);
                    nrm += col[x] * col[x];
                }
                nrm = std::sqrt(nrm);
                for (int x = 0; x < len; x++) b[(size_t)x * KM + i] = nrm > 1e-9 ? (float)(col[x] / nrm) : 0.f;
            }
            dst.ensure(b.size() * sizeof(float));
            EGX_CUDA(cudaMemcpy(dst.p, b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice));
        };
        basis(nx, n->bx);
        basis(ny, n->by);
        *out = n.release();
    });
}

int egx_net_free(egx_ctx *ctx, egx_net *net) {
    if (!ctx || !net) return EGX_ERR_INVALID;
    if (ctx->precond_kind == EGX_PRECOND_LEARNED && ctx->precond_user == net) {
        ctx->precond_kind = EGX_PRECOND_GMRES;
        ctx->precond_user = nullptr;
    }
    EGX_GUARD(ctx, {
        set_device(ctx);
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        delete net;
    });
}

long egx_net_size(const egx_net *net) { return net ? net->n_params : -1; }

int egx_net_params(egx_ctx *ctx, egx_net *net, float *host, int set) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(net && host, EGX_ERR_INVALID, "null network or buffer");
        set_device(ctx);
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        if (set)
            EGX_CUDA(cudaMemcpy(net->params.p, host, net->n_params * sizeof(float), cudaMemcpyHostToDevice));
        else
            EGX_CUDA(cudaMemcpy(host, net->params.p, net->n_params * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

int egx_net_set_models(egx_ctx *ctx, egx_net *net, const float *logsig, int count) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(net && logsig && count >= 1 && count <= 64, EGX_ERR_INVALID,
                  "null network or log-conductivity, or count outside 1..64");
        set_device(ctx);
        const size_t bytes = (size_t)count * net->ncell * net->nz * sizeof(float);
        net->logsig.ensure(bytes);
        EGX_CUDA(cudaMemcpyAsync(net->logsig.p, logsig, bytes, cudaMemcpyHostToDevice, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        net->nmodels = count;
    });
}

int egx_net_set_model(egx_ctx *ctx, egx_net *net, const float *logsig) {
    return egx_net_set_models(ctx, net, logsig, 1);
}

int egx_net_loss_grad(egx_ctx *ctx, egx_net *net, const float *v, const float *t, int batch, float *loss, float *grad,
                      int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(net && v && t && loss, EGX_ERR_INVALID, "bad training arguments");
        check_batch(batch);
        EGX_CHECK(net->logsig.p, EGX_ERR_STATE, "learned preconditioner has no model (egx_net_set_model)");
        set_device(ctx);
        const cudaStream_t s = ctx->stream;
        const long N = net->ncell * 3 * net->nz;
        const float2 *dv, *dt;
        if (where == EGX_DEVICE) {
            dv = reinterpret_cast<const float2 *>(v);
            dt = reinterpret_cast<const float2 *>(t);
        } else {
            ctx->xin32.ensure(2 * (size_t)batch * N * sizeof(float2));
            float2 *buf = ctx->xin32.as<float2>();
            EGX_CUDA(cudaMemcpyAsync(buf, v, (size_t)batch * N * sizeof(float2), cudaMemcpyHostToDevice, s));
            EGX_CUDA(cudaMemcpyAsync(buf + (size_t)batch * N, t, (size_t)batch * N * sizeof(float2),
                                     cudaMemcpyHostToDevice, s));
            dv = buf;
            dt = buf + (size_t)batch * N;
        }
        ensure_batch(net, batch);
        encode(net, dv, batch, s, &ctx->launches);
        const float *inv = net->scal.as<float>();
        k_encode_target<<<blocks_for((long)batch * net->nz * net->ncell * net->cout), 256, 0, s>>>(dt, inv, net->ncell, net->nz,
                                                                                         batch, net->T.as<float>());
        forward(net, batch, s, &ctx->launches);
        const long per = (long)net->nz * net->ncell * net->cout;  // one sample's outputs
        double *e2 = net->sums.as<double>() + batch, *t2 = e2 + batch;
        EGX_CUDA(cudaMemsetAsync(e2, 0, 2 * batch * sizeof(double), s));
        k_loss_sums<<<dim3((unsigned)std::min<long>((per + 255) / 256, 512), batch), 256, 0, s>>>(
            net->Out.as<float>(), net->T.as<float>(), per, e2, t2);
        k_loss_grad<<<blocks_for(per * batch), 256, 0, s>>>(net->Out.as<float>(), net->T.as<float>(), t2, per, batch,
                                                            net->dOut.as<float>());
        ctx->launches += 3;
        backward(net, batch, s, &ctx->launches);
        std::vector<double> h(2 * batch);
        EGX_CUDA(cudaMemcpyAsync(h.data(), e2, 2 * batch * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (grad) EGX_CUDA(cudaMemcpyAsync(grad, net->grads.p, net->n_params * sizeof(float), cudaMemcpyDeviceToHost, s));
        EGX_CUDA(cudaStreamSynchronize(s));
        check_device_error(ctx);
        double l = 0;
        for (int b = 0; b < batch; b++) l += h[batch + b] > 0 ? h[b] / h[batch + b] : 0.0;
        *loss = (float)(l / batch);
    });
}

int egx_net_use_tcgen05(egx_ctx *ctx, egx_net *net, int enable) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(net, EGX_ERR_INVALID, "null network");
        net->tc = enable ? 1 : 0;
    });
}

int egx_net_adam(egx_ctx *ctx, egx_net *net, float lr) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(net && lr > 0, EGX_ERR_INVALID, "bad Adam arguments");
        set_device(ctx);
        net->step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float bc1 = 1.f - std::pow(b1, (float)net->step), bc2 = 1.f - std::pow(b2, (float)net->step);
        k_adam<<<blocks_for(net->n_params), 256, 0, ctx->stream>>>(net->params.as<float>(), net->grads.as<float>(),
                                                                   net->adam_m.as<float>(), net->adam_v.as<float>(),
                                                                   net->n_params, lr, b1, b2, 1e-8f, bc1, bc2);
        ctx->launches++;
        EGX_CUDA(cudaGetLastError());
    });
}

int egx_net_apply(egx_ctx *ctx, egx_net *net, const float *v, float *z, int batch, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(net && v && z, EGX_ERR_INVALID, "bad apply arguments");
        set_device(ctx);
        const cudaStream_t s = ctx->stream;
        const long N = net->ncell * 3 * net->nz;
        if (where == EGX_DEVICE) {
            net_apply(net, reinterpret_cast<const float2 *>(v), reinterpret_cast<float2 *>(z), batch, s,
                      &ctx->launches);
        } else {
            check_batch(batch);
            ctx->xin32.ensure(2 * (size_t)batch * N * sizeof(float2));
            float2 *buf = ctx->xin32.as<float2>();
            EGX_CUDA(cudaMemcpyAsync(buf, v, (size_t)batch * N * sizeof(float2), cudaMemcpyHostToDevice, s));
            net_apply(net, buf, buf + (size_t)batch * N, batch, s, &ctx->launches);
            EGX_CUDA(cudaMemcpyAsync(z, buf + (size_t)batch * N, (size_t)batch * N * sizeof(float2),
                                     cudaMemcpyDeviceToHost, s));
        }
        EGX_CUDA(cudaStreamSynchronize(s));
        check_device_error(ctx);
    });
}

}  // extern "C"
