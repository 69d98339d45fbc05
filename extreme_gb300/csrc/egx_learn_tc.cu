// Pointwise GEMMs of the learned preconditioner's network on the fifth-
// generation tensor cores: C[m, n] = sum_k A[m, k] B(k, n) (+ C[m, n] when
// accumulating), A row-major [M x K] FP32 (activations: M = samples x depth
// x lateral cells, K <= 32), B a small weight matrix given by strides
// (K x N, N <= 32), C row-major [M x N] FP32.
//
// One CTA of 128 threads per 128-row tile (grid-stride over tiles): thread t
// owns row t of the tile. The weights are converted to BF16 once per CTA and
// the tile's rows on every iteration, both into shared memory in the
// canonical K-major, no-swizzle core-matrix layout (8 rows x 16 bytes per
// core matrix; 128 bytes between core matrices along K, KP/8 x 128 bytes
// between 8-row groups). One thread issues KP/16 tcgen05.mma kind::f16 (BF16
// operands, FP32 accumulator in tensor memory, M = 128, N = NP), commits
// them to an mbarrier, and every thread reads its row of the accumulator
// back with tcgen05.ld (lane = row). Each CTA holds 32 tensor-memory
// columns; at most 16 CTAs are resident on an SM (2048 threads), so the 512
// columns always suffice and the allocation never waits. The mbarrier wait
// is bounded (2 s, %globaltimer); on expiry the kernel records
// EGX_ERR_TIMEOUT in *err, skips its remaining tiles and frees its tensor
// memory. These GEMMs read and write ~130 bytes per row for ~2 K N flops:
// HBM-bound, so one tile in flight per CTA with many CTAs per SM suffices.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

#include "egx_common.cuh"
#include "egx_learn.cuh"
#include "egx_wait.cuh"

namespace egx {

namespace {

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading (K) and stride (8-row
// group) byte offsets >> 4, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3fff) | ((uint64_t)((lbo >> 4) & 0x3fff) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fff) << 32) | ((uint64_t)1 << 46);
}

// element (r, k) of an R x KP BF16 tile in the core-matrix layout
template <int KP>
__device__ __forceinline__ int cm(int r, int k) {
    return ((r >> 3) * (KP / 8) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

template <int NP>
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, float *v);
template <>
__device__ __forceinline__ void tmem_ld_row<16>(uint32_t t, float *v) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(t)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
template <>
__device__ __forceinline__ void tmem_ld_row<32>(uint32_t t, float *v) {
    tmem_ld_row<16>(t, v);
    tmem_ld_row<16>(t + 16, v + 16);
}

constexpr uint64_t kTcWait = 2000000000ull;

template <int KP, int NP>
__global__ void __launch_bounds__(128) k_pw_tc(const float *__restrict__ A, int M, int K, const float *__restrict__ B,
                                               long b_k, long b_n, int N, float *C, int accumulate, long ntiles,
                                               int *err) {
    __shared__ __align__(1024) __nv_bfloat16 sA[128 * KP];
    __shared__ __align__(1024) __nv_bfloat16 sB[NP * KP];
    __shared__ uint32_t tbase;
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tbase)), "r"(32)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // B^T into the core-matrix layout: row n, column k (zero beyond N, K)
    for (int e = tid; e < NP * KP; e += 128) {
        const int n = e / KP, k = e - n * KP;
        const float b = (n < N && k < K) ? B[k * b_k + n * b_n] : 0.f;
        sB[cm<KP>(n, k)] = __float2bfloat16_rn(b);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t dcol = tbase;
    // F32 accumulate, BF16 A and B, both K-major, N >> 3, M >> 4
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NP >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const uint32_t sa = saddr(sA), sb = saddr(sB);
    uint32_t parity = 0;
    for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long r = tile * 128 + tid;
        // this thread's row, converted to BF16, eight values per 16-byte store
#pragma unroll
        for (int k0 = 0; k0 < KP; k0 += 8) {
            __align__(16) __nv_bfloat16 h[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int k = k0 + j;
                h[j] = __float2bfloat16_rn((r < M && k < K) ? A[r * K + k] : 0.f);
            }
            *reinterpret_cast<uint4 *>(&sA[cm<KP>(tid, k0)]) = *reinterpret_cast<const uint4 *>(h);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < KP / 16; ks++) {
                const uint64_t da = sdesc(sa + ks * 256, 128, (KP / 8) * 128);
                const uint64_t db = sdesc(sb + ks * 256, 128, (KP / 8) * 128);
                const uint32_t acc = ks > 0;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                        dcol),
                    "l"(da), "l"(db), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(&bar))
                         : "memory");
        }
        const bool ok = mbar_wait_ns(saddr(&bar), parity, kTcWait);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(err, EGX_ERR_TIMEOUT);
                mbar_wait_ns(saddr(&bar), parity, kTcWait);  // the MMAs in flight, bounded again
            }
            __syncthreads();
            break;
        }
        parity ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        float v[NP];
        tmem_ld_row<NP>(dcol + ((uint32_t)(32 * warp) << 16), v);
        if (r < M) {
            float *c = C + r * N;
#pragma unroll
            for (int n = 0; n < NP; n++)
                if (n < N) c[n] = accumulate ? c[n] + v[n] : v[n];
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // the next tile's rows and MMAs wait for every read of this one
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(dcol), "r"(32) : "memory");
}

template <int KP, int NP>
void launch_pw(const float *A, int M, int K, const float *B, long b_k, long b_n, int N, float *C, bool accumulate,
               int *err, cudaStream_t s) {
    static int nsm = 0;
    if (!nsm) EGX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
    const long ntiles = ((long)M + 127) / 128;
    const unsigned grid = (unsigned)std::min<long>(ntiles, (long)nsm * 16);
    k_pw_tc<KP, NP><<<grid, 128, 0, s>>>(A, M, K, B, b_k, b_n, N, C, accumulate ? 1 : 0, ntiles, err);
    EGX_CUDA(cudaGetLastError());
}

}  // namespace

bool pw_gemm_tc_fits(int K, int N) { return K >= 1 && K <= 32 && N >= 1 && N <= 32; }

void pw_gemm_tc(const float *A, int M, int K, const float *B, long b_k, long b_n, int N, float *C, bool accumulate,
                int *err, cudaStream_t s) {
    EGX_CHECK(pw_gemm_tc_fits(K, N) && M >= 1 && err, EGX_ERR_INVALID, "pointwise tcgen05 GEMM: K, N must be in 1..32");
    if (K <= 16) {
        if (N <= 16)
            launch_pw<16, 16>(A, M, K, B, b_k, b_n, N, C, accumulate, err, s);
        else
            launch_pw<16, 32>(A, M, K, B, b_k, b_n, N, C, accumulate, err, s);
    } else {
        if (N <= 16)
            launch_pw<32, 16>(A, M, K, B, b_k, b_n, N, C, accumulate, err, s);
        else
            launch_pw<32, 32>(A, M, K, B, b_k, b_n, N, C, accumulate, err, s);
    }
}

}  // namespace egx
