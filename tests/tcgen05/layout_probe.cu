// Known-answer check of the tcgen05 operand encodings used for this design
// study: D[128 x 16] = A[128 x 32] B[32 x 16] with kind::tf32 MMAs
// (M = 128, N = 16, K = 8 per instruction), shared-memory operands in the
// K-major no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix,
// LBO = 128 B between core matrices along K, SBO between 8-row groups),
// accumulators in tensor memory read back with tcgen05.ld; once with A from
// shared memory and once with A written to tensor memory with tcgen05.st.
// Values are exactly representable in TF32 and the sums exact in FP32, so
// both results must equal the host product bit for bit. Every wait is
// bounded; every access stays inside the 18 KB of shared memory and the 64
// tensor-memory columns the kernel allocates.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

constexpr int M = 128, N = 16, K = 32;

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading and stride byte offsets
// (>> 4), version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3fff);
    d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < 2000000; i++) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// element (r, k) of an R x K fp32 tile in the core-matrix layout
__device__ __forceinline__ int cm_index(int r, int k) { return ((r >> 3) * (K / 4) + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3); }

__global__ void probe(const float *A, const float *B, float *D1, float *D2, int *status) {
    __shared__ __align__(1024) float sA[M * K];
    __shared__ __align__(1024) float sB[N * K];
    __shared__ uint32_t tbase;
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int e = tid; e < M * K; e += blockDim.x) { int r = e / K, k = e % K; sA[cm_index(r, k)] = A[e]; }
    for (int e = tid; e < N * K; e += blockDim.x) { int n = e / K, k = e % K; sB[cm_index(n, k)] = B[k * N + n]; }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(saddr(&tbase)), "r"(64) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t t0 = tbase;
    const uint32_t dcol1 = t0, dcol2 = t0 + 16, acol = t0 + 32;
    if (warp < 4) {  // A into tensor memory: lane = row, K columns
        const int r = 32 * warp + lane;
        uint32_t v[32];
        for (int k = 0; k < K; k++) v[k] = __float_as_uint(A[r * K + k]);
        const uint32_t ta = acol + ((uint32_t)(32 * warp) << 16);
        asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
                     :: "r"(ta), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
                        "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]) : "memory");
        asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
                     :: "r"(ta + 16), "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]),
                        "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31]) : "memory");
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
        // instruction descriptor: F32 accumulate, TF32 A and B, K-major, N >> 3, M >> 4
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
        const uint32_t sa = saddr(sA), sb = saddr(sB);
        for (int kk = 0; kk < K / 8; kk++) {
            const uint64_t da = sdesc(sa + kk * 256, 128, (K / 4) * 128);
            const uint64_t db = sdesc(sb + kk * 256, 128, (K / 4) * 128);
            const uint32_t acc = kk > 0;
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                         :: "r"(dcol1), "l"(da), "l"(db), "r"(idesc), "r"(acc) : "memory");
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}"
                         :: "r"(dcol2), "r"(acol + kk * 8), "l"(db), "r"(idesc), "r"(acc) : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(saddr(&bar)) : "memory");
    }
    const bool ok = bar_wait(saddr(&bar), 0);
    if (!ok && lane == 0) atomicExch(status, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp < 4 && ok) {
        const int r = 32 * warp + lane;
        for (int which = 0; which < 2; which++) {
            uint32_t v[16];
            const uint32_t ta = (which ? dcol2 : dcol1) + ((uint32_t)(32 * warp) << 16);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                           "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                         : "r"(ta) : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float *D = which ? D2 : D1;
            for (int c = 0; c < 16; c++) D[r * N + c] = __uint_as_float(v[c]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(t0), "r"(64) : "memory");
}

int main() {
    std::vector<float> A(M * K), B(K * N), D1(M * N), D2(M * N), R(M * N);
    srand(1);
    for (auto &x : A) x = (float)((rand() % 64) - 32) / 8.0f;
    for (auto &x : B) x = (float)((rand() % 64) - 32) / 16.0f;
    for (int m = 0; m < M; m++)
        for (int n = 0; n < N; n++) {
            double s = 0;
            for (int k = 0; k < K; k++) s += (double)A[m * K + k] * B[k * N + n];
            R[m * N + n] = (float)s;
        }
    float *dA, *dB, *dD1, *dD2;
    int *dst;
    cudaMalloc(&dA, A.size() * 4); cudaMalloc(&dB, B.size() * 4);
    cudaMalloc(&dD1, D1.size() * 4); cudaMalloc(&dD2, D2.size() * 4); cudaMalloc(&dst, 4);
    cudaMemset(dst, 0, 4); cudaMemset(dD1, 0, D1.size() * 4); cudaMemset(dD2, 0, D2.size() * 4);
    cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice);
    probe<<<1, 128>>>(dA, dB, dD1, dD2, dst);
    cudaError_t e = cudaDeviceSynchronize();
    printf("kernel: %s\n", cudaGetErrorString(e));
    if (e != cudaSuccess) return 1;
    int st = 0;
    cudaMemcpy(&st, dst, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(D1.data(), dD1, D1.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(D2.data(), dD2, D2.size() * 4, cudaMemcpyDeviceToHost);
    double e1 = 0, e2 = 0;
    for (int i = 0; i < M * N; i++) { e1 = fmax(e1, fabs(D1[i] - R[i])); e2 = fmax(e2, fabs(D2[i] - R[i])); }
    printf("status %d max_err_smem_a %g max_err_tmem_a %g\n", st, e1, e2);
    return (st == 0 && e1 == 0 && e2 == 0) ? 0 : 2;
}
