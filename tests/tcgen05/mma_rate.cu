// Issue cost of tcgen05.mma kind::tf32 (M = 128, K = 8 per instruction) by
// N and by the number of independent accumulators: one CTA per SM, one
// thread issuing 20,000 MMAs back to back into CH accumulator regions in
// round robin, A from tensor memory or shared memory; prints the cycles per
// MMA (clock64 around the issue loop and the commit's arrival) and the rate
// over the GPU. The operand encodings are those of layout_probe.cu. Every
// wait is bounded; the operands stay inside the kernel's shared arrays and
// its 256 tensor-memory columns.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3fff) | ((uint64_t)((lbo >> 4) & 0x3fff) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fff) << 32) | ((uint64_t)1 << 46);
}
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < 20000000; i++) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

template <int N, bool ATMEM, int CH>
__global__ void bench(int iters, long long *cycles, int *status) {
    __shared__ __align__(1024) float sA[128 * 8];
    __shared__ __align__(1024) float sB[64 * 8];
    __shared__ uint32_t tbase;
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int e = tid; e < 128 * 8; e += blockDim.x) sA[e] = 0.001f * (e % 7);
    for (int e = tid; e < 64 * 8; e += blockDim.x) sB[e] = 0.001f * (e % 5);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(saddr(&tbase)), "r"(256) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t t0 = tbase, dcol = t0, acol = t0 + 192;
    if (ATMEM && warp < 4) {
        uint32_t v[8];
        for (int k = 0; k < 8; k++) v[k] = __float_as_uint(0.001f * k);
        asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                     :: "r"(acol + ((uint32_t)(32 * warp) << 16)), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]),
                        "r"(v[5]), "r"(v[6]), "r"(v[7]) : "memory");
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    long long c0 = 0, c1 = 0;
    if (tid == 0) {
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
        const uint64_t da = sdesc(saddr(sA), 128, 256), db = sdesc(saddr(sB), 128, 256);
        c0 = clock64();
        for (int i = 0; i < iters; i++) {
            const uint32_t acc = i >= CH;
            const uint32_t dc = dcol + (uint32_t)((i % CH) * N);
            if (ATMEM)
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}"
                             :: "r"(dc), "r"(acol), "l"(db), "r"(idesc), "r"(acc) : "memory");
            else
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                             :: "r"(dc), "l"(da), "l"(db), "r"(idesc), "r"(acc) : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(saddr(&bar)) : "memory");
    }
    const bool ok = bar_wait(saddr(&bar), 0);
    if (tid == 0) {
        c1 = clock64();
        if (!ok) atomicExch(status, 1);
        atomicAdd((unsigned long long *)cycles, (unsigned long long)(c1 - c0));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(t0), "r"(256) : "memory");
}

template <int N, bool ATMEM, int CH>
void run(int nsm) {
    long long *dc; int *ds;
    cudaMalloc(&dc, 8); cudaMalloc(&ds, 4);
    const int iters = 20000;
    for (int rep = 0; rep < 2; rep++) {
        cudaMemset(dc, 0, 8); cudaMemset(ds, 0, 4);
        cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
        cudaEventRecord(a);
        bench<N, ATMEM, CH><<<nsm, 128>>>(iters, dc, ds);
        cudaEventRecord(b);
        cudaError_t e = cudaEventSynchronize(b);
        float ms = 0; cudaEventElapsedTime(&ms, a, b);
        long long cyc = 0; int st = 0;
        cudaMemcpy(&cyc, dc, 8, cudaMemcpyDeviceToHost); cudaMemcpy(&st, ds, 4, cudaMemcpyDeviceToHost);
        double flops = 2.0 * 128 * N * 8 * (double)iters * nsm;
        if (rep == 1)
            printf("CH=%d N=%3d A=%s: %s status %d  %.2f cycles/MMA  %.1f TFLOP/s (%.3f ms)\n", CH, N,
                   ATMEM ? "tmem" : "smem", cudaGetErrorString(e), st, (double)cyc / nsm / iters, flops / (ms * 1e-3) / 1e12, ms);
    }
    cudaFree(dc); cudaFree(ds);
}

int main() {
    int nsm = 0; cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
    run<16, true, 1>(nsm); run<16, true, 2>(nsm); run<16, true, 4>(nsm); run<16, true, 8>(nsm);
    run<16, false, 8>(nsm); run<32, true, 4>(nsm); run<64, true, 2>(nsm);
    return 0;
}
