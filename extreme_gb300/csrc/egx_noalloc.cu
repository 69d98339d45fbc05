// egx_dot_products_static: the DotProductRequest reduction of
// egx_dot_products on device vectors, for callers that cannot allocate
// device memory at the point of the call -- for example a host whose device
// memory is fully owned by its own pool allocator, or code running inside a
// solver callback, where a cudaMalloc would either fail or synchronise the
// whole device in the middle of a pipelined solve. The entry point allocates
// nothing: its per-block partial sums live in one file-scope device array of
// fixed size (128 KiB, kept by every GPU that loads the library until the
// process exits).
//
// The array is shared by every call on a device and keeps the last call's
// contents. Nothing in it has to start at zero: the first kernel writes every
// slot the second kernel reads, in the same call. Calls whose kernels overlap
// on the GPU (two streams, or two host threads) race on the array and give
// wrong results; serialise them.
//
// Host code may not use the array's name as a device address (on the host it
// is only a stand-in symbol): the address is looked up with
// cudaGetSymbolAddress once per device, with that device current, by the
// first call on that device.
//
// Every call ends by synchronising the context's stream, so it must not be
// made while that stream is being captured into a CUDA graph, nor from a
// CUDA host callback (cudaLaunchHostFunc), where CUDA calls are not allowed.
// "Inside a solver callback" means an ordinary host function that the
// solver calls between its own launches, such as the preconditioner or
// dot-product callback of a host-driven Krylov loop.
//
// V, w and out are read and written as double2 (16-byte loads and stores),
// so each must be 16-byte aligned; a misaligned pointer is rejected with
// EGX_ERR_INVALID before anything is launched.
#include <algorithm>
#include <mutex>
#include <string>

#include "egx_ctx.cuh"

using namespace egx;

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxBlocks = 128;
constexpr int kNaMaxCols = 64;   // the most columns one call may ask for
constexpr int kNaMaxDevices = 64;

// partial sums [column][block]
static __device__ __align__(256) double2 g_na_partials[kNaMaxCols * kNaMaxBlocks];

// block b: part[k * gridDim.x + b] = sum over its grid-stride elements of conj(V[k][i]) * w[i]
__global__ void __launch_bounds__(kNaThreads) k_na_dots(const double2 *__restrict__ V, int ncols,
                                                         const double2 *__restrict__ w, long n,
                                                         double2 *__restrict__ part) {
    __shared__ double2 red[kNaThreads / 32];
    const long stride = (long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k0 = 0; k0 < ncols; k0 += 4) {
        double2 acc[4];
#pragma unroll
        for (int j = 0; j < 4; j++) acc[j] = make_double2(0.0, 0.0);
        for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const double2 wi = w[i];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (k0 + j < ncols) {
                    const double2 v = V[(long)(k0 + j) * n + i];
                    acc[j].x += v.x * wi.x + v.y * wi.y;  // conj(v) * w
                    acc[j].y += v.x * wi.y - v.y * wi.x;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            double2 a = acc[j];
            for (int o = 16; o > 0; o >>= 1) {
                a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
                a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
            }
            if (lane == 0) red[warp] = a;
            __syncthreads();
            if (threadIdx.x == 0 && k0 + j < ncols) {
                double2 s = make_double2(0.0, 0.0);
                for (int q = 0; q < kNaThreads / 32; q++) {
                    s.x += red[q].x;
                    s.y += red[q].y;
                }
                part[(long)(k0 + j) * gridDim.x + blockIdx.x] = s;
            }
            __syncthreads();
        }
    }
}

// one warp per column: out[k] = sum over blocks of part[k * nblocks + b]
__global__ void k_na_reduce(const double2 *__restrict__ part, int nblocks, int ncols, double2 *__restrict__ out) {
    const int k = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (k >= ncols) return;
    double2 s = make_double2(0.0, 0.0);
    for (int b = lane; b < nblocks; b += 32) {
        s.x += part[(long)k * nblocks + b].x;
        s.y += part[(long)k * nblocks + b].y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) out[k] = s;
}

std::mutex g_na_mutex;
double2 *g_na_addr[kNaMaxDevices] = {};

// device address of g_na_partials on `device` (which must be current)
double2 *na_scratch(int device) {
    EGX_CHECK(device >= 0 && device < kNaMaxDevices, EGX_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_na_partials);
        if (e != cudaSuccess || !p)
            throw Error(EGX_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                          cudaGetErrorString(e));
        g_na_addr[device] = static_cast<double2 *>(p);
    }
    return g_na_addr[device];
}

}  // namespace

extern "C" int egx_dot_products_static(egx_ctx *ctx, const double *V, int ncols, const double *w, long n,
                                       double *out) {
    if (!ctx) return EGX_ERR_INVALID;
    try {
        EGX_CHECK(V && w && out && n >= 1 && ncols >= 1, EGX_ERR_INVALID, "bad dot-product arguments");
        EGX_CHECK(aligned16(V) && aligned16(w) && aligned16(out), EGX_ERR_INVALID,
                  "egx_dot_products_static: V, w and out must be 16-byte aligned device pointers");
        if (ncols > kNaMaxCols)
            throw Error(EGX_ERR_INVALID, "egx_dot_products_static: ncols = " + std::to_string(ncols) +
                                             " exceeds the static scratch limit of " + std::to_string(kNaMaxCols) +
                                             " columns");
        set_device(ctx);
        double2 *part = na_scratch(ctx->device);
        const int nblocks = (int)std::min<long>(kNaMaxBlocks, (n + kNaThreads - 1) / kNaThreads);
        k_na_dots<<<nblocks, kNaThreads, 0, ctx->stream>>>((const double2 *)V, ncols, (const double2 *)w, n, part);
        EGX_CUDA(cudaGetLastError());
        k_na_reduce<<<(ncols + 3) / 4, 128, 0, ctx->stream>>>(part, nblocks, ncols, (double2 *)out);
        EGX_CUDA(cudaGetLastError());
        ctx->launches += 2;
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (const egx::Error &e) {
        return fail(ctx, e.code, e.what());
    } catch (const std::exception &e) {
        return fail(ctx, EGX_ERR_INVALID, e.what());
    }
    return EGX_OK;
}
