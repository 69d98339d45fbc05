// Shared definitions of the egx CUDA library: complex arithmetic on
// double2/float2, error handling, the context object.
#pragma once

#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include <stdexcept>

#include "../../include/egx.h"

namespace egx {

// ---------------------------------------------------------------- complex
template <typename T> struct cvec;
template <> struct cvec<double> { typedef double2 type; };
template <> struct cvec<float> { typedef float2 type; };

template <typename T> using C = typename cvec<T>::type;

template <typename T> __host__ __device__ __forceinline__ C<T> mk(T re, T im) { C<T> r; r.x = re; r.y = im; return r; }
template <typename T> __host__ __device__ __forceinline__ C<T> cadd(C<T> a, C<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __host__ __device__ __forceinline__ C<T> csub(C<T> a, C<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __host__ __device__ __forceinline__ C<T> cmul(C<T> a, C<T> b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __host__ __device__ __forceinline__ C<T> cscale(C<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> __host__ __device__ __forceinline__ C<T> cconj(C<T> a) { return mk<T>(a.x, -a.y); }
// acc += a * b
template <typename T> __host__ __device__ __forceinline__ void cfma(C<T> &acc, C<T> a, C<T> b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename T> __host__ __device__ __forceinline__ void cfma_conj(C<T> &acc, C<T> a, C<T> b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}
// Complex division (Smith's algorithm, scaled to avoid overflow).
template <typename T> __host__ __device__ __forceinline__ C<T> cdiv(C<T> a, C<T> b) {
    T ar = b.x, ai = b.y;
    if (fabs(ar) >= fabs(ai)) {
        T r = ai / ar, d = ar + ai * r;
        return mk<T>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    } else {
        T r = ar / ai, d = ai + ar * r;
        return mk<T>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
    }
}

// ---------------------------------------------------------------- errors
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define EGX_CUDA(call)                                                                 \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            throw ::egx::Error(EGX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define EGX_CHECK(cond, code, msg)                                                     \
    do {                                                                               \
        if (!(cond)) throw ::egx::Error((code), (msg));                                \
    } while (0)

// Per-kernel device time, measured with CUDA events recorded on the launch
// stream around each launch of an instrumented kernel (enabled on demand).
struct Timers {
    static const int kKinds = 32;
    bool on = false;
    unsigned mask = ~0u;  // kinds recorded while on
    struct Rec {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double total_ms[kKinds] = {};
    long count[kKinds] = {};
    cudaEvent_t take() {
        if (pool.empty()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            return e;
        }
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    // returns the record index to close with end()
    int begin(int kind, cudaStream_t s) {
        if (!on || kind < 0 || kind >= kKinds || !((mask >> kind) & 1u)) return -1;
        Rec r{kind, take(), take()};
        cudaEventRecord(r.a, s);
        pending.push_back(r);
        return (int)pending.size() - 1;
    }
    void end(int idx, cudaStream_t s) {
        if (idx < 0) return;
        cudaEventRecord(pending[idx].b, s);
        if (pending.size() > 4000) flush();
    }
    void flush() {
        for (auto &r : pending) {
            cudaEventSynchronize(r.b);
            float ms = 0;
            cudaEventElapsedTime(&ms, r.a, r.b);
            if (r.kind >= 0 && r.kind < kKinds) {
                total_ms[r.kind] += ms;
                count[r.kind]++;
            }
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.clear();
    }
    void reset() {
        flush();
        for (int k = 0; k < kKinds; k++) {
            total_ms[k] = 0;
            count[k] = 0;
        }
    }
    ~Timers() {
        for (auto &r : pending) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

// Count of device allocations (cudaMalloc calls that succeeded) the library
// has made in this process; egx_device_allocations reports it.
inline std::atomic<long> &device_allocations() {
    static std::atomic<long> n{0};
    return n;
}

// cudaMalloc that counts the allocation; throws EGX_ERR_OOM (with `what`)
// when it fails.
inline void *device_alloc(size_t bytes, const char *what) {
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess)
        throw Error(EGX_ERR_OOM, std::string(what) + ": cudaMalloc of " + std::to_string(bytes) +
                                     " bytes failed: " + cudaGetErrorString(e));
    device_allocations()++;
    return p;
}

// True when p is 16-byte aligned (float4 / double2 loads).
inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// Raise a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device; never lower it. The limit belongs to the kernel, not to a
// context: contexts on other host threads may launch the same kernel with a
// larger size at any moment, so a per-launch set to the launch's own size
// would race with them.
inline void raise_smem_limit(const void *fn, size_t bytes) {
    if (bytes <= 48 * 1024) return;
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> limits;
    int dev = 0;
    EGX_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = limits[std::make_pair(fn, dev)];
    if (bytes <= cur) return;
    EGX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
}

// Device buffer owned by the context.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() {}
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t n) {
        if (n <= bytes) return;
        release();
        p = device_alloc(n, "device buffer");
        bytes = n;
    }
    template <typename X> X *as() const { return reinterpret_cast<X *>(p); }
    void swap(DevBuf &o) {
        std::swap(p, o.p);
        std::swap(bytes, o.bytes);
    }
};

}  // namespace egx
