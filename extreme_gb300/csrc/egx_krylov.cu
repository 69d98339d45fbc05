// Device vector kernels and the host-side GMRES driver (see egx_krylov.cuh).
#include <cmath>
#include <cstdint>

#include "egx_krylov.cuh"

namespace egx {

constexpr int kThreads = 256;

template <typename T> struct Acc { typedef T type; };

__device__ __forceinline__ double2 warp_sum2(double2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; result valid in thread 0.
__device__ double2 block_sum2(double2 v) {
    __shared__ double2 red[32];
    v = warp_sum2(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? red[lane] : make_double2(0, 0);
        v = warp_sum2(v);
    }
    return v;
}
__device__ double block_sum(double v) {
    __shared__ double red1[32];
    v = warp_sum(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red1[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? red1[lane] : 0.0;
        v = warp_sum(v);
    }
    return v;
}

// Each thread keeps the partial sums of up to kDotCols columns in
// registers, so w is read once per kDotCols columns (the stacked vectors are
// larger than L2), and reads DotRows<T> rows per pass, so that enough loads
// are in flight: eight rows reached 4.2-4.6 TB/s for 1-30 complex64 columns
// where two rows reached 2.5-3.7.
constexpr int kDotCols = 16;
template <typename T> struct DotRows { static constexpr int value = 8; };
template <> struct DotRows<double> { static constexpr int value = 4; };
template <typename T>
__global__ void k_multi_dot(const C<T> *__restrict__ V, int ncols, const C<T> *__restrict__ w, long n,
                            double2 *__restrict__ partials, const int *live) {
    if (live && !*live) return;
    constexpr int ROWS = DotRows<T>::value;
    const long stride = (long)gridDim.x * blockDim.x;
    for (int k0 = 0; k0 < ncols; k0 += kDotCols) {
        const int kc = min(kDotCols, ncols - k0);
        const C<T> *col = V + (long)k0 * n;
        C<T> acc[kDotCols];
#pragma unroll
        for (int j = 0; j < kDotCols; j++) acc[j] = mk<T>(0, 0);
        long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
        for (; r + (ROWS - 1) * stride < n; r += ROWS * stride) {
            C<T> x[ROWS];
#pragma unroll
            for (int u = 0; u < ROWS; u++) x[u] = w[r + u * stride];
#pragma unroll
            for (int j = 0; j < kDotCols; j++)
                if (j < kc) {
                    C<T> a[ROWS];
#pragma unroll
                    for (int u = 0; u < ROWS; u++) a[u] = col[(long)j * n + r + u * stride];
#pragma unroll
                    for (int u = 0; u < ROWS; u++) cfma_conj<T>(acc[j], a[u], x[u]);
                }
        }
        for (; r < n; r += stride) {
            const C<T> x = w[r];
#pragma unroll
            for (int j = 0; j < kDotCols; j++)
                if (j < kc) cfma_conj<T>(acc[j], col[(long)j * n + r], x);
        }
#pragma unroll
        for (int j = 0; j < kDotCols; j++) {
            if (j < kc) {  // kc is the same in every thread: the block sums stay uniform
                double2 s = block_sum2(make_double2((double)acc[j].x, (double)acc[j].y));
                if (threadIdx.x == 0) partials[(long)blockIdx.x * ncols + k0 + j] = s;
            }
        }
    }
}

// complex64 vectors of even length: the same dots with each load a float4
// (two complex entries), four per column and pass, eight columns per pass
// (66 registers: three CTAs per SM where sixteen columns allowed two)
__global__ void k_multi_dot_c2(const float4 *__restrict__ V, int ncols, const float4 *__restrict__ w, long n2,
                               double2 *__restrict__ partials, const int *live) {
    if (live && !*live) return;
    constexpr int ROWS = 4, kDotCols = 8;
    const long stride = (long)gridDim.x * blockDim.x;
    auto fma_conj2 = [](float2 &acc, float4 a, float4 b) {  // += conj(a) b, two entries
        acc.x = fmaf(a.x, b.x, acc.x);
        acc.x = fmaf(a.y, b.y, acc.x);
        acc.y = fmaf(a.x, b.y, acc.y);
        acc.y = fmaf(-a.y, b.x, acc.y);
        acc.x = fmaf(a.z, b.z, acc.x);
        acc.x = fmaf(a.w, b.w, acc.x);
        acc.y = fmaf(a.z, b.w, acc.y);
        acc.y = fmaf(-a.w, b.z, acc.y);
    };
    for (int k0 = 0; k0 < ncols; k0 += kDotCols) {
        const int kc = min(kDotCols, ncols - k0);
        const float4 *col = V + (long)k0 * n2;
        float2 acc[kDotCols];
#pragma unroll
        for (int j = 0; j < kDotCols; j++) acc[j] = make_float2(0.f, 0.f);
        long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
        for (; r + (ROWS - 1) * stride < n2; r += ROWS * stride) {
            float4 x[ROWS];
#pragma unroll
            for (int u = 0; u < ROWS; u++) x[u] = w[r + u * stride];
#pragma unroll
            for (int j = 0; j < kDotCols; j++)
                if (j < kc) {
                    float4 a[ROWS];
#pragma unroll
                    for (int u = 0; u < ROWS; u++) a[u] = col[(long)j * n2 + r + u * stride];
#pragma unroll
                    for (int u = 0; u < ROWS; u++) fma_conj2(acc[j], a[u], x[u]);
                }
        }
        for (; r < n2; r += stride) {
            const float4 x = w[r];
#pragma unroll
            for (int j = 0; j < kDotCols; j++)
                if (j < kc) fma_conj2(acc[j], col[(long)j * n2 + r], x);
        }
#pragma unroll
        for (int j = 0; j < kDotCols; j++) {
            if (j < kc) {
                double2 sm = block_sum2(make_double2((double)acc[j].x, (double)acc[j].y));
                if (threadIdx.x == 0) partials[(long)blockIdx.x * ncols + k0 + j] = sm;
            }
        }
    }
}

__global__ void k_reduce_cols(const double2 *__restrict__ partials, int nblocks, int ncols, double2 *__restrict__ out,
                              const int *live) {
    if (live && !*live) return;
    const int k = blockIdx.x;
    double2 s = make_double2(0, 0);
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        double2 p = partials[(long)b * ncols + k];
        s.x += p.x;
        s.y += p.y;
    }
    s = block_sum2(s);
    if (threadIdx.x == 0) out[k] = s;
}

__global__ void k_reduce_scalar(const double *__restrict__ partials, int nblocks, double *__restrict__ out,
                                const int *live) {
    if (live && !*live) return;
    double s = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[b];
    s = block_sum(s);
    if (threadIdx.x == 0) out[0] = s;
}

template <typename T>
__global__ void k_update_norm(const C<T> *__restrict__ V, int ncols, const double2 *__restrict__ dots, C<T> *w, long n,
                              double *__restrict__ partials, const int *live) {
    if (live && !*live) return;
    __shared__ C<T> sd[64];
    for (int k = threadIdx.x; k < ncols; k += blockDim.x) sd[k] = mk<T>((T)dots[k].x, (T)dots[k].y);
    __syncthreads();
    const long stride = (long)gridDim.x * blockDim.x;
    T acc = 0;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        C<T> v = w[r];
        for (int k = 0; k < ncols; k++) {
            C<T> a = V[(long)k * n + r];
            C<T> d = sd[k];
            // v -= a * d
            v.x = fma(-a.x, d.x, v.x);
            v.x = fma(a.y, d.y, v.x);
            v.y = fma(-a.x, d.y, v.y);
            v.y = fma(-a.y, d.x, v.y);
        }
        w[r] = v;
        acc = fma(v.x, v.x, acc);
        acc = fma(v.y, v.y, acc);
    }
    double s = block_sum((double)acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// complex64 vectors of even length: the update with float4 loads
__global__ void k_update_norm_c2(const float4 *__restrict__ V, int ncols, const double2 *__restrict__ dots, float4 *w,
                                 long n2, double *__restrict__ partials, const int *live) {
    if (live && !*live) return;
    __shared__ float2 sd[64];
    for (int k = threadIdx.x; k < ncols; k += blockDim.x) sd[k] = make_float2((float)dots[k].x, (float)dots[k].y);
    __syncthreads();
    const long stride = (long)gridDim.x * blockDim.x;
    float acc = 0.f;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n2; r += stride) {
        float4 v = w[r];
#pragma unroll 4
        for (int k = 0; k < ncols; k++) {
            const float4 a = V[(long)k * n2 + r];
            const float2 d = sd[k];
            v.x = fmaf(-a.x, d.x, v.x);
            v.x = fmaf(a.y, d.y, v.x);
            v.y = fmaf(-a.x, d.y, v.y);
            v.y = fmaf(-a.y, d.x, v.y);
            v.z = fmaf(-a.z, d.x, v.z);
            v.z = fmaf(a.w, d.y, v.z);
            v.w = fmaf(-a.z, d.y, v.w);
            v.w = fmaf(-a.w, d.x, v.w);
        }
        w[r] = v;
        acc = fmaf(v.x, v.x, acc);
        acc = fmaf(v.y, v.y, acc);
        acc = fmaf(v.z, v.z, acc);
        acc = fmaf(v.w, v.w, acc);
    }
    double sm = block_sum((double)acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = sm;
}

template <typename T>
__global__ void k_norm2(const C<T> *__restrict__ x, long n, double *__restrict__ partials, const int *live) {
    if (live && !*live) return;
    const long stride = (long)gridDim.x * blockDim.x;
    T acc = 0;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        C<T> v = x[r];
        acc = fma(v.x, v.x, acc);
        acc = fma(v.y, v.y, acc);
    }
    double s = block_sum((double)acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

template <typename T>
__global__ void k_scale(const C<T> *__restrict__ x, T a, C<T> *__restrict__ y, long n) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
        y[r] = mk<T>(x[r].x * a, x[r].y * a);
}
template <typename T>
__global__ void k_divide(const C<T> *__restrict__ x, T d, C<T> *__restrict__ y, long n) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
        y[r] = mk<T>(x[r].x / d, x[r].y / d);
}
template <typename T>
__global__ void k_divide_dev(const C<T> *__restrict__ x, const double *__restrict__ d, C<T> *__restrict__ y, long n,
                             const int *live) {
    if (live && !*live) return;
    const T dd = (T)*d;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
        y[r] = mk<T>(x[r].x / dd, x[r].y / dd);
}
template <typename T>
__global__ void k_sub(const C<T> *__restrict__ a, const C<T> *__restrict__ b, C<T> *__restrict__ y, long n,
                      const int *live) {
    if (live && !*live) return;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
        y[r] = csub<T>(a[r], b[r]);
}
template <typename T>
__global__ void k_add(const C<T> *__restrict__ x, C<T> *__restrict__ y, long n, const int *live) {
    if (live && !*live) return;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
        y[r] = cadd<T>(y[r], x[r]);
}
template <typename T>
__global__ void k_gemv(const C<T> *__restrict__ V, int ncols, const double2 *__restrict__ coef, C<T> *__restrict__ out,
                       long n, const int *ncols_dev) {
    if (ncols_dev) ncols = *ncols_dev;
    if (ncols <= 0) return;
    __shared__ C<T> sc[64];
    for (int k = threadIdx.x; k < ncols; k += blockDim.x) sc[k] = mk<T>((T)coef[k].x, (T)coef[k].y);
    __syncthreads();
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
        C<T> acc = mk<T>(0, 0);
        for (int k = 0; k < ncols; k++) cfma<T>(acc, V[(long)k * n + r], sc[k]);
        out[r] = acc;
    }
}

__global__ void k_d2f(const double2 *__restrict__ x, float2 *__restrict__ y, long n, double sc) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
        y[r] = make_float2((float)(x[r].x * sc), (float)(x[r].y * sc));
}
__global__ void k_f2d_add(const float2 *__restrict__ x, double2 *__restrict__ y, long n, double sc) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
        double2 v = y[r];
        v.x += (double)x[r].x * sc;
        v.y += (double)x[r].y * sc;
        y[r] = v;
    }
}

// the float4 kernels read two complex64 entries per load: 16-byte alignment

static int grid_for(long n) {
    long g = (n + kThreads - 1) / kThreads;
    if (g > 2048) g = 2048;
    if (g < 1) g = 1;
    return (int)g;
}

template <typename T>
void VecOps<T>::multi_dot(const C<T> *V, int ncols, const C<T> *w, long n, double2 *dots_dev, double2 *partials,
                          int nblocks, cudaStream_t s, const int *live) {
    if (sizeof(T) == sizeof(float) && n % 2 == 0 && aligned16(V) && aligned16(w))
        k_multi_dot_c2<<<nblocks, kThreads, 0, s>>>(reinterpret_cast<const float4 *>(V), ncols,
                                                    reinterpret_cast<const float4 *>(w), n / 2, partials, live);
    else
        k_multi_dot<T><<<nblocks, kThreads, 0, s>>>(V, ncols, w, n, partials, live);
    k_reduce_cols<<<ncols, kThreads, 0, s>>>(partials, nblocks, ncols, dots_dev, live);
}
template <typename T>
void VecOps<T>::update_norm(const C<T> *V, int ncols, const double2 *dots_dev, C<T> *w, long n, double *norm2_dev,
                            double *partials, int nblocks, cudaStream_t s, const int *live) {
    if (sizeof(T) == sizeof(float) && n % 2 == 0 && aligned16(V) && aligned16(w))
        k_update_norm_c2<<<nblocks, kThreads, 0, s>>>(reinterpret_cast<const float4 *>(V), ncols, dots_dev,
                                                      reinterpret_cast<float4 *>(w), n / 2, partials, live);
    else
        k_update_norm<T><<<nblocks, kThreads, 0, s>>>(V, ncols, dots_dev, w, n, partials, live);
    k_reduce_scalar<<<1, kThreads, 0, s>>>(partials, nblocks, norm2_dev, live);
}
template <typename T>
void VecOps<T>::norm2(const C<T> *x, long n, double *norm2_dev, double *partials, int nblocks, cudaStream_t s,
                      const int *live) {
    k_norm2<T><<<nblocks, kThreads, 0, s>>>(x, n, partials, live);
    k_reduce_scalar<<<1, kThreads, 0, s>>>(partials, nblocks, norm2_dev, live);
}
template <typename T>
void VecOps<T>::scale(const C<T> *x, double a, C<T> *y, long n, cudaStream_t s) {
    k_scale<T><<<grid_for(n), kThreads, 0, s>>>(x, (T)a, y, n);
}
template <typename T>
void VecOps<T>::divide(const C<T> *x, double d, C<T> *y, long n, cudaStream_t s) {
    k_divide<T><<<grid_for(n), kThreads, 0, s>>>(x, (T)d, y, n);
}
template <typename T>
void VecOps<T>::divide_dev(const C<T> *x, const double *d, C<T> *y, long n, cudaStream_t s, const int *live) {
    k_divide_dev<T><<<grid_for(n), kThreads, 0, s>>>(x, d, y, n, live);
}
template <typename T>
void VecOps<T>::sub(const C<T> *a, const C<T> *b, C<T> *y, long n, cudaStream_t s, const int *live) {
    k_sub<T><<<grid_for(n), kThreads, 0, s>>>(a, b, y, n, live);
}
template <typename T>
void VecOps<T>::add(const C<T> *x, C<T> *y, long n, cudaStream_t s, const int *live) {
    k_add<T><<<grid_for(n), kThreads, 0, s>>>(x, y, n, live);
}
template <typename T>
void VecOps<T>::gemv(const C<T> *V, int ncols, const double2 *coef, C<T> *out, long n, cudaStream_t s,
                     const int *ncols_dev) {
    k_gemv<T><<<grid_for(n), kThreads, 0, s>>>(V, ncols, coef, out, n, ncols_dev);
}
template <typename T>
void VecOps<T>::copy(const C<T> *x, C<T> *y, long n, cudaStream_t s) {
    if (x != y) EGX_CUDA(cudaMemcpyAsync(y, x, n * sizeof(C<T>), cudaMemcpyDeviceToDevice, s));
}
template <typename T>
void VecOps<T>::zero(C<T> *x, long n, cudaStream_t s) {
    EGX_CUDA(cudaMemsetAsync(x, 0, n * sizeof(C<T>), s));
}

void convert_d2f(const double2 *x, float2 *y, long n, double scale, cudaStream_t s) {
    k_d2f<<<grid_for(n), kThreads, 0, s>>>(x, y, n, scale);
}
void convert_f2d_add(const float2 *x, double2 *y, long n, double scale, cudaStream_t s) {
    k_f2d_add<<<grid_for(n), kThreads, 0, s>>>(x, y, n, scale);
}

template struct VecOps<double>;
template struct VecOps<float>;

// ------------------------------------------------------------------ driver

template <typename T>
Gmres<T>::Gmres(long n, int m, double tol, int max_restarts, bool check_true, cudaStream_t s)
    : n_(n), m_(m), tol_(tol), max_restarts_(max_restarts), check_true_(check_true), s_(s) {
    EGX_CHECK(m >= 1 && m <= 60, EGX_ERR_INVALID, "GMRES buffer length must be in [1, 60]");
    nblocks_ = grid_for(n);
    if (nblocks_ > 1024) nblocks_ = 1024;
    auto alloc = [](void **p, size_t b) { *p = device_alloc(b, "GMRES workspace"); };
    alloc((void **)&V_, sizeof(C<T>) * n * m);
    alloc((void **)&w_, sizeof(C<T>) * n);
    alloc((void **)&r0_, sizeof(C<T>) * n);
    alloc((void **)&xcur_, sizeof(C<T>) * n);
    alloc((void **)&dots_, sizeof(double2) * 64 + sizeof(double) * 2);
    norm_dev_ = reinterpret_cast<double *>(dots_ + 64);
    alloc((void **)&coef_, sizeof(double2) * 64);
    alloc((void **)&partials_, sizeof(double2) * (size_t)nblocks_ * 64);
    EGX_CUDA(cudaMallocHost((void **)&host_, sizeof(double2) * 64 + sizeof(double) * 2));
    alloc((void **)&st_, sizeof(GmState));
    alloc((void **)&napp_dev_, sizeof(long long));
    EGX_CUDA(cudaMemsetAsync(napp_dev_, 0, sizeof(long long), s));
    alloc((void **)&Hd_, sizeof(double2) * (m + 1) * (m + 1));
    alloc((void **)&csd_, sizeof(double) * m);
    alloc((void **)&snd_, sizeof(double2) * m);
    EGX_CUDA(cudaMallocHost((void **)&hst_, sizeof(GmState)));
    H_.assign((size_t)(m + 1) * (m + 1), 0.0);
    cs_.assign(m, 0.0);
    sn_.assign(m, 0.0);
}

template <typename T>
Gmres<T>::~Gmres() {
    cudaFree(V_);
    if (Z_) cudaFree(Z_);
    cudaFree(w_);
    cudaFree(r0_);
    cudaFree(xcur_);
    cudaFree(dots_);
    cudaFree(coef_);
    cudaFree(partials_);
    cudaFree(st_);
    cudaFree(napp_dev_);
    cudaFree(Hd_);
    cudaFree(csd_);
    cudaFree(snd_);
    cudaFreeHost(hst_);
    cudaFreeHost(host_);
}

template <typename T>
double Gmres<T>::norm(const C<T> *x) {
    VecOps<T>::norm2(x, n_, norm_dev_, reinterpret_cast<double *>(partials_), nblocks_, s_);
    kernel_launches += 2;
    EGX_CUDA(cudaMemcpyAsync(host_, norm_dev_, sizeof(double), cudaMemcpyDeviceToHost, s_));
    EGX_CUDA(cudaStreamSynchronize(s_));
    return std::sqrt(host_[0]);
}

template <typename T>
void Gmres<T>::construct(int jh, C<T> *result) {
    // y = H(0:jh, 0:jh) \ g (SimplifiedZtrsv, upper, non-unit)
    std::vector<std::complex<double>> y(jh > 0 ? jh : 1);
    for (int i = 0; i < jh; i++) y[i] = h(i, m_);
    for (int j = jh - 1; j >= 0; j--) {
        if (y[j] != std::complex<double>(0.0, 0.0)) {
            y[j] /= h(j, j);
            std::complex<double> t = y[j];
            for (int i = j - 1; i >= 0; i--) y[i] -= t * h(i, j);
        }
    }
    if (jh > 0) {
        EGX_CUDA(cudaMemcpyAsync(coef_, y.data(), sizeof(double2) * jh, cudaMemcpyHostToDevice, s_));
        VecOps<T>::gemv(precond ? Z_ : V_, jh, coef_, r0_, n_, s_);
        VecOps<T>::add(r0_, result, n_, s_);
        kernel_launches += 2;
        // the host vector y must outlive the async copy
        EGX_CUDA(cudaStreamSynchronize(s_));
    }
}

template <typename T>
double Gmres<T>::final_actions(int jh, const C<T> *rhs, C<T> *result) {
    construct(jh, result);
    if (!check_true_) return -1.0;
    VecOps<T>::copy(result, r0_, n_, s_);
    apply(r0_, w_);
    VecOps<T>::sub(rhs, w_, w_, n_, s_);
    kernel_launches += 1;
    double tn = norm(w_);
    return tn / bn_;
}

template <typename T>
double Gmres<T>::arnoldi(double bn, int &jh) {
    double bea = -1.0;
    const int m = m_;
    do {
        C<T> *vj = V_ + (long)jh * n_;
        // w = A M v_j straight into w (the apply leaves its input unchanged)
        if (precond) {
            C<T> *zj = Z_ + (long)jh * n_;
            precond(vj, zj);
            apply(zj, w_);
        } else {
            apply(vj, w_);
        }
        for (int j = 0; j <= jh; j++) h(j, jh) = 0.0;
        int northo = 0;
        double dloo = 0, dnormw = 0;
        do {
            northo++;
            const int koff = sizeof(T) == sizeof(double) ? 0 : EGX_K_C64;
            int ev = timers ? timers->begin(EGX_K_GS_DOTS + koff, s_) : -1;
            VecOps<T>::multi_dot(V_, jh + 1, w_, n_, dots_, partials_, nblocks_, s_);
            if (timers) timers->end(ev, s_);
            ev = timers ? timers->begin(EGX_K_GS_UPDATE + koff, s_) : -1;
            VecOps<T>::update_norm(V_, jh + 1, dots_, w_, n_, norm_dev_, reinterpret_cast<double *>(partials_),
                                   nblocks_, s_);
            if (timers) timers->end(ev, s_);
            kernel_launches += 4;
            EGX_CUDA(cudaMemcpyAsync(host_, dots_, sizeof(double2) * 64 + sizeof(double), cudaMemcpyDeviceToHost, s_));
            EGX_CUDA(cudaStreamSynchronize(s_));
            const double2 *hd = reinterpret_cast<const double2 *>(host_);
            double ss = 0;
            for (int j = 0; j <= jh; j++) {
                h(j, jh) += std::complex<double>(hd[j].x, hd[j].y);
                ss += hd[j].x * hd[j].x + hd[j].y * hd[j].y;
            }
            dloo = ss;
            dnormw = std::sqrt(host_[2 * 64]);
        } while (2.0 * dnormw <= std::sqrt(dloo) && northo < 3);
        h(jh + 1, jh) = dnormw;
        if (jh < m - 1) {
            VecOps<T>::divide(w_, dnormw, V_ + (long)(jh + 1) * n_, n_, s_);
            kernel_launches += 1;
        }
        auto rot = [](std::complex<double> &x, std::complex<double> &y, double c, std::complex<double> s) {
            std::complex<double> t = c * x + s * y;
            y = c * y - std::conj(s) * x;
            x = t;
        };
        for (int j = 0; j < jh; j++) rot(h(j, jh), h(j + 1, jh), cs_[j], sn_[j]);
        // zrotg (classic reference algorithm)
        {
            std::complex<double> a = h(jh, jh), b = h(jh + 1, jh);
            double c;
            std::complex<double> s;
            if (std::abs(a) == 0.0) {
                c = 0.0;
                s = 1.0;
            } else {
                double scale = std::abs(a) + std::abs(b);
                double a1 = std::abs(a / scale), b1 = std::abs(b / scale);
                double nrm = scale * std::sqrt(a1 * a1 + b1 * b1);
                std::complex<double> alpha = a / std::abs(a);
                c = std::abs(a) / nrm;
                s = alpha * std::conj(b) / nrm;
            }
            cs_[jh] = c;
            sn_[jh] = s;
        }
        rot(h(jh, m), h(jh + 1, m), cs_[jh], sn_[jh]);
        rot(h(jh, jh), h(jh + 1, jh), cs_[jh], sn_[jh]);
        h(jh + 1, jh) = 0.0;
        double dnormres = std::abs(h(jh + 1, m));
        bea = dnormres / bn;
        iterations_done_++;
        jh++;
    } while (bea > tol_ && jh < m);
    return bea;
}

template <typename T>
GmresResult Gmres<T>::solve(const C<T> *rhs, const C<T> *x0, C<T> *result) {
    if (precond && !Z_) Z_ = static_cast<C<T> *>(device_alloc(sizeof(C<T>) * n_ * m_, "FGMRES preconditioned basis"));
    return device_control ? solve_device(rhs, x0, result) : solve_host(rhs, x0, result);
}

template <typename T>
GmresResult Gmres<T>::solve_host(const C<T> *rhs, const C<T> *x0, C<T> *result) {
    GmresResult res;
    iterations_done_ = 0;
    double bn = norm(rhs);
    bn_ = bn;
    if (bn == 0) {
        res.converged = true;
        res.arnoldi_be = 0;
        res.true_be = 0;
        return res;
    }
    apply(x0, r0_);
    VecOps<T>::sub(rhs, r0_, r0_, n_, s_);
    VecOps<T>::copy(r0_, w_, n_, s_);
    kernel_launches += 1;
    double beta = norm(w_);
    if (!std::isfinite(beta)) {
        res.converged = false;
        res.arnoldi_be = beta;
        res.true_be = -1;
        return res;
    }
    if (beta == 0) {
        if (x0 != result) VecOps<T>::copy(x0, result, n_, s_);
        res.converged = true;
        res.arnoldi_be = 0;
        res.true_be = 0;
        res.iterations = 1;
        return res;
    }
    double bea = -1, be = -1;
    int iter = 0;
    if (x0 != result) VecOps<T>::copy(x0, result, n_, s_);
    while (true) {
        VecOps<T>::scale(w_, 1.0 / beta, V_, n_, s_);
        kernel_launches += 1;
        h(0, m_) = beta;
        for (int i = 1; i <= m_; i++) h(i, m_) = 0.0;
        int jh = 0;
        bea = arnoldi(bn, jh);
        if (!std::isfinite(bea)) {
            // a non-finite vector (NaN or Inf from the operator or the
            // preconditioner) never converges: stop at once, not converged,
            // instead of running out the restarts on NaN (the reference has
            // no such check; finite runs are unchanged)
            res.converged = false;
            res.arnoldi_be = bea;
            res.true_be = -1;
            res.iterations = iterations_done_;
            return res;
        }
        if (bea < tol_) {
            be = final_actions(jh, rhs, result);
            res.converged = true;
            res.arnoldi_be = bea;
            res.true_be = be;
            res.iterations = iterations_done_;
            return res;
        }
        iter++;
        if (iter >= max_restarts_) break;
        // PrepareRestart with the true residual
        construct(jh, result);
        VecOps<T>::copy(result, w_, n_, s_);
        apply(w_, r0_);
        VecOps<T>::sub(rhs, r0_, r0_, n_, s_);
        VecOps<T>::copy(r0_, w_, n_, s_);
        kernel_launches += 1;
        beta = norm(w_);
    }
    be = final_actions(m_, rhs, result);
    res.converged = false;
    res.arnoldi_be = bea;
    res.true_be = be;
    res.iterations = iterations_done_;
    return res;
}

// ------------------------------------------------------------ device control
//
// One-thread kernels that take the host's decisions of GmresSolver
// (Extreme.Fgmres/Gmres.cs:77-348) on the device state GmState: the
// right-hand side and initial residual norms (:80-107), the classical
// Gram-Schmidt pass bookkeeping and its re-orthogonalisation test
// (:252-262, :297-313), the Givens rotations and the Arnoldi backward error
// (:271-292), and the upper-triangular solve of the solution update
// (:187-196, SimplifiedZtrsv). The arithmetic is the host driver's, in the
// same order; complex moduli and quotients use hypot and Smith's division.

__device__ __forceinline__ double cabs2(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj2(double2 a) { return make_double2(a.x, -a.y); }
// x, y <- c x + s y, c y - conj(s) x (zrot)
__device__ __forceinline__ void zrot_dev(double2 &x, double2 &y, double c, double2 s) {
    const double2 sy = cmul2(s, y), sx = cmul2(cconj2(s), x);
    const double2 t = make_double2(c * x.x + sy.x, c * x.y + sy.y);
    y = make_double2(c * y.x - sx.x, c * y.y - sx.y);
    x = t;
}

// a fresh solve: ||rhs|| from its squared norm
__global__ void k_gm_start(GmState *st, const double *norm2) {
    GmState g;
    memset(&g, 0, sizeof g);
    g.bn = sqrt(*norm2);
    g.flags = !isfinite(g.bn) ? kGmNonFinite : (g.bn == 0 ? kGmZero : 0);
    g.active = g.flags == 0;
    g.true_be = -1;
    *st = g;
}

// beta = ||r0||: a cycle starts (active) unless beta is 0 (the initial guess
// is exact: CheckForExactSolution, one iteration) or not finite
__global__ void k_gm_beta(GmState *st, const double *norm2, int first) {
    if (st->flags) return;
    const double beta = sqrt(*norm2);
    st->beta = beta;
    if (!isfinite(beta)) {
        st->flags |= kGmNonFinite;
        st->active = 0;
    } else if (beta == 0) {
        st->flags |= kGmExact;
        if (first) st->iterations = 1;
        st->active = 0;
    } else {
        st->active = 1;
    }
}

// the rhs column of H = beta e1; no steps yet
__global__ void k_gm_cycle(GmState *st, double2 *H, int m) {
    if (!st->active) return;
    for (int i = threadIdx.x; i <= m; i += blockDim.x)
        H[(size_t)m * (m + 1) + i] = make_double2(i == 0 ? st->beta : 0.0, 0.0);
    if (threadIdx.x == 0) st->jh = 0;
}

// one Gram-Schmidt pass of step j (pass 1: while active; later passes:
// while the previous one asked for another): h(0..j, j) += dots, dloo,
// ||w|| and the re-orthogonalisation test 2 ||w|| <= sqrt(dloo)
__global__ void k_gm_ortho(GmState *st, double2 *H, const double2 *dots, const double *norm2, int j, int m,
                           int pass, int max_pass) {
    if (!(pass == 1 ? st->active : st->reorth)) return;
    double2 *h = H + (size_t)j * (m + 1);
    double ss = 0;
    for (int i = 0; i <= j; i++) {
        const double2 d = dots[i];
        const double2 o = pass == 1 ? make_double2(0.0, 0.0) : h[i];
        h[i] = make_double2(o.x + d.x, o.y + d.y);
        ss += d.x * d.x + d.y * d.y;
    }
    st->dloo = ss;
    st->dnormw = sqrt(*norm2);
    st->reorth = (2.0 * st->dnormw <= sqrt(ss) && pass < max_pass) ? 1 : 0;
}

// the rest of step j: h(j+1, j) = ||w||, the previous rotations, zrotg,
// the rotation of the rhs column, bea = |g_{j+1}| / ||b||; the cycle stops
// when bea <= tol, after m steps, or on a non-finite bea
__global__ void k_gm_step(GmState *st, double2 *H, double *cs, double2 *sn, int j, int m, double tol) {
    if (!st->active) return;
    double2 *h = H + (size_t)j * (m + 1);
    double2 *g = H + (size_t)m * (m + 1);
    h[j + 1] = make_double2(st->dnormw, 0.0);
    for (int i = 0; i < j; i++) zrot_dev(h[i], h[i + 1], cs[i], sn[i]);
    {  // zrotg (classic reference algorithm)
        const double2 a = h[j], b = h[j + 1];
        double c;
        double2 sv;
        const double aa = cabs2(a);
        if (aa == 0.0) {
            c = 0.0;
            sv = make_double2(1.0, 0.0);
        } else {
            const double scale = aa + cabs2(b);
            const double a1 = cabs2(make_double2(a.x / scale, a.y / scale));
            const double b1 = cabs2(make_double2(b.x / scale, b.y / scale));
            const double nrm = scale * sqrt(a1 * a1 + b1 * b1);
            const double2 alpha = make_double2(a.x / aa, a.y / aa);
            c = aa / nrm;
            const double2 t = cmul2(alpha, cconj2(b));
            sv = make_double2(t.x / nrm, t.y / nrm);
        }
        cs[j] = c;
        sn[j] = sv;
    }
    zrot_dev(g[j], g[j + 1], cs[j], sn[j]);
    zrot_dev(h[j], h[j + 1], cs[j], sn[j]);
    h[j + 1] = make_double2(0.0, 0.0);
    const double bea = cabs2(g[j + 1]) / st->bn;
    st->bea = bea;
    st->iterations++;
    st->jh = j + 1;
    if (!isfinite(bea)) st->flags |= kGmNonFinite;
    if (!(bea > tol && j + 1 < m)) st->active = 0;
}

// y = H(0:jh, 0:jh) \ g (upper triangular, SimplifiedZtrsv) into coef;
// ncols = jh, or 0 when the solve ended before a cycle (zero rhs, exact
// guess, non-finite)
__global__ void k_gm_construct(GmState *st, const double2 *H, int m, double2 *coef) {
    const int jh = (st->flags & (kGmZero | kGmNonFinite)) || ((st->flags & kGmExact) && st->jh == 0) ? 0 : st->jh;
    for (int i = 0; i < jh; i++) coef[i] = H[(size_t)m * (m + 1) + i];
    for (int j = jh - 1; j >= 0; j--) {
        double2 y = coef[j];
        if (y.x != 0.0 || y.y != 0.0) {
            y = cdiv<double>(y, H[(size_t)j * (m + 1) + j]);
            coef[j] = y;
            for (int i = j - 1; i >= 0; i--) {
                const double2 t = cmul2(y, H[(size_t)j * (m + 1) + i]);
                coef[i] = make_double2(coef[i].x - t.x, coef[i].y - t.y);
            }
        }
    }
    st->ncols = jh;
}

// true backward error ||b - A x|| / ||b||
__global__ void k_gm_true(GmState *st, const double *norm2) {
    st->true_be = st->flags & kGmZero ? 0.0 : sqrt(*norm2) / st->bn;
}

__global__ void k_gm_count(const int *live, long long *count) {
    if (*live) ++*count;
}

// an operator apply of the solve; in an enqueue-only solve it may be
// speculative (its cycle already stopped): it runs all the same, but only a
// live one is counted (on the device)
template <typename T>
void Gmres<T>::apply_counted(const C<T> *x, C<T> *y, const int *live) {
    apply(x, y);
    if (enqueue_only) {
        k_gm_count<<<1, 1, 0, s_>>>(live, napp_dev_);
        kernel_launches += 1;
    }
}

template <typename T>
long Gmres<T>::live_applies() {
    long long v = 0;
    EGX_CUDA(cudaMemcpyAsync(&v, napp_dev_, sizeof v, cudaMemcpyDeviceToHost, s_));
    EGX_CUDA(cudaStreamSynchronize(s_));
    return (long)v;
}

template <typename T>
void Gmres<T>::reset_apply_counts() {
    EGX_CUDA(cudaMemsetAsync(napp_dev_, 0, sizeof(long long), s_));
}

template <typename T>
void Gmres<T>::dc_norm(const C<T> *x, const int *live) {
    VecOps<T>::norm2(x, n_, norm_dev_, reinterpret_cast<double *>(partials_), nblocks_, s_, live);
    kernel_launches += 2;
}

template <typename T>
GmState Gmres<T>::read_state() {
    EGX_CUDA(cudaMemcpyAsync(hst_, st_, sizeof(GmState), cudaMemcpyDeviceToHost, s_));
    EGX_CUDA(cudaStreamSynchronize(s_));
    return *hst_;
}

// w = rhs - A x (x: the initial guess or the current solution, never one of
// this solver's vectors) and beta = ||w||; first: the initial residual
// (predicated on a non-zero right-hand side)
template <typename T>
void Gmres<T>::dc_residual(const C<T> *rhs, const C<T> *x, bool first) {
    const int *live = first ? &st_->active : nullptr;
    apply_counted(x, r0_, &st_->active);
    VecOps<T>::sub(rhs, r0_, w_, n_, s_, live);
    kernel_launches += 1;
    dc_norm(w_, live);
    k_gm_beta<<<1, 1, 0, s_>>>(st_, norm_dev_, first ? 1 : 0);
    kernel_launches += 1;
}

// Arnoldi step j of the cycle (KrylovSubspaceConstruction, one iteration)
template <typename T>
void Gmres<T>::dc_step(int j) {
    const int *live = &st_->active;
    const int *more = &st_->reorth;
    C<T> *vj = V_ + (long)j * n_;
    if (precond) {
        C<T> *zj = Z_ + (long)j * n_;
        precond(vj, zj);
        apply_counted(zj, w_, live);
    } else {
        apply_counted(vj, w_, live);
    }
    const int koff = sizeof(T) == sizeof(double) ? 0 : EGX_K_C64;
    for (int pass = 1; pass <= 3; pass++) {
        const int *p = pass == 1 ? live : more;
        int ev = timers ? timers->begin(EGX_K_GS_DOTS + koff, s_) : -1;
        VecOps<T>::multi_dot(V_, j + 1, w_, n_, dots_, partials_, nblocks_, s_, p);
        if (timers) timers->end(ev, s_);
        ev = timers ? timers->begin(EGX_K_GS_UPDATE + koff, s_) : -1;
        VecOps<T>::update_norm(V_, j + 1, dots_, w_, n_, norm_dev_, reinterpret_cast<double *>(partials_), nblocks_,
                               s_, p);
        if (timers) timers->end(ev, s_);
        k_gm_ortho<<<1, 1, 0, s_>>>(st_, Hd_, dots_, norm_dev_, j, m_, pass, 3);
        kernel_launches += 5;
    }
    if (j < m_ - 1) {
        VecOps<T>::divide_dev(w_, &st_->dnormw, V_ + (long)(j + 1) * n_, n_, s_, live);
        kernel_launches += 1;
    }
    k_gm_step<<<1, 1, 0, s_>>>(st_, Hd_, csd_, snd_, j, m_, tol_);
    kernel_launches += 1;
}

// ConstructCurrentSolution: result += (Z or V)[:, :jh] y
template <typename T>
void Gmres<T>::dc_construct(C<T> *result) {
    k_gm_construct<<<1, 1, 0, s_>>>(st_, Hd_, m_, coef_);
    VecOps<T>::gemv(precond ? Z_ : V_, m_, coef_, r0_, n_, s_, &st_->ncols);
    VecOps<T>::add(r0_, result, n_, s_, &st_->ncols);
    kernel_launches += 3;
}

template <typename T>
GmresResult Gmres<T>::solve_device(const C<T> *rhs, const C<T> *x0, C<T> *result) {
    GmresResult res;
    const int *live = &st_->active;
    dc_norm(rhs, nullptr);
    k_gm_start<<<1, 1, 0, s_>>>(st_, norm_dev_);
    kernel_launches += 1;
    if (!enqueue_only) {  // the reference applies nothing for a zero right-hand side
        const GmState g = read_state();
        if (g.flags & kGmZero) {
            res.converged = true;
            res.arnoldi_be = res.true_be = 0;
            return res;
        }
        if (g.flags) {
            res.arnoldi_be = g.bn;
            return res;
        }
    }
    dc_residual(rhs, x0, true);
    if (x0 != result) VecOps<T>::copy(x0, result, n_, s_);
    // one true-residual evaluation at the end (FinalActions / CheckBackwardError)
    auto true_be = [&]() {
        if (!check_true_) return -1.0;
        dc_residual(rhs, result, false);
        k_gm_true<<<1, 1, 0, s_>>>(st_, norm_dev_);
        kernel_launches += 1;
        return read_state().true_be;
    };
    int iter = 0;
    GmState g{};
    while (true) {
        if (!enqueue_only) {
            g = read_state();
            if (g.flags & kGmExact) {  // CheckForExactSolution, or a zero residual at a restart
                res.converged = true;
                res.arnoldi_be = res.true_be = 0;
                res.iterations = g.iterations;
                return res;
            }
            if (g.flags) {  // non-finite residual
                res.arnoldi_be = g.beta;
                res.iterations = g.iterations;
                return res;
            }
        }
        // V[:, 0] = w / beta, g = beta e1
        VecOps<T>::divide_dev(w_, &st_->beta, V_, n_, s_, live);
        k_gm_cycle<<<1, 32, 0, s_>>>(st_, Hd_, m_);
        kernel_launches += 2;
        for (int j = 0; j < m_; j++) {
            dc_step(j);
            if (!enqueue_only) {
                g = read_state();
                if (!g.active) break;
            }
        }
        if (enqueue_only) break;  // one cycle, the device decides everything
        if (g.flags & kGmNonFinite) {
            res.arnoldi_be = g.bea;
            res.iterations = g.iterations;
            return res;
        }
        if (g.bea < tol_) {  // FinalActions
            dc_construct(result);
            res.converged = true;
            res.arnoldi_be = g.bea;
            res.iterations = g.iterations;
            res.true_be = true_be();
            return res;
        }
        iter++;
        if (iter >= max_restarts_) break;
        // PrepareRestart with the true residual
        dc_construct(result);
        dc_residual(rhs, result, false);
    }
    // not converged within the restarts (or the enqueue-only single cycle)
    dc_construct(result);
    if (enqueue_only) return res;
    res.arnoldi_be = g.bea;
    res.iterations = g.iterations;
    res.true_be = true_be();
    return res;
}

template class Gmres<double>;
template class Gmres<float>;

}  // namespace egx
