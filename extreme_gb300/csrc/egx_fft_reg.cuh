// Register-resident batched DFT of BT interleaved columns of length
// N = R1 * R2 * R3 (R1 == R2 >= R3), three radix passes with two exchanges
// through one shared buffer S[N][BT] (BT columns of a row are contiguous, so
// every shared and global access of a warp covers whole 128-byte rows).
//
// Index maps (a mixed-radix decimation in frequency, written out for
// three digits): with M = R2 R3, n = m + M r1 and k = k1 + R1 k',
//   pass 1 (thread m):        y[k1][m]  = W_N^{m k1} DFT_R1(x[m + M r1])[k1]
//   pass 2 (thread k1, p):    z[k1][k2][p] = W_M^{p k2} DFT_R2(y[k1][p + R3 r2])[k2]
//   pass 3 (thread k1, k2):   X[k1 + R1 (k2 + R2 k3)] = DFT_R3(z[k1][k2][p])[k3]
// (W_N = exp(sign 2 pi i / N); sign -1 is FFTW's forward transform).
//
// Threads: TPC = N / R1 per column, TPC * BT per CTA; thread t handles
// column t % BT and row index t / BT of each pass.
#pragma once

#include "egx_fft.cuh"

namespace egx {

template <typename T, int R>
__device__ __forceinline__ void dft_r(C<T> *v, int sign) {
    if (R == 2) dft2<T>(v[0], v[1]);
    else if (R == 4) dft4<T>(v, sign);
    else if (R == 8) dft8<T>(v, sign);
    else dft_odd<T, R>(v, sign);
}

template <typename T>
__device__ __forceinline__ C<T> twiddle(const C<T> *__restrict__ tw, int idx, int sign) {
    C<T> w = tw[idx];
    if (sign > 0) w.y = -w.y;
    return w;
}

template <int N> struct RegFft;
template <> struct RegFft<64> { static constexpr int R1 = 4, R2 = 4, R3 = 4; };
template <> struct RegFft<128> { static constexpr int R1 = 8, R2 = 8, R3 = 2; };
template <> struct RegFft<256> { static constexpr int R1 = 8, R2 = 8, R3 = 4; };
template <> struct RegFft<512> { static constexpr int R1 = 8, R2 = 8, R3 = 8; };

inline bool reg_fft_ok(int n) { return n == 64 || n == 128 || n == 256 || n == 512; }

// columns per CTA: 128-byte rows (BT), or 64-byte rows (BTN: twice the CTAs
// of half the size, which overlap their load, exchange and store phases
// better where the pass is latency-bound)
template <typename T> struct RegCols {
    static constexpr int BT = 128 / (int)sizeof(C<T>);
    static constexpr int BTN = 64 / (int)sizeof(C<T>);
};

template <int N, typename T, int BT = RegCols<T>::BT> constexpr int reg_threads() { return N / RegFft<N>::R1 * BT; }

template <int N, typename T, int BT = RegCols<T>::BT> constexpr size_t reg_smem() {
    return (size_t)N * BT * sizeof(C<T>);
}

// resident CTAs per SM the latency-bound y passes are compiled for: a full
// SM of threads, at most four CTAs
template <int N, typename T, int BT = RegCols<T>::BT> constexpr int reg_min_blocks() {
    return 2048 / reg_threads<N, T, BT>() < 4 ? 2048 / reg_threads<N, T, BT>() : 4;
}

// load(n) -> C<T> (element n of this thread's column), store(k, v)
template <typename T, int N, int BT = RegCols<T>::BT, class Load, class Store>
__device__ __forceinline__ void fft_reg(C<T> *S, const C<T> *__restrict__ tw, int sign, Load load, Store store) {
    constexpr int R1 = RegFft<N>::R1, R2 = RegFft<N>::R2, R3 = RegFft<N>::R3;
    constexpr int M = R2 * R3, TPC = N / R1;
    static_assert(R1 == R2 && R3 <= R1 && R1 * R2 * R3 == N, "radix plan");
    const int c = threadIdx.x % BT, u = threadIdx.x / BT;
    // pass 1: thread m = u
    {
        C<T> v[R1];
#pragma unroll
        for (int r = 0; r < R1; r++) v[r] = load(u + M * r);
        dft_r<T, R1>(v, sign);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            if (k1) v[k1] = cmul<T>(v[k1], twiddle<T>(tw, (u * k1) % N, sign));
            S[(k1 * M + u) * BT + c] = v[k1];
        }
    }
    __syncthreads();
    // pass 2: thread (k1, p), TPC = R1 * R3 of them
    {
        const int k1 = u / R3, p = u - k1 * R3;
        C<T> v[R2];
#pragma unroll
        for (int r = 0; r < R2; r++) v[r] = S[(k1 * M + p + R3 * r) * BT + c];
        __syncthreads();
        dft_r<T, R2>(v, sign);
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) {
            if (k2) v[k2] = cmul<T>(v[k2], twiddle<T>(tw, (R1 * p * k2) % N, sign));
            S[((k1 * R2 + k2) * R3 + p) * BT + c] = v[k2];
        }
    }
    __syncthreads();
    // pass 3: items (k1, k2), R1 * R2 of them
#pragma unroll
    for (int it = 0; it < (R1 * R2) / TPC; it++) {
        const int u3 = u + it * TPC;
        C<T> v[R3];
#pragma unroll
        for (int p = 0; p < R3; p++) v[p] = S[(u3 * R3 + p) * BT + c];
        dft_r<T, R3>(v, sign);
        const int k1 = u3 / R2, k2 = u3 - k1 * R2;
#pragma unroll
        for (int k3 = 0; k3 < R3; k3++) store(k1 + R1 * (k2 + R2 * k3), v[k3]);
    }
}

}  // namespace egx
