// Batched, interleaved 2-D DFT building blocks (FFTW plan_many_dft rank 2,
// stride = howmany, dist = 1, unnormalised; Fft/FftW/FftWTransform.cs:218-225).
//
// One CTA transforms `bt` interleaved sequences of length n held in shared
// memory as buf[idx * bt + col]. The transform is a Stockham autosort FFT
// (Govindaraju et al., "High performance discrete Fourier transforms on
// graphics processors", SC 2008): each stage of radix R reads element
// j + r*n/R, multiplies by the twiddle W_n^{(j mod Ns) * r * n/(Ns R)}, does
// an in-register radix-R DFT and writes to (j/Ns)*Ns*R + (j mod Ns) + r*Ns,
// ping-ponging between two shared buffers. Radices 2..8 cover every
// 7-smooth length.
#pragma once

#include "egx_common.cuh"

namespace egx {

struct FftPlan {
    int n;
    int nstages;
    int radix[16];
};

// Host: radix sequence for n (prefers 8, then 4, 2, and 7, 6, 5, 3).
inline FftPlan make_fft_plan(int n) {
    FftPlan p;
    p.n = n;
    p.nstages = 0;
    int m = n;
    while (m > 1) {
        int r = 0;
        const int pref[] = {8, 4, 2, 7, 6, 5, 3};
        for (int c : pref) {
            if (m % c == 0) {
                r = c;
                break;
            }
        }
        if (r == 0) throw Error(EGX_ERR_INVALID, "FFT length " + std::to_string(n) + " is not 7-smooth");
        // keep a lone factor 2 from ending next to an 8 when 4*4 would do
        p.radix[p.nstages++] = r;
        m /= r;
        if (p.nstages >= 16) throw Error(EGX_ERR_INVALID, "FFT length too large");
    }
    return p;
}

template <typename T> struct Const;
template <> struct Const<double> {
    static __device__ __forceinline__ double h() { return 0.7071067811865476; }
};
template <> struct Const<float> {
    static __device__ __forceinline__ float h() { return 0.70710678f; }
};

// multiply by -i*sign ... helpers: rot(v, s) = v * (s * i)
template <typename T> __device__ __forceinline__ C<T> mul_i(C<T> v, int sign) {
    // v * (sign * i)
    return sign > 0 ? mk<T>(-v.y, v.x) : mk<T>(v.y, -v.x);
}

// In-register DFT of length R with exponent sign `sign` (-1 forward).
template <typename T> __device__ __forceinline__ void dft2(C<T> &a, C<T> &b) {
    C<T> t = a;
    a = cadd<T>(t, b);
    b = csub<T>(t, b);
}

template <typename T> __device__ __forceinline__ void dft4(C<T> *v, int sign) {
    C<T> a0 = cadd<T>(v[0], v[2]), a1 = csub<T>(v[0], v[2]);
    C<T> b0 = cadd<T>(v[1], v[3]), b1 = mul_i<T>(csub<T>(v[1], v[3]), sign);
    v[0] = cadd<T>(a0, b0);
    v[2] = csub<T>(a0, b0);
    v[1] = cadd<T>(a1, b1);
    v[3] = csub<T>(a1, b1);
}

template <typename T> __device__ __forceinline__ void dft8(C<T> *v, int sign) {
    C<T> e[4] = {v[0], v[2], v[4], v[6]};
    C<T> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<T>(e, sign);
    dft4<T>(o, sign);
    const T h = Const<T>::h();
    // o[k] *= W8^k (W8 = exp(sign*2*pi*i/8))
    o[1] = mk<T>(h * (o[1].x - sign * o[1].y), h * (o[1].y + sign * o[1].x));
    o[2] = mul_i<T>(o[2], sign);
    o[3] = mk<T>(h * (-o[3].x - sign * o[3].y), h * (-o[3].y + sign * o[3].x));
    for (int k = 0; k < 4; k++) {
        v[k] = cadd<T>(e[k], o[k]);
        v[k + 4] = csub<T>(e[k], o[k]);
    }
}

// Odd radices: direct DFT with the correctly rounded cos/sin of 2*pi*m/R.
template <typename T, int R> __device__ __forceinline__ void dft_odd(C<T> *v, int sign) {
    T cs[R], sn[R];
    cs[0] = 1;
    sn[0] = 0;
    if (R == 3) {
        cs[1] = -0.5; sn[1] = 0.8660254037844386;
    } else if (R == 5) {
        cs[1] = 0.30901699437494745; sn[1] = 0.9510565162951535;
        cs[2] = -0.8090169943749475; sn[2] = 0.5877852522924731;
    } else if (R == 7) {
        cs[1] = 0.6234898018587335; sn[1] = 0.7818314824680298;
        cs[2] = -0.2225209339563144; sn[2] = 0.9749279121818236;
        cs[3] = -0.9009688679024191; sn[3] = 0.4338837391175581;
    }
#pragma unroll
    for (int m = 1; m <= (R - 1) / 2; m++) {
        cs[R - m] = cs[m];
        sn[R - m] = -sn[m];
    }
    C<T> out[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        C<T> acc = v[0];
#pragma unroll
        for (int r = 1; r < R; r++) {
            int m = (r * k) % R;
            C<T> w = mk<T>(cs[m], sign * sn[m]);
            cfma<T>(acc, v[r], w);
        }
        out[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < R; k++) v[k] = out[k];
}

template <typename T> __device__ __forceinline__ void dft6(C<T> *v, int sign) {
    // 6 = 2 x 3 (Good-Thomas free: plain Cooley-Tukey with W6 twiddles)
    C<T> a[3] = {v[0], v[2], v[4]};
    C<T> b[3] = {v[1], v[3], v[5]};
    dft_odd<T, 3>(a, sign);
    dft_odd<T, 3>(b, sign);
    // b[k] *= W6^k
    const T c1 = 0.5, s1 = 0.8660254037844386;
    b[1] = mk<T>(b[1].x * c1 - sign * s1 * b[1].y, b[1].y * c1 + sign * s1 * b[1].x);
    b[2] = mk<T>(-b[2].x * c1 - sign * s1 * b[2].y, -b[2].y * c1 + sign * s1 * b[2].x);
    for (int k = 0; k < 3; k++) {
        v[k] = cadd<T>(a[k], b[k]);
        v[k + 3] = csub<T>(a[k], b[k]);
    }
}

template <typename T, int R>
__device__ __forceinline__ void stage_items(const C<T> *__restrict__ src, C<T> *__restrict__ dst, int n, int bt,
                                            int Ns, const C<T> *__restrict__ tw, int sign) {
    const int nb = n / R;
    const int items = nb * bt;
    const int tstep = n / (Ns * R);
    for (int item = threadIdx.x; item < items; item += blockDim.x) {
        int j = item / bt;
        int col = item - j * bt;
        int jm = j % Ns;
        C<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = src[(j + r * nb) * bt + col];
        if (Ns > 1) {
            int t = jm * tstep;
#pragma unroll
            for (int r = 1; r < R; r++) {
                C<T> w = tw[(t * r) % n];
                if (sign > 0) w.y = -w.y;
                v[r] = cmul<T>(v[r], w);
            }
        }
        if (R == 2) dft2<T>(v[0], v[1]);
        else if (R == 4) dft4<T>(v, sign);
        else if (R == 8) dft8<T>(v, sign);
        else if (R == 6) dft6<T>(v, sign);
        else dft_odd<T, R>(v, sign);
        int idxD = (j / Ns) * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) dst[(idxD + r * Ns) * bt + col] = v[r];
    }
}

// Transform bt columns of length n held in a; b is scratch of the same size.
// Returns the buffer that holds the result. Must be called by all threads.
// tw: forward twiddles W_n^m = exp(-2*pi*i*m/n), m = 0..n-1.
template <typename T>
__device__ C<T> *fft_smem(C<T> *a, C<T> *b, const FftPlan &plan, int bt, const C<T> *__restrict__ tw, int sign) {
    int Ns = 1;
    const int n = plan.n;
    for (int s = 0; s < plan.nstages; s++) {
        const int R = plan.radix[s];
        switch (R) {
            case 2: stage_items<T, 2>(a, b, n, bt, Ns, tw, sign); break;
            case 3: stage_items<T, 3>(a, b, n, bt, Ns, tw, sign); break;
            case 4: stage_items<T, 4>(a, b, n, bt, Ns, tw, sign); break;
            case 5: stage_items<T, 5>(a, b, n, bt, Ns, tw, sign); break;
            case 6: stage_items<T, 6>(a, b, n, bt, Ns, tw, sign); break;
            case 7: stage_items<T, 7>(a, b, n, bt, Ns, tw, sign); break;
            default: stage_items<T, 8>(a, b, n, bt, Ns, tw, sign); break;
        }
        __syncthreads();
        C<T> *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Host-side twiddle table W_n^m = exp(-2*pi*i*m/n).
std::vector<double> twiddles(int n);

// Columns per CTA so that the two shared buffers stay near 64 KB.
inline int fft_cols(int n, size_t elem) {
    int bt = (int)(32768 / ((size_t)n * elem));
    if (bt < 1) bt = 1;
    int p = 1;
    while (p * 2 <= bt && p < 16) p *= 2;
    return p;
}

}  // namespace egx
