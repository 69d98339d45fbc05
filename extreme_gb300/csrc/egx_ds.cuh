// Double-FP32 ("double-single") helpers: a complex128 value carried as a
// pair of floats hi + lo (47 significant bits) and dot products computed as
// Dot2 (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26 (2005), Algorithm 5.3) on the FP32 pipes, which GB300 runs at
// 64 times its complex128 FMA rate.
#pragma once

namespace egx {

// v = h + l: h keeps the sign, the exponent and the top 23 stored mantissa
// bits of v, l the next 23 bits; built from the bit pattern with integer
// and FP32 operations only (no complex128 conversion in the hot loop).
// |v| < 2^-80 keeps only h; |v| < 2^-126 flushes to zero.
__device__ __forceinline__ void ds_split(double v, float &h, float &l) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const unsigned w1 = (unsigned)(u >> 32), w0 = (unsigned)u;
    const unsigned sgn = w1 & 0x80000000u;
    const int e = (int)((w1 >> 20) & 0x7FFu);
    const int eh = e - 896;  // biased float exponent of h
    const unsigned mh = ((w1 & 0xFFFFFu) << 3) | (w0 >> 29);
    h = (eh >= 1 && eh <= 254) ? __int_as_float((int)(sgn | ((unsigned)eh << 23) | mh)) : 0.f;
    const unsigned r = (w0 & 0x1FFFFFFFu) >> 6;                                     // 23 bits
    const float fr = __fsub_rn(__int_as_float((int)(0x4B000000u | r)), 8388608.f);  // exactly r
    const int el = e - 942;  // biased float exponent of 2^(e - 1023 - 46)
    const float sc = (el >= 1 && el <= 254) ? __int_as_float(el << 23) : 0.f;
    l = __int_as_float(__float_as_int(__fmul_rn(fr, sc)) | (int)sgn);
}

// (s, c) += (ah + al)(bh + bl): TwoProduct of the high parts, the cross
// terms into its error, TwoSum into s, both errors into c
__device__ __forceinline__ void ds_dot2(float &s, float &c, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    c = __fadd_rn(c, __fadd_rn(err, e));
    s = t;
}

}  // namespace egx
