// pgb_f3.cuh -- FP64-accurate dot products and updates on the FP32 pipe,
// for the Gram-Schmidt kernels of the FP64 form.
//
// On GB300 the FP64 pipe retires two lanes per clock per SM, so a
// Gram-Schmidt pass (one FP64 FMA per basis element in the projections and
// one in the update) is bound by it well below the HBM bandwidth.  Here an
// FP64 value is split exactly into three FP32 pieces with integer
// operations (24 + 23 + 6 significant bits), and products are accumulated
// at three levels: the leading products exactly (two-product + two-sum),
// the cross products of relative size 2^-24 and 2^-48 in plain FP32.  The
// result of a dot product carries an error of about 2^-48 of the level-1
// sum, i.e. ~2^-53 relative to sum |w_i x_i| -- the size of an FP64 dot
// product's own rounding -- and costs ~40 FP32/INT operations per element
// instead of one FP64 FMA.
#pragma once
#include "pgb.cuh"

namespace pgb {

struct F3 {
    float a, b, c;  // value = a + b + c
};

// v 2^-shift as a + b + c, exactly when 2^-74 <= |v 2^-shift| < 2^128;
// smaller magnitudes give 0 (callers scale so that values are <= 1, where
// a dropped value is below 2^-74 of the largest), larger ones +-inf
__device__ __forceinline__ F3 f3_split(double v, int shift)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(bits >> 32), lo = (unsigned)bits;
    const int eb = (int)((hi >> 20) & 0x7ffu);
    const int e = eb - shift;
    const unsigned sgn = hi & 0x80000000u;
    F3 r;
    if (eb == 0 || e < 949) {
        r.a = r.b = r.c = 0.f;
    } else if (e > 1150) {
        r.a = __uint_as_float(sgn | 0x7F800000u);
        r.b = r.c = 0.f;
    } else {
        r.a = __uint_as_float(sgn | ((unsigned)(e - 896) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
        const unsigned R = lo & 0x1FFFFFFFu;  // the 29 bits below a, weight 2^(e - 1075)
        const float fb = __uint_as_float(0x4B000000u | (R >> 6)) - 8388608.0f;
        const float fc = __uint_as_float(0x4B000000u | (R & 63u)) - 8388608.0f;
        r.b = __uint_as_float(__float_as_uint(fb * __uint_as_float((unsigned)(e - 942) << 23)) | sgn);
        r.c = __uint_as_float(__float_as_uint(fc * __uint_as_float((unsigned)(e - 948) << 23)) | sgn);
    }
    return r;
}

// biased FP64 exponent field of v (0 for zero and subnormals)
__device__ __forceinline__ int f3_expo(double v)
{
    return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ffu);
}

// 2^k as an FP64 value (-1022 <= k <= 1023)
__device__ __forceinline__ double f3_pow2(int k) { return __longlong_as_double((long long)(k + 1023) << 52); }

// sum of products w x at three levels
struct F3Acc {
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, s2 = 0.f;
    __device__ __forceinline__ void add(const F3 &w, const F3 &x)
    {
        const float p = w.a * x.a;
        const float pe = fmaf(w.a, x.a, -p);  // p + pe = w.a x.a exactly
        const float t = s0 + p;
        const float bp = t - s0;
        c0 += (s0 - (t - bp)) + (p - bp);  // t + err = s0 + p exactly
        s0 = t;
        s1 = fmaf(w.a, x.b, s1);
        s1 = fmaf(w.b, x.a, s1);
        s1 += pe;
        s2 = fmaf(w.b, x.b, s2);
        s2 = fmaf(w.a, x.c, s2);
        s2 = fmaf(w.c, x.a, s2);
    }
    __device__ __forceinline__ double value() const
    {
        return (double)s0 + ((double)c0 + ((double)s1 + (double)s2));
    }
};

}  // namespace pgb
