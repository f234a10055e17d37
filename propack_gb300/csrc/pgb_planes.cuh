// pgb_planes.cuh -- FP64-accurate products on the FP32 pipe from "planes":
// an FP64 value w held as two FP32 numbers hi + lo (the leading 24 and the
// next 23 bits of w, cut with integer operations), so that a product costs
// 12 FP32 operations (hi*hi as an exact two-product folded into a two-sum,
// the cross terms hi*lo and lo*hi into the compensation) instead of one FMA
// on GB300's FP64 pipe, which retires two lanes per clock per SM.  The error
// of a sum of products is a few 2^-48 of sum |w_i x_i|.  Used by the
// Gram-Schmidt kernels of the single-problem path (pgb_lanczos.cu) and by
// the batched kernel (pgb_batch.cu).
#pragma once
#include "pgb.cuh"
#include "pgb_f3.cuh"

namespace pgb {

// s + c: a sum of products kept as an unevaluated FP32 pair
struct PlAcc {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float ah, float al, float bh, float bl)
    {
        const float p = ah * bh;
        const float pe = fmaf(ah, bh, -p);  // p + pe = ah bh exactly
        const float t = s + p;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (p - bp);  // t + err = s + p exactly
        c = fmaf(ah, bl, c);
        c = fmaf(al, bh, c);
        c += pe + err;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
    // the same sum widened with integer operations (no FP64-pipe conversion)
    __device__ __forceinline__ double value_int() const;
};

// f as an FP64 value with integer operations only (no FP64-pipe conversion);
// FP32 subnormals (|f| < 2^-126) become 0, infinities and NaNs stay so
__device__ __forceinline__ double pl_f2d(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    const unsigned long long ee = e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u);
    const unsigned long long m = (unsigned long long)(u & 0x7fffffu) << 29;
    return e == 0 ? 0.0 : __longlong_as_double((long long)(sgn | (ee << 52) | m));
}

// (s, c) += (s2, c2) for compensated pairs: the leading parts by a two-sum
__device__ __forceinline__ void pl_pair_add(float &s, float &c, float s2, float c2)
{
    const float t = s + s2;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (s2 - bp);
    c = (c + c2) + e;
    s = t;
}
// Sum four compensated pairs over the warp with FP32 operations only, by a
// transposed butterfly: at offset 16 a lane keeps two of the four sums and
// sends the other two, at offset 8 one of its two, then one sum travels
// the last three offsets (12 shuffles instead of 40).  Lanes 8u .. 8u+7
// end with the total of acc[u].  The order of additions is fixed.
__device__ __forceinline__ PlAcc pl_warp_sum4(const PlAcc *acc)
{
    const unsigned F = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool b4 = lane & 16, b3 = lane & 8;
    PlAcc k0 = b4 ? acc[2] : acc[0], k1 = b4 ? acc[3] : acc[1];
    const PlAcc g0 = b4 ? acc[0] : acc[2], g1 = b4 ? acc[1] : acc[3];
    pl_pair_add(k0.s, k0.c, __shfl_xor_sync(F, g0.s, 16), __shfl_xor_sync(F, g0.c, 16));
    pl_pair_add(k1.s, k1.c, __shfl_xor_sync(F, g1.s, 16), __shfl_xor_sync(F, g1.c, 16));
    PlAcc k = b3 ? k1 : k0;
    const PlAcc g = b3 ? k0 : k1;
    pl_pair_add(k.s, k.c, __shfl_xor_sync(F, g.s, 8), __shfl_xor_sync(F, g.c, 8));
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) pl_pair_add(k.s, k.c, __shfl_xor_sync(F, k.s, o), __shfl_xor_sync(F, k.c, o));
    return k;
}

// the planes of a basis element, with integer operations only: the leading
// 24 and the next 23 bits of w (|w| <= 1; parts below 2^-74 are dropped).
// Conversions between FP64 and FP32 run on the FP64 pipe, which retires two
// lanes per clock per SM on GB300.
__device__ __forceinline__ float2 pl_split(double w)
{
    const F3 f = f3_split(w, 0);
    return make_float2(f.a, f.b);
}
__device__ __forceinline__ float4 pl_split2(double2 w)
{
    const float2 a = pl_split(w.x), b = pl_split(w.y);
    return make_float4(a.x, a.y, b.x, b.y);
}
// x 2^-shift as (hi, lo) planes with integer operations only (the FP64
// pipe stays free): the leading 24 and the next 23 bits of the value
__device__ __forceinline__ float2 pl_xsplit(double x, int shift)
{
    const F3 f = f3_split(x, shift);
    return make_float2(f.a, f.b);
}

__device__ __forceinline__ double PlAcc::value_int() const { return pl_f2d(s) + pl_f2d(c); }

}  // namespace pgb
