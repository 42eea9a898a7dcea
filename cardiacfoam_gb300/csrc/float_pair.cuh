// Float-pair arithmetic: a value held as hi + lo, two floats with
// |lo| <= ulp(hi) / 2, about 48 significant bits, computed on the FP32 pipe.
// GB300 issues FP64 at 1/64 of the FP32 rate, so an FP64 multiply-add costs
// as much pipe time as several dozen FP32 operations; the error-free
// transformations below (Knuth's two-sum, Dekker's product with fmaf for the
// rounding error) give near-FP64 accuracy for a handful of FP32 operations.
//
// Every rounded operation is an _rn intrinsic, so that no multiply-add
// contraction or reassociation changes it.  The additions are the "sloppy"
// form: the error of a + b is within a few units of 2^-48 max(|a|, |b|),
// which is what the solvers need (their residual updates carry the same
// kind of absolute error in FP64).  Values below 2^-126 lose their low part
// gradually and read as zero below 2^-149: callers scale their systems so
// that the quantities stay well inside the float range.
#pragma once

#include <cuda_runtime.h>

namespace cfg {
namespace fp {

using P = float2;   // x: high part, y: low part

__device__ __forceinline__ P make(float h, float l = 0.0f) { return make_float2(h, l); }

// s + e with |e| <= ulp(s): renormalised pair
__device__ __forceinline__ P quick(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}

// a + b exactly as s + e (no precondition on the magnitudes)
__device__ __forceinline__ P two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}

__device__ __forceinline__ P add(P a, P b)
{
    const P s = two_sum(a.x, b.x);
    return quick(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}

__device__ __forceinline__ P neg(P a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ P sub(P a, P b) { return add(a, neg(b)); }

__device__ __forceinline__ P abs(P a) { return a.x < 0.0f ? neg(a) : a; }

__device__ __forceinline__ P mul(P a, P b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return quick(p, e);
}

// a * b + c
__device__ __forceinline__ P madd(P a, P b, P c)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const P s = two_sum(c.x, p);
    return quick(s.x, __fadd_rn(s.y, __fadd_rn(e, c.y)));
}

// a / b: the float quotient, corrected once by the pair remainder
__device__ __forceinline__ P div(P a, P b)
{
    const float q1 = __fdiv_rn(a.x, b.x);
    const P r = madd(make_float2(-q1, 0.0f), b, a);
    const float q2 = __fdiv_rn(r.x, b.x);
    return quick(q1, q2);
}

// a < b for renormalised pairs
__device__ __forceinline__ bool less(P a, P b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }

__device__ __forceinline__ double join(P a) { return double(a.x) + double(a.y); }

// Sum of products kept unrenormalised between terms (hi by two-sum, the
// rounding errors and low-order cross terms gathered in lo): fewer
// operations than madd per term; value() renormalises.
struct Acc {
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void add_prod(P a, P b)
    {
        const float p = __fmul_rn(a.x, b.x);
        float e = __fmaf_rn(a.x, b.x, -p);
        e = __fmaf_rn(a.x, b.y, e);
        e = __fmaf_rn(a.y, b.x, e);
        const P s = two_sum(h, p);
        h = s.x;
        l = __fadd_rn(l, __fadd_rn(s.y, e));
    }
    __device__ __forceinline__ void sub_prod(P a, P b) { add_prod(neg(a), b); }
    __device__ __forceinline__ P value() const { return quick(h, l); }
};

// v * 2^shift as a renormalised pair, from the bit pattern of v with integer
// operations (the FP64 pipe is not used): hi takes the leading 24
// significant bits (truncated), lo the next 29 rounded to 24, which leaves
// |v 2^shift - hi - lo| <= 2^-48 |v 2^shift|.  Results below 2^-126 read as
// zero, beyond the float range as infinity; NaN stays NaN.
__device__ __forceinline__ P split(double v, int shift = 0)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const unsigned hw = unsigned(b >> 32), lw = unsigned(b);
    const unsigned sign = hw & 0x80000000u;
    const int eb = int((hw >> 20) & 0x7ffu);
    if (eb == 0x7ff) return make_float2(__double2float_rn(v), 0.0f);
    const int e = eb + shift;
    const int ef = e - 896;                // biased float exponent of 2^(e - 1023)
    if (eb == 0 || ef <= 0) return make_float2(__uint_as_float(sign), 0.0f);
    if (ef >= 255) return make_float2(__uint_as_float(sign | 0x7f800000u), 0.0f);
    const float hi =
        __uint_as_float(sign | (unsigned(ef) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
    const int es = e - 948;                // biased float exponent of 2^(e - 1075)
    const float rem = es > 0 ? __fmul_rn(__uint2float_rn(lw & 0x1fffffffu),
                                         __uint_as_float(unsigned(es) << 23))
                             : 0.0f;
    return quick(hi, __uint_as_float(__float_as_uint(rem) | sign));
}

// Warp sum of pairs in a fixed tree (lane 0 holds the result)
__device__ __forceinline__ P warp_sum(P v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const P w = make_float2(__shfl_down_sync(0xffffffffu, v.x, o),
                                __shfl_down_sync(0xffffffffu, v.y, o));
        v = add(v, w);
    }
    return v;
}

}  // namespace fp
}  // namespace cfg
