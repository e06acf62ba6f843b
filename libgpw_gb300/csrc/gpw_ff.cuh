// Float-float ("double-single") arithmetic on the FP32 pipe.  GB300 runs FP64 at
// about 1/64 of its FP32 rate, so the mixed path keeps ~44-bit intermediates as
// unevaluated sums hi + lo of two floats.  All operations use round-to-nearest
// intrinsics so that the compiler cannot contract or reorder them.
#pragma once

#include <cuda_runtime.h>

namespace gpw {

// 8-byte aligned, so that shared-memory arrays of ff load and store as one
// 64-bit access per element
struct alignas(8) ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_make(float a) { return {a, 0.0f}; }

__device__ __forceinline__ ff ff_from_double(double d) {
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - (double)h)};
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// s + e == a + b exactly (Knuth)
__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// requires |a| >= |b|
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return fast_two_sum(p, e);
}

// a*b + c in one pass: exact product error by FMA, exact sum with c.hi, one renormalisation
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const ff s = two_sum(p, c.hi);
    const float t = __fadd_rn(s.lo, __fadd_rn(e, c.lo));
    return fast_two_sum(s.hi, t);
}

// s += a*b with the sum kept unnormalised: s.hi takes the rounded sum of the
// leading products (exact error by two-sum), s.lo gathers the errors and the
// cross terms.  |s.lo| stays a few ulps of s.hi over short sums; normalise with
// ff_add / fast_two_sum before the value is used elsewhere.
__device__ __forceinline__ void ff_acc_lazy(ff &s, ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const ff t = two_sum(s.hi, p);
    s.hi = t.hi;
    s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, e));
}

// 2^(j/32), j = 0..31, as float-float (hi = the float nearest, lo = the rest)
__constant__ float2 c_exp2_32[32] = {
    {1.0f, 0.0f},
    {1.0218971967697144f, -4.811559861650494e-08f},
    {1.0442737340927124f, 4.8334701574503924e-08f},
    {1.0671404600143433f, -5.9337519786595294e-08f},
    {1.0905077457427979f, -1.3077539939843064e-08f},
    {1.114386796951294f, -5.435540018083884e-08f},
    {1.1387885808944702f, 5.386222312608879e-08f},
    {1.1637248992919922f, -4.051441493402308e-08f},
    {1.1892070770263672f, 3.797635272917432e-08f},
    {1.215247392654419f, -3.267394887984665e-08f},
    {1.2418577671051025f, 4.496838101886169e-08f},
    {1.2690509557724f, 1.419333317542737e-09f},
    {1.2968395948410034f, -4.018999533172973e-08f},
    {1.3252366781234741f, -3.496373324196611e-08f},
    {1.3542555570602417f, -1.0123349269974824e-08f},
    {1.3839099407196045f, -5.875577357983275e-08f},
    {1.4142135381698608f, 2.4203234971764687e-08f},
    {1.4451807737350464f, 3.324199937537742e-08f},
    {1.4768261909484863f, -4.500898853621038e-08f},
    {1.5091644525527954f, -2.4959373234878512e-08f},
    {1.5422108173370361f, 8.070904833346049e-09f},
    {1.5759809017181396f, -5.661025426206834e-08f},
    {1.610490322113037f, 9.836217174097328e-09f},
    {1.6457555294036865f, -5.124972091152813e-08f},
    {1.6817928552627563f, -2.4755326677450284e-08f},
    {1.7186193466186523f, -4.8496175963919086e-08f},
    {1.7562521696090698f, -9.235770370707996e-09f},
    {1.7947090864181519f, -1.141504490931311e-08f},
    {1.8340080976486206f, -1.1239277952768134e-08f},
    {1.8741676807403564f, -4.663005626071026e-08f},
    {1.9152065515518188f, 9.845328108326612e-09f},
    {1.9571441411972046f, -1.7021804410433106e-08f}};

// exp(a) in float-float, table-driven (Tang's method): a = (32 m + j) ln2/32 + r
// with k = 32 m + j = round(a 32/ln2), |r| <= ln2/64, so exp(a) = 2^m 2^(j/32) exp(r).
// ln2/32 is split Cody-Waite style as C1 (11 significant bits: k C1 and a - k C1
// are exact for |k| < 2^13) plus the float-float C2 + C3.  exp(r) = 1 + r + r^2 h
// with h = 1/2 + r/6 + r^2/24 + r^3/120 (the tail after r^2/2 is below 2^-20 and
// needs only float precision; truncation r^6/720 < 2^-48).  Relative error about
// 2^-45 while the result is a normal float with a normal low part (a > -60);
// below, the low part underflows gradually; a.hi < -103 returns 0.  Valid for
// a.hi < 88.
__device__ __forceinline__ ff ff_exp(ff a) {
    if (a.hi < -103.0f) return {0.0f, 0.0f};
    const float kf = rintf(__fmul_rn(a.hi, 46.16624069213867f));
    const int k = (int)kf;
    ff r = two_sum(__fmaf_rn(-kf, 0.02166748046875f, a.hi), a.lo);
    r = ff_add(r, ff_mul_f(ff{-6.631076303165173e-06f, 5.14560928046269e-14f}, -kf));
    const float s = r.hi;
    const float t = __fmul_rn(s, __fmaf_rn(s, __fmaf_rn(s, 0.008333333767950535f, 0.0416666679084301f),
                                           0.1666666716337204f));
    const ff h = fast_two_sum(0.5f, t);
    ff p = ff_add(ff_add(ff{1.0f, 0.0f}, r), ff_mul(ff_mul(r, r), h));
    const float2 tj = c_exp2_32[k & 31];
    p = ff_mul(p, ff{tj.x, tj.y});
    // 2^m in two normal-range factors (m >= -149 here)
    const int m = k >> 5, m1 = m >> 1, m2 = m - m1;
    const float s1 = __int_as_float((127 + m1) << 23), s2 = __int_as_float((127 + m2) << 23);
    return {__fmul_rn(__fmul_rn(p.hi, s1), s2), __fmul_rn(__fmul_rn(p.lo, s1), s2)};
}

}  // namespace gpw
