// Float-float ("double-single") arithmetic on the FP32 pipe.  GB300 runs FP64 at
// about 1/64 of its FP32 rate, so the mixed path keeps ~44-bit intermediates as
// unevaluated sums hi + lo of two floats.  All operations use round-to-nearest
// intrinsics so that the compiler cannot contract or reorder them.
#pragma once

#include <cuda_runtime.h>

namespace gpw {

struct ff {
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

// exp(a) for -87 < a.hi < 80.  Cody-Waite reduction r = a - k ln2 with ln2 split
// as L1 (16 significant bits, so k*L1 is exact for |k| < 2^8) plus a float-float
// remainder, then the degree-11 Taylor polynomial of exp(r), |r| <= ln2/2, by
// Horner in float-float (truncation < 2^-45).  Constants: 1/n! and ln2 - L1 rounded
// to float-float.
__device__ __forceinline__ ff ff_exp(ff a) {
    const float kf = rintf(__fmul_rn(a.hi, 1.44269502162933350f));
    const float L1 = 0.693145751953125f;
    const ff ln2_rest = {1.428606765330187e-06f, 5.497923148104107e-14f};
    ff r = two_sum(__fmaf_rn(-kf, L1, a.hi), a.lo);
    r = ff_add(r, ff_mul_f(ln2_rest, -kf));
    const float ih[12] = {1.0f, 1.0f, 0.5f, 0.1666666716337204f, 0.0416666679084301f, 0.008333333767950535f,
                          0.0013888889225199819f, 0.00019841270113829523f, 2.4801587642286904e-05f,
                          2.7557318844628753e-06f, 2.755731998149713e-07f, 2.5052107943679403e-08f};
    const float il[12] = {0.0f, 0.0f, 0.0f, -4.967053879312289e-09f, -1.2417634698280722e-09f,
                          -4.34617203337595e-10f, -3.3631094437103215e-11f, -2.725596874933456e-12f,
                          -3.40699609366682e-13f, 3.793571224297229e-14f, -7.575112209051195e-15f,
                          4.4176230446483665e-16f};
    ff p = {ih[11], il[11]};
#pragma unroll
    for (int n = 10; n >= 0; n--) p = ff_add(ff_mul(p, r), ff{ih[n], il[n]});
    const int k = (int)kf;
    return {ldexpf(p.hi, k), ldexpf(p.lo, k)};
}

}  // namespace gpw
