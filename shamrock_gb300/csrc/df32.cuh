// Double-float ("double-word") arithmetic on the FP32 pipes: a value is the unevaluated
// sum hi + lo of two floats, carrying about 44 significant bits.  GB300 runs FP64 at a
// small fraction of its FP32 rate, so the compensated tier of the mixed-precision path
// evaluates the sums that cancel (the background-pressure part of the force, the
// density sums behind h and Omega) with these error-free transformations instead of
// FP64 arithmetic.
//
// Algorithms: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), Fast2Sum (Dekker 1971), TwoProd by
// fused multiply-add, and the double-word sums and products of Joldes, Muller & Popescu,
// "Tight and rigorous error bounds for basic building blocks of double-word arithmetic"
// (ACM TOMS 44, 2017): the "sloppy" sum (absolute error about 2^-46 (|x| + |y|), which is
// what a sum of many terms needs) and the product with one FMA per cross term.
// The unit that includes this header must not reassociate FP32 arithmetic (nvcc never
// does without fast-math); flushed denormals only affect values below 1e-38.
#pragma once

#include <cuda_runtime.h>

namespace gbsph {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo) { return df{hi, lo}; }

// s + e = a + b exactly
__device__ __forceinline__ df two_sum(float a, float b) {
    float s  = a + b;
    float bb = s - a;
    float e  = (a - (s - bb)) + (b - bb);
    return df{s, e};
}
// s + e = a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    float s = a + b;
    return df{s, b - (s - a)};
}
// p + e = a * b exactly (barring underflow)
__device__ __forceinline__ df two_prod(float a, float b) {
    float p = a * b;
    return df{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ df df_add(df x, df y) {
    df s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ df df_add_f(df x, float b) {
    df s = two_sum(x.hi, b);
    return fast_two_sum(s.hi, s.lo + x.lo);
}
__device__ __forceinline__ df df_neg(df x) { return df{-x.hi, -x.lo}; }
__device__ __forceinline__ df df_mul(df x, df y) {
    df p = two_prod(x.hi, y.hi);
    float e = fmaf(x.hi, y.lo, p.lo);
    e       = fmaf(x.lo, y.hi, e);
    return fast_two_sum(p.hi, e);
}
__device__ __forceinline__ df df_mul_f(df x, float b) {
    df p = two_prod(x.hi, b);
    return fast_two_sum(p.hi, fmaf(x.lo, b, p.lo));
}
__device__ __forceinline__ df df_sqr(df x) {
    df p = two_prod(x.hi, x.hi);
    return fast_two_sum(p.hi, fmaf(x.hi + x.hi, x.lo, p.lo));
}
// 1/sqrt(x), x > 0: the hardware estimate (relative error ~1e-7) and one Newton step
// y + y (1 - x y^2) / 2 with the residual formed exactly enough (relative error ~1e-13)
__device__ __forceinline__ df df_rsqrt(df x) {
    float y  = rsqrtf(x.hi);
    df y2    = two_prod(y, y);
    df m     = df_mul(x, y2);
    float r  = (1.f - m.hi) - m.lo;
    return fast_two_sum(y, 0.5f * y * r);
}
__device__ __forceinline__ double df_to_f64(df x) { return (double) x.hi + (double) x.lo; }

} // namespace gbsph
