// Helpers shared by the FP32 pair kernels (sph_mixed.cu) and the compensated tier
// (sph_comp.cu): M4 in FP32, compensated sums, hi/lo splits, bf16 residual packing and
// the CSR entry batches.  Included by translation units compiled with approximate FP32
// division and square root.
#pragma once

#include "sph_mixed.cuh"
#include "split64.cuh"

#include <cuda_bf16.h>

namespace gbsph {
namespace {

constexpr float kNorm3dF = 0.318309886183790671538f; // 1/pi

__device__ __forceinline__ float m4_f32(float q) {
    float t1 = 2.f - q, t2 = 1.f - q;
    t1 = t1 * t1 * t1 * 0.25f;
    t2 = -(t2 * t2 * t2);
    return q < 1.f ? t1 + t2 : (q < 2.f ? t1 : 0.f);
}
__device__ __forceinline__ float m4_df32(float q) {
    return q < 1.f ? (-3.f * q + 2.25f * q * q) : (q < 2.f ? (-3.f + 3.f * q - 0.75f * q * q) : 0.f);
}
// sqrt(x) for x >= 0 from the hardware reciprocal square root (about 2 ulp; the pair
// loops need 1e-5, and the correctly rounded sqrtf costs several more instructions per
// pair); 0 for x = 0
__device__ __forceinline__ float sqrt_approx(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }
__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
    float y = v - c;
    float t = s + y;
    c       = (t - s) - y;
    s       = t;
}
__device__ __forceinline__ float hi32(f64 v) { return __double2float_rn(v); }
__device__ __forceinline__ float lo32(f64 v) { return __double2float_rn(v - (f64) __double2float_rn(v)); }
// 1/v from the FP32 reciprocal refined by one FP64 Newton step (relative error ~1e-14,
// so its FP32 rounding is the correctly rounded 1/v but for rare ties); plain FP64
// division where the FP32 reciprocal leaves the normal range
__device__ __forceinline__ f64 rcp64(f64 v) {
    const float y0 = __frcp_rn(__double2float_rn(v));
    if (!(fabsf(y0) < 3.0e38f && fabsf(y0) > 1.0e-37f)) return 1.0 / v;
    const f64 y = (f64) y0;
    return y * (2.0 - v * y);
}
// kNorm3d / hfact^3: rho_sum / rho_h = kC sum f(q), h (d rho/dh) / rho_h = -kC sum (3f + q f')
constexpr float kDensRatio = (float) (kNorm3d / (kHfact * kHfact * kHfact));

// Two residuals in one 32-bit word as bfloat16 (8 exponent bits: the range of a float,
// so no residual underflows): with hi = fl32(v) the pair hi + bf16(lo) carries v to
// about 2^-33 relative.
__device__ __forceinline__ float pack_bf16x2(float a, float b) {
    u32 ha = __bfloat16_as_ushort(__float2bfloat16_rn(a));
    u32 hb = __bfloat16_as_ushort(__float2bfloat16_rn(b));
    return __uint_as_float((ha << 16) | hb);
}
__device__ __forceinline__ float bf_hi(float w) { return __uint_as_float(__float_as_uint(w) & 0xffff0000u); }
__device__ __forceinline__ float bf_lo(float w) { return __uint_as_float(__float_as_uint(w) << 16); }

__device__ __forceinline__ f64 rho_h64(f64 m, f64 h) {
    return m * (kHfact / h) * (kHfact / h) * (kHfact / h);
}

// Four CSR entries from k on as a uint4, slots at or past k1 set to `pad`.  vec: the row
// is padded to 4-entry boundaries (library cache) and is read with one 128-bit load.
__device__ __forceinline__ uint4 load_entries(const u32 *__restrict__ ent, u32 k, u32 k1, bool vec,
                                              u32 pad) {
    uint4 v;
    if (vec) {
        v = __ldg((const uint4 *) (ent + k));
    } else {
        v.x = __ldg(&ent[k]);
        v.y = (k + 1 < k1) ? __ldg(&ent[k + 1]) : pad;
        v.z = (k + 2 < k1) ? __ldg(&ent[k + 2]) : pad;
        v.w = (k + 3 < k1) ? __ldg(&ent[k + 3]) : pad;
    }
    if (k + 1 >= k1) v.y = pad;
    if (k + 2 >= k1) v.z = pad;
    if (k + 3 >= k1) v.w = pad;
    return v;
}

struct MixedParams {
    float alpha_u, alpha_AV, beta_AV;
    float mh3; // m hfact^3: rho = mh3 / h^3
};

inline MixedParams mixed_params(f64 pmass, f64 alpha_u, f64 alpha_AV, f64 beta_AV) {
    f64 mh3 = pmass * kHfact * kHfact * kHfact;
    return MixedParams{(float) alpha_u, (float) alpha_AV, (float) beta_AV, (float) mh3};
}

// Block maxima of the error-estimate inputs of a derivatives pass (bare sums; the pair
// mass is a common factor of numerator and denominator), folded into the step's
// scalars: the largest condition sums of force and du/dt, and the largest |F| and |U|.
// All values are non-negative, so the ordered-bit maximum is the float maximum.
__device__ __forceinline__ void cond_reduce(Scalars *sc, float fa, float fu, float a, float du) {
    u64 m0 = block_reduce(f64_to_ordered((f64) fa), OpMaxU64{}, 0ull);
    u64 m1 = block_reduce(f64_to_ordered((f64) fu), OpMaxU64{}, 0ull);
    u64 m2 = block_reduce(f64_to_ordered((f64) a), OpMaxU64{}, 0ull);
    u64 m3 = block_reduce(f64_to_ordered((f64) du), OpMaxU64{}, 0ull);
    if (threadIdx.x == 0) {
        atomicMax((unsigned long long *) &sc->cond_fa, (unsigned long long) m0);
        atomicMax((unsigned long long *) &sc->cond_fu, (unsigned long long) m1);
        atomicMax((unsigned long long *) &sc->cond_a, (unsigned long long) m2);
        atomicMax((unsigned long long *) &sc->cond_du, (unsigned long long) m3);
    }
}

} // namespace
} // namespace gbsph
