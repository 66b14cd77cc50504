// Exact hi/lo split of a double with integer operations only.
//
// hi = fl32(v) (round to nearest, ties to even) and lo = fl32(v - hi), the pair the
// mixed-precision records store for positions, velocities and pressures.  Converting
// and subtracting in FP64 costs several FP64-pipe operations per value, and GB300's
// FP64 rate is a small fraction of its FP32 rate; here the 53-bit significand is cut
// with integer shifts and the remainder converted with one int -> float conversion.
//
// The fast path covers binary exponents E in [-74, 126] (about 5e-23 <= |v| < 1.7e38),
// where hi, lo and the scale 2^(E - 52) are normal floats, so the results equal
// __double2float_rn(v) and __double2float_rn(v - (double) hi) bit for bit.  Other values
// (0, tiny, huge, inf, nan) take the FP64 route, so the function is exact everywhere.
// Header-only and free of CUDA intrinsics so the same code is checked on the host
// (tests/native/split64_check.cpp).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define GBSPH_HD __host__ __device__ __forceinline__
#else
#define GBSPH_HD inline
#endif

namespace gbsph {

GBSPH_HD float split64_bits_to_float(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

GBSPH_HD void split64(double v, float &hi, float &lo) {
    uint64_t b;
    std::memcpy(&b, &v, 8);
    const int E = (int) ((b >> 52) & 0x7ffu) - 1023;
    if (E < -74 || E > 126) {
        hi = (float) v;
        lo = (float) (v - (double) hi);
        return;
    }
    const uint32_t sgn = (uint32_t) (b >> 63) << 31;
    const uint64_t M   = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52); // v = M 2^(E - 52)
    uint32_t mh        = (uint32_t) (M >> 29);                    // top 24 bits
    const uint32_t R   = (uint32_t) (M & 0x1FFFFFFFu);            // low 29 bits
    int32_t r          = (int32_t) R;
    if (R > 0x10000000u || (R == 0x10000000u && (mh & 1u))) { // round up
        mh += 1u;
        r -= 0x20000000;
    }
    const uint32_t hb = (mh == (1u << 24)) ? ((uint32_t) (E + 128) << 23)
                                           : (((uint32_t) (E + 127) << 23) | (mh & 0x7FFFFFu));
    hi = split64_bits_to_float(hb | sgn);
    // v - hi = r 2^(E - 52) exactly, |r| <= 2^28; (float) r rounds it to 24 bits and the
    // power-of-two scale (normal for E >= -74) is exact
    // (an exact difference of zero is +0, as the FP64 subtraction gives)
    const float scale = split64_bits_to_float((uint32_t) (E + 75) << 23);
    lo                = (float) (sgn ? -r : r) * scale;
}

} // namespace gbsph
