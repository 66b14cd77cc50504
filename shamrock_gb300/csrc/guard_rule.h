// The refresh rule of the error-controlled mixed precision (GBSPH_MIXED_GUARDED), as a
// plain host function so that it can be checked on its own.
//
// After a step that refreshed the FP32 tier's error estimate est (the step ran in `tier`;
// prev_est is the refresh before it, since the steps from that one to this, prev_est < 0
// when there is none), the next refresh comes after `skip` steps more, 3 or 0: three when
// the estimate cannot reach the tolerance in the three steps between, i.e. it lies below
// an eighth of the tolerance, or below 0.8 of it with its growth since the last refresh,
// doubled and carried over four steps, still below 0.8 of it; otherwise none (and none
// after a step that ran in the compensated tier).
#pragma once

#include <algorithm>
#include <cstdint>

namespace gbsph {

inline uint32_t guard_refresh_skip(double est, double prev_est, uint32_t since, double tol,
                                   bool fp32_tier) {
    if (!fp32_tier) return 0;
    if (est <= tol / 8) return 3;
    if (prev_est >= 0 && since > 0 && est <= 0.8 * tol) {
        const double rate = std::max(0.0, est - prev_est) / double(since);
        if (est + 2 * 4 * rate <= 0.8 * tol) return 3;
    }
    return 0;
}

} // namespace gbsph
