// Checks of the mixed precision's estimate refresh rule (shamrock_gb300/csrc/guard_rule.h).
#include "../../shamrock_gb300/csrc/guard_rule.h"

#include <cstdio>

int main() {
    using gbsph::guard_refresh_skip;
    int bad = 0;
    auto expect = [&](unsigned got, unsigned want, const char *what) {
        if (got != want) {
            std::printf("FAIL %s: %u != %u\n", what, got, want);
            bad++;
        }
    };
    const double tol = 1e-5;
    expect(guard_refresh_skip(1e-6, -1, 0, tol, true), 3, "far below, first refresh");
    expect(guard_refresh_skip(tol / 8, -1, 0, tol, true), 3, "at an eighth");
    expect(guard_refresh_skip(5e-6, -1, 0, tol, true), 0, "near, no earlier refresh");
    expect(guard_refresh_skip(5e-6, 5e-6, 1, tol, true), 3, "near, steady");
    expect(guard_refresh_skip(5e-6, 5.5e-6, 4, tol, true), 3, "near, falling");
    expect(guard_refresh_skip(7.2e-6, 7.0e-6, 4, tol, true), 3, "near, slow growth");
    expect(guard_refresh_skip(7.5e-6, 7.0e-6, 4, tol, true), 0, "near, growth reaches 0.8 tol");
    expect(guard_refresh_skip(5e-6, 4e-6, 1, tol, true), 0, "near, fast growth");
    expect(guard_refresh_skip(8.1e-6, 8.1e-6, 1, tol, true), 0, "above 0.8 tol");
    expect(guard_refresh_skip(1e-7, 1e-7, 1, tol, false), 0, "compensated tier");
    expect(guard_refresh_skip(5e-6, 5e-6, 0, tol, true), 0, "no steps between refreshes");
    std::printf("failures %d\n", bad);
    return bad ? 1 : 0;
}
