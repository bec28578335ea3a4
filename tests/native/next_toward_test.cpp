// Compares umcx_dev::next_toward (the device code's nextafterf restatement) with the C library's nextafterf on edge
// values and pseudo-random finite floats; prints the number of mismatches.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>

#include "../../umcx_gb300/csrc/next_toward.h"

static float from_bits(uint32_t u) {
    float f;
    std::memcpy(&f, &u, sizeof(f));
    return f;
}

int main() {
    const float edges[] = {0.f, -0.f, 1.f, -1.f, 0.5f, 2.f, 59.f, 60.f, 199.f, 1e-38f, -1e-38f, 1e-45f, -1e-45f,
                           std::numeric_limits<float>::min(), std::numeric_limits<float>::max() / 2,
                           std::numeric_limits<float>::denorm_min(), 3.5f, -7.25f};
    const float dirs[] = {1.f, -1.f, 0.f, -0.f, 2.f, -2.f, 60.f, 1e-45f};
    long checked = 0, bad = 0;
    auto check = [&](float x, float y) {
        const float a = umcx_dev::next_toward(x, y), b = std::nextafter(x, y);
        uint32_t ua, ub;
        std::memcpy(&ua, &a, 4);
        std::memcpy(&ub, &b, 4);
        checked++;
        if (ua != ub) {
            if (bad < 10) std::printf("mismatch x=%a y=%a: %a vs %a\n", x, y, a, b);
            bad++;
        }
    };
    for (float x : edges)
        for (float y : dirs) check(x, y);
    uint32_t s = 12345u;
    for (int i = 0; i < 2000000; i++) {
        s = s * 1664525u + 1013904223u;
        const uint32_t u = s & 0x7F7FFFFFu;  // finite magnitudes below the largest exponent
        const float x = from_bits(u | ((s >> 3) & 1u) << 31);
        check(x, (s & 2u) ? 1.f : -1.f);
        check(x, from_bits((s >> 5) | 0u) * 0.f + ((s & 4u) ? x * 2.f : -x));
    }
    std::printf("checked %ld mismatches %ld\n", checked, bad);
    return bad != 0;
}
