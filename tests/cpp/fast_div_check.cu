// Host-only check of the invariant-divisor magic numbers (fast_div in
// pg_internal.cuh) used to split flat indices in the advection, RHS and
// projection kernels: the quotient the device computes with __umulhi,
// restated here with a 64-bit product, must equal n / d for every divisor
// and index tried.  No kernel runs.
#include <cstdint>
#include <cstdio>
#include <random>

#include "pg_internal.cuh"

static unsigned quotient(unsigned n, pg::FastDiv f) {  // fdiv with __umulhi written out
    const unsigned t = (unsigned)(((uint64_t)n * f.m) >> 32);
    return f.m ? (t + ((n - t) >> 1)) >> f.s : n;
}

int main() {
    std::mt19937_64 rng(7);
    long checked = 0, bad = 0;
    auto check_div = [&](unsigned d) {
        const pg::FastDiv f = pg::fast_div(d);
        const unsigned edge[] = {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 2 * d, 0x7fffffffu, 0xffffffffu,
                                 0xffffffffu - d, (0xffffffffu / d) * d, (0xffffffffu / d) * d - 1};
        for (unsigned n : edge) {
            ++checked;
            if (quotient(n, f) != n / d) ++bad;
        }
        for (int k = 0; k < 256; ++k) {
            const unsigned n = (unsigned)rng();
            ++checked;
            if (quotient(n, f) != n / d) ++bad;
        }
    };
    for (unsigned d = 1; d <= 70000; ++d) check_div(d);  // every grid side and plane size up to 70000
    for (int s = 1; s < 32; ++s) {
        check_div(1u << s);
        check_div((1u << s) - 1);
        check_div((1u << s) + 1);
    }
    for (int k = 0; k < 20000; ++k) check_div((unsigned)(rng() % 0xfffffffeu) + 2u);
    std::printf("%ld checked, %ld wrong\n", checked, bad);
    return bad != 0;
}
