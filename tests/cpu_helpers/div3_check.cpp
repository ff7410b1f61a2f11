// Checks the FP64 division by 3 of the face kernel (fv2d_kernels.cuh div3: q0 = RN(a y) with
// y = RN(1/3), one residual correction q = RN(q0 + RN-exact(a - 3 q0) y)) against IEEE a / 3 on
// random operands over the whole range whose quotient stays normal, and on operands whose
// quotient lies next to a rounding midpoint.  Exits non-zero on any mismatch.
// Build: g++ -std=c++17 -O2 -ffp-contract=off div3_check.cpp
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

static uint64_t bits(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }
static double dbl(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }

static double div3(double a) {
    const double y = 1.0 / 3.0, q0 = a * y;
    if ((bits(a) << 1) == 0) return q0;
    return std::fma(std::fma(-3.0, q0, a), y, q0);
}

int main(int argc, char** argv) {
    const uint64_t N = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 2000000ull;
    std::mt19937_64 rng(2024);
    uint64_t n = 0, bad = 0;
    auto check = [&](double a) {
        n++;
        const double got = div3(a), want = a / 3.0;
        if (bits(got) != bits(want)) {
            if (bad < 10) std::printf("a = %a: got %a want %a\n", a, got, want);
            bad++;
        }
    };
    for (double a : {0.0, -0.0, 1.0, -1.0, 3.0, 1.5, 0.1, 1e300, -1e300, 1e-300, 7.0, 9.0})
        check(a);
    for (uint64_t i = 0; i < N; i++) {
        // any sign and significand, exponent with a normal quotient
        const uint64_t e = 3 + rng() % 2043;
        check(dbl((rng() & 0x800fffffffffffffull) | (e << 52)));
        // solver-like magnitudes
        check(dbl((rng() & 0x800fffffffffffffull) | ((uint64_t)(990 + rng() % 70) << 52)));
        // quotients next to a midpoint: a = RN(3 (q + ulp/2)) for a random q, +- a few ulps
        const double q = dbl((rng() & 0x000fffffffffffffull) | ((uint64_t)(1000 + rng() % 40) << 52));
        const double a = 3.0 * q + 1.5 * (std::nextafter(q, 1e308) - q);
        for (int k = -3; k <= 3; k++) check(dbl(bits(a) + k));
    }
    std::printf("div3: %" PRIu64 " checked, %" PRIu64 " mismatches\n", n, bad);
    return bad ? 1 : 0;
}
