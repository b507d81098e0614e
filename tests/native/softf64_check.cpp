// Host check of csrc/svm_softf64.cuh: every operation against the host's IEEE operations on random
// operands (any bit patterns, exponents near 1, near-cancelling pairs, short significands, divisors
// next to powers of two) and on exact cases (products divided back, squares); the float <-> double
// conversions likewise.  Prints the number of mismatches per operation; exit status 1 if any.
//   Usage: softf64_check [cases]
#include "svm_softf64.cuh"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

static bool same(double x, double y) { return (std::isnan(x) && std::isnan(y)) || sf::bits(x) == sf::bits(y); }

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
    std::mt19937_64 g(20261204);
    long bad[5] = {0, 0, 0, 0, 0};
    auto draw = [&](bool any) {
        const unsigned long long u = g();
        if (any) return sf::dbl(u);
        const unsigned long long e = 1023 + (long long)(g() % 81) - 40;
        return sf::dbl((u & (sf::kMant | sf::kSign)) | (e << 52));
    };
    for (long i = 0; i < n; ++i) {
        double a = draw(i % 3 == 0), b = draw(i % 3 == 0);
        if (i % 7 == 0) b = sf::dbl(sf::bits(a) ^ (g() & 0xFFFF) ^ (g() & 1 ? sf::kSign : 0));
        if (i % 11 == 0) b = sf::dbl(sf::bits(b) & ~0xFFFFFFull);
        if (i % 13 == 0) a = sf::dbl(sf::bits(a) & ~0xFFFFFFFFull);
        if (i % 17 == 0) b = sf::dbl((sf::bits(b) & ~sf::kMant) | (g() & 0xFull));
        if (i % 19 == 0) b = sf::dbl((sf::bits(b) | sf::kMant) ^ (g() & 0xFull));
        if (i % 23 == 0) a = sf::dbl(sf::bits(b) + (long long)(g() % 9) - 4);
        const double got[5] = {sf::mul(a, b), sf::add(a, b), sf::div(a, b), sf::sqrt(std::fabs(a)), sf::sub(a, b)};
        const double want[5] = {sf::hw_mul(a, b), sf::hw_add(a, b), sf::hw_div(a, b), sf::hw_sqrt(std::fabs(a)),
                                sf::hw_add(a, -b)};
        for (int k = 0; k < 5; ++k) bad[k] += !same(got[k], want[k]);
    }
    for (long i = 0; i < n / 10; ++i) {
        const double x = sf::dbl(((1023ull + g() % 40 - 20) << 52) | (g() & sf::kMant & ~0xFFFFFFFFull));
        const double y = sf::dbl(((1023ull + g() % 40 - 20) << 52) | (g() & sf::kMant & ~0xFFFFFFFFull));
        const double p = sf::hw_mul(x, y), s = sf::hw_mul(x, x);
        bad[2] += !same(sf::div(p, y), sf::hw_div(p, y));
        bad[3] += !same(sf::sqrt(s), sf::hw_sqrt(s));
    }
    // conversions: every float bit pattern at a stride (plus every pattern of the special and the
    // smallest exponents), and doubles around the float range, at and next to rounding ties
    long badW = 0, badN = 0;
    auto sameF = [](float x, float y) { return (x != x && y != y) || sf::f32bits(x) == sf::f32bits(y); };
    for (unsigned long long u = 0; u < (1ull << 32); u += 251) {
        const float f = sf::f32of((unsigned)u);
        badW += !same(sf::widen(f), sf::hw_widen(f));
    }
    for (unsigned e : {0u, 1u, 254u, 255u})
        for (unsigned m = 0; m < (1u << 23); m += 7)
            for (unsigned sgn : {0u, 0x80000000u}) {
                const float f = sf::f32of(sgn | (e << 23) | m);
                badW += !same(sf::widen(f), sf::hw_widen(f));
            }
    for (long i = 0; i < n; ++i) {
        const unsigned long long r = g();
        unsigned long long u = g();
        if (i % 2) u = (u & (sf::kMant | sf::kSign)) | ((unsigned long long)(1023 - 150 + (int)(r % 300)) << 52);
        if (i % 5 == 1) u = (u & ~0x1FFFFFFFull) | 0x10000000ull;                      // exact tie
        if (i % 5 == 2) u = (u & ~0x1FFFFFFFull) | (0x10000000ull + (r >> 40) % 5) - 2;  // next to a tie
        if (i % 5 == 3) u = (u & ~0x1FFFFFFFull) | 0x1FFFFFFFull;                        // carries upwards
        if (i % 7 == 0) u = (u & ~(0x7FFull << 52)) | ((unsigned long long)(1023 + 127) << 52) | 0xFFFFFE0000000ull;
        const double d = sf::dbl(u);
        badN += !sameF(sf::narrow(d), sf::hw_narrow(d));
    }
    std::printf("{\"cases\": %ld, \"mul\": %ld, \"add\": %ld, \"div\": %ld, \"sqrt\": %ld, \"sub\": %ld, "
                "\"widen\": %ld, \"narrow\": %ld}\n", n, bad[0], bad[1], bad[2], bad[3], bad[4], badW, badN);
    return (bad[0] | bad[1] | bad[2] | bad[3] | bad[4] | badW | badN) ? 1 : 0;
}
