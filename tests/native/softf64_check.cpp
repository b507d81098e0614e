// Host check of csrc/svm_softf64.cuh: every operation against the host's IEEE operations on random
// operands (any bit patterns, exponents near 1, near-cancelling pairs, short significands, divisors
// next to powers of two) and on exact cases (products divided back, squares).  Prints the number of
// mismatches per operation; exit status 1 if any.   Usage: softf64_check [cases]
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
    std::printf("{\"cases\": %ld, \"mul\": %ld, \"add\": %ld, \"div\": %ld, \"sqrt\": %ld, \"sub\": %ld}\n", n, bad[0],
                bad[1], bad[2], bad[3], bad[4]);
    return (bad[0] | bad[1] | bad[2] | bad[3] | bad[4]) ? 1 : 0;
}
