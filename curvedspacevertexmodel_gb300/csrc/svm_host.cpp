// Host-side initialisation helpers of libsvm (no device code).
#include <cmath>
#include <random>
#include <vector>
#include "svm.h"

namespace {
const double kPI = 3.141592653589793115997963468544185161590576171875;

// p <- R p / |p| with the reference's rounding order (inc/sphericalDomain.h:183-187).
void renormalise(double* p, double R) {
    double s = 0.0;
    s += p[0] * p[0]; s += p[1] * p[1]; s += p[2] * p[2];
    const double inv = 1.0 / std::sqrt(s);
    for (int d = 0; d < 3; ++d) p[d] = R * (inv * p[d]);
}
}  // namespace

extern "C" int svm_random_cell_centres(int seed, int n, double* out) {
    if (n < 4 || !out) return SVM_ERR_ARG;
    std::mt19937 gen(13377);
    if (seed >= 0) gen = std::mt19937(seed);
    auto uniform = [&]() { std::uniform_real_distribution<double> u(0.0, 1.0); return u(gen); };
    for (int i = 0; i < n; ++i) {
        const double u = uniform(), v = uniform();
        const double phi = 2.0 * kPI * u, theta = std::acos(2.0 * v - 1);
        double* p = out + 3 * i;
        p[0] = 1.0 * std::sin(theta) * std::cos(phi);
        p[1] = 1.0 * std::sin(theta) * std::sin(phi);
        p[2] = 1.0 * std::cos(theta);
        renormalise(p, 1.0);
    }
    const double R = std::sqrt(n / (4.0 * kPI));
    for (int i = 0; i < n; ++i) renormalise(out + 3 * i, R);
    return SVM_OK;
}
