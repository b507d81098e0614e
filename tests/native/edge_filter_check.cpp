// Host check of csrc/svm_edge_filter.h: clearly_longer(p1, p2, R, t) may only answer true for an
// edge whose exact chord (long double, from the same double coordinates) exceeds t by a clear
// margin, so that the FP64 test it skips would have answered "not shorter" too.  Random edges of
// spheres of radius 0.5 .. 3e4 around thresholds of 1e-4 .. 2 radii: arcs from 0.2 t to 5 t (and
// a broad population), both points rounded to doubles and renormalised in double as the model's
// moves leave them.  Prints counts as JSON; exit status 1 on any violation.
//   Usage: edge_filter_check [cases]
#include "svm_edge_filter.h"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
    std::mt19937_64 g(4117);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::normal_distribution<double> N(0.0, 1.0);
    long violations = 0, decided = 0, nearDecided = 0, near = 0;
    long double worst = 1e30L;   // smallest (chord - t) / t over the edges called clearly longer
    for (long i = 0; i < n; ++i) {
        const double R = 0.5 * std::pow(6e4, U(g));
        const double a = std::pow(10.0, -4.0 + 4.3 * U(g));           // t / R in [1e-4, 2)
        const double t = a * R;
        const bool isNear = i % 2 == 0;
        const double arc = isNear ? t * (0.98 + 0.04 * U(g)) * (i % 4 == 0 ? 1.0 : 1.0 + 0.002 * N(g))
                                  : t * std::pow(25.0, U(g)) / 5.0;    // 0.2 t .. 5 t
        double x[3] = {N(g), N(g), N(g)};
        double nx = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        for (double& c : x) c *= R / nx;
        // a unit tangent at x, then the point at angle arc / R along the great circle
        double r[3] = {N(g), N(g), N(g)};
        double d = (r[0] * x[0] + r[1] * x[1] + r[2] * x[2]) / (R * R);
        for (int k = 0; k < 3; ++k) r[k] -= d * x[k];
        double nr = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double th = arc / R;
        double y[3];
        for (int k = 0; k < 3; ++k) y[k] = std::cos(th) * x[k] + std::sin(th) * R * r[k] / nr;
        double ny = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
        for (double& c : y) c *= R / ny;
        const bool longer = svm_edge::clearly_longer(x[0], x[1], x[2], y[0], y[1], y[2], R, t);
        long double c2 = 0;
        for (int k = 0; k < 3; ++k) {
            const long double dk = (long double)x[k] - (long double)y[k];
            c2 += dk * dk;
        }
        const long double chord = std::sqrt(c2);
        if (isNear) ++near;
        if (longer) {
            ++decided;
            if (isNear) ++nearDecided;
            const long double m = (chord - t) / t;
            if (m < worst) worst = m;
            // the documented margin: chord > t + 9e-4 t + 6e-6 R
            if (!(chord > (long double)t * (1.0L + 9e-4L) + 6e-6L * R)) ++violations;
        }
    }
    // edge cases: coincident points, infinities and NaN (undecided), antipodes
    const double inf = INFINITY, nan = NAN;
    long special = 0;
    special += svm_edge::clearly_longer(1, 2, 3, 1, 2, 3, 4, 0.1);                   // coincident: false
    special += svm_edge::clearly_longer(inf, 0, 0, 1, 0, 0, 1, 0.1);                 // inf - 1: undecided
    special += svm_edge::clearly_longer(nan, 0, 0, 1, 0, 0, 1, 0.1);                 // NaN: undecided
    special += svm_edge::clearly_longer(1, 0, 0, -1, 0, 0, 1, inf);                  // infinite threshold
    special += !svm_edge::clearly_longer(1, 0, 0, -1, 0, 0, 1, 0.1);                 // antipodes: longer
    special += svm_edge::hi_word_float(1e-200) != 0.0f;
    special += svm_edge::hi_word_float(-3.0) != -3.0f;
    special += !std::isnan(svm_edge::hi_word_float(1e300));
    std::printf("{\"cases\": %ld, \"decided\": %ld, \"near\": %ld, \"near_decided\": %ld, "
                "\"violations\": %ld, \"special_failures\": %ld, \"worst_margin\": %.6Lg}\n",
                n, decided, near, nearDecided, violations, special, worst);
    return violations || special ? 1 : 0;
}
