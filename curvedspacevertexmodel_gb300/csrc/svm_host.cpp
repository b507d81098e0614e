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

// The vertex model's random directors, made as sphericalVertexModel.cpp:58-70 makes them: two
// uniforms per vertex give a random unit vector, projected onto the tangent plane at the vertex and
// normalised (sphericalDomain.h:173-177).  The draws continue the seeded stream after the cell
// centres and the cell model's own director draws (sphericalModel.cpp:37-63, 4 nCells uniforms);
// the reference uses the model's own default noise source instead, which random_device seeds
// (noiseSource.h:21-30), so only the distribution is the reference's.
extern "C" int svm_random_vertex_directors(int seed, int nCells, const double* vertexPos, int nV, double* out) {
    if (nCells < 4 || nV < 1 || !vertexPos || !out) return SVM_ERR_ARG;
    std::mt19937 gen(13377);
    if (seed >= 0) gen = std::mt19937(seed);
    auto uniform = [&]() { std::uniform_real_distribution<double> u(0.0, 1.0); return u(gen); };
    for (long i = 0; i < 4L * nCells; ++i) uniform();
    for (int i = 0; i < nV; ++i) {
        const double u2 = uniform(), v2 = uniform();
        const double phi = 2.0 * kPI * u2, theta = std::acos(2.0 * v2 - 1);
        double n[3] = {1.0 * std::sin(theta) * std::cos(phi), 1.0 * std::sin(theta) * std::sin(phi),
                       1.0 * std::cos(theta)};
        const double* p = vertexPos + 3 * i;
        double vn = 0.0, pp = 0.0;
        vn += n[0] * p[0]; vn += n[1] * p[1]; vn += n[2] * p[2];
        pp += p[0] * p[0]; pp += p[1] * p[1]; pp += p[2] * p[2];
        const double s = vn / pp;
        for (int d = 0; d < 3; ++d) n[d] = n[d] - s * p[d];
        double nn = 0.0;
        nn += n[0] * n[0]; nn += n[1] * n[1]; nn += n[2] * n[2];
        const double inv = 1.0 / std::sqrt(nn);
        for (int d = 0; d < 3; ++d) out[3 * i + d] = inv * n[d];
    }
    return SVM_OK;
}
