// Internal state and FP64 device math of libsvm.
//
// Device layout (structure of arrays, one GPU):
//   pos[2]      double4_32a[Nv]   vertex positions (x,y,z,0); two buffers so the fused
//                             force+integrate+move kernel reads old and writes new positions
//   vsph        double4_32a[Nv]   per-vertex spherical coordinates (cos t, sin t, cos p, sin p)
//   vcell/vnbr  int4[Nv]      vertex->cell and vertex->vertex slots (w unused)
//   vlast/vnext int4[Nv]      ring predecessor / successor of the vertex in each of its cells
//   vrpos       int4[Nv]      position of the vertex in each of its cells' rings
//   ring        int[N*Wc]     clockwise ring of each cell, capacity Wc; ringCount int[N]
//   corner      double2[N*Wc] per ring position k: (arc(ring[k-1], ring[k]), included angle at k)
//   cellPos     double4_32a[N]    renormalised ring centroid; cellSph double4_32a[N] its (cos t, ...)
//   ap, pref    double2[N]    (area, perimeter) and (A0, P0)
//   force, vel  double4_32a[Nv]
// The reference keeps AoS double[3] vertices and scatters (last, cur, next) vertex copies into
// per-(vertex, cell) slots every step (src/model/sphericalVertexModel.cu:94-96); here the force
// kernel gathers them through vlast/vnext instead, which removes 3 x 24 B x 3Nv of writes.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "../../include/svm.h"
#include "svm_acos.h"
#include "svm_softf64.cuh"
#include "svm_edge_filter.h"

namespace svm {

constexpr double kPI = 3.141592653589793115997963468544185161590576171875;
// pi - kPI (the next term of pi's double-double expansion)
constexpr double kPILo = 1.2246467991473532e-16;

struct D3 { double x, y, z; };

// Division and square root of the FP64 kernels.  Both are the IEEE correctly rounded operations
// either way; by default they run on the integer and FP32 pipes (svm_softf64.cuh), which leaves
// GB300's FP64 pipe -- 2 lanes per clock per SM, the bound of these kernels -- to the products and
// sums, where a hardware division or square root would take about eight FP64 instructions.  kHw
// (the T1 pass's kernels, where one warp's chain of dependent operations, not the FP64 pipe's
// issue rate, sets the time) takes the hardware sequences, whose latency is shorter; so does a
// build with -DSVM_NATIVE_FP64_DIV.  The results are the same bits.
template <bool kHw = false>
__device__ __forceinline__ double f64_div(double a, double b) {
#ifdef SVM_NATIVE_FP64_DIV
    return __ddiv_rn(a, b);
#else
    if constexpr (kHw) return __ddiv_rn(a, b);
    else return sf::div(a, b);
#endif
}
template <bool kHw = false>
__device__ __forceinline__ double f64_sqrt(double a) {
#ifdef SVM_NATIVE_FP64_DIV
    return __dsqrt_rn(a);
#else
    if constexpr (kHw) return __dsqrt_rn(a);
    else return sf::sqrt(a);
#endif
}

// The arccosine of the FP64 geometry (arcs, included angles, triangle areas, T1 length tests).
// The default build uses CUDA's acos; a build with -DSVM_PORTABLE_ACOS uses svm_portable::acos,
// the same operations as the CPU restatement's portable mode, which makes GPU and CPU trajectories
// comparable bit for bit.
__device__ __forceinline__ double svm_acos(double x) {
#ifdef SVM_PORTABLE_ACOS
    return svm_portable::acos(x);
#else
    return acos(x);
#endif
}

__device__ __forceinline__ D3 ld3(const double4_32a* p, int i) {
    double4_32a t = p[i];
    return D3{t.x, t.y, t.z};
}
__device__ __forceinline__ void st3(double4_32a* p, int i, D3 v) { p[i] = make_double4_32a(v.x, v.y, v.z, 0.0); }
// FP32 positions (mixed-precision form): widened exactly on load, rounded to nearest on store (the
// conversions on the integer pipes: sf::widen, sf::narrow).
__device__ __forceinline__ D3 ld3(const float4* p, int i) {
    const float4 t = p[i];
    return D3{sf::widen(t.x), sf::widen(t.y), sf::widen(t.z)};
}
__device__ __forceinline__ void st3(float4* p, int i, D3 v) {
    p[i] = make_float4(sf::narrow(v.x), sf::narrow(v.y), sf::narrow(v.z), 0.f);
}
// In the mixed form the w component of a vertex's FP32 position holds its replica index (0 for a
// single sphere); rounded stores of a vertex keep it.
__device__ __forceinline__ void st3_keep(float4* p, int i, D3 v) {
    p[i] = make_float4(sf::narrow(v.x), sf::narrow(v.y), sf::narrow(v.z), p[i].w);
}
__device__ __forceinline__ int rep_of(const float4& p) { return (int)p.w; }
__device__ __forceinline__ int rep_of(const double4_32a&) { return 0; }
__device__ __forceinline__ D3 add3(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 sub3(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 scl3(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
// dot (inc/functions.h:131-138): accumulated in component order
__device__ __forceinline__ double dot3(D3 a, D3 b) { double s = a.x * b.x; s += a.y * b.y; s += a.z * b.z; return s; }
__device__ __forceinline__ D3 cross3(D3 p1, D3 p2) {          // inc/functions.h:160-167
    return D3{p1.y * p2.z - p1.z * p2.y, p1.z * p2.x - p1.x * p2.z, p1.x * p2.y - p1.y * p2.x};
}
// A product on the integer pipes (sf::mul: the same bits as the hardware multiply) for the products
// that start the FP64 kernels' dependency chains -- the pair terms of the geodesic and triangle-area
// gradients, which depend only on the spherical coordinates, and the cross and dot products ahead of
// the geometry's divisions and arccosines.  The FP64 pipe, which bounds the force
// kernel, keeps the rest; the integer pipes, otherwise busy only with the divisions and square
// roots, take these early, mutually independent products, whose latency the resident warps hide.
// Measured at 100k cells: 0.476 -> 0.447 ms per force launch, and 0.442 with grad_triangle's
// d/dtheta numerators, which are formed while the denominators' square roots run.  Moving the
// d/dphi numerators too (chains of three products: 0.487 ms), the products at the end of
// grad_triangle's chains (0.509 ms), all its products, or the pair terms' sums (0.531 ms) was slower.
// The corner phase (k_edges' cross products and arcs, the included angles' products): 0.159 -> 0.151 ms;
// the norms ahead of the centroids', vertices' and fan triangles' square roots: cells and fallback
// phases 2-3% shorter.
// (kHw: the hardware multiply, for the T1 pass's latency-bound chains.)
template <bool kHw = false>
__device__ __forceinline__ double early_mul(double x, double y) {
    if constexpr (kHw) return __dmul_rn(x, y);
    else return sf::mul(x, y);
}
// dot3 and cross3 with their products on the integer pipes (the same bits)
template <bool kHw = false>
__device__ __forceinline__ double dot3e(D3 a, D3 b) {
    double s = early_mul<kHw>(a.x, b.x);
    s += early_mul<kHw>(a.y, b.y);
    s += early_mul<kHw>(a.z, b.z);
    return s;
}
template <bool kHw = false>
__device__ __forceinline__ D3 cross3e(D3 p1, D3 p2) {
    return D3{early_mul<kHw>(p1.y, p2.z) - early_mul<kHw>(p1.z, p2.y),
              early_mul<kHw>(p1.z, p2.x) - early_mul<kHw>(p1.x, p2.z),
              early_mul<kHw>(p1.x, p2.y) - early_mul<kHw>(p1.y, p2.x)};
}
__device__ __forceinline__ double det3(D3 a, D3 b, D3 c) {    // a . (b x c), sphericalDomain.h:123-125
    return a.x * (b.y * c.z - b.z * c.y) + a.y * (b.z * c.x - b.x * c.z) + a.z * (b.x * c.y - b.y * c.x);
}

// putInBoxReal (sphericalDomain.h:183-187): p <- R p / |p|
__device__ __forceinline__ D3 renorm(D3 p, double R) {
    double inv = f64_div(1.0, f64_sqrt(dot3e(p, p)));
    return scl3(R, scl3(inv, p));
}
// move(p, v) (sphericalDomain.h:203-209): project v onto the tangent plane at p, add, renormalise
__device__ __forceinline__ D3 sphere_move(D3 p, D3 v, double R) {
    double s = f64_div(dot3(v, p), dot3(p, p));
    D3 d = sub3(v, scl3(s, p));
    return renorm(add3(p, d), R);
}
// geodesicDistance (sphericalDomain.h:94-112)
template <bool kHw = false>
__device__ __forceinline__ double geodesic(D3 p1, D3 p2, double R) {
    double num = p1.x * p2.x + p1.y * p2.y + p1.z * p2.z;
    double den = f64_sqrt<kHw>(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z) *
                 f64_sqrt<kHw>(p2.x * p2.x + p2.y * p2.y + p2.z * p2.z);
    return R * svm_acos(f64_div<kHw>(num, den));
}
// |p| as geodesic and sph_coords evaluate it (same operations, so the same value)
template <bool kHw = false>
__device__ __forceinline__ double pos_norm(D3 p) { return f64_sqrt<kHw>(dot3e<kHw>(p, p)); }
// geodesic with the two norms given (n1 = pos_norm(p1), n2 = pos_norm(p2)): the same value
__device__ __forceinline__ double geodesic_n(D3 p1, D3 p2, double n1, double n2, double R) {
    return R * svm_acos(f64_div(dot3e(p1, p2), early_mul(n1, n2)));
}
// The T1 length test geodesic(p1, p2) < t, i.e. R acos(c) < t with c = p1.p2 / (|p1||p2|).  acos
// is decreasing, so away from c = cos(t / R) the answer is c > cos(t / R); the formula itself is
// evaluated only when c lies within [cosLo, cosHi], a bracket around cos(t / R) of half-width
// 1e-9, which is many orders wider than the error of acos and of the rounding of c, or when c > 1.
__host__ __device__ inline void t1_bracket(double t, double R, double* lo, double* hi) {
    if (!(t > 0.0)) {   // an arc is never below a threshold of 0 or less: every c < lo decides "no"
        *lo = *hi = 2.0;
        return;
    }
    const double c = cos(t / R);
    *lo = c - 1e-9;
    *hi = c + 1e-9;
}
// A pre-test decides the edges away from the threshold without square roots or divisions:
// sin^2(angle) = |p1 x p2|^2 / (|p1|^2 |p2|^2) against sin^2(a) (1 -/+ eps) (s2Lo, s2Hi), a = t / R,
// for angles below pi / 2 (p1.p2 > 0) and above 3e-7 (|p1 x p2|^2 > 1e-13 |p1|^2 |p2|^2: closer
// to 0, c can round to 1 or past it, where the reference's acos is 0 or NaN).  The formula's
// decision is c > c* with c* within 1e-30 of cos(a), and c within 5e-16 of the cosine of the angle;
// outside the band, the cosine differs from cos(a) by at least a^2 eps / 2 >= 5e-13, and the
// pre-test's own relative error is below 1e-9 / a, so every decision it takes is the formula's.
// eps = max(1e-6, 1e-12 / a^2); thresholds of 0 or of 1 radian or more skip the pre-test.
__host__ inline void t1_sin2_bracket(double t, double R, double* lo, double* hi) {
    const double a = t / R;
    if (!(a > 0.0 && a < 1.0)) {   // never decides: xx < -d and xx > 2 d are impossible
        *lo = -1.0;
        *hi = 2.0;
        return;
    }
    const double s = sin(a);
    double eps = 1e-12 / (a * a);
    if (eps < 1e-6) eps = 1e-6;
    *lo = s * s * (1.0 - eps);
    *hi = s * s * (1.0 + eps);
}
template <bool kHw = false>
__device__ __forceinline__ bool shorter_than(D3 p1, D3 p2, double R, double t, double cosLo, double cosHi,
                                             double s2Lo, double s2Hi) {
    if (svm_edge::clearly_longer(p1.x, p1.y, p1.z, p2.x, p2.y, p2.z, R, t)) return false;
    const double num = p1.x * p2.x + p1.y * p2.y + p1.z * p2.z;
    if (num > 0) {
        const D3 x = cross3(p1, p2);
        const double xx = dot3(x, x), d = dot3(p1, p1) * dot3(p2, p2);
        if (xx < s2Lo * d && xx > 1e-13 * d) return true;
        if (xx > s2Hi * d) return false;
    }
    const double den = f64_sqrt<kHw>(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z) *
                       f64_sqrt<kHw>(p2.x * p2.x + p2.y * p2.y + p2.z * p2.z);
    const double c = f64_div<kHw>(num, den);
    if (c > cosHi && c <= 1.0) return true;   // c > 1 (rounding) makes acos NaN: not shorter
    if (c < cosLo) return false;
    return R * svm_acos(c) < t;
}
// Arc length in the mixed-precision form: 2 R asin(|q - p| / 2R) in FP32 from the raw chord
// (exact for nearby FP32 points), well conditioned for the short arcs of the model (the acos form
// loses half its digits there).
__device__ __forceinline__ float arc32(float4 p, float4 q, float R) {
    const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
    return 2.0f * R * asinf(sqrtf(dx * dx + dy * dy + dz * dz) / (2.0f * R));
}
// includedAngle (sphericalDomain.h:114-133)
template <bool kHw = false>
__device__ __forceinline__ double included_angle(D3 p1, D3 p2, D3 p3) {
    D3 ci = cross3(p2, p3), cim1 = cross3(p1, p2);
    double det = det3(p1, p2, p3);
    double a = svm_acos(f64_div<kHw>(-dot3(ci, cim1), f64_sqrt<kHw>(dot3(ci, ci)) * f64_sqrt<kHw>(dot3(cim1, cim1))));
    if (det > 0) a = -a;
    if (a < 0) a += 2. * kPI;
    return a;
}
// includedAngle(pl, p, px) from the cross products Cx = p x px and Cl = p x pl and their norms,
// computed once per neighbour of p: cross(pl, p) = -(p x pl) exactly, the negations cancel exactly
// in the dot product and the norms, and det(pl, p, px) = pl . (p x px) in the same operation
// order, so the result is bitwise included_angle(pl, p, px).
//
// With `clamp` (the mixed form) the cosine is clamped to [-1, 1]: for a nearly straight corner its
// rounding can leave the domain, where acos is NaN (the reference does not clamp, and the FP64
// form keeps that behaviour).
template <bool clamp = false>
__device__ __forceinline__ double included_angle_pre(D3 Cx, D3 Cl, double nx, double nl, D3 pl) {
    const double det = dot3e(pl, Cx);
    double c = f64_div(dot3e(Cx, Cl), early_mul(nx, nl));
    if (clamp) c = fmin(1.0, fmax(-1.0, c));
    double a = svm_acos(c);
    if (det > 0) a = -a;
    if (a < 0) a += 2. * kPI;
    return a;
}
// element j of a three-element register array (selects, no local-memory indexing)
template <class T>
__device__ __forceinline__ T pick3(const T* a, int j) { return j == 0 ? a[0] : (j == 1 ? a[1] : a[2]); }
// slot of vertex u among the three neighbour slots nb (-1 if absent)
__device__ __forceinline__ int nbr_slot(int4 nb, int u) { return u == nb.x ? 0 : (u == nb.y ? 1 : (u == nb.z ? 2 : -1)); }
// included_angle with the cosine clamped to [-1, 1] (the mixed form)
template <bool kHw = false>
__device__ __forceinline__ double included_angle_clamped(D3 p1, D3 p2, D3 p3) {
    D3 ci = cross3(p2, p3), cim1 = cross3(p1, p2);
    double det = det3(p1, p2, p3);
    double c = f64_div<kHw>(-dot3(ci, cim1), f64_sqrt<kHw>(dot3(ci, ci)) * f64_sqrt<kHw>(dot3(cim1, cim1)));
    double a = svm_acos(fmin(1.0, fmax(-1.0, c)));
    if (det > 0) a = -a;
    if (a < 0) a += 2. * kPI;
    return a;
}
// sphericalTriangleArea (sphericalDomain.h:135-166)
// q / |q| as sphericalTriangleArea normalises each corner
__device__ __forceinline__ D3 unit_corner(D3 q) { return scl3(f64_div(1.0, f64_sqrt(dot3e(q, q))), q); }
__device__ __forceinline__ double triangle_area_unit(D3 p1, D3 p2, D3 p3, double R);
__device__ __forceinline__ double triangle_area(D3 q1, D3 q2, D3 q3, double R) {
    return triangle_area_unit(unit_corner(q1), unit_corner(q2), unit_corner(q3), R);
}
// the same from the normalised corners
__device__ __forceinline__ double triangle_area_unit(D3 p1, D3 p2, D3 p3, double R) {
    double d12 = dot3e(p1, p2), d13 = dot3e(p1, p3), d23 = dot3e(p2, p3);
    double area = -kPI;
    area += svm_acos(f64_div(d23 - d12 * d13, f64_sqrt(1 - d12 * d12) * f64_sqrt(1 - d13 * d13)));
    area += svm_acos(f64_div(d12 - d13 * d23, f64_sqrt(1 - d13 * d13) * f64_sqrt(1 - d23 * d23)));
    area += svm_acos(f64_div(d13 - d12 * d23, f64_sqrt(1 - d12 * d12) * f64_sqrt(1 - d23 * d23)));
    return area * (R * R);
}

// Spherical coordinates of a point as the reference's gradients compute them
// (sphericalDomain.h:218-232, 251-261): cos t = z/|p|, sin t = sqrt(1 - cos^2 t),
// cos p = x / sqrt(x^2+y^2), sin p = y / sqrt(x^2+y^2).
template <bool kHw = false>
__device__ __forceinline__ double4_32a sph_coords_n(D3 p, double r) {  // r = pos_norm(p)
    double cosT = f64_div<kHw>(p.z, r);
    double sinT = f64_sqrt<kHw>(1. - cosT * cosT);
    double rxy = f64_sqrt<kHw>(early_mul<kHw>(p.x, p.x) + early_mul<kHw>(p.y, p.y));
    return make_double4_32a(cosT, sinT, f64_div<kHw>(p.x, rxy), f64_div<kHw>(p.y, rxy));
}
template <bool kHw = false>
__device__ __forceinline__ double4_32a sph_coords(D3 p) { return sph_coords_n<kHw>(p, pos_norm<kHw>(p)); }

// gradientGeodesicDistance (sphericalDomain.h:248-273) in the (theta, phi) basis of v1:
// returns (d/dtheta, d/dphi) components.
__device__ __forceinline__ double2 grad_geodesic(double4_32a s1, double4_32a s2) {
    const auto E = [](double x, double y) { return early_mul(x, y); };
    double sP12 = E(s1.w, s2.z) - E(s1.z, s2.w);
    double cP12 = E(s1.z, s2.z) + E(s1.w, s2.w);
    double dp = E(s1.x, s2.x) + E(E(cP12, s1.y), s2.y);
    double dinv = f64_div(1., f64_sqrt(1 - dp * dp));
    double gT = 1.0 * (E(s2.x, s1.y) - E(E(s1.x, cP12), s2.y)) * dinv;
    double gP = E(s2.y, sP12) * dinv;
    return make_double2(gT, gP);
}

// The other products of grad_triangle: the hardware multiply, spelled out.
__device__ __forceinline__ double tri_mul(double x, double y) { return __dmul_rn(x, y); }

// gradientTriangleArea (sphericalDomain.h:347-411) in the (theta, phi) basis of v1; the sign
// follows det(v1, v2, v3).  Returns (d/dtheta, d/dphi) components.  Every product and sum in the
// order the reference's expressions evaluate them (left to right, products first).
__device__ __forceinline__ double2 grad_triangle(double4_32a a, double4_32a b, double4_32a c, D3 v1, D3 v2, D3 v3, double R) {
    const auto M = tri_mul;
    const auto E = [](double x, double y) { return early_mul(x, y); };
    const double sP12 = E(a.w, b.z) - E(a.z, b.w);
    const double sP13 = E(a.w, c.z) - E(a.z, c.w);
    const double cP12 = E(a.z, b.z) + E(a.w, b.w);
    const double cP13 = E(a.z, c.z) + E(a.w, c.w);
    const double cP23 = E(b.z, c.z) + E(b.w, c.w);
    const double s12 = E(a.x, b.x) + E(E(cP12, a.y), b.y);
    const double s13 = E(a.x, c.x) + E(E(cP13, a.y), c.y);
    const double s23 = E(b.x, c.x) + E(E(cP23, b.y), c.y);
    const double d12 = E(E(a.x, cP12), b.y) - E(b.x, a.y);
    const double d13 = E(E(a.x, cP13), c.y) - E(c.x, a.y);
    const double s12s12 = M(s12, s12), s13s13 = M(s13, s13), s12s13 = M(s12, s13);
    const double g = (((1 - s12s12) - s13s13) - M(s23, s23)) + M(M(M(2.0, s12), s13), s23);
    const double q12 = -1. + s12s12, q13 = -1. + s13s13;
    const double den1 = f64_sqrt(M(M(q12, q12), g));
    const double den2 = f64_sqrt(M(M(q13, q13), g));
    const double a12 = s12s12 - 1., a13 = s13s13 - 1.;
    const double den3 = f64_sqrt(M(M(M(M(a12, a13), a12), a13), g));
    const double s12s23 = M(s12, s23), s13s23 = M(s13, s23);
    // the d/dtheta numerators are formed while the square roots of the denominators run: integer pipes
    double gT = f64_div(E(d13, a12) + E(d12, s23 - s12s13), den1)
              + f64_div(E(d12, a13) + E(d13, s23 - s12s13), den2)
              - f64_div(E(E(d12, a13), s13 - s12s23) + E(E(d13, a12), s12 - s13s23), den3);
    gT = M(gT, R);
    double gP = f64_div(M(M(s12s13 - s23, sP12), b.y) - M(M(-1 + s12s12, sP13), c.y), den1)
              - f64_div(M(M(-1 + s13s13, sP12), b.y) + M(M(-s12s13 + s23, sP13), c.y), den2)
              + f64_div(M(M(M(-1 + s13s13, s13 - s12s23), sP12), b.y) + M(M(M(-1 + s12s12, s12 - s13s23), sP13), c.y), den3);
    gP = M(gP, R);
    if (det3(v1, v2, v3) < 0) { gT = -gT; gP = -gP; }
    return make_double2(gT, gP);
}

// (theta, phi) components to Cartesian with the basis of sphericalDomain.h:218-232:
// thetaHat = (cos t cos p, cos t sin p, -sin t), phiHat = (-sin p, cos p, 0).
__device__ __forceinline__ D3 from_basis(double4_32a s, double2 g) {
    return D3{g.x * (s.x * s.z) + g.y * (-s.w), g.x * (s.x * s.w) + g.y * s.z, g.x * (-s.y) + g.y * 0};
}

// ---- host-side state -----------------------------------------------------------------------
// Old values of everything one T1 flip overwrites, so a parallel pass can be rolled back.
struct UndoEntry {
    int v1, v2, b, c;              // vertices whose vertex->vertex slots change
    int cells[4];                  // cells i, j, k, l whose rings change
    double4_32a p1, p2;            // old positions of v1, v2
    int4 vc1, vc2;                 // old vertex->cell slots of v1, v2
    int4 vn[4];                    // old vertex->vertex slots of v1, v2, b, c
    int counts[4];                 // old ring sizes
    int logIdx;                    // the flip's entry in the flip log
};

// Counters of one parallel T1 pass: in shared memory for a single-block pass, in global memory
// (T1Scratch::ctl) for a pass spread over a cooperative grid, with the grid barrier's words.
struct T1Ctl {
    int nCur, flag, nWordsHit, undo, late, rollback, exec, flips, next[2];
    unsigned barCount, barGen;
};
constexpr int kT1CtlInts = sizeof(T1Ctl) / sizeof(int);

struct T1Scratch {
    unsigned* bits = nullptr;      // one bit per (vertex, slot) position, 3*Nv bits
    unsigned* summary = nullptr;   // one bit per word of `bits`
    int* count = nullptr;          // number of candidate positions found by the test
    int* flipLog = nullptr;        // (pass, position, v1, v2) per flip, capacity flipLogCap
    int* flipCount = nullptr;
    int* pass = nullptr;           // T1 passes so far (orders the flip log across passes)
    int* touched = nullptr;        // cells whose rings changed during the apply kernel
    int nWords = 0, nSummary = 0, flipLogCap = 0, touchedCap = 0;
    // parallel pass (deterministic reservations), capacity `cap` pending positions
    int* listA = nullptr;          // pending positions of this round
    int* listB = nullptr;          // pending positions of the next round
    int* listOrig = nullptr;       // the candidates as flagged by the test (for a rollback)
    int* fp = nullptr;             // footprint of each pending position, kFootprint ints
    int* resV = nullptr;           // per vertex: lowest position reserving it this round
    int* resC = nullptr;           // per cell: same
    int* comV = nullptr;           // per vertex: highest position that has executed on it
    int* comC = nullptr;           // per cell: same
    int* comList = nullptr;        // footprints of executed positions (to clear comV/comC)
    UndoEntry* undo = nullptr;     // one entry per committed flip
    int* undoRings = nullptr;      // old rings of the four cells, 4*Wc ints per entry
    int* ctr = nullptr;            // [0] pending, [1] next, [2] undo entries, [3] rollback, [4] executed
    int* stats = nullptr;          // svm_model_t1_stats counters
    unsigned long long* clocks = nullptr;  // svm_model_t1_clocks: SM cycles per phase (null: off)
    T1Ctl* ctl = nullptr;          // counters of a cooperative pass (inside the ctr allocation)
    int cap = 0, undoCap = 0;
};
constexpr int kFootprint = 14;     // 8 vertex slots + 6 cell slots (duplicates allowed)
constexpr int kListPad = 1024;     // list slack of a single-sphere parallel pass
constexpr int kListPadBatch = 64;  // list slack per replica of a batch's parallel pass
constexpr int kResFree = 0x7f7f7f7f;

}  // namespace svm

struct svm_model {
    int nCells = 0, nVertices = 0, Wc = 0;
    // Ring capacity grows as the reference's growCellVerticesList widens its ring storage: the T1
    // commits keep the largest ring count in ringMax, every T1 pass copies it to the page-locked
    // ringMaxHost, and before a pass the host grows the capacity whenever ringHeadroom or fewer
    // slots are free in the largest ring.  passEv: the ends of the last two passes launched outside
    // a capture (the host waits for the older before the next pass, so its reading is recent).
    int* ringMax = nullptr;            // device
    int* ringMaxHost = nullptr;        // page-locked, mapped
    int* ringMaxHostDev = nullptr;     // its device address
    int ringHeadroom = 2;
    int ringGrowths = 0;
    cudaEvent_t passEv[2] = {nullptr, nullptr};
    int passSlot = 0;
    double R = 1.0, Kr = 1.0, t1Threshold = 0.1;
    bool restricted = false;
    bool ownStream = false;
    cudaStream_t stream = nullptr;
    int cur = 0;                       // index of the current position buffer
    bool cornersValid = false;         // corner/vsph arrays match the current state
    int t1Blocks = 0;                  // svm_model_set_t1_blocks (0: automatic)
    int t1WaitLimit = 1 << 20;         // polls of a cooperative T1 pass's grid-barrier wait
    double4_32a* pos[2] = {nullptr, nullptr};
    double4_32a* vsph = nullptr;
    double* vnorm = nullptr;           // |p| per vertex, from the last corner pass (FP64 form)
    double4_32a* dir = nullptr;        // directors (self-propelled updater; single spheres only)
    double4_32a* dirTarget = nullptr;  // the Vicsek updater's target directors (allocated on first use)
    double4_32a* cellRef = nullptr;    // reference cell positions of the dynamical observables
    double4_32a* edgeC = nullptr;      // per owned edge slot 3v+j (v < u): p_v x p_u and its norm
    double* edgeArc = nullptr;         // and the arc (FP64 corner pass; single spheres only)
    int4 *vcell = nullptr, *vnbr = nullptr, *vlast = nullptr, *vnext = nullptr, *vrpos = nullptr;
    int* ring = nullptr;
    int* ringCount = nullptr;
    double2* corner = nullptr;
    double4_32a* cellPos = nullptr;
    double4_32a* cellSph = nullptr;
    double2* ap = nullptr;
    double2* pref = nullptr;
    double4_32a* force = nullptr;
    double4_32a* vel = nullptr;
    // mixed-precision form (SVM_PRECISION_MIXED): FP32 positions, centroids and forces
    int precision = SVM_PRECISION_FP64;
    float4* pos32[2] = {nullptr, nullptr};
    float4* cellPos32 = nullptr;
    float4* force32 = nullptr;
    float2* dap32 = nullptr;           // per cell (A - A0, P - P0) in FP32, written with the geometry
    // replicas (mixed form): per-replica radius, noise amplitude and reductions.  A single sphere
    // is one replica; vertex v of replica r has pos32[v].w = r, replica r owns cells
    // [repCellOff[r], repCellOff[r+1]) and vertices [repVertOff[r], repVertOff[r+1]).
    int nRep = 1;
    double* repR = nullptr;            // device [nRep]
    float* repNp = nullptr;            // device [nRep], sqrt(2 dt mu T_r) of the batch's last step
    int* repCellOff = nullptr;         // device [nRep + 1]
    int* repVertOff = nullptr;         // device [nRep + 1]
    int* repFlag = nullptr;            // device [nRep], area-check fallback flags
    double* repScal = nullptr;         // device [3 nRep]: total area, excess, energy
    std::vector<double> repT;          // host, per-replica temperatures of a batch
    std::vector<int> hRepCellOff, hRepVertOff;
    double repNpDt = -1, repNpMu = -1; // (dt, mu) repNp was computed for
    unsigned repTVersion = 0, repNpVersion = ~0u;
    // block sizes of the batch's per-element kernels (picked by the autotuner)
    int blkCorners = 256, blkCells = 256, blkForce = 256;
    void* tuners = nullptr;            // svm::BatchTuners when autotuning is on
    // FIRE minimizers created on this model; destroying the model detaches them
    std::vector<svm_fire*> fires;
    double* noiseBuf = nullptr;        // [3*Nv] staging for host-supplied noise / displacements
    double* dispBuf = nullptr;         // [3*Nv]
    double* ioHostOut = nullptr;       // while a host-buffer step is issued: the caller's mapped output
                                       // positions (AoS), written by the force kernel and the T1 patch
    // reductions: per-block partials + ticket (last-block-done pattern)
    double* partials = nullptr;
    double* dotPartials = nullptr;     // svm_reduce_dots: 4 per block of 64 vertices (allocated on first use)
    unsigned* ticket = nullptr;
    double* scalars = nullptr;         // [0] total area, [1] excess, [2] energy ...
    int* fallbackFlag = nullptr;
    int* status = nullptr;             // SVM_DEV_* bits
    unsigned long long* stepCounter = nullptr;
    svm::T1Scratch t1;
    int maxPartialBlocks = 0;
    int sms = 152;                     // SMs of the model's device
    // graph cache for svm_brownian_run
    cudaGraphExec_t bdGraph = nullptr;
    cudaEvent_t runEv[2] = {nullptr, nullptr};   // svm_brownian_run: ends of the last two chunks
    double bdT = 0, bdDt = 0, bdMu = 0;
    uint64_t bdSeed = 0;
    int bdGraphCur = -1;
    // per-phase event timing (svm_model_profile)
    bool prof = false;
    int profMask = 0xff;               // phases bracketed by events while profiling (bit per phase)
    std::vector<cudaEvent_t> profEvents[SVM_PHASE_COUNT];   // start/stop pairs, in launch order
    int profUsed[SVM_PHASE_COUNT] = {0};
    double profMs[SVM_PHASE_COUNT] = {0};
    int profLaunches[SVM_PHASE_COUNT] = {0};   // kernel launches (a bracket may hold several)
    std::vector<int> profKernels[SVM_PHASE_COUNT];
    // bumped by every setter whose value a captured graph bakes in (Kr, threshold, restriction)
    unsigned paramsVersion = 0;
    unsigned bdGraphVersion = ~0u;
    // graph cache for svm_brownian_step_io with pinned host buffers, one per position-buffer role
    struct IoGraph {
        cudaGraphExec_t exec = nullptr;
        double T = 0, dt = 0, mu = 0;
        uint64_t seed = 0;
        const void *in = nullptr, *out = nullptr;
        const void* outDev = nullptr;   // the output's mapped device address the kernels write, or null
        unsigned version = ~0u;
        int precision = -1;
    } ioGraph[2];
    double* ioEnergy = nullptr;        // page-locked landing slot of the graph's energy copy
};

namespace svm {
// Brackets one phase launch with profiling events when profiling is on and the stream is not
// being captured.
struct PhaseTimer {
    svm_model* m;
    int phase;
    bool on;       // profiling on: the phase's launches are counted
    bool timed;    // and bracketed by events (the phase is in the profile mask)
    PhaseTimer(svm_model* m_, int phase_, int kernels = 1);
    ~PhaseTimer();
};
// launch helpers shared across translation units (svm_model.cu)
int launch_geometry(svm_model* m);
// vnormReady: the kernel that last moved every vertex also wrote its norm (pos_norm) to m->vnorm, so
// the corner pass skips k_vnorm.
int launch_corners(svm_model* m, bool t1test, bool vnormReady = false);
int launch_t1_apply(svm_model* m, int bump);
int grow_rings(svm_model* m, int newCapacity);
// Threads per block for a one-thread-per-item FP64 kernel over n items: the largest of 256, 128, 64
// and 32 that still gives every SM four blocks (or 32).  An SM's FP64 pipe -- one warp instruction
// per 16 clocks -- is kept busy by a few warps, so a small grid goes over all SMs in small blocks
// rather than over some of them in full ones.
inline int spread_block(const svm_model* m, long n) {
    int bs = 256;
    while (bs > 32 && n < 4L * m->sms * bs) bs >>= 1;
    return bs;
}
int ensure_ring_headroom(svm_model* m);
int check_launch();
// A binned view of device points (svm_celllist.cu): per-bin counts and slots (ascending point
// index), grid side nside and bin side h over [-radius, radius]^3.
struct CellGrid {
    const unsigned* counts;
    const int* slots;
    int cap, nside;
    double h, radius;
};
// Bins the points (AoS double[3n] on the device), widening the slots until no bin overflows;
// synchronises.  SVM_ERR_DEVICE when a point lies outside the grid.
int cell_list_bin(svm_cell_list* cl, const double* pointsDevice, int n, CellGrid* view);
void fire_detach(svm_fire* F);          // svm_fire.cu: the model is going away
int model_alloc(int nCells, int nVertices, int Wc, const double* radius, int nRep, void* stream, svm_model** out);
// replicas (svm_batch.cu)
int launch_rep_check(svm_model* m);
int update_rep_noise(svm_model* m, double dt, double mu);
void batch_release(svm_model* m);
int batch_tuned_corners(svm_model* m, bool t1test);
int batch_tuned_cells(svm_model* m, int (*launch)(svm_model*));
int batch_tuned_force_bd(svm_model* m, double T, double dt, double mu, int noiseMode, const double* noise,
                         uint64_t seed, int nxt);
bool batch_tuning(svm_model* m);
int mixed_max_block_corners();
int mixed_max_block_force();
int max_block_cells_batch();
void batch_tuner_untimed(svm_model* m, int calls);
// FP64 force kernels (svm_force_kernels.cu)
int zig_init();  // the device's normal-sampling table (svm_force_kernels.cu), before the first Brownian step
int launch_force_fp64(svm_model* m);
int launch_force_bd_fp64(svm_model* m, double np, double fp, int noiseMode, const double* noise, uint64_t seed,
                         int nxt);
// mixed-precision kernels (svm_mixed.cu)
int mixed_launch_corners(svm_model* m, bool t1test);
int mixed_launch_force(svm_model* m);
int mixed_launch_force_bd(svm_model* m, double T, double dt, double mu, int noiseMode, const double* noise,
                          uint64_t seed, int nxt);
int mixed_launch_move(svm_model* m, const double* disp, double scale);
int mixed_upload_positions(svm_model* m, const double* deviceAos);
int mixed_download(svm_model* m, const float4* src, int n, double* deviceAos);
}  // namespace svm
