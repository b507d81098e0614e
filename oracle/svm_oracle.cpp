// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's CPU path for the spherical vertex-model step
// (DanielMSussman/curvedSpaceVertexModel).  Only tests/, __graft_entry__.smoke() and
// bench.py's cpu_baseline / reference legs may load this library, and only as the checker or
// as the timed CPU baseline; the product path (libsvm) never links or calls it.
//
// Each routine cites the reference file:line it restates.  The arithmetic is written so that,
// compiled with -ffp-contract=off, it performs the same IEEE-754 operations in the same order
// as the reference's own CPU code; the tests pin it bit-for-bit against the reference compiled
// from its sources (oracle/ref) and against golden fixtures made from that build.
//
// Noise: the reference draws Brownian noise from std::mt19937 through the libstdc++
// std::normal_distribution<double> (src/utilities/noiseSource.{h,cpp}); this file uses the same
// standard-library engine and distributions, so a seed gives the same stream.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include <algorithm>

#include "svm_acos.h"   // the portable arccosine shared with the device build (product csrc/)

namespace {

// The arccosine of the geometry: the C library's (as the reference calls std::acos), or, when
// switched on by orc_set_portable_acos, svm_portable::acos -- the function the device library's
// -DSVM_PORTABLE_ACOS build evaluates with the same operations, so that GPU and CPU trajectories
// can be compared bit for bit.
//
// Mode 2 (orc_set_acos_mode) is another faithful arccosine: the C library's with one result in four
// moved by one ulp, up or down, chosen by a hash of the argument's bits and a seed -- a fixed
// function of the argument, like any library's.  An ensemble of such variants measures how far
// the reference's own trajectory moves when only the last bits of acos change.
int gAcosMode = 0;
unsigned long long gAcosSeed = 0;
inline unsigned long long mix64(unsigned long long z) {   // splitmix64 finaliser (Steele et al. 2014)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double racos(double x) {
    if (gAcosMode == 0) return std::acos(x);
    if (gAcosMode == 1) return svm_portable::acos(x);
    const double y = std::acos(x);
    unsigned long long b;
    std::memcpy(&b, &x, sizeof b);
    const unsigned long long h = mix64(b ^ gAcosSeed);
    if ((h & 3ull) != 0 || !(y > 0.0)) return y;
    return std::nextafter(y, (h >> 2) & 1ull ? 4.0 : 0.0);
}

const double kPI = 3.141592653589793115997963468544185161590576171875;  // inc/std_include.h:47

struct V3 { double x[3]; };

inline V3 v3(double a, double b, double c) { V3 r; r.x[0] = a; r.x[1] = b; r.x[2] = c; return r; }
inline V3 add(const V3& a, const V3& b) { return v3(a.x[0] + b.x[0], a.x[1] + b.x[1], a.x[2] + b.x[2]); }
inline V3 sub(const V3& a, const V3& b) { return v3(a.x[0] - b.x[0], a.x[1] - b.x[1], a.x[2] - b.x[2]); }
inline V3 scale(double s, const V3& a) { return v3(s * a.x[0], s * a.x[1], s * a.x[2]); }
// dot: accumulate from 0.0 in component order (inc/functions.h:131-138)
inline double dot(const V3& a, const V3& b) {
    double s = 0.0;
    s += a.x[0] * b.x[0]; s += a.x[1] * b.x[1]; s += a.x[2] * b.x[2];
    return s;
}
inline double norm(const V3& a) { return std::sqrt(dot(a, a)); }           // inc/functions.h:170-173
inline V3 cross(const V3& p1, const V3& p2) {                              // inc/functions.h:160-167
    return v3(p1.x[1] * p2.x[2] - p1.x[2] * p2.x[1],
              p1.x[2] * p2.x[0] - p1.x[0] * p2.x[2],
              p1.x[0] * p2.x[1] - p1.x[1] * p2.x[0]);
}
// rodriguesRotation (inc/functions.h:175-181)
inline void rodrigues(V3& v, const V3& k, double theta) {
    V3 cp = cross(k, v);
    double c = std::cos(theta), s = std::sin(theta);
    double kv = dot(k, v);
    double w = (1.0 - c) * kv;
    V3 ans;
    for (int d = 0; d < 3; ++d) ans.x[d] = (c * v.x[d] + s * cp.x[d]) + w * k.x[d];
    v = ans;
}

// ---- sphericalDomain (inc/sphericalDomain.h) -------------------------------------------
struct Sphere {
    double radius = 1.0;
    // putInBoxVirtual / putInBoxReal (sphericalDomain.h:179-187)
    void putVirtual(V3& p) const { double inv = 1.0 / norm(p); p = scale(inv, p); }
    void putReal(V3& p) const { double inv = 1.0 / norm(p); V3 t = scale(inv, p); p = scale(radius, t); }
    // projectToTangentPlane (sphericalDomain.h:169-172)
    static void project(V3& vec, const V3& n) {
        double s = dot(vec, n) / dot(n, n);
        vec = sub(vec, scale(s, n));
    }
    // move(p, v) (sphericalDomain.h:203-209)
    void move(V3& p, const V3& v) const { V3 d = v; project(d, p); p = add(p, d); putReal(p); }
    // geodesicDistance (sphericalDomain.h:94-112)
    double geodesic(const V3& p1, const V3& p2) const {
        double num = p1.x[0] * p2.x[0] + p1.x[1] * p2.x[1] + p1.x[2] * p2.x[2];
        double den = std::sqrt(p1.x[0] * p1.x[0] + p1.x[1] * p1.x[1] + p1.x[2] * p1.x[2]) *
                     std::sqrt(p2.x[0] * p2.x[0] + p2.x[1] * p2.x[1] + p2.x[2] * p2.x[2]);
        return radius * racos(num / den);
    }
    // includedAngle (sphericalDomain.h:114-133)
    static double includedAngle(const V3& p1, const V3& p2, const V3& p3) {
        V3 ci = cross(p2, p3), cim1 = cross(p1, p2);
        double det = p1.x[0] * (p2.x[1] * p3.x[2] - p2.x[2] * p3.x[1]) +
                     p1.x[1] * (p2.x[2] * p3.x[0] - p2.x[0] * p3.x[2]) +
                     p1.x[2] * (p2.x[0] * p3.x[1] - p2.x[1] * p3.x[0]);
        double a = racos(-dot(ci, cim1) / (norm(ci) * norm(cim1)));
        if (det > 0) a *= -1;
        if (a < 0) a += 2. * kPI;
        return a;
    }
    // sphericalTriangleArea (sphericalDomain.h:135-166)
    double triangleArea(const V3& q1, const V3& q2, const V3& q3) const {
        V3 p1 = q1, p2 = q2, p3 = q3;
        putVirtual(p1); putVirtual(p2); putVirtual(p3);
        double d12 = dot(p1, p2), d13 = dot(p1, p3), d23 = dot(p2, p3);
        double area = -kPI;
        area += racos((d23 - d12 * d13) / (std::sqrt(1 - d12 * d12) * std::sqrt(1 - d13 * d13)));
        area += racos((d12 - d13 * d23) / (std::sqrt(1 - d13 * d13) * std::sqrt(1 - d23 * d23)));
        area += racos((d13 - d12 * d23) / (std::sqrt(1 - d12 * d12) * std::sqrt(1 - d23 * d23)));
        area *= (radius * radius);
        return area;
    }
    // cartesianSphericalBasisChange(p, thetaHat, phiHat) (sphericalDomain.h:218-232)
    static void basis(const V3& p, V3& th, V3& ph) {
        double r = std::sqrt(p.x[0] * p.x[0] + p.x[1] * p.x[1] + p.x[2] * p.x[2]);
        double cosT = p.x[2] / r;
        double sinT = std::sqrt(1. - cosT * cosT);
        double den = std::sqrt(p.x[0] * p.x[0] + p.x[1] * p.x[1]);
        double cosP = p.x[0] / den, sinP = p.x[1] / den;
        th = v3(cosT * cosP, cosT * sinP, -sinT);
        ph = v3(-sinP, cosP, 0);
    }
    // gradientGeodesicDistance with a known basis (sphericalDomain.h:248-273)
    static V3 gradGeodesic(const V3& v1, const V3& v2, const V3& th, const V3& ph) {
        double r1 = std::sqrt(dot(v1, v1)), r2 = std::sqrt(dot(v2, v2));
        double cosT1 = v1.x[2] / r1, cosT2 = v2.x[2] / r2;
        double sinT1 = std::sqrt(1 - cosT1 * cosT1), sinT2 = std::sqrt(1 - cosT2 * cosT2);
        double cosP1 = v1.x[0] / std::sqrt(v1.x[0] * v1.x[0] + v1.x[1] * v1.x[1]);
        double cosP2 = v2.x[0] / std::sqrt(v2.x[0] * v2.x[0] + v2.x[1] * v2.x[1]);
        double sinP1 = v1.x[1] / std::sqrt(v1.x[0] * v1.x[0] + v1.x[1] * v1.x[1]);
        double sinP2 = v2.x[1] / std::sqrt(v2.x[0] * v2.x[0] + v2.x[1] * v2.x[1]);
        double sP12 = sinP1 * cosP2 - cosP1 * sinP2;
        double cP12 = cosP1 * cosP2 + sinP1 * sinP2;
        double dp = cosT1 * cosT2 + cP12 * sinT1 * sinT2;
        double dinv = 1. / std::sqrt(1 - dp * dp);
        double gT = 1.0 * (cosT2 * sinT1 - cosT1 * cP12 * sinT2) * dinv;
        double gP = sinT2 * sP12 * dinv;
        V3 r;
        for (int d = 0; d < 3; ++d) r.x[d] = gT * th.x[d] + gP * ph.x[d];
        return r;
    }
    // gradientTriangleArea with a known basis (sphericalDomain.h:347-411)
    V3 gradTriangle(const V3& v1, const V3& v2, const V3& v3v, const V3& th, const V3& ph) const {
        double r1 = std::sqrt(dot(v1, v1)), r2 = std::sqrt(dot(v2, v2)), r3 = std::sqrt(dot(v3v, v3v));
        double cosT1 = v1.x[2] / r1, cosT2 = v2.x[2] / r2, cosT3 = v3v.x[2] / r3;
        double sinT1 = std::sqrt(1 - cosT1 * cosT1), sinT2 = std::sqrt(1 - cosT2 * cosT2), sinT3 = std::sqrt(1 - cosT3 * cosT3);
        double cosP1 = v1.x[0] / std::sqrt(v1.x[0] * v1.x[0] + v1.x[1] * v1.x[1]);
        double cosP2 = v2.x[0] / std::sqrt(v2.x[0] * v2.x[0] + v2.x[1] * v2.x[1]);
        double cosP3 = v3v.x[0] / std::sqrt(v3v.x[0] * v3v.x[0] + v3v.x[1] * v3v.x[1]);
        double sinP1 = v1.x[1] / std::sqrt(v1.x[0] * v1.x[0] + v1.x[1] * v1.x[1]);
        double sinP2 = v2.x[1] / std::sqrt(v2.x[0] * v2.x[0] + v2.x[1] * v2.x[1]);
        double sinP3 = v3v.x[1] / std::sqrt(v3v.x[0] * v3v.x[0] + v3v.x[1] * v3v.x[1]);
        double sP12 = sinP1 * cosP2 - cosP1 * sinP2;
        double sP13 = sinP1 * cosP3 - cosP1 * sinP3;
        double cP12 = cosP1 * cosP2 + sinP1 * sinP2;
        double cP13 = cosP1 * cosP3 + sinP1 * sinP3;
        double cP23 = cosP2 * cosP3 + sinP2 * sinP3;
        double s12 = cosT1 * cosT2 + cP12 * sinT1 * sinT2;
        double s13 = cosT1 * cosT3 + cP13 * sinT1 * sinT3;
        double s23 = cosT2 * cosT3 + cP23 * sinT2 * sinT3;
        double d12 = cosT1 * cP12 * sinT2 - cosT2 * sinT1;
        double d13 = cosT1 * cP13 * sinT3 - cosT3 * sinT1;
        double g = 1 - s12 * s12 - s13 * s13 - s23 * s23 + 2.0 * s12 * s13 * s23;
        double den1 = std::sqrt((-1. + s12 * s12) * (-1. + s12 * s12) * g);
        double den2 = std::sqrt((-1. + s13 * s13) * (-1. + s13 * s13) * g);
        double den3 = std::sqrt((s12 * s12 - 1.) * (s13 * s13 - 1.) * (s12 * s12 - 1.) * (s13 * s13 - 1.) * g);
        double gT = (d13 * (s12 * s12 - 1.0) + d12 * (s23 - s12 * s13)) / den1
                  + (d12 * (s13 * s13 - 1.0) + d13 * (s23 - s12 * s13)) / den2
                  - (d12 * (s13 * s13 - 1.) * (s13 - s12 * s23) + d13 * (s12 * s12 - 1.0) * (s12 - s13 * s23)) / den3;
        gT *= radius;
        double gP = ((s12 * s13 - s23) * sP12 * sinT2 - (-1 + s12 * s12) * sP13 * sinT3) / (den1)
                  - ((-1 + s13 * s13) * sP12 * sinT2 + (-(s12 * s13) + s23) * sP13 * sinT3) / (den2)
                  + ((-1 + s13 * s13) * (s13 - s12 * s23) * sP12 * sinT2 + (-1 + s12 * s12) * (s12 - s13 * s23) * sP13 * sinT3) / (den3);
        gP *= radius;
        double det = v1.x[0] * (v2.x[1] * v3v.x[2] - v2.x[2] * v3v.x[1]) +
                     v1.x[1] * (v2.x[2] * v3v.x[0] - v2.x[0] * v3v.x[2]) +
                     v1.x[2] * (v2.x[0] * v3v.x[1] - v2.x[1] * v3v.x[0]);
        V3 r;
        for (int d = 0; d < 3; ++d) r.x[d] = gT * th.x[d] + gP * ph.x[d];
        if (det < 0) r = scale(-1., r);
        return r;
    }
};

struct Int4 { int x, y, z, w; };

}  // namespace

// ---- model state: the reference's arrays (src/model/sphericalVertexModel.h:208-230) -------
struct orc_model {
    int nCells = 0, N = 0;           // N = number of vertices (sphericalVertexModel.cpp:30)
    int W = 0;                       // maximumVerticesPerCell = cellNeighborIndex width
    Sphere sphere;
    double Kr = 1.0, t1Threshold = 0.1;
    bool restrictedMotion = false;
    std::vector<V3> pos, forces, vel, cellPos, curV, lastV, nextV;
    std::vector<V3> dir;                     // directors (simpleModel.h:113), one per vertex
    std::vector<double> mass;
    std::vector<int> cellNeighbors;          // [nCells*W], index c*W + k (inc/indexer.h:41-44)
    std::vector<unsigned> cellCount;         // cellNumberOfNeighbors
    std::vector<int> vcn;                    // vertexCellNeighbors [3N]
    std::vector<int> vn;                     // neighbors (vertex-vertex) [3N]
    std::vector<double> ap, app;             // areaPerimeter / preference, pairs (x=area, y=perimeter)
    std::vector<int> flipLog;                // (vertex1, vertex2) per performed T1, in order
    double lastExcessArea = 0.0;
    int fallbackCount = 0;
};

extern "C" {

// Selects the arccosine of the geometry: 0 the C library's (the reference's), 1 the portable one,
// 2 the C library's with a seeded one-ulp perturbation of one result in four.
void orc_set_acos_mode(int mode, unsigned long long seed) {
    gAcosMode = mode;
    gAcosSeed = seed;
}
void orc_set_portable_acos(int on) { orc_set_acos_mode(on ? 1 : 0, 0); }
// svm_portable::acos over an array (checks of the portable function itself).
void orc_acos_portable(const double* x, double* out, long n) {
    for (long i = 0; i < n; ++i) out[i] = svm_portable::acos(x[i]);
}

orc_model* orc_create(int nCells, int nVertices, int W, const double* pos, const int* cellNeighbors,
                      const unsigned* cellCount, const int* vcn, const int* vn, double radius) {
    orc_model* m = new orc_model();
    m->nCells = nCells; m->N = nVertices; m->W = W;
    m->sphere.radius = radius;
    m->pos.resize(nVertices);
    m->dir.assign(nVertices, v3(0.0, 0.0, 0.0));
    for (int i = 0; i < nVertices; ++i) m->pos[i] = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    m->cellNeighbors.assign(cellNeighbors, cellNeighbors + (size_t)nCells * W);
    m->cellCount.assign(cellCount, cellCount + nCells);
    m->vcn.assign(vcn, vcn + 3 * (size_t)nVertices);
    m->vn.assign(vn, vn + 3 * (size_t)nVertices);
    m->forces.assign(nVertices, v3(0, 0, 0));
    m->vel.assign(nVertices, v3(0, 0, 0));
    m->mass.assign(nVertices, 1.0);
    m->cellPos.assign(nCells, v3(0, 0, 0));
    m->curV.assign(3 * (size_t)nVertices, v3(0, 0, 0));
    m->lastV = m->curV; m->nextV = m->curV;
    m->ap.assign(2 * (size_t)nCells, 0.0);
    m->app.assign(2 * (size_t)nCells, 0.0);
    for (int c = 0; c < nCells; ++c) { m->app[2 * c] = 1.0; m->app[2 * c + 1] = 3.8; }
    return m;
}

void orc_destroy(orc_model* m) { delete m; }

// setPreferredParameters (sphericalVertexModel.cpp:103-109)
void orc_set_preferred(orc_model* m, double a0, double p0) {
    for (int c = 0; c < m->nCells; ++c) { m->app[2 * c] = a0; m->app[2 * c + 1] = p0; }
}
void orc_set_preferred_array(orc_model* m, const double* a0p0) {
    std::memcpy(m->app.data(), a0p0, sizeof(double) * 2 * m->nCells);
}
void orc_set_kr(orc_model* m, double kr) { m->Kr = kr; }
void orc_set_t1_threshold(orc_model* m, double t) { m->t1Threshold = t; }
void orc_set_restricted(orc_model* m, int r) { m->restrictedMotion = r != 0; }

// recomputeAreasCPU (sphericalVertexModel.cpp:162-207)
static void recomputeAreas(orc_model* m) {
    for (int cc = 0; cc < m->nCells; ++cc) {
        int neighs = (int)m->cellCount[cc];
        V3 cp = m->cellPos[cc];
        V3 last = m->pos[m->cellNeighbors[cc * m->W + neighs - 2]];
        V3 cur = m->pos[m->cellNeighbors[cc * m->W + neighs - 1]];
        double area = 0;
        for (int nn = 0; nn < neighs; ++nn) {
            V3 next = m->pos[m->cellNeighbors[cc * m->W + nn]];
            area += m->sphere.triangleArea(cp, last, cur);
            last = cur; cur = next;
        }
        m->ap[2 * cc] = area;
    }
}

// computeGeometryCPU (sphericalVertexModel.cpp:209-311)
void orc_compute_geometry(orc_model* m) {
    double totalArea = 0;
    const int W = m->W;
    for (int cc = 0; cc < m->nCells; ++cc) {
        int neighs = (int)m->cellCount[cc];
        V3 cpos = v3(0.0, 0.0, 0.0);
        for (int nn = 0; nn < neighs; ++nn) cpos = add(cpos, m->pos[m->cellNeighbors[cc * W + nn]]);
        m->sphere.putReal(cpos);
        m->cellPos[cc] = cpos;
        int lastIdx = m->cellNeighbors[cc * W + neighs - 3];
        int curIdx = m->cellNeighbors[cc * W + neighs - 2];
        int nextIdx = m->cellNeighbors[cc * W + neighs - 1];
        V3 last = m->pos[lastIdx], cur = m->pos[curIdx], next = m->pos[nextIdx];
        double perimeter = 0, area = 0;
        for (int nn = 0; nn < neighs; ++nn) {
            int slot = -1;
            for (int vn = 0; vn < 3; ++vn)
                if (m->vcn[3 * curIdx + vn] == cc) slot = 3 * curIdx + vn;
            int plus2 = m->cellNeighbors[cc * W + nn];
            V3 p2 = m->pos[plus2];
            perimeter += m->sphere.geodesic(last, cur);
            area += Sphere::includedAngle(last, cur, next);
            m->curV[slot] = cur; m->lastV[slot] = last; m->nextV[slot] = next;
            last = cur; curIdx = nextIdx; cur = next; nextIdx = plus2; next = p2;
        }
        area = (area - (neighs - 2) * kPI);
        int extra = (int)std::floor(area / (1.0 * kPI));
        if (extra > 0) area -= extra * kPI;
        area = area * m->sphere.radius * m->sphere.radius;
        m->ap[2 * cc] = area;
        m->ap[2 * cc + 1] = perimeter;
        totalArea += area;
    }
    double excess = totalArea - 4.0 * kPI * m->sphere.radius * m->sphere.radius;
    m->lastExcessArea = excess;
    if (std::fabs(excess) > 1e-6) { recomputeAreas(m); m->fallbackCount += 1; }
}

// computeForceCPU (sphericalVertexModel.cpp:356-420)
void orc_compute_forces(orc_model* m) {
    orc_compute_geometry(m);
    for (int v = 0; v < m->N; ++v) {
        V3 f = v3(0.0, 0.0, 0.0);
        for (int cc = 0; cc < 3; ++cc) {
            V3 fs = v3(0.0, 0.0, 0.0);
            int cni = 3 * v + cc;
            int cell = m->vcn[cni];
            const V3 cp = m->cellPos[cell], vl = m->lastV[cni], vc = m->curV[cni], vx = m->nextV[cni];
            double dA = m->ap[2 * cell] - m->app[2 * cell];
            double dP = m->ap[2 * cell + 1] - m->app[2 * cell + 1];
            V3 th, ph, t;
            Sphere::basis(vc, th, ph);
            double pp = 2.0 * dP;
            double aa = 2.0 * m->Kr * dA;
            t = Sphere::gradGeodesic(vc, vl, th, ph);
            for (int d = 0; d < 3; ++d) fs.x[d] -= pp * t.x[d];
            t = Sphere::gradGeodesic(vc, vx, th, ph);
            for (int d = 0; d < 3; ++d) fs.x[d] -= pp * t.x[d];
            t = m->sphere.gradTriangle(vc, vl, cp, th, ph);
            for (int d = 0; d < 3; ++d) fs.x[d] -= aa * t.x[d];
            t = m->sphere.gradTriangle(vc, cp, vx, th, ph);
            for (int d = 0; d < 3; ++d) fs.x[d] -= aa * t.x[d];
            if (!std::isnan(fs.x[0])) f = add(f, fs);
        }
        m->forces[v] = f;
    }
}

// computeEnergy (sphericalVertexModel.cpp:150-160)
double orc_energy(orc_model* m) {
    double e = 0.0;
    for (int i = 0; i < m->nCells; ++i) {
        double da = m->ap[2 * i] - m->app[2 * i], dp = m->ap[2 * i + 1] - m->app[2 * i + 1];
        e += m->Kr * da * da + dp * dp;
    }
    return e;
}

// getCellVertexSetForT1 (sphericalVertexModel.cpp:611-731).  The unused search for "c" and
// "d" at lines 630-640 has no effect on any output and is omitted.
static void cellVertexSet(orc_model* m, int v1, int v2, Int4& cs, Int4& vs, bool& grow) {
    const int W = m->W;
    int c[3] = {m->vcn[3 * v1], m->vcn[3 * v1 + 1], m->vcn[3 * v1 + 2]};
    for (int ff = 0; ff < 3; ++ff) {
        int t = m->vcn[3 * v2 + ff];
        if (t != c[0] && t != c[1] && t != c[2]) cs.w = t;
    }
    auto around = [&](int cell, int target, int& vlast, int& vnext) {
        int n = (int)m->cellCount[cell];
        vlast = m->cellNeighbors[cell * W + n - 2];
        int vcur = m->cellNeighbors[cell * W + n - 1];
        for (int k = 0; k < n; ++k) {
            vnext = m->cellNeighbors[cell * W + k];
            if (vcur == target) break;
            vlast = vcur; vcur = vnext;
        }
    };
    for (int q = 0; q < 3; ++q) {
        int vl, vx;
        around(c[q], v1, vl, vx);
        if (vl == v2) cs.x = c[q];
        else if (vx == v2) cs.z = c[q];
        else cs.y = c[q];
    }
    int vl, vx;
    around(cs.y, v1, vl, vx); vs.x = vl; vs.y = vx;
    around(cs.w, v2, vl, vx); vs.w = vl; vs.z = vx;
    const unsigned Wm = (unsigned)m->W;
    if (m->cellCount[cs.x] == Wm || m->cellCount[cs.y] == Wm || m->cellCount[cs.z] == Wm || m->cellCount[cs.w] == Wm)
        grow = true;
}

// growCellVerticesList (sphericalVertexModel.cpp:733-758)
static void growRings(orc_model* m, int newVertexMax) {
    int oldW = m->W, newW = newVertexMax + 1;
    std::vector<int> nc((size_t)newW * m->nCells, 0);
    for (int c = 0; c < m->nCells; ++c)
        for (int k = 0; k < (int)m->cellCount[c]; ++k) nc[(size_t)c * newW + k] = m->cellNeighbors[(size_t)c * oldW + k];
    m->cellNeighbors.swap(nc);
    m->W = newW;
}

// testAndPerformT1TransitionsCPU (sphericalVertexModel.cpp:439-604)
static void t1Transitions(orc_model* m) {
    int vMax = m->W;
    Int4 cs = {0, 0, 0, 0}, vs = {0, 0, 0, 0};
    for (int vertex1 = 0; vertex1 < m->N; ++vertex1) {
        V3 v1 = m->pos[vertex1];
        for (int vv = 0; vv < 3; ++vv) {
            int vertex2 = m->vn[3 * vertex1 + vv];
            if (!(vertex1 < vertex2)) continue;
            V3 v2 = m->pos[vertex2];
            double arc = m->sphere.geodesic(v1, v2);
            if (!(arc < m->t1Threshold)) continue;
            bool grow = false;
            cellVertexSet(m, vertex1, vertex2, cs, vs, grow);
            if (m->cellCount[cs.x] == 3 || m->cellCount[cs.z] == 3) continue;
            if (grow) { vMax += 1; growRings(m, vMax); }
            const int W = m->W;
            V3 mid = scale(0.5, add(v1, v2));
            m->sphere.putVirtual(mid);
            V3 vC = m->pos[vs.z];
            double det = vC.x[0] * (v1.x[1] * v2.x[2] - v1.x[2] * v2.x[1]) +
                         vC.x[1] * (v1.x[2] * v2.x[0] - v1.x[0] * v2.x[2]) +
                         vC.x[2] * (v1.x[0] * v2.x[1] - v1.x[1] * v2.x[0]);
            det = det > 0 ? 1. : -1.;
            rodrigues(v1, mid, -0.5 * det * kPI);
            rodrigues(v2, mid, -0.5 * det * kPI);
            V3 diff = scale(0.5, sub(v1, v2));
            v1 = add(v1, diff);
            v2 = sub(v2, diff);
            m->sphere.putReal(v1);
            m->sphere.putReal(v2);
            m->pos[vertex1] = v1;
            m->pos[vertex2] = v2;
            for (int k = 0; k < 3; ++k) {
                if (m->vcn[3 * vertex1 + k] == cs.z) m->vcn[3 * vertex1 + k] = cs.w;
                if (m->vcn[3 * vertex2 + k] == cs.x) m->vcn[3 * vertex2 + k] = cs.y;
                if (m->vn[3 * vs.y + k] == vertex1) m->vn[3 * vs.y + k] = vertex2;
                if (m->vn[3 * vs.z + k] == vertex2) m->vn[3 * vs.z + k] = vertex1;
                if (m->vn[3 * vertex1 + k] == vs.y) m->vn[3 * vertex1 + k] = vs.z;
                if (m->vn[3 * vertex2 + k] == vs.z) m->vn[3 * vertex2 + k] = vs.y;
            }
            auto removeFrom = [&](int cell, int target) {
                int n = (int)m->cellCount[cell];
                int idx = 0;
                for (int k = 0; k < n - 1; ++k) {
                    if (m->cellNeighbors[cell * W + k] == target) idx += 1;
                    m->cellNeighbors[cell * W + k] = m->cellNeighbors[cell * W + idx];
                    idx += 1;
                }
                m->cellCount[cell] -= 1;
            };
            auto insertAfter = [&](int cell, int after, int added) {
                int n = (int)m->cellCount[cell];
                std::vector<int> cp(n + 1);
                int idx = 0;
                for (int k = 0; k < n; ++k) {
                    int x = m->cellNeighbors[cell * W + k];
                    cp[idx++] = x;
                    if (x == after) cp[idx++] = added;
                }
                for (int k = 0; k < n + 1; ++k) m->cellNeighbors[cell * W + k] = cp[k];
                m->cellCount[cell] = n + 1;
            };
            removeFrom(cs.x, vertex2);
            insertAfter(cs.y, vertex1, vertex2);
            removeFrom(cs.z, vertex1);
            insertAfter(cs.w, vertex2, vertex1);
            m->flipLog.push_back(vertex1);
            m->flipLog.push_back(vertex2);
        }
    }
}

// moveParticlesCPU (sphericalVertexModel.cpp:111-135) + enforceTopology (422-433)
void orc_move(orc_model* m, const double* disp, double scaleFactor) {
    for (int i = 0; i < m->N; ++i) {
        V3 d = v3(disp[3 * i], disp[3 * i + 1], disp[3 * i + 2]);
        if (scaleFactor != 1.) d = scale(scaleFactor, d);
        m->sphere.move(m->pos[i], d);
    }
    if (!m->restrictedMotion) t1Transitions(m);
}

void orc_enforce_topology(orc_model* m) { t1Transitions(m); }

// ---- accessors ------------------------------------------------------------------------
int orc_num_vertices(orc_model* m) { return m->N; }
int orc_ring_width(orc_model* m) { return m->W; }
void orc_get_positions(orc_model* m, double* out) {
    for (int i = 0; i < m->N; ++i) for (int d = 0; d < 3; ++d) out[3 * i + d] = m->pos[i].x[d];
}
void orc_set_positions(orc_model* m, const double* in) {
    for (int i = 0; i < m->N; ++i) for (int d = 0; d < 3; ++d) m->pos[i].x[d] = in[3 * i + d];
}
void orc_get_forces(orc_model* m, double* out) {
    for (int i = 0; i < m->N; ++i) for (int d = 0; d < 3; ++d) out[3 * i + d] = m->forces[i].x[d];
}
void orc_get_velocities(orc_model* m, double* out) {
    for (int i = 0; i < m->N; ++i) for (int d = 0; d < 3; ++d) out[3 * i + d] = m->vel[i].x[d];
}
void orc_set_velocities(orc_model* m, const double* in) {
    for (int i = 0; i < m->N; ++i) for (int d = 0; d < 3; ++d) m->vel[i].x[d] = in[3 * i + d];
}
void orc_get_cell_positions(orc_model* m, double* out) {
    for (int i = 0; i < m->nCells; ++i) for (int d = 0; d < 3; ++d) out[3 * i + d] = m->cellPos[i].x[d];
}
void orc_get_area_perimeter(orc_model* m, double* out) { std::memcpy(out, m->ap.data(), sizeof(double) * 2 * m->nCells); }
// Rings are returned in a caller-chosen width Wout >= max ring (padding -1).
int orc_get_rings(orc_model* m, int* out, int Wout, unsigned* counts) {
    for (int c = 0; c < m->nCells; ++c) {
        int n = (int)m->cellCount[c];
        if (n > Wout) return -1;
        counts[c] = (unsigned)n;
        for (int k = 0; k < Wout; ++k) out[(size_t)c * Wout + k] = k < n ? m->cellNeighbors[(size_t)c * m->W + k] : -1;
    }
    return 0;
}
void orc_get_vertex_cells(orc_model* m, int* out) { std::memcpy(out, m->vcn.data(), sizeof(int) * 3 * m->N); }
void orc_get_vertex_neighbors(orc_model* m, int* out) { std::memcpy(out, m->vn.data(), sizeof(int) * 3 * m->N); }
int orc_flip_count(orc_model* m) { return (int)m->flipLog.size() / 2; }
void orc_get_flips(orc_model* m, int* out) { std::memcpy(out, m->flipLog.data(), sizeof(int) * m->flipLog.size()); }
void orc_clear_flips(orc_model* m) { m->flipLog.clear(); }
double orc_last_excess_area(orc_model* m) { return m->lastExcessArea; }
int orc_fallback_count(orc_model* m) { return m->fallbackCount; }

// ---- noise source (src/utilities/noiseSource.{h,cpp}) ---------------------------------------
struct orc_noise {
    std::mt19937 gen{13377};                        // noiseSource.h:24
    std::normal_distribution<> unitNormal;           // noiseSource.h:75
};
orc_noise* orc_noise_create(int seed) {              // setReproducibleSeed (noiseSource.cpp:72-82)
    orc_noise* n = new orc_noise();
    if (seed >= 0) n->gen = std::mt19937(seed);
    return n;
}
void orc_noise_destroy(orc_noise* n) { delete n; }
double orc_noise_uniform(orc_noise* n, double lo, double hi) {   // getRealUniform (noiseSource.cpp:18-27)
    std::uniform_real_distribution<double> u(lo, hi);
    return u(n->gen);
}
void orc_noise_normals(orc_noise* n, double* out, long count) {  // getRealNormalStandardized (29-37)
    for (long i = 0; i < count; ++i) out[i] = n->unitNormal(n->gen);
}

// Cell centres of sphericalModel: setParticlePositionsRandomly at radius 1 (sphericalModel.cpp:37-51),
// the director draws that follow it (52-63; consumed, not returned), then setRadius(sqrt(n/4pi))
// (sphericalVertexModel.cpp:12, sphericalModel.cpp:11-22).
void orc_random_cell_centres(orc_noise* nz, int n, double* out) {
    Sphere unit; unit.radius = 1.0;
    std::vector<V3> p(n);
    for (int i = 0; i < n; ++i) {
        double u = orc_noise_uniform(nz, 0., 1.), v = orc_noise_uniform(nz, 0., 1.);
        double phi = 2.0 * kPI * u, theta = std::acos(2.0 * v - 1);
        p[i] = v3(1.0 * std::sin(theta) * std::cos(phi), 1.0 * std::sin(theta) * std::sin(phi), 1.0 * std::cos(theta));
        unit.putReal(p[i]);
    }
    for (int i = 0; i < n; ++i) { orc_noise_uniform(nz, 0., 1.); orc_noise_uniform(nz, 0., 1.); }
    Sphere big; big.radius = std::sqrt(n / (4.0 * kPI));
    for (int i = 0; i < n; ++i) { big.putReal(p[i]); for (int d = 0; d < 3; ++d) out[3 * i + d] = p[i].x[d]; }
}

// ---- Brownian dynamics: integrateEOMCPU (src/updaters/brownianDynamics.cpp:29-48) -------------
// Forces, then disp = xi*sqrt(2 dt mu T) + F dt mu with xi drawn in (vertex, dim) order, then move.
void orc_brownian_step(orc_model* m, orc_noise* nz, double T, double dt, double mu, double* dispOut) {
    orc_compute_forces(m);
    double fp = dt * mu;
    double np = std::sqrt(2.0 * fp * T);
    std::vector<double> disp(3 * (size_t)m->N);
    for (int i = 0; i < m->N; ++i)
        for (int d = 0; d < 3; ++d) disp[3 * i + d] = nz->unitNormal(nz->gen) * np + m->forces[i].x[d] * fp;
    if (dispOut) std::memcpy(dispOut, disp.data(), sizeof(double) * disp.size());
    orc_move(m, disp.data(), 1.0);
}

// Same step with the standard normals supplied by the caller (Nv*3, vertex-major).
void orc_brownian_step_noise(orc_model* m, const double* xi, double T, double dt, double mu) {
    orc_compute_forces(m);
    double fp = dt * mu;
    double np = std::sqrt(2.0 * fp * T);
    std::vector<double> disp(3 * (size_t)m->N);
    for (int i = 0; i < m->N; ++i)
        for (int d = 0; d < 3; ++d) disp[3 * i + d] = xi[3 * i + d] * np + m->forces[i].x[d] * fp;
    orc_move(m, disp.data(), 1.0);
}

// ---- self-propelled particles on the vertex model's directors -----------------------------
// projectToTangentPlaneAndNormalize (sphericalDomain.h:173-177)
static void projectNormalize(V3& vec, const V3& n) {
    double s = dot(vec, n) / dot(n, n);
    vec = sub(vec, scale(s, n));
    vec = scale(1.0 / norm(vec), vec);
}
void orc_set_directors(orc_model* m, const double* d) {
    for (int i = 0; i < m->N; ++i) m->dir[i] = v3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
}
void orc_get_directors(orc_model* m, double* out) {
    for (int i = 0; i < m->N; ++i)
        for (int d = 0; d < 3; ++d) out[3 * i + d] = m->dir[i].x[d];
}
// The vertex model's random directors, made as sphericalVertexModel.cpp:58-70 makes them, drawn from
// the noise source that made the cell centres, after them (the reference draws them from the
// model's own random_device-seeded source; the library's seeded choice is restated here).
void orc_init_directors(orc_model* m, orc_noise* nz) {
    for (int i = 0; i < m->N; ++i) {
        double u2 = orc_noise_uniform(nz, 0., 1.), v2 = orc_noise_uniform(nz, 0., 1.);
        double phi = 2.0 * kPI * u2, theta = std::acos(2.0 * v2 - 1);
        V3 n = v3(1.0 * std::sin(theta) * std::cos(phi), 1.0 * std::sin(theta) * std::sin(phi), 1.0 * std::cos(theta));
        projectNormalize(n, m->pos[i]);
        m->dir[i] = n;
    }
}
// sphericalSelfPropelledParticle::integrateEOMCPU (src/updaters/sphericalSelfPropelledParticle.cpp:
// 16-47): forces; disp = dt (v0 n + mu F); move (with T1 unless restricted); then each director is
// projected onto the tangent plane at its vertex's new position, normalised, and rotated about
// that position vector by theta = r sqrt(2 dt tau), r the vertex's uniform draw in [-1/2, 1/2)
// (here supplied by the caller, Nv values).
void orc_spp_step_noise(orc_model* m, const double* r, double dt, double mu, double v0, double tau) {
    orc_compute_forces(m);
    std::vector<double> disp(3 * (size_t)m->N);
    for (int i = 0; i < m->N; ++i)
        for (int d = 0; d < 3; ++d) disp[3 * i + d] = dt * (v0 * m->dir[i].x[d] + mu * m->forces[i].x[d]);
    orc_move(m, disp.data(), 1.0);
    for (int i = 0; i < m->N; ++i) {
        double theta = r[i] * std::sqrt(2.0 * dt * tau);
        projectNormalize(m->dir[i], m->pos[i]);
        V3 nd = m->dir[i];
        rodrigues(nd, m->pos[i], theta);
        m->dir[i] = nd;
    }
}
// sphericalVectorialVicsek::integrateEOMCPU (src/updaters/sphericalVectorialVicsek.cpp:5-60) on the
// vertex model, whose neighbours (numberOfNeighbors, neighbors) are the three vertex neighbours:
// forces; disp = dt (v0 n + mu F); move (with T1 unless restricted); then, from the directors before
// the update, per vertex a random unit vector (u, w: phi = 2 pi u, theta = acos(2w - 1)) projected
// onto the tangent plane at the vertex's new position and normalised, the target
// (n + neighbours' n) * (1/4) + point * eta projected and normalised; then each director
// n += (dt/tau)(target - n), projected onto the tangent plane and normalised.  uw: the caller's
// 2 Nv uniform draws in [0, 1), (u, w) per vertex in vertex order.
void orc_vicsek_step_noise(orc_model* m, const double* uw, double dt, double mu, double v0, double eta, double tau) {
    orc_compute_forces(m);
    std::vector<double> disp(3 * (size_t)m->N);
    for (int i = 0; i < m->N; ++i)
        for (int d = 0; d < 3; ++d) disp[3 * i + d] = dt * (v0 * m->dir[i].x[d] + mu * m->forces[i].x[d]);
    orc_move(m, disp.data(), 1.0);
    std::vector<V3> target(m->N);
    for (int i = 0; i < m->N; ++i) {
        const V3& p = m->pos[i];
        const double u = uw[2 * i], w = uw[2 * i + 1];
        const double phi = 2.0 * kPI * u, theta = std::acos(2.0 * w - 1);
        V3 sp = v3(1.0 * std::sin(theta) * std::cos(phi), 1.0 * std::sin(theta) * std::sin(phi), 1.0 * std::cos(theta));
        const double s = dot(sp, p) / dot(p, p);
        sp = sub(sp, scale(s, p));
        sp = scale(1.0 / norm(sp), sp);
        V3 nd = m->dir[i];
        int cnt = 3;
        for (int jj = 0; jj < cnt; ++jj) nd = add(nd, m->dir[m->vn[3 * i + jj]]);
        cnt += 1;
        const double mi = 1.0 / cnt;
        nd = add(scale(mi, nd), scale(eta, sp));
        projectNormalize(nd, p);
        target[i] = nd;
    }
    for (int i = 0; i < m->N; ++i) {
        const V3& p = m->pos[i];
        V3 n = add(m->dir[i], scale(dt / tau, sub(target[i], m->dir[i])));
        const double s = dot(n, p) / dot(p, p);
        n = sub(n, scale(s, p));
        m->dir[i] = scale(1.0 / norm(n), n);
    }
}
// Uniform draws getRealUniform(lo, hi) (noiseSource.cpp:18-27), count of them.
void orc_noise_uniforms(orc_noise* nz, double lo, double hi, double* out, long count) {
    for (long i = 0; i < count; ++i) out[i] = orc_noise_uniform(nz, lo, hi);
}

// ---- dynamicalFeatures (src/analysis/dynamicalFeatures.cpp:6-53) --------------------------
// computeMSD and computeOverlapFunction over the first floor(n fraction) points (all when
// fraction >= 1), in index order; NaN distances are skipped by the MSD (the reference prints them).
void orc_dynamics(const double* init, const double* cur, int n, double fraction, double radius, double cutoff,
                  double* msdOut, double* overlapOut) {
    Sphere s; s.radius = radius;
    int N = n;
    if (fraction < 1) N = (int)std::floor(N * fraction);
    double msd = 0.0, overlap = 0.0;
    for (int i = 0; i < N; ++i) {
        V3 a = v3(init[3 * i], init[3 * i + 1], init[3 * i + 2]), b = v3(cur[3 * i], cur[3 * i + 1], cur[3 * i + 2]);
        double d = s.geodesic(a, b);
        if (!std::isnan(d)) msd += d * d;
        if (d < cutoff) overlap += 1;
    }
    *msdOut = msd / N;
    *overlapOut = overlap / N;
}

// ---- logSpacedIntegers (inc/simpleUtilities.h:5-41) ---------------------------------------
// The first `count` save steps: the constructor's nextSave, then nextSave after each update().
void orc_log_spaced(int firstSave, double exponent, int count, int* out) {
    int nextSave = firstSave, logSaveIdx = 0;
    const double base = std::pow(10.0, exponent);
    if (nextSave != 0) {
        int tempCur = 0;
        while (tempCur < nextSave) { logSaveIdx += 1; tempCur = (int)std::round(std::pow(base, logSaveIdx)); }
    }
    for (int i = 0; i < count; ++i) {
        out[i] = nextSave;
        logSaveIdx += 1;
        int curSave = (int)std::round(std::pow(base, logSaveIdx));
        while (curSave == nextSave) { logSaveIdx += 1; curSave = (int)std::round(std::pow(base, logSaveIdx)); }
        nextSave = curSave;
    }
}

// ---- FIRE (src/updaters/energyMinimizerFIRE.cpp, velocityVerlet.cpp) ----------------------
struct orc_fire {
    double deltaT = 0.01, deltaTMin = 0.0001, deltaTMax = 0.1, deltaTInc = 1.05, deltaTDec = 0.95;
    double alpha = 0.99, alphaStart = 0.99, alphaDec = 0.9, alphaMin = 0.0;
    double forceCutoff = 1e-7, forceMax = 100., Power = 0, maxAbsForce = 0;
    int NMin = 5, NSince = 0, iterations = 0, maxIterations = 1000;
};
// initializeParameters defaults (energyMinimizerFIRE.cpp:22-41) then setFIREParameters (203-214)
orc_fire* orc_fire_create(double dt, double alphaStart, double dtMax, double dtInc, double dtDec,
                          double alphaDec, int nMin, double forceCutoff, double alphaMin, int maxIt) {
    orc_fire* f = new orc_fire();
    f->deltaT = dt; f->deltaTMin = dt * .01;
    f->alphaStart = alphaStart; f->alpha = alphaStart;
    f->deltaTMax = dtMax; f->deltaTInc = dtInc; f->deltaTDec = dtDec; f->alphaDec = alphaDec;
    f->NMin = nMin; f->forceCutoff = forceCutoff; f->alphaMin = alphaMin; f->maxIterations = maxIt;
    return f;
}
void orc_fire_destroy(orc_fire* f) { delete f; }

// velocityVerlet::integrateEOMCPU (velocityVerlet.cpp:6-38)
static void vvStep(orc_model* m, double dt) {
    std::vector<double> disp(3 * (size_t)m->N);
    for (int i = 0; i < m->N; ++i) {
        double hv = (0.5 / m->mass[i]) * dt;
        double h2 = 0.5 * dt * dt;
        for (int d = 0; d < 3; ++d) {
            disp[3 * i + d] = dt * m->vel[i].x[d] + h2 * m->forces[i].x[d];
            m->vel[i].x[d] += hv * m->forces[i].x[d];
        }
    }
    orc_move(m, disp.data(), 1.0);
    orc_compute_forces(m);
    for (int i = 0; i < m->N; ++i) {
        double hv = (0.5 / m->mass[i]) * dt;
        for (int d = 0; d < 3; ++d) m->vel[i].x[d] += hv * m->forces[i].x[d];
    }
}

// fireStepCPU (energyMinimizerFIRE.cpp:122-174); also records max_i |F_i|.
static void fireStep(orc_model* m, orc_fire* f) {
    f->Power = 0.0;
    double forceNorm = 0.0, velocityNorm = 0.0, maxF2 = 0.0;
    for (int i = 0; i < m->N; ++i) {
        f->Power += dot(m->forces[i], m->vel[i]);
        double fdot = dot(m->forces[i], m->forces[i]);
        forceNorm += fdot;
        velocityNorm += dot(m->vel[i], m->vel[i]);
        if (fdot > maxF2) maxF2 = fdot;
    }
    f->forceMax = std::sqrt(forceNorm) / (double)m->N;
    f->maxAbsForce = std::sqrt(maxF2);
    double s = 0.0;
    if (forceNorm > 0.) s = std::sqrt(velocityNorm / forceNorm);
    double a1 = 1.0 - f->alpha, as = f->alpha * s;
    for (int i = 0; i < m->N; ++i)
        for (int d = 0; d < 3; ++d) m->vel[i].x[d] = a1 * m->vel[i].x[d] + as * m->forces[i].x[d];
    if (f->Power > 0) {
        if (f->NSince > f->NMin) {
            f->deltaT = std::min(f->deltaT * f->deltaTInc, f->deltaTMax);
            f->alpha = f->alpha * f->alphaDec;
            f->alpha = std::max(f->alpha, f->alphaMin);
        }
        f->NSince += 1;
    } else {
        f->NSince = 0;
        f->deltaT = f->deltaT * f->deltaTDec;
        f->deltaT = std::max(f->deltaT, f->deltaTMin);
        f->alpha = f->alphaStart;
        for (int i = 0; i < m->N; ++i) m->vel[i] = v3(0.0, 0.0, 0.0);
    }
}

// minimize (energyMinimizerFIRE.cpp:180-200).  criterion 0: the reference's
// sqrt(sum F^2)/N; criterion 1: max_i |F_i|.  Returns iterations done in this call.
int orc_fire_minimize(orc_model* m, orc_fire* f, int criterion) {
    orc_compute_forces(m);
    f->forceMax = 110.0;
    f->maxAbsForce = 110.0;
    int done = 0;
    while (f->iterations < f->maxIterations &&
           (criterion == 0 ? f->forceMax : f->maxAbsForce) > f->forceCutoff) {
        f->iterations += 1;
        vvStep(m, f->deltaT);
        fireStep(m, f);
        done += 1;
    }
    return done;
}
// The pieces of an iteration on their own: velocityVerlet::integrateEOMCPU at dt, and fireStepCPU.
void orc_vv_step(orc_model* m, double dt) { vvStep(m, dt); }
void orc_fire_step(orc_model* m, orc_fire* f) { fireStep(m, f); }
// One VV + FIRE iteration without the stopping test (forces must be current).
void orc_fire_iterate(orc_model* m, orc_fire* f, int count) {
    for (int k = 0; k < count; ++k) { f->iterations += 1; vvStep(m, f->deltaT); fireStep(m, f); }
}
void orc_fire_state(orc_fire* f, double* out) {
    out[0] = f->deltaT; out[1] = f->alpha; out[2] = f->Power; out[3] = f->forceMax;
    out[4] = f->maxAbsForce; out[5] = (double)f->NSince; out[6] = (double)f->iterations;
}

// ---- hyperrectangularCellList (src/utilities/hyperrectangularCellList.cpp) --------------------
// setGridSize (27-51) and computeCPU (165-214).  `nmaxInOut` carries Nmax across calls as the
// class member does.  Outputs: per-point bin, per-bin counts [nside^3], slot table
// [nside^3 * Nmax] (index bin*Nmax + slot, -1 where empty).
int orc_cell_list_dims(double a, double radius, int* nsideOut, double* hOut) {
    double b = 2. * radius;
    unsigned n = (unsigned)std::floor(b / a);
    if (n % 2 == 1) n -= 1;
    *nsideOut = (int)n;
    *hOut = b / n;
    return 0;
}
int orc_cell_list(const double* pts, int np, double a, double radius, int* nmaxInOut,
                  int* binOut, unsigned* countsOut, int* idxOut, long idxCapacity) {
    int nside; double h;
    orc_cell_list_dims(a, radius, &nside, &h);
    long total = (long)nside * nside * nside;
    int Nmax = *nmaxInOut;
    bool recompute = true;
    std::vector<unsigned> counts;
    std::vector<int> idx;
    while (recompute) {
        recompute = false;
        counts.assign(total, 0u);
        idx.assign((size_t)total * Nmax, 0);
        for (int nn = 0; nn < np; ++nn) {
            int b[3];
            for (int d = 0; d < 3; ++d) b[d] = (int)std::floor((pts[3 * nn + d] + radius) / h);
            long bin = b[0] + (long)b[1] * nside + (long)b[2] * nside * nside;
            binOut[nn] = (int)bin;
            int off = (int)counts[bin];
            if (off < Nmax && !recompute) idx[(size_t)bin * Nmax + off] = nn;
            else { Nmax = std::max(Nmax, off + 1); recompute = true; }
            counts[bin]++;
        }
    }
    *nmaxInOut = Nmax;
    std::memcpy(countsOut, counts.data(), sizeof(unsigned) * total);
    if ((long)total * Nmax > idxCapacity) return -1;
    for (long bin = 0; bin < total; ++bin)
        for (int s = 0; s < Nmax; ++s)
            idxOut[bin * Nmax + s] = s < (int)counts[bin] ? idx[(size_t)bin * Nmax + s] : -1;
    return 0;
}

// neighborList (src/utilities/neighborList.cpp:6-18, 96-151): a cell list of grid size
// range / subGridReduction over [-radius, radius]^3, adjacent cells within `width` =
// subGridReduction (computeAdjacentCells, hyperrectangularCellList.cpp:219-262: the offsets in
// iVecIterate order, x fastest, kept if the nearest corner is within width cells, wrapped
// periodically), then per point, in cell-list slot order, every other point at minimum-image
// distance (periodic box of side 2 radius, periodicBoundaryConditions.h:124-132) below `range`.
// Nmax starts at 4 and grows to the largest count.  Outputs [Np] counts and [Np * Nmax] index,
// displacement (3 doubles) and distance, zero past each count; returns Nmax.
int orc_neighbor_list(const double* pts, int np, double range, double radius, int subGrid, int nmaxIn,
                      unsigned* nppOut, int* idxOut, double* vecOut, double* distOut, long capacity) {
    int nside; double h;
    const double a = range * (1. / (double)subGrid);
    orc_cell_list_dims(a, radius, &nside, &h);
    const long total = (long)nside * nside * nside;
    int cellNmax = 2;  // the cell list's own width, grown by its first pass
    std::vector<int> bins(np);
    std::vector<unsigned> counts(total);
    orc_cell_list(pts, np, a, radius, &cellNmax, bins.data(), counts.data(), nullptr, 0);
    std::vector<int> slots((size_t)total * cellNmax, -1);
    orc_cell_list(pts, np, a, radius, &cellNmax, bins.data(), counts.data(), slots.data(), (long)total * cellNmax);
    const int width = subGrid;
    std::vector<int> mask;
    for (int z = -width; z <= width; ++z)
        for (int y = -width; y <= width; ++y)
            for (int x = -width; x <= width; ++x) {
                const int g[3] = {x, y, z};
                double rmin = 0.0;
                for (int d = 0; d < 3; ++d) {
                    double t = h * (std::max(std::abs(g[d]) - 1., 0.0));
                    rmin += t * t;
                }
                rmin = std::sqrt(rmin);
                if (rmin < h * width + 1e-6) { mask.push_back(x); mask.push_back(y); mask.push_back(z); }
            }
    const int K = (int)mask.size() / 3;
    int Nmax = nmaxIn;
    bool recompute = true;
    std::vector<unsigned> npp;
    std::vector<int> idx;
    std::vector<double> vec, dist;
    while (recompute) {
        recompute = false;
        npp.assign(np, 0u);
        idx.assign((size_t)np * Nmax, 0);
        vec.assign((size_t)np * Nmax * 3, 0.0);
        dist.assign((size_t)np * Nmax, 0.0);
        int nmax = Nmax;
        for (int pp = 0; pp < np; ++pp) {
            const double* t = pts + 3 * pp;
            int c[3];
            for (int d = 0; d < 3; ++d) c[d] = std::max(0, std::min(nside - 1, (int)std::floor((t[d] + radius) / h)));
            for (int cc = 0; cc < K; ++cc) {
                int nb[3];
                for (int d = 0; d < 3; ++d) {
                    nb[d] = (c[d] + mask[3 * cc + d]) % nside;
                    if (nb[d] < 0) nb[d] += nside;
                }
                const long cell = nb[0] + (long)nb[1] * nside + (long)nb[2] * nside * nside;
                for (unsigned p1 = 0; p1 < counts[cell]; ++p1) {
                    const int j = slots[(size_t)cell * cellNmax + p1];
                    if (j == pp) continue;
                    double disp[3];
                    for (int d = 0; d < 3; ++d) {
                        disp[d] = t[d] - pts[3 * j + d];
                        while (disp[d] < -radius) disp[d] += 2. * radius;
                        while (disp[d] > radius) disp[d] -= 2. * radius;
                    }
                    double dd = 0.0;
                    dd += disp[0] * disp[0]; dd += disp[1] * disp[1]; dd += disp[2] * disp[2];
                    const double r = std::sqrt(dd);
                    if (r >= range) continue;
                    const int off = (int)npp[pp];
                    if (off < Nmax && !recompute) {
                        const size_t at = (size_t)pp * Nmax + off;
                        idx[at] = j;
                        for (int d = 0; d < 3; ++d) vec[3 * at + d] = disp[d];
                        dist[at] = r;
                    } else {
                        nmax = std::max(nmax, off + 1);
                        Nmax = nmax;
                        recompute = true;
                    }
                    npp[pp] += 1;
                }
            }
        }
    }
    if ((long)np * Nmax > capacity) return -Nmax;
    std::memcpy(nppOut, npp.data(), sizeof(unsigned) * np);
    std::memcpy(idxOut, idx.data(), sizeof(int) * idx.size());
    std::memcpy(vecOut, vec.data(), sizeof(double) * vec.size());
    std::memcpy(distOut, dist.data(), sizeof(double) * dist.size());
    return Nmax;
}

}  // extern "C"
