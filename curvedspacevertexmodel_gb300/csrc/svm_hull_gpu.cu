// The initial topology on the device: the convex hull of the cell centres (a spherical Delaunay
// triangulation) and the vertex-model arrays built from it, with the contract of svm_hull.h
// (convexHullCGAL.cpp:82-186: one vertex per facet at the normalised centroid, CCW facet corners,
// neighbours across facet edges, clockwise rings) and the same canonical numbering, so the result
// equals svm_topology_from_points array for array.
//
// A hull built point by point instead of by incremental insertion:
//   k_hull_star   a thread per centre p.  Candidates are the centres in the bins within w of p's
//                 bin (a ball of radius w h around p lies inside them).  The nearest candidate q0
//                 spans a hull edge (for points on a sphere, the plane through p and q0 with
//                 normal p + q0 has every other point strictly below it).  Gift wrapping around p
//                 from the edge p -> q0: the next corner s of edge p -> q is the candidate that no
//                 other candidate lies above, i.e. the last one to win "orient(p, q, s, x) > 0",
//                 until the wrap returns to q0.  Each triangle of the star is then certified: its
//                 circumcircle's cap (the part of the sphere above its plane, smaller than a
//                 hemisphere) lies within 2 rho of p, rho the triangle's circumradius, so when
//                 2 rho < w h every point that could lie in the cap was a candidate and the
//                 triangle is a hull facet.  A star with an uncertified triangle is computed
//                 again with w + 1 (in a second launch over the centres that need it).  A closed
//                 cycle of hull facets around p is p's whole star.
//   k_hull_check  every triangle of a star appears, rotated, in the stars of its other two corners
//                 (the stars form one triangulated sphere), and counts the triangles whose
//                 smallest corner is the star's own point.
//   (scan)        facet offsets: the facets of the smallest corner a are numbered in (b, c) order
//                 after those of smaller a -- the lexicographic order of the host builder.
//   k_hull_emit   writes each point's facets (a, b, c), sorted by (b, c).
//   k_hull_vertex per facet: position (radius / |c|) c with c = (p_a + p_b + p_c) / 3 summed and
//                 scaled as convexHullCGAL.cpp:118-127, cells, and the facets across its edges.
//   k_hull_ring   per cell: its facets clockwise from the lowest-numbered one.
// The orientation test is the host hull's: the FP64 determinant with a relative filter, and a
// double-double evaluation where the filter cannot decide (the host uses long double there).
#include <algorithm>
#include <cmath>
#include <vector>
#include "svm_internal.cuh"
#include "svm_hull.h"

using namespace svm;

namespace {
constexpr int kHB = 128;          // threads per block of the star kernel (local candidate arrays)
constexpr int kMaxCand = 512;     // candidates a star may draw on
constexpr int kMaxDeg = 32;       // facets around one centre
constexpr int kMaxW = 4;          // widest search, in bins
constexpr int kB = 256;

struct DD { double hi, lo; };

__device__ __forceinline__ DD two_sum(double a, double b) {
    const double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DD quick_two_sum(double a, double b) {
    const double s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
    const DD s = two_sum(a.hi, b.hi);
    return quick_two_sum(s.hi, s.lo + a.lo + b.lo);
}
__device__ __forceinline__ DD dd_neg(DD a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ DD dd_mul(DD a, DD b) {
    const double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e += a.hi * b.lo + a.lo * b.hi;
    return quick_two_sum(p, e);
}
__device__ __forceinline__ DD dd_diff(double a, double b) { return two_sum(a, -b); }  // a - b, exactly

__device__ double orient_dd(const double* A, const double* B, const double* C, const double* D) {
    DD b[3], c[3], d[3];
    for (int k = 0; k < 3; ++k) { b[k] = dd_diff(B[k], A[k]); c[k] = dd_diff(C[k], A[k]); d[k] = dd_diff(D[k], A[k]); }
    const DD nx = dd_add(dd_mul(b[1], c[2]), dd_neg(dd_mul(b[2], c[1])));
    const DD ny = dd_add(dd_mul(b[2], c[0]), dd_neg(dd_mul(b[0], c[2])));
    const DD nz = dd_add(dd_mul(b[0], c[1]), dd_neg(dd_mul(b[1], c[0])));
    const DD det = dd_add(dd_add(dd_mul(nx, d[0]), dd_mul(ny, d[1])), dd_mul(nz, d[2]));
    return det.hi + det.lo;
}

// Positive when D lies on the side the normal (B - A) x (C - A) points to; the FP64 value and
// filter of the host hull's orient.
__device__ double orient(const double* A, const double* B, const double* C, const double* D) {
    const double bx = B[0] - A[0], by = B[1] - A[1], bz = B[2] - A[2];
    const double cx = C[0] - A[0], cy = C[1] - A[1], cz = C[2] - A[2];
    const double dx = D[0] - A[0], dy = D[1] - A[1], dz = D[2] - A[2];
    const double nx = by * cz - bz * cy, ny = bz * cx - bx * cz, nz = bx * cy - by * cx;
    const double det = nx * dx + ny * dy + nz * dz;
    const double perm = (fabs(by * cz) + fabs(bz * cy)) * fabs(dx) + (fabs(bz * cx) + fabs(bx * cz)) * fabs(dy) +
                        (fabs(bx * cy) + fabs(by * cx)) * fabs(dz);
    if (fabs(det) > 1e-13 * perm) return det;
    return orient_dd(A, B, C, D);
}

__device__ __forceinline__ void load3(const double* P, int i, double* o) {
    o[0] = P[3 * i]; o[1] = P[3 * i + 1]; o[2] = P[3 * i + 2];
}

// The cap above the plane of (p, q, s) lies within `reach` of p.
__device__ bool cap_within(const double* p, const double* q, const double* s, double reach) {
    double a[3], b[3], ab[3];
    for (int k = 0; k < 3; ++k) { a[k] = q[k] - p[k]; b[k] = s[k] - p[k]; ab[k] = a[k] - b[k]; }
    const double nx = a[1] * b[2] - a[2] * b[1], ny = a[2] * b[0] - a[0] * b[2], nz = a[0] * b[1] - a[1] * b[0];
    if (nx * p[0] + ny * p[1] + nz * p[2] <= 0.0) return false;  // cap not smaller than a hemisphere
    const double la = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    const double lb = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    const double lab = sqrt(ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]);
    const double ln = sqrt(nx * nx + ny * ny + nz * nz);
    const double diameter = la * lb * lab / ln;  // twice the circumradius
    return diameter * (1.0 + 1e-9) < reach;
}

// The plane of (p, q, s) for the pivot's FP32 sign test: n = b x c with b = q - p, c = s - p in
// FP32, and the coefficients of the filter's permanent (|b1 c2| + |b2 c1|, ...).
struct Plane32 { float n[3], k[3]; };
__device__ __forceinline__ Plane32 plane32(const float* b, const float* c) {
    Plane32 t;
    t.n[0] = b[1] * c[2] - b[2] * c[1]; t.n[1] = b[2] * c[0] - b[0] * c[2]; t.n[2] = b[0] * c[1] - b[1] * c[0];
    t.k[0] = fabsf(b[1] * c[2]) + fabsf(b[2] * c[1]);
    t.k[1] = fabsf(b[2] * c[0]) + fabsf(b[0] * c[2]);
    t.k[2] = fabsf(b[0] * c[1]) + fabsf(b[1] * c[0]);
    return t;
}

// Centres list[0..count) (all centres when list is null) with searches of wFirst..wLast bins.  A
// centre whose stars all fail certification in that range is queued in retry (when given) for a
// second launch with the wider searches, so that warps of the first launch do not wait on them.
__global__ void __launch_bounds__(kHB) k_hull_star(const double* __restrict__ P, const int* __restrict__ list,
                                                  int count, int wFirst, int wLast, CellGrid g,
                                                  int* __restrict__ deg, int* __restrict__ star,
                                                  int* __restrict__ retry, int* __restrict__ retryCount,
                                                  int* __restrict__ err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int p = list ? list[t] : t;
    // candidates and their offsets from p, fl32(x - p) of the FP64 difference (relative error
    // within 2^-24 (1 + 2^-29) per component)
    int cand[kMaxCand];
    float dv[kMaxCand][3];
    int st[kMaxDeg];
    double pp[3];
    load3(P, p, pp);
    int c[3];
    for (int d = 0; d < 3; ++d) c[d] = max(0, min(g.nside - 1, (int)floor((pp[d] + g.radius) / g.h)));
    bool hard = false;  // a failure no wider search can repair
    for (int w = wFirst; w <= wLast; ++w) {
        int lo[3], hi[3];
        bool whole = true;
        for (int d = 0; d < 3; ++d) {
            lo[d] = max(0, c[d] - w); hi[d] = min(g.nside - 1, c[d] + w);
            whole &= lo[d] == 0 && hi[d] == g.nside - 1;
        }
        int nc = 0, iq0 = -1;
        bool overflow = false;
        float b1 = INFINITY, b2 = INFINITY;
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    const long cell = x + (long)y * g.nside + (long)z * g.nside * g.nside;
                    const int m = min((int)g.counts[cell], g.cap);
                    for (int k = 0; k < m; ++k) {
                        const int j = g.slots[cell * g.cap + k];
                        if (j == p) continue;
                        if (nc >= kMaxCand) { overflow = true; continue; }
                        double xx[3];
                        load3(P, j, xx);
                        cand[nc] = j;
                        dv[nc][0] = (float)(xx[0] - pp[0]);
                        dv[nc][1] = (float)(xx[1] - pp[1]);
                        dv[nc][2] = (float)(xx[2] - pp[2]);
                        // the nearest in FP32 (squared length within 5 2^-24 relative of the exact one)
                        const float d2 = dv[nc][0] * dv[nc][0] + dv[nc][1] * dv[nc][1] + dv[nc][2] * dv[nc][2];
                        if (d2 < b1) { b2 = b1; b1 = d2; iq0 = nc; }
                        else if (d2 < b2) b2 = d2;
                        ++nc;
                    }
                }
        if (overflow) { hard = true; break; }
        if (nc < 3) { if (whole) { hard = true; break; } continue; }
        if (!(b2 > b1 * (1.0f + 1e-5f))) {  // a near tie: the FP64 squared lengths, lowest index on ties
            double best = 0.0;
            iq0 = -1;
            for (int i = 0; i < nc; ++i) {
                double xx[3];
                load3(P, cand[i], xx);
                const double dx = xx[0] - pp[0], dy = xx[1] - pp[1], dz = xx[2] - pp[2];
                const double d2 = dx * dx + dy * dy + dz * dz;
                if (iq0 < 0 || d2 < best || (d2 == best && cand[i] < cand[iq0])) { best = d2; iq0 = i; }
            }
        }
        // gift wrapping around p from the edge to the nearest candidate.  The pivot's sign test
        // runs in FP32 with the plane hoisted out of the candidate loop: with every input within
        // 2^-24 relative, |det32 - det| <= 8 2^-24 perm, so |det32| > 1e-5 perm32 fixes the sign;
        // anything closer (or so small that FP32 could underflow) takes the FP64 test.
        int d = 0, iq = iq0;
        bool ok = true;
        do {
            if (d >= kMaxDeg) { ok = false; break; }
            st[d++] = cand[iq];
            const float b[3] = {dv[iq][0], dv[iq][1], dv[iq][2]};
            int is = -1;
            Plane32 pl;
            for (int i = 0; i < nc; ++i) {
                if (i == iq) continue;
                if (is < 0) { is = i; pl = plane32(b, dv[i]); continue; }
                const float det = pl.n[0] * dv[i][0] + pl.n[1] * dv[i][1] + pl.n[2] * dv[i][2];
                const float perm = pl.k[0] * fabsf(dv[i][0]) + pl.k[1] * fabsf(dv[i][1]) + pl.k[2] * fabsf(dv[i][2]);
                bool above;
                if (perm > 1e-30f && fabsf(det) > 1e-5f * perm) {
                    above = det > 0.f;
                } else {
                    double qq[3], ss[3], xx[3];
                    load3(P, cand[iq], qq); load3(P, cand[is], ss); load3(P, cand[i], xx);
                    above = orient(pp, qq, ss, xx) > 0.0;
                }
                if (above) { is = i; pl = plane32(b, dv[i]); }
            }
            if (is < 0) { ok = false; break; }
            iq = is;
        } while (iq != iq0);
        if (ok && d < 3) ok = false;
        if (ok && !whole) {
            const double reach = w * g.h;
            for (int i = 0; i < d && ok; ++i) {
                double a[3], b[3];
                load3(P, st[i], a);
                load3(P, st[(i + 1) % d], b);
                ok = cap_within(pp, a, b, reach);
            }
        }
        if (ok) {
            deg[p] = d;
            for (int i = 0; i < d; ++i) star[(long)p * kMaxDeg + i] = st[i];
            return;
        }
        if (whole) { hard = true; break; }
    }
    deg[p] = 0;
    if (retry && !hard) { retry[atomicAdd(retryCount, 1)] = p; return; }
    atomicOr(err, 1);
}

__device__ __forceinline__ int star_next(const int* star, const int* deg, int a, int b) {
    // in a's star, the corner after b (-1 if b is not a neighbour of a)
    const int da = deg[a];
    const int* s = star + (long)a * kMaxDeg;
    for (int i = 0; i < da; ++i)
        if (s[i] == b) return s[i + 1 < da ? i + 1 : 0];
    return -1;
}

__global__ void k_hull_check(const int* __restrict__ star, const int* __restrict__ deg, int n,
                             int* __restrict__ own, int* __restrict__ err) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int d = deg[p];
    const int* s = star + (long)p * kMaxDeg;
    int count = 0;
    bool ok = d >= 3;
    for (int i = 0; i < d && ok; ++i) {
        const int a = s[i], b = s[i + 1 < d ? i + 1 : 0];
        ok = star_next(star, deg, a, b) == p && star_next(star, deg, b, p) == a;
        count += p < a && p < b;
    }
    own[p] = count;
    if (!ok) atomicOr(err, 2);
}

__global__ void k_hull_emit(const int* __restrict__ star, const int* __restrict__ deg, int n,
                            const int* __restrict__ off, int* __restrict__ F) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int d = deg[p];
    const int* s = star + (long)p * kMaxDeg;
    int b[kMaxDeg], c[kMaxDeg], m = 0;
    for (int i = 0; i < d; ++i) {
        const int u = s[i], v = s[i + 1 < d ? i + 1 : 0];
        if (p < u && p < v) {
            int k = m++;
            while (k > 0 && (b[k - 1] > u || (b[k - 1] == u && c[k - 1] > v))) { b[k] = b[k - 1]; c[k] = c[k - 1]; --k; }
            b[k] = u; c[k] = v;
        }
    }
    const int o = off[p];
    for (int k = 0; k < m; ++k) { F[3 * (o + k)] = p; F[3 * (o + k) + 1] = b[k]; F[3 * (o + k) + 2] = c[k]; }
}

// Index of the facet with corners u, v, w (CCW), in canonical numbering.
__device__ int facet_of(int u, int v, int w, const int* off, const int* F) {
    int a = u, b = v, c = w;
    if (v < u && v < w) { a = v; b = w; c = u; }
    else if (w < u && w < v) { a = w; b = u; c = v; }
    for (int k = off[a]; k < off[a + 1]; ++k)
        if (F[3 * k + 1] == b && F[3 * k + 2] == c) return k;
    return -1;
}

__global__ void k_hull_vertex(const double* __restrict__ P, const int* __restrict__ F, int nf,
                              const int* __restrict__ off, const int* __restrict__ star, const int* __restrict__ deg,
                              double radius, double* __restrict__ vpos, int* __restrict__ vcells,
                              int* __restrict__ vnbrs, int* __restrict__ err) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int t[3] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]};
    double c[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k)
        for (int d = 0; d < 3; ++d) c[d] += P[3 * t[k] + d];
    for (int d = 0; d < 3; ++d) c[d] = (1.0 / 3.0) * c[d];
    const double nrm = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    for (int d = 0; d < 3; ++d) vpos[3 * (long)f + d] = (radius / nrm) * c[d];
    for (int k = 0; k < 3; ++k) {
        vcells[3 * (long)f + k] = t[k];
        const int from = t[(k + 2) % 3], to = t[k];  // the facet across the edge ending at corner k
        const int x = star_next(star, deg, to, from);
        const int gidx = x < 0 ? -1 : facet_of(to, from, x, off, F);
        if (gidx < 0) atomicOr(err, 4);
        vnbrs[3 * (long)f + k] = gidx;
    }
}

__global__ void k_hull_ring(const int* __restrict__ star, const int* __restrict__ deg, int n,
                            const int* __restrict__ off, const int* __restrict__ F,
                            const int* __restrict__ ringOff, int* __restrict__ ring, int* __restrict__ err) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const int d = deg[x];
    const int* s = star + (long)x * kMaxDeg;
    int gi[kMaxDeg];
    int start = 0;
    for (int i = 0; i < d; ++i) {
        gi[i] = facet_of(x, s[i], s[i + 1 < d ? i + 1 : 0], off, F);
        if (gi[i] < 0) atomicOr(err, 8);
        if (gi[i] < gi[start]) start = i;
    }
    const int o = ringOff[x];
    for (int j = 0; j < d; ++j) ring[o + j] = gi[(start - j + d) % d];  // clockwise: decreasing i
}

// Exclusive scan of n ints in place; a block scans 2 kB entries, the block totals are scanned the
// same way, then added back.
__global__ void k_scan_block(int* a, int n, int* sums) {
    __shared__ int sh[2 * kB];
    const int base = blockIdx.x * 2 * kB;
    const int i0 = base + threadIdx.x, i1 = base + kB + threadIdx.x;
    sh[threadIdx.x] = i0 < n ? a[i0] : 0;
    sh[kB + threadIdx.x] = i1 < n ? a[i1] : 0;
    __syncthreads();
    for (int o = 1; o < 2 * kB; o <<= 1) {  // Hillis-Steele over the block's 2 kB entries
        int v0 = 0, v1 = 0;
        if (threadIdx.x >= o) v0 = sh[threadIdx.x - o];
        if (kB + threadIdx.x >= o) v1 = sh[kB + threadIdx.x - o];
        __syncthreads();
        sh[threadIdx.x] += v0;
        sh[kB + threadIdx.x] += v1;
        __syncthreads();
    }
    const int e0 = threadIdx.x == 0 ? 0 : sh[threadIdx.x - 1];
    const int e1 = sh[kB + threadIdx.x - 1];
    if (i0 < n) a[i0] = e0;
    if (i1 < n) a[i1] = e1;
    if (threadIdx.x == 0) sums[blockIdx.x] = sh[2 * kB - 1];
}
__global__ void k_scan_add(int* a, int n, const int* sums) {
    const int i = blockIdx.x * 2 * kB + threadIdx.x;
    const int add = sums[blockIdx.x];
    if (i < n) a[i] += add;
    if (i + kB < n) a[i + kB] += add;
}

int exclusive_scan(int* a, int n, cudaStream_t s, int* total) {
    const int nb = (n + 2 * kB - 1) / (2 * kB);
    int* sums = nullptr;
    if (cudaMalloc(&sums, sizeof(int) * (nb + 1)) != cudaSuccess) return SVM_ERR_CUDA;
    k_scan_block<<<nb, kB, 0, s>>>(a, n, sums);
    int rc = check_launch();
    if (!rc && nb > 1) rc = exclusive_scan(sums, nb, s, nullptr);
    else if (!rc) rc = cudaMemsetAsync(sums, 0, sizeof(int), s) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
    if (!rc) { k_scan_add<<<nb, kB, 0, s>>>(a, n, sums); rc = check_launch(); }
    if (!rc && total) {  // callers end the array with a zero, so its last entry is the sum
        rc = cudaMemcpyAsync(total, a + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) rc = SVM_ERR_CUDA;
    cudaFree(sums);
    return rc;
}

struct DevBuf {
    std::vector<void*> ptrs;
    template <typename T> T* get(size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T*)p;
    }
    ~DevBuf() { for (void* p : ptrs) cudaFree(p); }
};
}  // namespace

extern "C" int svm_topology_from_points_gpu(const double* pts, int n, void* stream, svm_topology** out) {
    if (!pts || n < 4 || !out) return SVM_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf buf;
    double* P = buf.get<double>(3 * (size_t)n);
    int* deg = buf.get<int>(n);
    int* star = buf.get<int>((size_t)n * kMaxDeg);
    int* own = buf.get<int>((size_t)n + 1);
    int* err = buf.get<int>(2);          // [0] error bits, [1] centres queued for the wider search
    int* retry = buf.get<int>(n);
    if (!P || !deg || !star || !own || !err || !retry) return SVM_ERR_CUDA;
    if (cudaMemcpyAsync(P, pts, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(err, 0, 2 * sizeof(int), s) != cudaSuccess || cudaMemsetAsync(own + n, 0, sizeof(int), s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)  // the cell list bins on a stream of its own
        return SVM_ERR_CUDA;
    // bins of side 2.5 mean spacings (a unit-density sphere has ~70 candidates at w = 1)
    double rmax = 0.0;
    for (int i = 0; i < n; ++i)
        rmax = std::max(rmax, std::sqrt(pts[3 * i] * pts[3 * i] + pts[3 * i + 1] * pts[3 * i + 1] + pts[3 * i + 2] * pts[3 * i + 2]));
    const double gridR = rmax * (1.0 + 1e-6) + 1e-3;
    const double spacing = std::sqrt(4.0 * 3.141592653589793 * rmax * rmax / n);
    const double a = std::min(2.5 * spacing, gridR);
    svm_cell_list* cl = nullptr;
    int rc = svm_cell_list_create(a, gridR, n, 32, stream, &cl);
    if (rc) return rc;
    CellGrid g;
    rc = cell_list_bin(cl, P, n, &g);
    if (!rc) {
        k_hull_star<<<(n + kHB - 1) / kHB, kHB, 0, s>>>(P, nullptr, n, 1, 1, g, deg, star, retry, err + 1, err);
        rc = check_launch();
    }
    int nRetry = 0;
    if (!rc) rc = (cudaMemcpyAsync(&nRetry, err + 1, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                   cudaStreamSynchronize(s) == cudaSuccess) ? SVM_OK : SVM_ERR_CUDA;
    if (!rc && nRetry > 0) {
        k_hull_star<<<(nRetry + kHB - 1) / kHB, kHB, 0, s>>>(P, retry, nRetry, 2, kMaxW, g, deg, star, nullptr,
                                                            nullptr, err);
        rc = check_launch();
    }
    if (!rc) {
        k_hull_check<<<(n + kB - 1) / kB, kB, 0, s>>>(star, deg, n, own, err);
        rc = check_launch();
    }
    int nf = 0, e = 0;
    if (!rc) rc = exclusive_scan(own, n + 1, s, &nf);
    if (!rc) rc = (cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                   cudaStreamSynchronize(s) == cudaSuccess) ? SVM_OK : SVM_ERR_CUDA;
    svm_cell_list_destroy(cl);
    if (rc) return rc;
    if (e || nf != 2 * n - 4) return SVM_ERR_HULL;
    int* F = buf.get<int>(3 * (size_t)nf);
    double* vpos = buf.get<double>(3 * (size_t)nf);
    int* vcells = buf.get<int>(3 * (size_t)nf);
    int* vnbrs = buf.get<int>(3 * (size_t)nf);
    int* ringOff = buf.get<int>((size_t)n + 1);
    int* ring = buf.get<int>(3 * (size_t)nf);
    if (!F || !vpos || !vcells || !vnbrs || !ringOff || !ring) return SVM_ERR_CUDA;
    const double radius = std::sqrt(pts[0] * pts[0] + pts[1] * pts[1] + pts[2] * pts[2]);
    k_hull_emit<<<(n + kB - 1) / kB, kB, 0, s>>>(star, deg, n, own, F);
    if (check_launch()) return SVM_ERR_CUDA;
    k_hull_vertex<<<(nf + kB - 1) / kB, kB, 0, s>>>(P, F, nf, own, star, deg, radius, vpos, vcells, vnbrs, err);
    if (check_launch()) return SVM_ERR_CUDA;
    if (cudaMemcpyAsync(ringOff, deg, sizeof(int) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(ringOff + n, 0, sizeof(int), s) != cudaSuccess)
        return SVM_ERR_CUDA;
    int nr = 0;
    if (exclusive_scan(ringOff, n + 1, s, &nr)) return SVM_ERR_CUDA;
    if (nr != 3 * nf) return SVM_ERR_HULL;
    k_hull_ring<<<(n + kB - 1) / kB, kB, 0, s>>>(star, deg, n, own, F, ringOff, ring, err);
    if (check_launch()) return SVM_ERR_CUDA;
    svm_topology* t = new svm_topology();
    Topology& T = t->t;
    T.nCells = n;
    T.nVertices = nf;
    T.vertexPos.resize(3 * (size_t)nf);
    T.vertexCells.resize(3 * (size_t)nf);
    T.vertexNeighbors.resize(3 * (size_t)nf);
    T.ringOffsets.resize((size_t)n + 1);
    T.ringVertices.resize(3 * (size_t)nf);
    std::vector<int> degs(n);
    bool ok = cudaMemcpyAsync(T.vertexPos.data(), vpos, sizeof(double) * 3 * nf, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaMemcpyAsync(T.vertexCells.data(), vcells, sizeof(int) * 3 * nf, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaMemcpyAsync(T.vertexNeighbors.data(), vnbrs, sizeof(int) * 3 * nf, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaMemcpyAsync(T.ringOffsets.data(), ringOff, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaMemcpyAsync(T.ringVertices.data(), ring, sizeof(int) * 3 * nf, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaMemcpyAsync(degs.data(), deg, sizeof(int) * n, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
              cudaStreamSynchronize(s) == cudaSuccess;
    if (!ok || e) { delete t; return ok ? SVM_ERR_HULL : SVM_ERR_CUDA; }
    T.maxRing = *std::max_element(degs.begin(), degs.end());
    *out = t;
    return SVM_OK;
}
