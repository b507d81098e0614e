// Per-vertex force of the quadratic spherical vertex model, shared by the Brownian, FIRE and
// plain force kernels.
//
// Restates computeForceCPU (src/model/sphericalVertexModel.cpp:356-420) /
// gpu_quadratic_spherical_cellular_force_kernel (src/model/sphericalVertexModel.cu:141-195):
// for each of the vertex's three cells,
//   fSet = -2 dP [grad d(v,last) + grad d(v,next)] - 2 Kr dA [grad A(v,last,c) + grad A(v,c,next)]
// in the spherical basis at v, skipping a cell whose contribution is NaN.  (last, next) are the
// ring neighbours of v in that cell, c the cell's renormalised centroid.
#pragma once
#include "svm_internal.cuh"

namespace svm {

struct ForceArgs {
    const double4_32a* pos;
    const double4_32a* vsph;
    const int4* vcell;
    const int4* vlast;
    const int4* vnext;
    const double4_32a* cellPos;
    const double4_32a* cellSph;
    const double2* ap;
    const double2* pref;
    double Kr, R;
    int vec;   // SVM_PRECISION_FP64_VECTOR: the exact gradient as vectors (vertex_force_vec)
};

__device__ __forceinline__ int comp(const int4& a, int s) { return s == 0 ? a.x : (s == 1 ? a.y : a.z); }

// Unit tangent at a pointing away from the neighbour at v + d: gradient of the geodesic length
// (any radius), from the raw position difference d.
__device__ __forceinline__ D3 grad_geo_vec(D3 a, D3 d) {
    const D3 t = sub3(d, scl3(dot3(d, a), a));
    return scl3(-1.0 / sqrt(dot3(t, t)), t);
}
// Gradient w.r.t. v = |v| a of the signed spherical triangle area R^2 E(a, a + beta, a + gamma),
// beta and gamma the raw differences to the other corners over |v|: tan(E/2) = N/D (Van Oosterom
// and Strackee, 1983) differentiated, projected onto the tangent plane.
__device__ __forceinline__ D3 grad_tri_vec(D3 a, D3 beta, D3 gamma, double R) {
    const D3 bg = cross3(beta, gamma);
    const D3 bxc = add3(add3(cross3(a, gamma), cross3(beta, a)), bg);
    const double N = dot3(a, bg);
    const double D = 4.0 - dot3(beta, beta) - dot3(gamma, gamma) + dot3(beta, gamma);
    const double w = 2.0 / (N * N + D * D);
    const D3 g = scl3(w, sub3(scl3(D, bxc), scl3(N, add3(beta, gamma))));
    return scl3(R, sub3(g, scl3(dot3(g, a), a)));
}

// The same force as vertex_force (the negative energy gradient) with well-conditioned vector
// formulas; the reference's formulas below lose digits for short edges and thin fan triangles.
__device__ __forceinline__ D3 vertex_force_vec(const ForceArgs& A, int v) {
    const D3 P = ld3(A.pos, v);
    const double inv = 1.0 / sqrt(dot3(P, P));
    const D3 a = scl3(inv, P);
    const int4 cells = A.vcell[v], lasts = A.vlast[v], nexts = A.vnext[v];
    D3 f{0.0, 0.0, 0.0};
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int c = comp(cells, s);
        const D3 dc = sub3(ld3(A.cellPos, c), P);
        const D3 dl = sub3(ld3(A.pos, comp(lasts, s)), P), dx = sub3(ld3(A.pos, comp(nexts, s)), P);
        const double2 apc = A.ap[c], pr = A.pref[c];
        const double pp = 2.0 * (apc.y - pr.y), aa = 2.0 * A.Kr * (apc.x - pr.x);
        const D3 bl = scl3(inv, dl), bc = scl3(inv, dc), bx = scl3(inv, dx);
        const D3 fs = add3(scl3(-pp, add3(grad_geo_vec(a, dl), grad_geo_vec(a, dx))),
                           scl3(-aa, add3(grad_tri_vec(a, bl, bc, A.R), grad_tri_vec(a, bc, bx, A.R))));
        if (!isnan(fs.x)) f = add3(f, fs);
    }
    return f;
}

__device__ __forceinline__ D3 vertex_force(const ForceArgs& A, int v) {
    if (A.vec) return vertex_force_vec(A, v);
    const D3 p = ld3(A.pos, v);
    const double4_32a sv = A.vsph[v];
    const int4 cells = A.vcell[v], lasts = A.vlast[v], nexts = A.vnext[v];
    // The ring predecessors (and successors) of v in its three cells are its three neighbours, so
    // each neighbour's geodesic gradient serves two cells: evaluated once per neighbour, keyed by
    // the neighbours' order in `lasts` (a successor is found among them).
    D3 gG[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) gG[j] = from_basis(sv, grad_geodesic(sv, A.vsph[comp(lasts, j)]));
    D3 f{0.0, 0.0, 0.0};
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int c = comp(cells, s), L = comp(lasts, s), X = comp(nexts, s);
        const D3 cp = ld3(A.cellPos, c);
        const double4_32a sc = A.cellSph[c];
        const double2 apc = A.ap[c], pr = A.pref[c];
        const double dA = apc.x - pr.x, dP = apc.y - pr.y;
        const D3 pl = ld3(A.pos, L), px = ld3(A.pos, X);
        const double4_32a sl = A.vsph[L], sx = A.vsph[X];
        const double pp = 2.0 * dP;
        const double aa = 2.0 * A.Kr * dA;
        const int jx = X == lasts.x ? 0 : (X == lasts.y ? 1 : (X == lasts.z ? 2 : -1));
        D3 fs{0.0, 0.0, 0.0}, t;
        t = gG[s];
        fs = sub3(fs, scl3(pp, t));
        t = jx >= 0 ? pick3(gG, jx) : from_basis(sv, grad_geodesic(sv, sx));
        fs = sub3(fs, scl3(pp, t));
        t = from_basis(sv, grad_triangle(sv, sl, sc, p, pl, cp, A.R));
        fs = sub3(fs, scl3(aa, t));
        t = from_basis(sv, grad_triangle(sv, sc, sx, p, cp, px, A.R));
        fs = sub3(fs, scl3(aa, t));
        if (!isnan(fs.x)) f = add3(f, fs);
    }
    return f;
}

}  // namespace svm
