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
};

__device__ __forceinline__ int comp(const int4& a, int s) { return s == 0 ? a.x : (s == 1 ? a.y : a.z); }

__device__ __forceinline__ D3 vertex_force(const ForceArgs& A, int v) {
    const D3 p = ld3(A.pos, v);
    const double4_32a sv = A.vsph[v];
    const int4 cells = A.vcell[v], lasts = A.vlast[v], nexts = A.vnext[v];
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
        D3 fs{0.0, 0.0, 0.0}, t;
        t = from_basis(sv, grad_geodesic(sv, sl));
        fs = sub3(fs, scl3(pp, t));
        t = from_basis(sv, grad_geodesic(sv, sx));
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
