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
    int vec;   // SVM_PRECISION_FP64_VECTOR: the exact gradient as vectors (grad_geo_vec, grad_tri_vec)
};

__device__ __forceinline__ int comp(const int4& a, int s) { return s == 0 ? a.x : (s == 1 ? a.y : a.z); }

// Unit tangent at a pointing away from the neighbour at v + d: gradient of the geodesic length
// (any radius), from the raw position difference d.
__device__ __forceinline__ D3 grad_geo_vec(D3 a, D3 d) {
    const D3 t = sub3(d, scl3(dot3(d, a), a));
    return scl3(f64_div(-1.0, f64_sqrt(dot3(t, t))), t);
}
// Gradient w.r.t. v = |v| a of the signed spherical triangle area R^2 E(a, a + beta, a + gamma),
// beta and gamma the raw differences to the other corners over |v|: tan(E/2) = N/D (Van Oosterom
// and Strackee, 1983) differentiated, projected onto the tangent plane.
__device__ __forceinline__ D3 grad_tri_vec(D3 a, D3 beta, D3 gamma, double R) {
    const D3 bg = cross3(beta, gamma);
    const D3 bxc = add3(add3(cross3(a, gamma), cross3(beta, a)), bg);
    const double N = dot3(a, bg);
    const double D = 4.0 - dot3(beta, beta) - dot3(gamma, gamma) + dot3(beta, gamma);
    const double w = f64_div(2.0, N * N + D * D);
    const D3 g = scl3(w, sub3(scl3(D, bxc), scl3(N, add3(beta, gamma))));
    return scl3(R, sub3(g, scl3(dot3(g, a), a)));
}

// The geodesic-length gradient at v towards its ring predecessor in cell slot s, in Cartesian
// form.  Each neighbour of v is the predecessor in one of its cells and the successor in another,
// so the three of them cover both geodesic terms of every slot, each evaluated once.
__device__ __forceinline__ D3 slot_geodesic(const ForceArgs& A, int v, int s) {
    const double4_32a sv = A.vsph[v];
    return from_basis(sv, grad_geodesic(sv, A.vsph[comp(A.vlast[v], s)]));
}

// The contribution of cell slot s to the force on vertex v: the fSet term of the header's sum for
// the vertex's cell s, which block_slot_force adds in slot order, skipping a NaN term, as the
// reference's loop over the three cells does.  Three threads share a vertex (more warps in flight
// when the vertex count is small).  gG: the vertex's three slot_geodesic values (reference form
// only).  The vector form (A.vec: the exact gradient as vectors, well conditioned where the
// reference's closed forms lose digits -- short edges, thin fan triangles) uses grad_geo_vec and
// grad_tri_vec on the position differences instead.
// The force form of a kernel: chosen per launch from A.vec (kFormAny), or fixed at compile time, which
// lets a kernel that runs one form drop the other's registers.
constexpr int kFormAny = 0, kFormVector = 1, kFormReference = 2;
template <int kForm = kFormAny>
__device__ __forceinline__ D3 slot_force(const ForceArgs& A, int v, int s, const D3* gG) {
    const int4 cells = A.vcell[v], lasts = A.vlast[v], nexts = A.vnext[v];
    const int c = comp(cells, s), L = comp(lasts, s), X = comp(nexts, s);
    if (kForm == kFormVector || (kForm == kFormAny && A.vec)) {
        const D3 P = ld3(A.pos, v);
        const double inv = f64_div(1.0, f64_sqrt(dot3(P, P)));
        const D3 a = scl3(inv, P);
        const D3 dc = sub3(ld3(A.cellPos, c), P);
        const D3 dl = sub3(ld3(A.pos, L), P), dx = sub3(ld3(A.pos, X), P);
        const double2 apc = A.ap[c], pr = A.pref[c];
        const double pp = 2.0 * (apc.y - pr.y), aa = 2.0 * A.Kr * (apc.x - pr.x);
        const D3 bl = scl3(inv, dl), bc = scl3(inv, dc), bx = scl3(inv, dx);
        return add3(scl3(-pp, add3(grad_geo_vec(a, dl), grad_geo_vec(a, dx))),
                    scl3(-aa, add3(grad_tri_vec(a, bl, bc, A.R), grad_tri_vec(a, bc, bx, A.R))));
    }
    const D3 p = ld3(A.pos, v);
    const double4_32a sv = A.vsph[v];
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
    t = pick3(gG, s);
    fs = sub3(fs, scl3(pp, t));
    t = jx >= 0 ? pick3(gG, jx) : from_basis(sv, grad_geodesic(sv, sx));
    fs = sub3(fs, scl3(pp, t));
    t = from_basis(sv, grad_triangle(sv, sl, sc, p, pl, cp, A.R));
    fs = sub3(fs, scl3(aa, t));
    t = from_basis(sv, grad_triangle(sv, sc, sx, p, cp, px, A.R));
    fs = sub3(fs, scl3(aa, t));
    return fs;
}

// Block-level force of kSlotVerts vertices by 3 kSlotVerts threads (thread 3 i + s computes slot s
// of vertex i of the block); threads i < kSlotVerts receive vertex i's force in slot order.  The
// geodesic gradients of the reference form are evaluated once per neighbour (thread 3 i + s for
// the predecessor in slot s) and shared through the block.
constexpr int kSlotVerts = 64;
// Resident blocks per SM the slot-force kernels are compiled for: three blocks of 3 kSlotVerts
// threads (the register budget falls from 120 to 96 with a few bytes of spill), whose 18 warps hide
// the latency of the integer-pipe divisions and square roots better than two blocks' 12 (the
// Brownian step's force kernel at 100k cells: 0.49 -> 0.475 ms per launch; FIRE's at 20k cells
// likewise).  Blocks of 32 vertices (six per SM) measured no faster at 20k or 100k cells.
constexpr int kSlotMinBlocks = 3;
struct SlotShared { double x[3 * kSlotVerts], y[3 * kSlotVerts], z[3 * kSlotVerts]; };
template <int kForm = kFormAny>
__device__ __forceinline__ D3 block_slot_force(const ForceArgs& A, int nV, SlotShared& sh) {
    const bool vec = kForm == kFormVector || (kForm == kFormAny && A.vec);
    const int t = threadIdx.x, base = blockIdx.x * kSlotVerts;
    const int vi = t / 3, s = t - 3 * (t / 3);
    const int v = base + vi;
    if (!vec) {
        if (v < nV) {
            const D3 g = slot_geodesic(A, v, s);
            sh.x[t] = g.x; sh.y[t] = g.y; sh.z[t] = g.z;
        }
        __syncthreads();
    }
    D3 fs{0.0, 0.0, 0.0};
    if (v < nV) {
        D3 gG[3];
        if (!vec)
#pragma unroll
            for (int j = 0; j < 3; ++j) gG[j] = D3{sh.x[3 * vi + j], sh.y[3 * vi + j], sh.z[3 * vi + j]};
        fs = slot_force<kForm>(A, v, s, gG);
    }
    __syncthreads();
    if (v < nV) { sh.x[t] = fs.x; sh.y[t] = fs.y; sh.z[t] = fs.z; }
    __syncthreads();
    D3 f{0.0, 0.0, 0.0};
    if (t < kSlotVerts && base + t < nV) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const D3 fq{sh.x[3 * t + q], sh.y[3 * t + q], sh.z[3 * t + q]};
            if (!isnan(fq.x)) f = add3(f, fq);
        }
    }
    return f;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11): ten rounds of two 32x32->64 multiplies with a Weyl-sequence key schedule.
__device__ __forceinline__ uint4 philox4x32_10(uint4 ctr, uint2 key) {
    const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { key.x += W0; key.y += W1; }
        const unsigned hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
        const unsigned hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
        ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
    }
    return ctr;
}
// 53-bit uniform in (0, 1) from two 32-bit words.
__device__ __forceinline__ double u53(unsigned a, unsigned b) {
    const unsigned long long x = ((unsigned long long)a << 21) ^ (unsigned long long)(b >> 11);
    return ((double)(x & ((1ull << 53) - 1)) + 0.5) * 0x1.0p-53;
}

// Standard normals by the ziggurat method (G. Marsaglia and W. W. Tsang, "The Ziggurat Method for
// Generating Random Variables", J. Stat. Softw. 5(8), 2000) with 256 layers of equal area v under
// f(x) = exp(-x^2/2): layer i >= 1 is the box [0, x_i) x [f(x_i), f(x_{i+1})), layer 0 the box
// [0, v / f(r)) x [0, f(r)) together with the tail beyond r = x_1.  A uniform layer, sign and
// u in [0, 1) give x = u x_i, accepted at once when x < x_{i+1} (98.5% of draws); otherwise layer 0
// samples the tail (Marsaglia's x = -ln(u1) / r, y = -ln(u2), accepted when 2y > x^2) and the other
// layers test the wedge against f(x), starting over on rejection.  The bits: one Philox draw's
// 64-bit halves for the fast path, a fresh draw per retry.
struct ZigTable {
    double x[257];  // x_0 = v / f(r), x_1 = r, ..., x_256 = 0
    double f[257];  // f(x_i) (f_0 unused)
};
constexpr double kZigR = 3.654152885361009;  // r for 256 layers
// Layer, sign and a 53-bit u in [0, 1) from 64 bits.
__device__ __forceinline__ double zig_draw(const ZigTable* __restrict__ Z, unsigned a, unsigned b, int& i, bool& neg) {
    i = (int)(a & 255u);
    neg = (a >> 8) & 1u;
    const unsigned long long n = ((unsigned long long)(a >> 9) << 30) | (unsigned long long)(b >> 2);
    return (double)n * 0x1.0p-53 * __ldg(Z->x + i);
}
static __device__ __noinline__ double zig_slow(const ZigTable* __restrict__ Z, int i, double x, bool neg, uint4 ctr, uint2 key) {
    for (int attempt = 0; attempt < 32; ++attempt) {  // each round fails with probability < 0.02
        ctr.w += 1u;
        const uint4 r = philox4x32_10(ctr, key);
        if (i == 0) {
            const double xt = -log(u53(r.x, r.y)) / kZigR, y = -log(u53(r.z, r.w));
            if (y + y > xt * xt) return neg ? -(kZigR + xt) : kZigR + xt;
            continue;
        }
        const double y = __ldg(Z->f + i) + u53(r.x, r.y) * (__ldg(Z->f + i + 1) - __ldg(Z->f + i));
        if (y < exp(-0.5 * x * x)) return neg ? -x : x;
        x = zig_draw(Z, r.z, r.w, i, neg);
        if (x < __ldg(Z->x + i + 1)) return neg ? -x : x;
    }
    return neg ? -x : x;
}
__device__ __forceinline__ double zig_normal(const ZigTable* __restrict__ Z, unsigned a, unsigned b, uint4 ctr, uint2 key) {
    int i;
    bool neg;
    const double x = zig_draw(Z, a, b, i, neg);
    if (x < __ldg(Z->x + i + 1)) return neg ? -x : x;
    return zig_slow(Z, i, x, neg, ctr, key);
}
// Three standard normals for (vertex, step): two Philox draws (counter words 0 and 1) give the
// three fast-path draws; normal j retries on counter words 64 (j + 1) + 1, 2, ...
__device__ __forceinline__ D3 philox_normals3(const ZigTable* __restrict__ Z, uint64_t seed, unsigned long long step, int v) {
    const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    const uint4 c0 = make_uint4((unsigned)v, (unsigned)step, (unsigned)(step >> 32), 0u);
    const uint4 r0 = philox4x32_10(c0, key);
    const uint4 r1 = philox4x32_10(make_uint4(c0.x, c0.y, c0.z, 1u), key);
    return D3{zig_normal(Z, r0.x, r0.y, make_uint4(c0.x, c0.y, c0.z, 64u), key),
              zig_normal(Z, r0.z, r0.w, make_uint4(c0.x, c0.y, c0.z, 128u), key),
              zig_normal(Z, r1.x, r1.y, make_uint4(c0.x, c0.y, c0.z, 192u), key)};
}

// disp_d = xi_d sqrt(2 dt mu T) + F_d dt mu (brownianDynamics.cpp:37-44), products rounded
// before the sum as on the CPU.
__device__ __forceinline__ double bd_disp(double xi, double np, double f, double fp) {
    return __dadd_rn(__dmul_rn(xi, np), __dmul_rn(f, fp));
}
// sphericalDomain::move with every product and sum rounded separately (no contraction), so the
// renormalised positions follow the CPU's sequence of roundings.
__device__ __forceinline__ D3 move_exact(D3 p, D3 v, double R) {
    const double vp = __dadd_rn(__dadd_rn(__dmul_rn(v.x, p.x), __dmul_rn(v.y, p.y)), __dmul_rn(v.z, p.z));
    const double pp = __dadd_rn(__dadd_rn(__dmul_rn(p.x, p.x), __dmul_rn(p.y, p.y)), __dmul_rn(p.z, p.z));
    const double s = f64_div(vp, pp);
    D3 q{__dadd_rn(p.x, __dsub_rn(v.x, __dmul_rn(s, p.x))), __dadd_rn(p.y, __dsub_rn(v.y, __dmul_rn(s, p.y))),
         __dadd_rn(p.z, __dsub_rn(v.z, __dmul_rn(s, p.z)))};
    const double qq = __dadd_rn(__dadd_rn(__dmul_rn(q.x, q.x), __dmul_rn(q.y, q.y)), __dmul_rn(q.z, q.z));
    const double inv = f64_div(1.0, f64_sqrt(qq));
    return D3{__dmul_rn(R, __dmul_rn(inv, q.x)), __dmul_rn(R, __dmul_rn(inv, q.y)), __dmul_rn(R, __dmul_rn(inv, q.z))};
}


inline ForceArgs force_args(svm_model* m, int buf) {
    ForceArgs A;
    A.pos = m->pos[buf]; A.vsph = m->vsph; A.vcell = m->vcell; A.vlast = m->vlast; A.vnext = m->vnext;
    A.cellPos = m->cellPos; A.cellSph = m->cellSph; A.ap = m->ap; A.pref = m->pref; A.Kr = m->Kr; A.R = m->R;
    A.vec = m->precision == SVM_PRECISION_FP64_VECTOR ? 1 : 0;
    return A;
}
}  // namespace svm
