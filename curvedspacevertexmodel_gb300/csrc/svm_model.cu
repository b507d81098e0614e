// Spherical vertex model on one GB300: geometry, forces, Brownian step, moves and T1 flips,
// plus the model half of the C ABI declared in include/svm.h.
//
// Kernel sequence of one Brownian timestep (invariant: `corner` and `vsph` describe the current
// positions and topology when a step starts):
//   k_cells         per cell: centroid, area (spherical excess), perimeter, total-area check
//   k_fallback      per cell: triangle-fan areas, only when the total area is off by > 1e-6
//   k_force_bd      per vertex: force, Brownian displacement, move onto the sphere (new buffer)
//   k_corners       per vertex: spherical coordinates, per-corner arc and angle, T1 edge test
//   k_t1_apply      one block: the CPU's sequential T1 order over the flagged edges; patches
//                   corners of every cell whose ring changed
// None of them synchronises with the host, so a run of steps is captured as one CUDA graph.
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include <atomic>
#include <type_traits>
#include "svm_internal.cuh"
#include "svm_force.cuh"
#include "svm_hull.h"

using namespace svm;

namespace svm {

constexpr int kBlock = 256;
constexpr int kApplyThreads = 256;
constexpr int kExtractCap = 1024;  // positions extracted per bitmap chunk (32 words)
constexpr int kHeapCap = 512;

inline int blocksFor(long n, int b = kBlock) { return (int)((n + b - 1) / b); }

static bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &st);
    return st != cudaStreamCaptureStatusNone;
}

static void profile_drain(svm_model* m) {
    cudaStreamSynchronize(m->stream);
    for (int ph = 0; ph < SVM_PHASE_COUNT; ++ph) {
        for (int k = 0; k + 1 < m->profUsed[ph]; k += 2) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, m->profEvents[ph][k], m->profEvents[ph][k + 1]) == cudaSuccess) {
                m->profMs[ph] += ms;
                m->profLaunches[ph] += m->profKernels[ph][k / 2];
            }
        }
        m->profUsed[ph] = 0;
        m->profKernels[ph].clear();
    }
}

PhaseTimer::PhaseTimer(svm_model* m_, int phase_, int kernels)
    : m(m_), phase(phase_), on(m_->prof && !capturing(m_->stream)), timed(false) {
    if (!on) return;
    timed = ((m->profMask >> phase) & 1) != 0;
    if (!timed) {  // counted, not timed
        m->profLaunches[phase] += kernels;
        return;
    }
    auto& ev = m->profEvents[phase];
    if (m->profUsed[phase] + 2 > 512) profile_drain(m);
    m->profKernels[phase].push_back(kernels);
    while ((int)ev.size() < m->profUsed[phase] + 2) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ev.push_back(e);
    }
    cudaEventRecord(ev[m->profUsed[phase]], m->stream);
}
PhaseTimer::~PhaseTimer() {
    if (!on || !timed) return;
    cudaEventRecord(m->profEvents[phase][m->profUsed[phase] + 1], m->stream);
    m->profUsed[phase] += 2;
}

int check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "libsvm: CUDA error %s\n", cudaGetErrorString(e));
        return SVM_ERR_CUDA;
    }
    return SVM_OK;
}

// Block-wide sum in a fixed order (warp shuffle tree, then warps in index order).
__device__ double block_sum(double v) {
    __shared__ double warpSums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) warpSums[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int w = 0; w < nw; ++w) r += warpSums[w];
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// ---- geometry ------------------------------------------------------------------------------

// Per vertex: spherical coordinates and, for each of its three cells, the arc from the ring
// predecessor and the included angle at the vertex (the per-corner terms of
// computeGeometryCPU, sphericalVertexModel.cpp:257-276).  With `t1test`, also marks every edge
// (v, u), v < u, shorter than the T1 threshold (sphericalVertexModel.cpp:469-481).
// One thread per vertex (large vertex counts: keeps each vertex's shared values in registers).
// |p| of every vertex, once per corner pass: each is read by the vertex and its three neighbours.
__global__ void k_vnorm(const double4_32a* __restrict__ pos, double* __restrict__ vnorm, int nV) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nV) vnorm[v] = pos_norm(ld3(pos, v));
}

// Position of the n-th (from 0) set bit of m, n < popc(m).
__device__ __forceinline__ int nth_set(unsigned m, int n) {
    int pos = 0, c = __popc(m & 0xFFFFu);
    if (n >= c) { n -= c; m >>= 16; pos += 16; }
    c = __popc(m & 0xFFu);
    if (n >= c) { n -= c; m >>= 8; pos += 8; }
    c = __popc(m & 0xFu);
    if (n >= c) { n -= c; m >>= 4; pos += 4; }
    c = __popc(m & 0x3u);
    if (n >= c) { n -= c; m >>= 2; pos += 2; }
    return pos + ((n >= (int)(m & 1u)) ? 1 : 0);
}

// Edge terms of the corner pass, once per edge: for every edge (v, u) with v < u, stored at slot
// e = 3 v + j (u = vnbr[v][j]): p_v x p_u with its norm, and the arc geodesic(p_u, p_v) (both
// endpoints' corners read them; from u's side the cross product is the exact negative and the arc
// and norm are the same bit for bit, since the products commute); with `t1test`, the T1 test of
// the edge (sphericalVertexModel.cpp:469-481).  Also each vertex's spherical coordinates.  A
// warp's owned edges (about half of its 96 slots) are compacted over its lanes first, so that the
// FP64 work runs on full warps.
__global__ void k_edges(const double4_32a* __restrict__ pos, const double* __restrict__ vnorm,
                        double4_32a* __restrict__ vsph, const int4* __restrict__ vnbr,
                        double4_32a* __restrict__ edgeC, double* __restrict__ edgeArc, int nV, double R, int t1test,
                        double t1Threshold, T1Scratch t1) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    const bool live = v < nV;
    int4 nb = make_int4(-1, -1, -1, -1);
    if (live) {
        nb = vnbr[v];
        vsph[v] = sph_coords_n(ld3(pos, v), vnorm[v]);
    }
    const unsigned b0 = __ballot_sync(0xffffffffu, live && v < nb.x);
    const unsigned b1 = __ballot_sync(0xffffffffu, live && v < nb.y);
    const unsigned b2 = __ballot_sync(0xffffffffu, live && v < nb.z);
    const int n0 = __popc(b0), n1 = __popc(b1), total = n0 + n1 + __popc(b2);
    const int base = v - lane;
    for (int k = lane; k < total; k += 32) {
        int j, src;
        if (k < n0) { j = 0; src = nth_set(b0, k); }
        else if (k < n0 + n1) { j = 1; src = nth_set(b1, k - n0); }
        else { j = 2; src = nth_set(b2, k - n0 - n1); }
        const int w = base + src, u = comp(vnbr[w], j);
        const D3 p = ld3(pos, w), U = ld3(pos, u);
        const D3 C = cross3e(p, U);
        const double arc = geodesic_n(U, p, vnorm[u], vnorm[w], R);
        const int e = 3 * w + j;
        edgeC[e] = make_double4_32a(C.x, C.y, C.z, f64_sqrt(dot3e(C, C)));
        edgeArc[e] = arc;
        // geodesic(u, p) < t is the reference's test (sphericalVertexModel.cpp:475)
        if (t1test && arc < t1Threshold) {
            atomicOr(&t1.bits[e >> 5], 1u << (e & 31));
            atomicOr(&t1.summary[e >> 10], 1u << ((e >> 5) & 31));
            atomicAdd(t1.count, 1);
        }
    }
}

// The edge terms of slot j of vertex v (neighbour u) from its owner: C = p_v x p_u, its norm and
// the arc.  False if u does not list v (inconsistent lists).
__device__ __forceinline__ bool edge_terms(int v, int j, int u, const int4* __restrict__ vnbr,
                                           const double4_32a* __restrict__ edgeC,
                                           const double* __restrict__ edgeArc, D3& C, double& nC, double& arc) {
    int e;
    bool neg = false;
    if (v < u) {
        e = 3 * v + j;
    } else {
        const int ju = nbr_slot(vnbr[u], v);
        if (ju < 0) return false;
        e = 3 * u + ju;
        neg = true;
    }
    const double4_32a q = edgeC[e];
    C = neg ? D3{-q.x, -q.y, -q.z} : D3{q.x, q.y, q.z};
    nC = q.w;
    arc = edgeArc[e];
    return true;
}

// k_corner with three threads per vertex (below ~100k vertices, where one thread per vertex
// leaves the FP64 pipe short of warps): thread (v, j) fetches the edge terms of neighbour j into
// shared memory, then, after a block barrier, computes the corner of cell slot j.
constexpr int kCornerVerts = 64;
constexpr int kCornerSlotsBelow = 100000;  // vertices
struct CornerShared {
    double cx[3 * kCornerVerts], cy[3 * kCornerVerts], cz[3 * kCornerVerts], n[3 * kCornerVerts];
    double ux[3 * kCornerVerts], uy[3 * kCornerVerts], uz[3 * kCornerVerts], arc[3 * kCornerVerts];
    int ok[kCornerVerts];
};
__global__ void __launch_bounds__(3 * kCornerVerts) k_corner_s(
    const double4_32a* __restrict__ pos, const int4* __restrict__ vcell, const int4* __restrict__ vlast,
    const int4* __restrict__ vnext, const int4* __restrict__ vrpos, const int4* __restrict__ vnbr,
    const double4_32a* __restrict__ edgeC, const double* __restrict__ edgeArc, double2* __restrict__ corner, int Wc,
    int nV, double R) {
    __shared__ CornerShared sh;
    const int t = threadIdx.x, vi = t / 3, j = t - 3 * (t / 3), b = 3 * vi;
    const int v = blockIdx.x * kCornerVerts + vi;
    const bool live = v < nV;
    if (j == 0) sh.ok[vi] = 1;
    __syncthreads();
    int4 nb = make_int4(0, 0, 0, 0);
    if (live) {
        nb = vnbr[v];
        const int u = comp(nb, j);
        const D3 U = ld3(pos, u);
        D3 C{0.0, 0.0, 0.0};
        double nC = 0.0, arc = 0.0;
        if (!edge_terms(v, j, u, vnbr, edgeC, edgeArc, C, nC, arc)) sh.ok[vi] = 0;
        sh.cx[t] = C.x; sh.cy[t] = C.y; sh.cz[t] = C.z; sh.n[t] = nC;
        sh.ux[t] = U.x; sh.uy[t] = U.y; sh.uz[t] = U.z; sh.arc[t] = arc;
    }
    __syncthreads();
    if (!live) return;
    const int s = j;
    const int4 cells = vcell[v], lasts = vlast[v], nexts = vnext[v], rp = vrpos[v];
    const int jl = nbr_slot(nb, comp(lasts, s)), jx = nbr_slot(nb, comp(nexts, s));
    double2 cr;
    if (sh.ok[vi] && jl >= 0 && jx >= 0) {
        const int l = b + jl, x = b + jx;
        cr = make_double2(sh.arc[l], included_angle_pre(D3{sh.cx[x], sh.cy[x], sh.cz[x]}, D3{sh.cx[l], sh.cy[l], sh.cz[l]},
                                                        sh.n[x], sh.n[l], D3{sh.ux[l], sh.uy[l], sh.uz[l]}));
    } else {  // inconsistent lists: evaluate directly
        const D3 p = ld3(pos, v), pl = ld3(pos, comp(lasts, s)), px = ld3(pos, comp(nexts, s));
        cr = make_double2(geodesic(pl, p, R), included_angle(pl, p, px));
    }
    corner[(long)comp(cells, s) * Wc + comp(rp, s)] = cr;
}

// Per vertex: for each of its three cells, the arc from the ring predecessor and the included
// angle at the vertex (the per-corner terms of computeGeometryCPU, sphericalVertexModel.cpp:257-276)
// from the edge terms of k_edges.  Compiled for three blocks of 256 per SM (80 registers, with some
// spill, instead of 114 at two): the FP64-bound kernel's last of 2.6 waves shrinks (159 against 162 us
// per corner phase at 100k cells).
__global__ void __launch_bounds__(256, 3) k_corner(const double4_32a* __restrict__ pos, const int4* __restrict__ vcell,
                         const int4* __restrict__ vlast, const int4* __restrict__ vnext, const int4* __restrict__ vrpos,
                         const int4* __restrict__ vnbr, const double4_32a* __restrict__ edgeC,
                         const double* __restrict__ edgeArc, double2* __restrict__ corner, int Wc, int nV, double R) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const int4 nb = vnbr[v], cells = vcell[v], lasts = vlast[v], nexts = vnext[v], rp = vrpos[v];
    D3 C[3], U[3];
    double nC[3], arc[3];
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int u = comp(nb, j);
        U[j] = ld3(pos, u);
        ok &= edge_terms(v, j, u, vnbr, edgeC, edgeArc, C[j], nC[j], arc[j]);
    }
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int jl = nbr_slot(nb, comp(lasts, s)), jx = nbr_slot(nb, comp(nexts, s));
        double2 cr;
        if (ok && jl >= 0 && jx >= 0) {
            cr = make_double2(pick3(arc, jl), included_angle_pre(pick3(C, jx), pick3(C, jl), pick3(nC, jx),
                                                                 pick3(nC, jl), pick3(U, jl)));
        } else {  // inconsistent lists: evaluate directly
            const D3 p = ld3(pos, v), pl = ld3(pos, comp(lasts, s)), px = ld3(pos, comp(nexts, s));
            cr = make_double2(geodesic(pl, p, R), included_angle(pl, p, px));
        }
        corner[(long)comp(cells, s) * Wc + comp(rp, s)] = cr;
    }
}

// Per cell: centroid (sum of ring vertices in ring order, renormalised), perimeter and angle sum
// in the CPU's order (ring positions n-2, n-1, 0, ..., n-3), area = (sum - (n-2) pi) wrapped
// by floor(area / pi), times R^2 (sphericalVertexModel.cpp:228-303).  The last block to finish
// totals the areas and raises the fallback flag when |sum A - 4 pi R^2| > 1e-6 (304-310).
//
// Replicas (mixed form, repR non-null): the radius is the replica's, read through the first ring
// vertex; with `ticket` null the area check is left to k_rep_check (per replica).
template <class PT>
__global__ void k_cells(const PT* __restrict__ pos, const int* __restrict__ ring,
                        const int* __restrict__ ringCount, const double2* __restrict__ corner, int Wc, int nC,
                        double R0, const double* __restrict__ repR, PT* __restrict__ cellPos,
                        double4_32a* __restrict__ cellSph, double2* __restrict__ ap, double* __restrict__ partials,
                        unsigned* __restrict__ ticket, double* __restrict__ scalars, int* __restrict__ fallbackFlag,
                        const double2* __restrict__ pref = nullptr, float2* __restrict__ dap32 = nullptr) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double area = 0.0;
    if (c < nC) {
        const int n = ringCount[c];
        const int* rg = ring + (long)c * Wc;
        const double R = repR ? repR[rep_of(pos[rg[0]])] : R0;
        D3 cp{0.0, 0.0, 0.0};
        for (int k = 0; k < n; ++k) cp = add3(cp, ld3(pos, rg[k]));
        cp = renorm(cp, R);
        st3(cellPos, c, cp);
        if (cellSph) cellSph[c] = sph_coords(cp);
        const double2* cr = corner + (long)c * Wc;
        double per = 0.0, ang = 0.0;
        int k = n - 2;
        for (int t = 0; t < n; ++t) {
            const double2 q = cr[k];
            per += q.x;
            ang += q.y;
            k = (k + 1 == n) ? 0 : k + 1;
        }
        area = __dsub_rn(ang, __dmul_rn((double)(n - 2), kPI));
        // The mixed form also subtracts (n - 2) times the part of pi below the double kPI: the
        // reference's excess is biased by +(n - 2)(pi - kPI) per cell, which over a sphere sums to
        // ~4N (pi - kPI) R^2 (4e-7 at N = 100k, 4e-5 at N = 1M) and trips its absolute 1e-6 area
        // check by itself at large N.  The FP64 form keeps the reference's arithmetic.
        if (std::is_same<PT, float4>::value) area = __dsub_rn(area, __dmul_rn((double)(n - 2), kPILo));
        const int extra = (int)floor(f64_div(area, 1.0 * kPI));
        if (extra > 0) area = __dsub_rn(area, __dmul_rn((double)extra, kPI));
        area = __dmul_rn(__dmul_rn(area, R), R);
        ap[c] = make_double2(area, per);
        if (dap32) {
            const double2 pr = pref[c];
            dap32[c] = make_float2(sf::narrow(area - pr.x), sf::narrow(per - pr.y));
        }
    }
    if (!ticket) return;
    const double R = R0;
    const double bs = block_sum(area);
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        amLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (amLast) {
        double s = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(partials + b);
        const double total = block_sum(s);
        if (threadIdx.x == 0) {
            const double excess = total - 4.0 * kPI * R * R;
            scalars[0] = total;
            scalars[1] = excess;
            const int taken = fabs(excess) > 1e-6 ? 1 : 0;
            fallbackFlag[0] = taken;
            fallbackFlag[1] += taken;  // geometry passes that took the fallback (svm_model_fallback_count)
            *ticket = 0u;
        }
    }
}

// recomputeAreasCPU (sphericalVertexModel.cpp:162-207): area as a sum of spherical triangles
// (centroid, ring[k-1], ring[k]) starting from (ring[n-2], ring[n-1]).
// Replicas (repFlag non-null): the flag and the radius are the cell's replica's.
template <class PT>
__global__ void k_fallback(const PT* __restrict__ pos, const int* __restrict__ ring,
                           const int* __restrict__ ringCount, const PT* __restrict__ cellPos, int Wc, int nC,
                           double R0, const int* __restrict__ fallbackFlag, const int* __restrict__ repFlag,
                           const double* __restrict__ repR, double2* __restrict__ ap,
                           const double2* __restrict__ pref = nullptr, float2* __restrict__ dap32 = nullptr) {
    if (!repFlag && *fallbackFlag == 0) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nC) return;
    const int n = ringCount[c];
    const int* rg = ring + (long)c * Wc;
    const int rep = rep_of(pos[rg[0]]);
    if (repFlag && repFlag[rep] == 0) return;
    const double R = repR ? repR[rep] : R0;
    const D3 cp = ld3(cellPos, c);
    D3 last = ld3(pos, rg[n - 2]), cur = ld3(pos, rg[n - 1]);
    double area = 0.0;
    for (int k = 0; k < n; ++k) {
        const D3 next = ld3(pos, rg[k]);
        area += triangle_area(cp, last, cur, R);
        last = cur;
        cur = next;
    }
    ap[c].x = area;
    if (dap32) dap32[c].x = sf::narrow(area - pref[c].x);
}

// k_fallback with a block's fan triangles packed densely over its threads (the triangle areas are
// FP64 acos chains, and the FP64 pipe charges a warp instruction whatever its active lanes) and
// every corner normalised once (a ring vertex serves two triangles, the centroid all of them),
// then each cell's triangles summed in the CPU's order by one thread: the same areas bit for bit.
// kFanCells cells per block; ring capacity <= 32.
constexpr int kFanCells = 32;
constexpr int kFanThreads = 256;
template <class PT>
__global__ void __launch_bounds__(kFanThreads) k_fallback_fan(
    const PT* __restrict__ pos, const int* __restrict__ ring, const int* __restrict__ ringCount,
    const PT* __restrict__ cellPos, int Wc, int nC, double R0, const int* __restrict__ fallbackFlag,
    const int* __restrict__ repFlag, const double* __restrict__ repR, double2* __restrict__ ap,
    const double2* __restrict__ pref = nullptr, float2* __restrict__ dap32 = nullptr) {
    if (!repFlag && *fallbackFlag == 0) return;
    __shared__ int cnt[kFanCells], off[kFanCells + 1], owner[kFanCells * 32];
    __shared__ double radius[kFanCells];
    __shared__ double ux[kFanCells * 32], uy[kFanCells * 32], uz[kFanCells * 32];
    __shared__ double cx[kFanCells], cy[kFanCells], cz[kFanCells];
    __shared__ double tri[kFanCells * 32];
    const int t = threadIdx.x, c0 = blockIdx.x * kFanCells;
    if (t < kFanCells) {
        const int c = c0 + t;
        int n = 0;
        if (c < nC) {
            n = ringCount[c];
            const int rep = rep_of(pos[ring[(long)c * Wc]]);
            if (repFlag && repFlag[rep] == 0) n = 0;  // this replica keeps its areas
            radius[t] = repR ? repR[rep] : R0;
            if (n > 0) {
                const D3 u = unit_corner(ld3(cellPos, c));
                cx[t] = u.x; cy[t] = u.y; cz[t] = u.z;
            }
        }
        cnt[t] = n;
        // exclusive scan of the counts over the first warp
        int incl = n;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (t >= o) incl += y;
        }
        off[t] = incl - n;
        if (t == kFanCells - 1) off[kFanCells] = incl;
        for (int k = 0; k < n; ++k) owner[incl - n + k] = t;
    }
    __syncthreads();
    const int total = off[kFanCells];
    for (int e = t; e < total; e += kFanThreads) {  // each ring corner, normalised once
        const int lc = owner[e];
        const D3 u = unit_corner(ld3(pos, ring[(long)(c0 + lc) * Wc + (e - off[lc])]));
        ux[e] = u.x; uy[e] = u.y; uz[e] = u.z;
    }
    __syncthreads();
    for (int e = t; e < total; e += kFanThreads) {
        // triangle k of cell lc in the CPU's loop: (centroid, ring[k - 2], ring[k - 1]), indices mod n
        const int lc = owner[e], b = off[lc], n = cnt[lc], k = e - b;
        const int i2 = b + (k + n - 2) % n, i3 = b + (k + n - 1) % n;
        tri[e] = triangle_area_unit(D3{cx[lc], cy[lc], cz[lc]}, D3{ux[i2], uy[i2], uz[i2]}, D3{ux[i3], uy[i3], uz[i3]},
                                    radius[lc]);
    }
    __syncthreads();
    if (t >= kFanCells || cnt[t] == 0) return;
    const int c = c0 + t;
    double area = 0.0;
    for (int k = 0; k < cnt[t]; ++k) area += tri[off[t] + k];
    ap[c].x = area;
    if (dap32) dap32[c].x = sf::narrow(area - pref[c].x);
}

// ---- forces and integration ------------------------------------------------------------------

// moveParticles (sphericalVertexModel.cpp:111-148): p <- move(p, scale * disp), in place.
__global__ void k_move(double4_32a* __restrict__ pos, const double* __restrict__ disp, double scale, int nV, double R) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const D3 d{__dmul_rn(scale, disp[3 * v]), __dmul_rn(scale, disp[3 * v + 1]), __dmul_rn(scale, disp[3 * v + 2])};
    st3(pos, v, move_exact(ld3(pos, v), d, R));
}

// Standalone T1 edge test (gpu_vm_test_edges_for_T1, sphericalVertexModel.cu:225-273).
__global__ void k_t1_test(const double4_32a* __restrict__ pos, const float4* __restrict__ pos32,
                          const double* __restrict__ repR, const int4* __restrict__ vnbr, int nV, double R,
                          double t1Threshold, double cosLo, double cosHi, double s2Lo, double s2Hi, T1Scratch t1) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const int4 nb = vnbr[v];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int u = comp(nb, s);
        if (!(v < u)) continue;
        const bool shortEdge = pos32 ? arc32(pos32[v], pos32[u], (float)repR[rep_of(pos32[v])]) < (float)t1Threshold
                                     : shorter_than<true>(ld3(pos, v), ld3(pos, u), R, t1Threshold, cosLo, cosHi, s2Lo, s2Hi);
        if (shortEdge) {
            const int q = 3 * v + s;
            atomicOr(&t1.bits[q >> 5], 1u << (q & 31));
            atomicOr(&t1.summary[q >> 10], 1u << ((q >> 5) & 31));
            atomicAdd(t1.count, 1);
        }
    }
}

// ---- T1 apply ------------------------------------------------------------------------------
struct ApplyArgs {
    double cosLo, cosHi;   // shorter_than bracket of cos(t1Threshold / R)
    double s2Lo, s2Hi;     // and its pre-test bracket of sin^2(t1Threshold / R)
    float4* pos32;         // FP32 positions in the mixed-precision form, else null
    const double* repR;    // per-replica radius (mixed form)
    double4_32a* pos;
    double4_32a* vsph;
    int4 *vcell, *vnbr, *vlast, *vnext, *vrpos;
    int* ring;
    int* ringCount;
    double2* corner;
    int Wc, nV, nC;
    double R, t1Threshold;
    int* status;
    unsigned long long* stepCounter;
    int bumpStep;
    int barrierSpins;      // polls of a grid-barrier wait before it gives up
    int* ringMax;          // largest ring count produced (atomicMax by the commits)
    int* ringMaxOut;       // host-visible copy, written once per pass by k_t1_patch
    double* hostOut;       // a host-buffer step's mapped AoS output (FP64 form), else null: k_t1_patch
                           // rewrites the vertices the pass may have moved
};

__device__ __forceinline__ int& compRef(int4* a, int v, int s) { return reinterpret_cast<int*>(a + v)[s]; }
__device__ __forceinline__ D3 apos(const ApplyArgs& A, int i) { return A.pos32 ? ld3(A.pos32, i) : ld3(A.pos, i); }
__device__ __forceinline__ void apos_st(const ApplyArgs& A, int i, D3 v) {
    if (A.pos32) st3_keep(A.pos32, i, v);
    else st3(A.pos, i, v);
}
// radius of the sphere vertex i lives on
__device__ __forceinline__ double aR(const ApplyArgs& A, int i) { return A.pos32 ? A.repR[rep_of(A.pos32[i])] : A.R; }
__device__ __forceinline__ double4_32a apos4(const ApplyArgs& A, int i) {
    const D3 p = apos(A, i);
    return make_double4_32a(p.x, p.y, p.z, 0.0);
}

// Locate `target` in ring `cell` the way getCellVertexSetForT1 does
// (sphericalVertexModel.cpp:642-652): returns its predecessor and successor.
__device__ void ring_neighbours(const ApplyArgs& A, int cell, int target, int& vlast, int& vnext) {
    const int n = A.ringCount[cell];
    const int* rg = A.ring + (long)cell * A.Wc;
    vlast = rg[n - 2];
    int vcur = rg[n - 1];
    vnext = vcur;
    for (int k = 0; k < n; ++k) {
        vnext = rg[k];
        if (vcur == target) break;
        vlast = vcur;
        vcur = vnext;
    }
}

__device__ void ring_remove(const ApplyArgs& A, int cell, int target) {
    int* rg = A.ring + (long)cell * A.Wc;
    const int n = A.ringCount[cell];
    int idx = 0;
    for (int k = 0; k < n - 1; ++k) {
        if (rg[k] == target) idx += 1;
        rg[k] = rg[idx];
        idx += 1;
    }
    A.ringCount[cell] = n - 1;
}

__device__ void ring_insert_after(const ApplyArgs& A, int cell, int after, int added) {
    int* rg = A.ring + (long)cell * A.Wc;
    const int n = A.ringCount[cell];
    int k = 0;
    while (k < n && rg[k] != after) ++k;
    for (int j = n; j > k + 1; --j) rg[j] = rg[j - 1];
    rg[k + 1] = added;
    A.ringCount[cell] = n + 1;
}

// rodriguesRotation (inc/functions.h:175-181)
// with c = cos(theta), s = sin(theta) given.  A flip rotates by theta = -det kPI / 2, det = +-1;
// kPI / 2 falls short of pi / 2 by kPILo / 2, so cos(theta) = sin(kPILo / 2), which is kPILo / 2
// to double precision (the cubic term is 1e-49), and sin(theta) = -det cos(kPILo / 2), which
// rounds to -det (1 - 1.9e-33 is within half an ulp of 1).
constexpr double kCosHalfPi = 0.5 * kPILo;
__device__ __forceinline__ D3 rodrigues(D3 v, D3 k, double c, double s) {
    const D3 cp{__dsub_rn(__dmul_rn(k.y, v.z), __dmul_rn(k.z, v.y)), __dsub_rn(__dmul_rn(k.z, v.x), __dmul_rn(k.x, v.z)),
                __dsub_rn(__dmul_rn(k.x, v.y), __dmul_rn(k.y, v.x))};
    const double w = __dmul_rn(1.0 - c, __dadd_rn(__dadd_rn(__dmul_rn(k.x, v.x), __dmul_rn(k.y, v.y)), __dmul_rn(k.z, v.z)));
    return D3{__dadd_rn(__dadd_rn(__dmul_rn(c, v.x), __dmul_rn(s, cp.x)), __dmul_rn(w, k.x)),
              __dadd_rn(__dadd_rn(__dmul_rn(c, v.y), __dmul_rn(s, cp.y)), __dmul_rn(w, k.y)),
              __dadd_rn(__dadd_rn(__dmul_rn(c, v.z), __dmul_rn(s, cp.z)), __dmul_rn(w, k.z))};
}
__device__ __forceinline__ D3 renorm_exact(D3 p, double R) {  // the T1 moves: hardware sequences
    const double pp = __dadd_rn(__dadd_rn(__dmul_rn(p.x, p.x), __dmul_rn(p.y, p.y)), __dmul_rn(p.z, p.z));
    const double inv = f64_div<true>(1.0, f64_sqrt<true>(pp));
    return D3{__dmul_rn(R, __dmul_rn(inv, p.x)), __dmul_rn(R, __dmul_rn(inv, p.y)), __dmul_rn(R, __dmul_rn(inv, p.z))};
}

// One flip as testAndPerformT1TransitionsCPU does it (sphericalVertexModel.cpp:483-599).
// Returns false when the flip is forbidden or does not fit the ring capacity.
//
// Rings of capacity 16 (the default) take a faster path: the four rings the flip reads and
// rewrites are loaded once as four 16-byte vectors each, searched and edited in thread-local
// copies (L1), and stored back whole; every value written is the same as the general path's.
struct Ring16 {
    int r[16];
    int n;
};
__device__ __forceinline__ void ring16_load(const ApplyArgs& A, int cell, Ring16& R) {
    const int4* q = reinterpret_cast<const int4*>(A.ring + (long)cell * A.Wc);
    const int4 a = q[0], b = q[1], c = q[2], d = q[3];
    R.r[0] = a.x; R.r[1] = a.y; R.r[2] = a.z; R.r[3] = a.w; R.r[4] = b.x; R.r[5] = b.y; R.r[6] = b.z; R.r[7] = b.w;
    R.r[8] = c.x; R.r[9] = c.y; R.r[10] = c.z; R.r[11] = c.w; R.r[12] = d.x; R.r[13] = d.y; R.r[14] = d.z; R.r[15] = d.w;
    R.n = A.ringCount[cell];
}
__device__ __forceinline__ void ring16_store(int* dst, const Ring16& R) {
    int4* q = reinterpret_cast<int4*>(dst);
    q[0] = make_int4(R.r[0], R.r[1], R.r[2], R.r[3]);
    q[1] = make_int4(R.r[4], R.r[5], R.r[6], R.r[7]);
    q[2] = make_int4(R.r[8], R.r[9], R.r[10], R.r[11]);
    q[3] = make_int4(R.r[12], R.r[13], R.r[14], R.r[15]);
}
// ring_neighbours, ring_remove and ring_insert_after on a local copy
__device__ __forceinline__ void ring16_neighbours(const Ring16& R, int target, int& vlast, int& vnext) {
    const int n = R.n;
    vlast = R.r[n - 2];
    int vcur = R.r[n - 1];
    vnext = vcur;
    for (int k = 0; k < n; ++k) {
        vnext = R.r[k];
        if (vcur == target) break;
        vlast = vcur;
        vcur = vnext;
    }
}
__device__ __forceinline__ void ring16_remove(Ring16& R, int target) {
    const int n = R.n;
    int idx = 0;
    for (int k = 0; k < n - 1; ++k) {
        if (R.r[k] == target) idx += 1;
        R.r[k] = R.r[idx];
        idx += 1;
    }
    R.n = n - 1;
}
__device__ __forceinline__ void ring16_insert_after(Ring16& R, int after, int added) {
    const int n = R.n;
    int k = 0;
    while (k < n && R.r[k] != after) ++k;
    for (int j = n; j > k + 1; --j) R.r[j] = R.r[j - 1];
    R.r[k + 1] = added;
    R.n = n + 1;
}

__device__ void t1_flip_positions(const ApplyArgs& A, int v1, int v2, const int4& cs, const int4& vs);
__device__ void t1_move_pair(const ApplyArgs& A, int v1, int v2, D3 p1, D3 p2, D3 vC);
// Replaces `from` by `to` in the three slots of a vertex's list.
__device__ __forceinline__ void slots_replace(int4& a, int from, int to) {
    if (a.x == from) a.x = to;
    if (a.y == from) a.y = to;
    if (a.z == from) a.z = to;
}

// A flip of 16-entry rings in three parts: t1_plan16 reads the two vertices' lists and the four
// rings, classifies the cells (cs), finds the outer neighbours (vs) and checks that the flip is
// allowed; t1_move_pair moves v1 and v2; t1_commit16 writes the undo entry, the rewired vertex
// lists (edited in registers, stored whole) and the edited rings.  The loads are grouped by level
// of dependence so that a flip waits for memory a few times instead of once per access.
struct FlipPlan16 {
    int4 c1, c2, n1, n2, ny, nz;   // vertex lists of v1, v2 and of the outer neighbours vs.y, vs.z
    Ring16 Rc[3], Rw;              // the rings of v1's three cells and of v2's fourth cell
    int qx, qy, qz;                // which of Rc is cell cs.x, cs.y, cs.z
};
// Returns 1 for a planned flip, 0 for none (forbidden, or a broken topology), 2 when a ring
// involved holds (or would hold) more than 16 entries: then the general path decides.
__device__ int t1_plan16(const ApplyArgs& A, int v1, int v2, int4& cs, int4& vs, FlipPlan16& F) {
    F.c1 = A.vcell[v1]; F.c2 = A.vcell[v2]; F.n1 = A.vnbr[v1]; F.n2 = A.vnbr[v2];
    const int c[3] = {F.c1.x, F.c1.y, F.c1.z};
    cs.w = -1;
    for (int ff = 0; ff < 3; ++ff) {
        const int t = comp(F.c2, ff);
        if (t != c[0] && t != c[1] && t != c[2]) cs.w = t;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) ring16_load(A, c[q], F.Rc[q]);
    if (cs.w >= 0) ring16_load(A, cs.w, F.Rw);
    if (F.Rc[0].n > 16 || F.Rc[1].n > 16 || F.Rc[2].n > 16 || (cs.w >= 0 && F.Rw.n > 16)) return 2;
    cs.x = cs.y = cs.z = -1;
    F.qx = F.qy = F.qz = 0;
    int yl = 0, yx = 0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        int vl, vx;
        ring16_neighbours(F.Rc[q], v1, vl, vx);
        if (vl == v2) { cs.x = c[q]; F.qx = q; }
        else if (vx == v2) { cs.z = c[q]; F.qz = q; }
        else { cs.y = c[q]; F.qy = q; yl = vl; yx = vx; }
    }
    if (cs.x < 0 || cs.y < 0 || cs.z < 0 || cs.w < 0) { atomicOr(A.status, SVM_DEV_BAD_TOPOLOGY); return 0; }
    vs.x = yl; vs.y = yx;
    int vl, vx;
    ring16_neighbours(F.Rw, v2, vl, vx);
    vs.w = vl; vs.z = vx;
    // forbid a T1 that would shrink a triangular cell (sphericalVertexModel.cpp:485-487)
    if (F.Rc[F.qx].n == 3 || F.Rc[F.qz].n == 3) return 0;
    if (F.Rc[F.qy].n + 1 > 16 || F.Rw.n + 1 > 16) return 2;
    F.ny = A.vnbr[vs.y];
    F.nz = A.vnbr[vs.z];
    return 1;
}
// p1, p2: the old positions of v1 and v2.
__device__ void t1_commit16(const ApplyArgs& A, int v1, int v2, const int4& cs, const int4& vs, FlipPlan16& F,
                            UndoEntry* undo, int* undoRings, D3 p1, D3 p2) {
    Ring16& RX = F.Rc[F.qx];
    Ring16& RY = F.Rc[F.qy];
    Ring16& RZ = F.Rc[F.qz];
    const bool yz = vs.y == vs.z;  // a vertex next to both (never v1 or v2 themselves)
    if (undo) {
        undo->v1 = v1; undo->v2 = v2; undo->b = vs.y; undo->c = vs.z;
        undo->cells[0] = cs.x; undo->cells[1] = cs.y; undo->cells[2] = cs.z; undo->cells[3] = cs.w;
        undo->p1 = make_double4_32a(p1.x, p1.y, p1.z, 0.0); undo->p2 = make_double4_32a(p2.x, p2.y, p2.z, 0.0);
        undo->vc1 = F.c1; undo->vc2 = F.c2;
        undo->vn[0] = F.n1; undo->vn[1] = F.n2; undo->vn[2] = F.ny; undo->vn[3] = F.nz;
        undo->counts[0] = RX.n; undo->counts[1] = RY.n; undo->counts[2] = RZ.n; undo->counts[3] = F.Rw.n;
        ring16_store(undoRings, RX);
        ring16_store(undoRings + A.Wc, RY);
        ring16_store(undoRings + 2 * A.Wc, RZ);
        ring16_store(undoRings + 3 * A.Wc, F.Rw);
    }
    // the slot rewiring of t1_flip_positions, slot by slot in the same order (for a shared outer
    // neighbour both of its replacements apply, the first one first)
    slots_replace(F.c1, cs.z, cs.w);
    slots_replace(F.c2, cs.x, cs.y);
    slots_replace(F.ny, v1, v2);
    if (yz) slots_replace(F.ny, v2, v1);
    else slots_replace(F.nz, v2, v1);
    slots_replace(F.n1, vs.y, vs.z);
    slots_replace(F.n2, vs.z, vs.y);
    A.vcell[v1] = F.c1; A.vcell[v2] = F.c2; A.vnbr[v1] = F.n1; A.vnbr[v2] = F.n2; A.vnbr[vs.y] = F.ny;
    if (!yz) A.vnbr[vs.z] = F.nz;
    ring16_remove(RX, v2);
    ring16_insert_after(RY, v1, v2);
    ring16_remove(RZ, v1);
    ring16_insert_after(F.Rw, v2, v1);
    ring16_store(A.ring + (long)cs.x * A.Wc, RX);
    ring16_store(A.ring + (long)cs.y * A.Wc, RY);
    ring16_store(A.ring + (long)cs.z * A.Wc, RZ);
    ring16_store(A.ring + (long)cs.w * A.Wc, F.Rw);
    A.ringCount[cs.x] = RX.n; A.ringCount[cs.y] = RY.n; A.ringCount[cs.z] = RZ.n; A.ringCount[cs.w] = F.Rw.n;
    atomicMax(A.ringMax, RY.n > F.Rw.n ? RY.n : F.Rw.n);
}
__device__ bool t1_flip_any(const ApplyArgs& A, int v1, int v2, int4& cs, int4& vs, UndoEntry* undo, int* undoRings);
__device__ bool t1_flip16(const ApplyArgs& A, int v1, int v2, int4& cs, int4& vs, UndoEntry* undo, int* undoRings) {
    FlipPlan16 F;
    const int plan = t1_plan16(A, v1, v2, cs, vs, F);
    if (plan == 2) return t1_flip_any(A, v1, v2, cs, vs, undo, undoRings);
    if (!plan) return false;
    const D3 p1 = apos(A, v1), p2 = apos(A, v2);
    t1_move_pair(A, v1, v2, p1, p2, apos(A, vs.z));
    t1_commit16(A, v1, v2, cs, vs, F, undo, undoRings, p1, p2);
    return true;
}

// The 16-entry fast path reads rings as int4 vectors at stride Wc, so it serves capacities that are
// multiples of 4 from 16 on (and hands rings of more than 16 entries to the general path).
__device__ __forceinline__ bool ring16_ok(const ApplyArgs& A) { return A.Wc >= 16 && (A.Wc & 3) == 0; }
// The general path: any capacity, rings edited in place.
__device__ bool t1_flip_any(const ApplyArgs& A, int v1, int v2, int4& cs, int4& vs, UndoEntry* undo, int* undoRings) {
    const int c[3] = {A.vcell[v1].x, A.vcell[v1].y, A.vcell[v1].z};
    cs.w = -1;
    for (int ff = 0; ff < 3; ++ff) {
        const int t = compRef(A.vcell, v2, ff);
        if (t != c[0] && t != c[1] && t != c[2]) cs.w = t;
    }
    cs.x = cs.y = cs.z = -1;
    for (int q = 0; q < 3; ++q) {
        int vl, vx;
        ring_neighbours(A, c[q], v1, vl, vx);
        if (vl == v2) cs.x = c[q];
        else if (vx == v2) cs.z = c[q];
        else cs.y = c[q];
    }
    if (cs.x < 0 || cs.y < 0 || cs.z < 0 || cs.w < 0) { atomicOr(A.status, SVM_DEV_BAD_TOPOLOGY); return false; }
    int vl, vx;
    ring_neighbours(A, cs.y, v1, vl, vx);
    vs.x = vl; vs.y = vx;
    ring_neighbours(A, cs.w, v2, vl, vx);
    vs.w = vl; vs.z = vx;
    // forbid a T1 that would shrink a triangular cell (sphericalVertexModel.cpp:485-487)
    if (A.ringCount[cs.x] == 3 || A.ringCount[cs.z] == 3) return false;
    if (A.ringCount[cs.y] + 1 > A.Wc || A.ringCount[cs.w] + 1 > A.Wc) { atomicOr(A.status, SVM_DEV_RING_OVERFLOW); return false; }
    if (undo) {
        undo->v1 = v1; undo->v2 = v2; undo->b = vs.y; undo->c = vs.z;
        undo->cells[0] = cs.x; undo->cells[1] = cs.y; undo->cells[2] = cs.z; undo->cells[3] = cs.w;
        undo->p1 = apos4(A, v1); undo->p2 = apos4(A, v2);
        undo->vc1 = A.vcell[v1]; undo->vc2 = A.vcell[v2];
        undo->vn[0] = A.vnbr[v1]; undo->vn[1] = A.vnbr[v2]; undo->vn[2] = A.vnbr[vs.y]; undo->vn[3] = A.vnbr[vs.z];
        for (int q = 0; q < 4; ++q) {
            const int cell = undo->cells[q];
            const int n = A.ringCount[cell];
            undo->counts[q] = n;
            for (int k = 0; k < n; ++k) undoRings[q * A.Wc + k] = A.ring[(long)cell * A.Wc + k];
        }
    }
    t1_flip_positions(A, v1, v2, cs, vs);
    ring_remove(A, cs.x, v2);
    ring_insert_after(A, cs.y, v1, v2);
    ring_remove(A, cs.z, v1);
    ring_insert_after(A, cs.w, v2, v1);
    atomicMax(A.ringMax, max(A.ringCount[cs.y], A.ringCount[cs.w]));
    return true;
}
__device__ bool t1_flip(const ApplyArgs& A, int v1, int v2, int4& cs, int4& vs, UndoEntry* undo = nullptr,
                        int* undoRings = nullptr) {
    if (ring16_ok(A)) return t1_flip16(A, v1, v2, cs, vs, undo, undoRings);
    return t1_flip_any(A, v1, v2, cs, vs, undo, undoRings);
}

// The rotation and separation of v1 and v2 and the rewiring of the vertex lists
// (sphericalVertexModel.cpp:513-573), shared by both paths of t1_flip.
__device__ void t1_flip_positions(const ApplyArgs& A, int v1, int v2, const int4& cs, const int4& vs) {
    t1_move_pair(A, v1, v2, apos(A, v1), apos(A, v2), apos(A, vs.z));
    for (int k = 0; k < 3; ++k) {
        if (compRef(A.vcell, v1, k) == cs.z) compRef(A.vcell, v1, k) = cs.w;
        if (compRef(A.vcell, v2, k) == cs.x) compRef(A.vcell, v2, k) = cs.y;
        if (compRef(A.vnbr, vs.y, k) == v1) compRef(A.vnbr, vs.y, k) = v2;
        if (compRef(A.vnbr, vs.z, k) == v2) compRef(A.vnbr, vs.z, k) = v1;
        if (compRef(A.vnbr, v1, k) == vs.y) compRef(A.vnbr, v1, k) = vs.z;
        if (compRef(A.vnbr, v2, k) == vs.z) compRef(A.vnbr, v2, k) = vs.y;
    }
}
// The rotation of v1 and v2 by a quarter turn about their midpoint and their separation
// (sphericalVertexModel.cpp:495-515), from their positions and that of the third vertex vC.
__device__ void t1_move_pair(const ApplyArgs& A, int v1, int v2, D3 p1, D3 p2, D3 vC) {
    D3 mid{__dmul_rn(0.5, __dadd_rn(p1.x, p2.x)), __dmul_rn(0.5, __dadd_rn(p1.y, p2.y)), __dmul_rn(0.5, __dadd_rn(p1.z, p2.z))};
    mid = renorm_exact(mid, 1.0);
    double det = vC.x * (p1.y * p2.z - p1.z * p2.y) + vC.y * (p1.z * p2.x - p1.x * p2.z) + vC.z * (p1.x * p2.y - p1.y * p2.x);
    det = det > 0 ? 1. : -1.;
    // theta = -0.5 det kPI (sphericalVertexModel.cpp:507-508)
    p1 = rodrigues(p1, mid, kCosHalfPi, -det);
    p2 = rodrigues(p2, mid, kCosHalfPi, -det);
    const D3 diff{__dmul_rn(0.5, __dsub_rn(p1.x, p2.x)), __dmul_rn(0.5, __dsub_rn(p1.y, p2.y)), __dmul_rn(0.5, __dsub_rn(p1.z, p2.z))};
    p1 = D3{__dadd_rn(p1.x, diff.x), __dadd_rn(p1.y, diff.y), __dadd_rn(p1.z, diff.z)};
    p2 = D3{__dsub_rn(p2.x, diff.x), __dsub_rn(p2.y, diff.y), __dsub_rn(p2.z, diff.z)};
    const double R = aR(A, v1);
    apos_st(A, v1, renorm_exact(p1, R));
    apos_st(A, v2, renorm_exact(p2, R));
}
constexpr unsigned kFull = 0xffffffffu;
// t1_move_pair by a whole warp: the rotation and renormalisation of v1 on the even lanes and of v2
// on the odd ones, the rest on every lane alike (an FP64 instruction costs a warp the same
// whatever its active lanes, so the pair takes two-thirds of the instructions of one thread).
// Lane 0 stores v1, lane 1 stores v2; the values are t1_move_pair's.
__device__ void t1_move_pair_warp(const ApplyArgs& A, int v1, int v2, D3 p1, D3 p2, D3 vC, int lane) {
    D3 mid{__dmul_rn(0.5, __dadd_rn(p1.x, p2.x)), __dmul_rn(0.5, __dadd_rn(p1.y, p2.y)), __dmul_rn(0.5, __dadd_rn(p1.z, p2.z))};
    mid = renorm_exact(mid, 1.0);
    double det = vC.x * (p1.y * p2.z - p1.z * p2.y) + vC.y * (p1.z * p2.x - p1.x * p2.z) + vC.z * (p1.x * p2.y - p1.y * p2.x);
    det = det > 0 ? 1. : -1.;
    const bool second = lane & 1;
    const D3 q = rodrigues(second ? p2 : p1, mid, kCosHalfPi, -det);
    const D3 o{__shfl_xor_sync(kFull, q.x, 1), __shfl_xor_sync(kFull, q.y, 1), __shfl_xor_sync(kFull, q.z, 1)};
    const D3 r1 = second ? o : q, r2 = second ? q : o;
    const D3 diff{__dmul_rn(0.5, __dsub_rn(r1.x, r2.x)), __dmul_rn(0.5, __dsub_rn(r1.y, r2.y)), __dmul_rn(0.5, __dsub_rn(r1.z, r2.z))};
    const D3 w = second ? D3{__dsub_rn(r2.x, diff.x), __dsub_rn(r2.y, diff.y), __dsub_rn(r2.z, diff.z)}
                        : D3{__dadd_rn(r1.x, diff.x), __dadd_rn(r1.y, diff.y), __dadd_rn(r1.z, diff.z)};
    const D3 n = renorm_exact(w, aR(A, v1));
    if (lane == 0) apos_st(A, v1, n);
    else if (lane == 1) apos_st(A, v2, n);
}
__device__ __forceinline__ int4 shfl0(int4 a) {
    return make_int4(__shfl_sync(kFull, a.x, 0), __shfl_sync(kFull, a.y, 0), __shfl_sync(kFull, a.z, 0),
                     __shfl_sync(kFull, a.w, 0));
}
// t1_flip by a whole warp (every lane calls it with the same arguments; p1, p2 are the old
// positions of v1 and v2): lane 0 plans and commits the topology, the warp moves the pair.  Same
// writes as t1_flip; the warp's lanes see them after it returns.
__device__ bool t1_flip_warp(const ApplyArgs& A, int v1, int v2, int4& cs, int4& vs, UndoEntry* undo, int* undoRings,
                             D3 p1, D3 p2, int lane) {
    int ok = 0;
    FlipPlan16 F;
    if (ring16_ok(A) && lane == 0) ok = t1_plan16(A, v1, v2, cs, vs, F);
    ok = ring16_ok(A) ? __shfl_sync(kFull, ok, 0) : 2;
    if (ok == 2) {  // other ring capacities, or rings of more than 16 entries: lane 0 alone
        if (lane == 0) ok = t1_flip_any(A, v1, v2, cs, vs, undo, undoRings) ? 1 : 0;
        ok = __shfl_sync(kFull, ok, 0);
        cs = shfl0(cs);
        vs = shfl0(vs);
        __syncwarp();
        return ok != 0;
    }
    if (!ok) return false;
    cs = shfl0(cs);
    vs = shfl0(vs);
    t1_move_pair_warp(A, v1, v2, p1, p2, apos(A, vs.z), lane);
    if (lane == 0) t1_commit16(A, v1, v2, cs, vs, F, undo, undoRings, p1, p2);
    __syncwarp();
    return true;
}

// Ring bookkeeping (vrpos/vlast/vnext) and corners of the cells whose rings a T1 pass changed,
// and fresh spherical coordinates of their vertices.  Grid-stride over (touched cell, ring
// position); every written value depends only on the final rings and positions, so duplicate
// entries and concurrent writers of the same vertex agree.
__global__ void k_t1_patch(ApplyArgs A, T1Scratch t1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the pass's largest ring, for the host's capacity check
        *(volatile int*)A.ringMaxOut = *(volatile int*)A.ringMax;
        __threadfence_system();
    }
    // appends past the list's capacity roll the pass back; a pass cut short by an exhausted barrier
    // wait may leave the counter above it, and only the stored entries are read
    const int ntRaw = *(volatile int*)(t1.ctr + 5);
    const int nt = min(ntRaw, t1.touchedCap);
    const long gs = (long)gridDim.x * blockDim.x, g0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
    // A host-buffer step's output: the force kernel wrote the moved positions; the flips moved
    // vertices of the touched cells, whose ring entries below rewrite them.  A list that may have
    // lost entries (full) rewrites every vertex instead.
    const bool hostAll = A.hostOut && ntRaw > t1.touchedCap - 4;
    if (hostAll)
        for (long v = g0; v < A.nV; v += gs) {
            const D3 p = ld3(A.pos, (int)v);
            A.hostOut[3 * v] = p.x; A.hostOut[3 * v + 1] = p.y; A.hostOut[3 * v + 2] = p.z;
        }
    // The touched cells go round-robin over the blocks (cell i to block i mod gridDim, 32 of a
    // block's at a time), and each block packs its cells' ring entries onto consecutive threads: the
    // few hundred cells of a pass then spread over all SMs, with every lane of a busy warp on a real
    // entry (a flat index over (cell, slot < capacity) leaves most lanes and most SMs idle).
    __shared__ int patchCell[32], patchOff[33];
    for (int base = blockIdx.x; base < nt; base += 32 * gridDim.x) {
        if (threadIdx.x < 32) {
            const int i = base + (int)gridDim.x * (int)threadIdx.x;
            const int cell = i < nt ? t1.touched[i] : -1;
            const int cnt = cell >= 0 ? A.ringCount[cell] : 0;
            int incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)threadIdx.x >= o) incl += y;
            }
            patchCell[threadIdx.x] = cell;
            patchOff[threadIdx.x] = incl - cnt;
            if (threadIdx.x == 31) patchOff[32] = incl;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < patchOff[32]; e += blockDim.x) {
            int j = 0;
            while (patchOff[j + 1] <= e) ++j;
            const int cell = patchCell[j], k = e - patchOff[j];
            const int n = A.ringCount[cell];
            const int* rg = A.ring + (long)cell * A.Wc;
            const int u = rg[k];
            const int last = rg[k == 0 ? n - 1 : k - 1], next = rg[k + 1 == n ? 0 : k + 1];
            for (int s = 0; s < 3; ++s)
                if (compRef(A.vcell, u, s) == cell) {
                    compRef(A.vrpos, u, s) = k;
                    compRef(A.vlast, u, s) = last;
                    compRef(A.vnext, u, s) = next;
                }
            const D3 pl = apos(A, last), p = apos(A, u), px = apos(A, next);
            if (A.hostOut && !hostAll) { A.hostOut[3L * u] = p.x; A.hostOut[3L * u + 1] = p.y; A.hostOut[3L * u + 2] = p.z; }
            if (A.pos32) {
                A.corner[(long)cell * A.Wc + k] =
                    make_double2((double)arc32(A.pos32[last], A.pos32[u], (float)aR(A, u)), included_angle_clamped<true>(pl, p, px));
            } else {
                A.corner[(long)cell * A.Wc + k] = make_double2(geodesic<true>(pl, p, A.R), included_angle<true>(pl, p, px));
                A.vsph[u] = sph_coords<true>(p);
            }
        }
        __syncthreads();
    }
}

// Restores everything a committed flip overwrote.
__device__ void t1_undo(const ApplyArgs& A, const UndoEntry& u, const int* undoRings) {
    apos_st(A, u.v1, D3{u.p1.x, u.p1.y, u.p1.z});
    apos_st(A, u.v2, D3{u.p2.x, u.p2.y, u.p2.z});
    A.vcell[u.v1] = u.vc1; A.vcell[u.v2] = u.vc2;
    A.vnbr[u.v1] = u.vn[0]; A.vnbr[u.v2] = u.vn[1]; A.vnbr[u.b] = u.vn[2]; A.vnbr[u.c] = u.vn[3];
    for (int q = 0; q < 4; ++q) {
        const int cell = u.cells[q];
        A.ringCount[cell] = u.counts[q];
        for (int k = 0; k < u.counts[q]; ++k) A.ring[(long)cell * A.Wc + k] = undoRings[q * A.Wc + k];
    }
}

// A position as the T1 test reads it: FP64, or FP32 with the replica index (mixed form; the
// conversions to double and back are exact).
struct TPos { double x, y, z; int rep; };
__device__ __forceinline__ TPos tpos(const ApplyArgs& A, int i) {
    if (A.pos32) {
        const float4 q = A.pos32[i];
        return TPos{q.x, q.y, q.z, rep_of(q)};
    }
    const D3 p = ld3(A.pos, i);
    return TPos{p.x, p.y, p.z, 0};
}
// The length test of t1_candidate on positions already loaded (a = vertex v, b = neighbour u).
__device__ __forceinline__ bool t1_short(const ApplyArgs& A, const TPos& a, const TPos& b) {
    if (A.pos32)
        return arc32(make_float4((float)a.x, (float)a.y, (float)a.z, 0.f), make_float4((float)b.x, (float)b.y, (float)b.z, 0.f),
                     (float)A.repR[a.rep]) < (float)A.t1Threshold;
    return shorter_than<true>(D3{a.x, a.y, a.z}, D3{b.x, b.y, b.z}, A.R, A.t1Threshold, A.cosLo, A.cosHi, A.s2Lo, A.s2Hi);
}

__device__ __forceinline__ bool t1_candidate(const ApplyArgs& A, int q) {
    const int v = q / 3, s = q - 3 * (q / 3);
    const int u = compRef(A.vnbr, v, s);
    if (!(v < u)) return false;
    if (A.pos32) return arc32(A.pos32[v], A.pos32[u], (float)aR(A, v)) < (float)A.t1Threshold;
    return shorter_than<true>(ld3(A.pos, v), ld3(A.pos, u), A.R, A.t1Threshold, A.cosLo, A.cosHi, A.s2Lo, A.s2Hi);
}

// Applies the flagged T1 flips in the order of the CPU loop (ascending vertex1, then slot),
// re-testing each edge against the current state when it is reached and re-testing, after every
// flip, the edges of the six vertices whose slots or positions the flip changed.  Flags ahead of
// the extracted window live in the bitmap; flags inside it in a small heap.  Afterwards every
// cell whose ring changed gets its ring bookkeeping (vrpos/vlast/vnext) and corners rebuilt.
__global__ void __launch_bounds__(kApplyThreads) k_t1_apply(ApplyArgs A, T1Scratch t1) {
    __shared__ int buf[kExtractCap];
    __shared__ int heap[kHeapCap];
    __shared__ int nbuf, head, nheap, extractWord, nTouched;
    __shared__ int nSummaryHit;
    const int tid = threadIdx.x;
    const int total = *t1.count;
    if (total == 0) {
        if (tid == 0) {
            *t1.pass += 1;
            t1.stats[0] += 1;
            if (A.bumpStep) *A.stepCounter += 1ull;
        }
        return;
    }
    // touched cells are appended after those of the parallel pass's segments that succeeded
    if (tid == 0) { nbuf = 0; head = 0; nheap = 0; extractWord = 0; nTouched = t1.ctr[5]; t1.stats[6] = *t1.flipCount; }
    __syncthreads();
    int lastProcessed = -1;
    while (true) {
        // Refill the window from the bitmap when both the window and the heap are empty.
        if (head == nbuf && nheap == 0) {
            __syncthreads();
            if (tid == 0) { nSummaryHit = 0x7fffffff; }
            __syncthreads();
            const int sw0 = extractWord >> 5;
            for (int sw = sw0 + tid; sw < t1.nSummary; sw += blockDim.x) {
                if (t1.summary[sw] != 0u) { atomicMin(&nSummaryHit, sw); break; }
            }
            __syncthreads();
            const int sw = nSummaryHit;
            if (sw == 0x7fffffff) break;  // uniform: nothing left
            // positions of the 32 bitmap words under summary word sw, in ascending order
            unsigned word = 0u;
            const int w = sw * 32 + tid;
            if (tid < 32 && w < t1.nWords) word = t1.bits[w];
            int cnt = __popc(word);
            int incl = cnt;
            if (tid < 32) {
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if ((tid & 31) >= o) incl += y;
                }
            }
            if (tid < 32) {
                int at = incl - cnt;
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1u;
                    buf[at++] = w * 32 + b;
                }
                if (w < t1.nWords) t1.bits[w] = 0u;
                if (tid == 31) { nbuf = incl; head = 0; extractWord = (sw + 1) * 32; t1.summary[sw] = 0u; }
            }
            __syncthreads();
            continue;
        }
        // Sequential part: one candidate by thread 0.
        if (tid == 0) {
            int q;
            const bool fromHeap = nheap > 0 && (head == nbuf || heap[0] < buf[head]);
            if (fromHeap) {
                q = heap[0];
                const int x = heap[--nheap];
                int i = 0;
                while (true) {
                    int l = 2 * i + 1, r = l + 1, mI = i;
                    int mv = x;
                    if (l < nheap && heap[l] < mv) { mI = l; mv = heap[l]; }
                    if (r < nheap && heap[r] < mv) { mI = r; mv = heap[r]; }
                    if (mI == i) break;
                    heap[i] = heap[mI];
                    i = mI;
                }
                if (nheap > 0) heap[i] = x;
            } else {
                q = buf[head++];
            }
            if (q != lastProcessed) {
                lastProcessed = q;
                if (t1_candidate(A, q)) {
                    const int v1 = q / 3, v2 = compRef(A.vnbr, v1, q - 3 * v1);
                    int4 cs, vs;
                    if (t1_flip(A, v1, v2, cs, vs)) {
                        const int fc = atomicAdd(t1.flipCount, 1);
                        if (fc < t1.flipLogCap) {
                            int* e = t1.flipLog + 4 * fc;
                            e[0] = *t1.pass; e[1] = q; e[2] = v1; e[3] = v2;
                        }
                        if (nTouched + 4 <= t1.touchedCap) {
                            t1.touched[nTouched++] = cs.x; t1.touched[nTouched++] = cs.y;
                            t1.touched[nTouched++] = cs.z; t1.touched[nTouched++] = cs.w;
                        } else {
                            atomicOr(A.status, SVM_DEV_T1_OVERFLOW);
                        }
                        const int aff[6] = {v1, v2, vs.x, vs.y, vs.z, vs.w};
                        const int windowEnd = extractWord * 32;
                        for (int a = 0; a < 6; ++a)
                            for (int s = 0; s < 3; ++s) {
                                const int r = 3 * aff[a] + s;
                                if (r <= q || !t1_candidate(A, r)) continue;
                                if (r >= windowEnd) {
                                    t1.bits[r >> 5] |= 1u << (r & 31);
                                    t1.summary[r >> 10] |= 1u << ((r >> 5) & 31);
                                } else if (nheap < kHeapCap) {
                                    int i = nheap++;
                                    while (i > 0 && heap[(i - 1) / 2] > r) { heap[i] = heap[(i - 1) / 2]; i = (i - 1) / 2; }
                                    heap[i] = r;
                                } else {
                                    atomicOr(A.status, SVM_DEV_T1_OVERFLOW);
                                }
                            }
                    }
                }
            }
        }
        __syncthreads();
    }
    // ring bookkeeping and corners of the touched cells: k_t1_patch
    __syncthreads();
    if (tid == 0) {
        t1.ctr[5] = nTouched;
        *t1.count = 0;
        *t1.pass += 1;
        t1.stats[0] += 1;
        t1.stats[3] += *t1.flipCount - t1.stats[6];
        if (A.bumpStep) *A.stepCounter += 1ull;
    }
}


// ---- parallel T1 pass -------------------------------------------------------------------------
// Footprint of the edge at position p: every vertex and cell that testing, flipping and
// re-testing after the flip can read or write (v1, v2 and their neighbours; the cells of v1 and
// v2).  Two positions with disjoint footprints commute.
__device__ __forceinline__ void t1_footprint(const ApplyArgs& A, int p, int* f) {
    const int v1 = p / 3, v2 = compRef(A.vnbr, v1, p - 3 * v1);
    const int4 n1 = A.vnbr[v1], n2 = A.vnbr[v2], c1 = A.vcell[v1], c2 = A.vcell[v2];
    f[0] = v1; f[1] = v2; f[2] = n1.x; f[3] = n1.y; f[4] = n1.z; f[5] = n2.x; f[6] = n2.y; f[7] = n2.z;
    f[8] = c1.x; f[9] = c1.y; f[10] = c1.z; f[11] = c2.x; f[12] = c2.y; f[13] = c2.z;
}

// Vertex a of (v1, v2, vs.x, vs.y, vs.z, vs.w): the six whose slots a flip re-tests.
__device__ __forceinline__ int pick_aff(int a, int v1, int v2, const int4& vs) {
    return a == 0 ? v1 : a == 1 ? v2 : a == 2 ? vs.x : a == 3 ? vs.y : a == 4 ? vs.z : vs.w;
}

constexpr int kParThreads = 512;        // one segment: the whole sphere
constexpr int kParThreadsBatch = 128;   // one segment per replica (4 resident blocks per SM at 128 registers)
constexpr int kCoopThreads = 256;       // per block of a cooperative single-sphere pass

// Block-wide exclusive scan of one int per thread; returns the block total in *total.
__device__ int block_excl_scan(int v, int* total) {
    __shared__ int warpTot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warpTot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int t = lane < nw ? warpTot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warpTot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    const int before = (warp == 0 ? 0 : warpTot[warp - 1]) + incl - v;
    *total = warpTot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

// Barrier of all blocks of a cooperative launch (co-resident by construction): the last block
// to arrive resets the count and advances the generation; the others poll the generation, at most
// kBarrierSpins times, after which the wait gives up and the barrier returns false.  Fences before
// the arrival and after the wait order every block's writes before the barrier with every read
// after it.
constexpr int kBarrierSpins = 1 << 20;  // at least 67 ms with 64 ns naps (svm_model_set_t1_wait_limit)
__device__ bool grid_barrier(T1Ctl* ctl, int spinLimit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned gen = *(volatile unsigned*)&ctl->barGen;
        __threadfence();
        if (atomicAdd(&ctl->barCount, 1u) == gridDim.x - 1) {
            *(volatile unsigned*)&ctl->barCount = 0u;
            __threadfence();
            atomicAdd(&ctl->barGen, 1u);
        } else {
            int spins = 0;
            while (*(volatile unsigned*)&ctl->barGen == gen) {
                if (++spins > spinLimit) { ok = 0; break; }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Applies the flagged flips with the result of the CPU's sequential order, in parallel rounds of
// deterministic reservations: every pending position writes its own value into the footprint
// cells (atomicMin); a position whose whole footprint holds its value runs (test, flip,
// re-test of the affected edges), the others wait for the next round.  Overlapping positions
// therefore run in ascending order and disjoint ones commute.  A position created by a re-test
// that overlaps a higher position which has already run would need the CPU order broken; that is
// detected through the per-vertex/per-cell record of the highest position that ran, and then
// every flip of the pass is undone and the bitmap restored for k_t1_apply, which then applies
// the flips one by one.  On success *t1.count is cleared so k_t1_apply returns at once.
//
// kCoop = false: one block per segment of the position space: the whole sphere, or one replica
// of a batch (whose flagged edges share no vertex or cell with another replica's, and whose
// positions are a contiguous range).  A block's lists, footprints, commit list and undo log are
// its own slices of the scratch arrays; the touched-cell list and the flip log are shared (atomic
// appends).  A block whose pass is not the sequential order undoes its own flips, marks their log
// entries invalid (pass -1) and restores its segment's flags, which k_t1_apply then replays; the
// counter of flagged positions drops by the positions of every block that succeeded.  The last
// block to finish (ticket) folds the round count into the statistics and clears summary bits
// whose bitmap words are empty.
// kCoop = true: one segment (the whole sphere) over all blocks of a cooperative launch, so that the
// flips' FP64 work spreads over many SMs instead of one: block 0 extracts the flagged positions,
// position i of a round runs on block i mod gridDim.x, the phases are separated by grid barriers
// instead of block barriers, the counters live in global memory (t1.ctl), and block 0 alone
// finishes the pass (rollback, statistics, cleanup).  Same decisions, same results.
template <bool kCoop>
__global__ void __launch_bounds__(kCoop ? kCoopThreads : kParThreads) k_t1_parallel(ApplyArgs A, T1Scratch t1, const int* __restrict__ segOff,
                                                             int listPad, int undoPer) {
    __shared__ T1Ctl sctl;
    T1Ctl* ctl = kCoop ? t1.ctl : &sctl;
    const int tid = threadIdx.x, seg = kCoop ? 0 : blockIdx.x;
    const bool leader = !kCoop || blockIdx.x == 0;  // extracts the positions and finishes the pass
    // this thread's first position of a round and the stride (reserve and release phases), and
    // this warp's (run phase: one warp per position).  Consecutive positions go to different
    // blocks of a cooperative grid.
    const int lane = tid & 31, warps = blockDim.x >> 5;
    const int gi = kCoop ? blockIdx.x + gridDim.x * tid : tid;
    const int gs = kCoop ? gridDim.x * blockDim.x : blockDim.x;
    const int wi = kCoop ? blockIdx.x + gridDim.x * (tid >> 5) : (tid >> 5);
    const int ws = kCoop ? gridDim.x * warps : warps;
    // one segment and nothing flagged: nothing to do.  (With several segments every block runs:
    // the last one to finish does the pass's cleanup.)  The count is read by every block before
    // the first grid barrier, so before block 0 can change it.
    if ((kCoop || gridDim.x == 1) && *t1.count == 0) return;
    auto group_sync = [&]() -> bool {
        if (!kCoop) { __syncthreads(); return true; }
        if (grid_barrier(ctl, A.barrierSpins)) return true;
        if (tid == 0) atomicOr(A.status, SVM_DEV_T1_TIMEOUT);
        return false;
    };
    const int qLo = segOff ? 3 * segOff[seg] : 0;
    const int qHi = segOff ? 3 * segOff[seg + 1] : 3 * A.nV;
    const int base = qLo / 2 + listPad * seg;
    const int capB = (qHi - qLo) / 2 + listPad;
    int* cur = t1.listA + base;
    int* nxt = t1.listB + base;
    int* orig = t1.listOrig + base;
    int* fpB = t1.fp + (long)base * kFootprint;
    int* comB = t1.comList + (long)base * kFootprint;
    UndoEntry* undoB = t1.undo + (long)seg * undoPer;
    int* undoRingsB = t1.undoRings + (long)seg * undoPer * 4 * A.Wc;
    // a cooperative pass starts from zeroed counters (cleared with the launch's memset)
    if (!kCoop && tid == 0) {
        sctl.nCur = 0; sctl.flag = 0; sctl.nWordsHit = 0; sctl.undo = 0; sctl.rollback = 0; sctl.exec = 0;
        sctl.flips = 0; sctl.next[0] = 0; sctl.next[1] = 0; sctl.late = 0;
    }
    __syncthreads();
    // phase clocks (block 0, thread 0; svm_model_t1_clocks): extraction, reserve, run, release, end
    const bool clk = t1.clocks && seg == 0 && blockIdx.x == 0 && tid == 0;
    long long c0 = clk ? clock64() : 0, c1 = c0;
    auto lap = [&](int slot) {
        if (!clk) return;
        c1 = clock64();
        atomicAdd(t1.clocks + slot, (unsigned long long)(c1 - c0));
        c0 = c1;
    };
    // 1. the segment's flagged positions, ascending: the bitmap words whose summary bit is set
    //    (a superset of the non-empty words) into `nxt`, then their set bits inside [qLo, qHi)
    const int wLo = qLo >> 5, wHi = (qHi + 31) >> 5;  // words [wLo, wHi)
    if (leader) {
        for (int base2 = wLo >> 5; base2 < ((wHi + 31) >> 5); base2 += blockDim.x) {
            const int sw = base2 + tid;
            unsigned sword = sw < ((wHi + 31) >> 5) && sw < t1.nSummary ? t1.summary[sw] : 0u;
            // keep the summary bits of words inside [wLo, wHi)
            if (sw == (wLo >> 5)) sword &= ~0u << (wLo & 31);
            if (sw == ((wHi - 1) >> 5) && (wHi & 31)) sword &= (1u << (wHi & 31)) - 1u;
            int tot;
            const int off = block_excl_scan(__popc(sword), &tot);
            unsigned x = sword;
            int at = ctl->nWordsHit + off;
            while (x) {
                const int b = __ffs(x) - 1;
                x &= x - 1u;
                const int w = sw * 32 + b;
                if (w < t1.nWords && at < capB) nxt[at] = w;
                ++at;
            }
            __syncthreads();
            if (tid == 0) ctl->nWordsHit = min(ctl->nWordsHit + tot, capB);
            __syncthreads();
        }
        const int nHit = ctl->nWordsHit;
        for (int b0 = 0; b0 < nHit; b0 += blockDim.x) {
            const int i = b0 + tid;
            const int w = i < nHit ? nxt[i] : -1;
            unsigned word = (w >= 0 && w < t1.nWords) ? t1.bits[w] : 0u;
            if (w == (qLo >> 5)) word &= ~0u << (qLo & 31);
            if (w >= 0 && w == ((qHi - 1) >> 5) && (qHi & 31)) word &= (1u << (qHi & 31)) - 1u;
            int tot;
            const int off = block_excl_scan(__popc(word), &tot);
            const int n0 = ctl->nCur;
            if (n0 + tot > capB) { if (tid == 0) ctl->flag = 1; __syncthreads(); break; }
            unsigned x = word;
            int at = n0 + off;
            while (x) {
                const int b = __ffs(x) - 1;
                x &= x - 1u;
                cur[at] = w * 32 + b;
                orig[at] = w * 32 + b;
                ++at;
            }
            __syncthreads();
            if (tid == 0) ctl->nCur = n0 + tot;
            __syncthreads();
        }
    }
    if (!group_sync()) return;
    // uniform over the group from here on: every thread reads the same counters after a barrier
    const int nOrig = *(volatile int*)&ctl->nCur;
    int nCur = nOrig;
    int par = 0;  // the round's next-list counter: ctl->next[par]
    int rounds = 0;
    bool rollback = *(volatile int*)&ctl->flag != 0;  // more candidates than the slice holds: k_t1_apply takes them all
    lap(0);
    // 2. rounds
    while (!rollback && nCur > 0) {
        ++rounds;
        // reserve
        for (int i = gi; i < nCur; i += gs) {
            const int p = cur[i];
            int* f = fpB + (long)i * kFootprint;
            t1_footprint(A, p, f);
            bool late = false;
            for (int k = 0; k < 8; ++k) { late |= t1.comV[f[k]] > p; atomicMin(t1.resV + f[k], p); }
            for (int k = 8; k < kFootprint; ++k) { late |= t1.comC[f[k]] > p; atomicMin(t1.resC + f[k], p); }
            if (late) atomicExch(&ctl->late, 1);
        }
        if (!group_sync()) return;
        lap(1);
        // `late` is written only while reserving and `rollback` only while running, so each is
        // read after the barrier that ends its phase, by every block alike
        if (*(volatile int*)&ctl->late) {
            // release this round's reservations before leaving
            for (int i = gi; i < nCur; i += gs) {
                const int* f = fpB + (long)i * kFootprint;
                for (int k = 0; k < 8; ++k) t1.resV[f[k]] = kResFree;
                for (int k = 8; k < kFootprint; ++k) t1.resC[f[k]] = kResFree;
            }
            rollback = true;
            break;
        }
        // run the positions that hold their whole footprint.  While the round's positions fit the
        // warps: one warp per position, its lanes sharing the reservation checks, the pair's
        // rotation and the 18 re-tests (an FP64 warp instruction costs the same for 1 or 32 lanes,
        // so a flip's FP64 chain shortens ~2.6x); beyond that (segments with many flips in a
        // round): one thread per position.  The same decisions and writes either way.
        if (nCur <= ws) {
        for (int i = wi; i < nCur; i += ws) {
            const int p = cur[i];
            const int* f = fpB + (long)i * kFootprint;
            // the edge (f[0], f[1]) is p's; its positions load alongside the reservation words (if
            // p does not hold its footprint they may be changing, and are not used)
            const int v1 = f[0], v2 = f[1];
            const TPos P1 = tpos(A, v1), P2 = tpos(A, v2);
            const int fk = lane < kFootprint ? f[lane] : 0;
            bool held = true;
            if (lane < kFootprint) held = (lane < 8 ? t1.resV[fk] : t1.resC[fk]) == p;
            if (!__all_sync(kFull, held)) {
                if (lane == 0) {
                    const int ni = atomicAdd(&ctl->next[par], 1);
                    if (ni < capB) nxt[ni] = p;
                    else atomicExch(&ctl->rollback, 1);
                }
                continue;
            }
            int ci = 0;
            if (lane == 0) ci = atomicAdd(&ctl->exec, 1);
            ci = __shfl_sync(kFull, ci, 0);
            if (ci >= capB) { if (lane == 0) atomicExch(&ctl->rollback, 1); continue; }
            if (lane < kFootprint) {
                comB[(long)ci * kFootprint + lane] = fk;
                atomicMax((lane < 8 ? t1.comV : t1.comC) + fk, p);
            }
            if (lane == 0) atomicAnd(t1.bits + (p >> 5), ~(1u << (p & 31)));
            if (!(v1 < v2 && t1_short(A, P1, P2))) continue;  // t1_candidate(A, p), on every lane alike
            int ui = 0;
            if (lane == 0) ui = atomicAdd(&ctl->undo, 1);
            ui = __shfl_sync(kFull, ui, 0);
            if (ui >= undoPer) { if (lane == 0) atomicExch(&ctl->rollback, 1); continue; }
            int4 cs, vs;
            UndoEntry* u = undoB + ui;
            if (!t1_flip_warp(A, v1, v2, cs, vs, u, undoRingsB + (long)ui * 4 * A.Wc, D3{P1.x, P1.y, P1.z},
                              D3{P2.x, P2.y, P2.z}, lane)) {
                if (lane == 0) u->v1 = -1;  // nothing was written
                continue;
            }
            if (lane == 0) {
                atomicAdd(&ctl->flips, 1);
                const int fc = atomicAdd(t1.flipCount, 1);
                u->logIdx = fc;
                if (fc < t1.flipLogCap) {
                    int* e = t1.flipLog + 4 * fc;
                    e[0] = *t1.pass; e[1] = p; e[2] = v1; e[3] = v2;
                }
                const int tc = atomicAdd(t1.ctr + 5, 4);
                if (tc + 4 <= t1.touchedCap) {
                    t1.touched[tc] = cs.x; t1.touched[tc + 1] = cs.y; t1.touched[tc + 2] = cs.z; t1.touched[tc + 3] = cs.w;
                } else {
                    atomicExch(&ctl->rollback, 1);
                }
            }
            // re-test the 18 slots of the six vertices whose slots or positions the flip changed
            // (t1_candidate on each): lane l < 18 tests slot l % 3 of vertex l / 3 of
            // (v1, v2, vs.x, vs.y, vs.z, vs.w); lane 0 then flags the new candidates in that order
            bool again = false;
            if (lane < 18) {
                const int a = lane / 3, sl = lane - 3 * (lane / 3);
                const int v = pick_aff(a, v1, v2, vs);
                const int r = 3 * v + sl;
                const int w = compRef(A.vnbr, v, sl);
                again = r > p && r < qHi && v < w && t1_short(A, tpos(A, v), tpos(A, w));
            }
            const unsigned hits = __ballot_sync(kFull, again);
            if (lane == 0) {
                for (unsigned m = hits; m; m &= m - 1u) {
                    const int l = __ffs(m) - 1;
                    const int r = 3 * pick_aff(l / 3, v1, v2, vs) + (l - 3 * (l / 3));
                    const unsigned bit = 1u << (r & 31);
                    if (!(atomicOr(t1.bits + (r >> 5), bit) & bit)) {
                        atomicOr(t1.summary + (r >> 10), 1u << ((r >> 5) & 31));
                        const int ni = atomicAdd(&ctl->next[par], 1);
                        if (ni < capB) nxt[ni] = r;
                        else atomicExch(&ctl->rollback, 1);
                    }
                }
            }
        }
        } else {
        for (int i = gi; i < nCur; i += gs) {
            const int p = cur[i];
            const int* f = fpB + (long)i * kFootprint;
            bool ready = true;
            for (int k = 0; k < 8; ++k) ready &= t1.resV[f[k]] == p;
            for (int k = 8; k < kFootprint; ++k) ready &= t1.resC[f[k]] == p;
            if (!ready) {
                const int ni = atomicAdd(&ctl->next[par], 1);
                if (ni < capB) nxt[ni] = p;
                else atomicExch(&ctl->rollback, 1);
                continue;
            }
            const int ci = atomicAdd(&ctl->exec, 1);
            if (ci >= capB) { atomicExch(&ctl->rollback, 1); continue; }
            for (int k = 0; k < kFootprint; ++k) comB[(long)ci * kFootprint + k] = f[k];
            for (int k = 0; k < 8; ++k) atomicMax(t1.comV + f[k], p);
            for (int k = 8; k < kFootprint; ++k) atomicMax(t1.comC + f[k], p);
            atomicAnd(t1.bits + (p >> 5), ~(1u << (p & 31)));
            if (!t1_candidate(A, p)) continue;
            const int ui = atomicAdd(&ctl->undo, 1);
            if (ui >= undoPer) { atomicExch(&ctl->rollback, 1); continue; }
            const int v1 = f[0], v2 = f[1];
            int4 cs, vs;
            UndoEntry* u = undoB + ui;
            if (!t1_flip(A, v1, v2, cs, vs, u, undoRingsB + (long)ui * 4 * A.Wc)) {
                u->v1 = -1;  // nothing was written
                continue;
            }
            atomicAdd(&ctl->flips, 1);
            const int fc = atomicAdd(t1.flipCount, 1);
            u->logIdx = fc;
            if (fc < t1.flipLogCap) {
                int* e = t1.flipLog + 4 * fc;
                e[0] = *t1.pass; e[1] = p; e[2] = v1; e[3] = v2;
            }
            const int tc = atomicAdd(t1.ctr + 5, 4);
            if (tc + 4 <= t1.touchedCap) {
                t1.touched[tc] = cs.x; t1.touched[tc + 1] = cs.y; t1.touched[tc + 2] = cs.z; t1.touched[tc + 3] = cs.w;
            } else {
                atomicExch(&ctl->rollback, 1);
            }
            const int aff[6] = {v1, v2, vs.x, vs.y, vs.z, vs.w};
            for (int a = 0; a < 6; ++a)
                for (int sl = 0; sl < 3; ++sl) {
                    const int r = 3 * aff[a] + sl;
                    if (!(r > p && r < qHi && t1_candidate(A, r))) continue;
                    const unsigned bit = 1u << (r & 31);
                    if (!(atomicOr(t1.bits + (r >> 5), bit) & bit)) {
                        atomicOr(t1.summary + (r >> 10), 1u << ((r >> 5) & 31));
                        const int ni = atomicAdd(&ctl->next[par], 1);
                        if (ni < capB) nxt[ni] = r;
                        else atomicExch(&ctl->rollback, 1);
                    }
                }
        }
        }
        if (!group_sync()) return;
        lap(2);
        // release this round's reservations; the other next-list counter starts the next round at 0
        for (int i = gi; i < nCur; i += gs) {
            const int* f = fpB + (long)i * kFootprint;
            for (int k = 0; k < 8; ++k) t1.resV[f[k]] = kResFree;
            for (int k = 8; k < kFootprint; ++k) t1.resC[f[k]] = kResFree;
        }
        if (leader && tid == 0) ctl->next[par ^ 1] = 0;
        if (!group_sync()) return;
        nCur = min(*(volatile int*)&ctl->next[par], capB);
        par ^= 1;
        int* t = cur; cur = nxt; nxt = t;
        lap(3);
        if (*(volatile int*)&ctl->rollback) rollback = true;
    }
    if (!group_sync()) return;
    if (!leader) return;
    if (rollback) {
        if (tid == 0) {
            // undo this segment's flips, newest first, and invalidate their log entries
            const int nu = min(*(volatile int*)&ctl->undo, undoPer);
            for (int i = nu - 1; i >= 0; --i) {
                const UndoEntry& u = undoB[i];
                if (u.v1 < 0) continue;
                t1_undo(A, u, undoRingsB + (long)i * 4 * A.Wc);
                if (u.logIdx >= 0 && u.logIdx < t1.flipLogCap) t1.flipLog[4 * u.logIdx] = -1;
            }
        }
        __syncthreads();
        // the segment's flags back to the ones the test set: clear, then set the originals
        for (int w = wLo + tid; w < wHi; w += blockDim.x) {
            unsigned keep = 0u;  // bits of other segments in a shared boundary word
            if (w == (qLo >> 5)) keep |= ~(~0u << (qLo & 31));
            if (w == ((qHi - 1) >> 5) && (qHi & 31)) keep |= ~((1u << (qHi & 31)) - 1u);
            atomicAnd(t1.bits + w, keep);
        }
        __syncthreads();
        for (int i = tid; i < nOrig; i += blockDim.x) {
            const int q = orig[i];
            atomicOr(t1.bits + (q >> 5), 1u << (q & 31));
            atomicOr(t1.summary + (q >> 10), 1u << ((q >> 5) & 31));
        }
    }
    __syncthreads();
    const int ne = min(*(volatile int*)&ctl->exec, capB);
    for (int i = tid; i < ne; i += blockDim.x) {
        const int* f = comB + (long)i * kFootprint;
        for (int k = 0; k < 8; ++k) t1.comV[f[k]] = -1;
        for (int k = 8; k < kFootprint; ++k) t1.comC[f[k]] = -1;
    }
    __shared__ bool amLast;
    if (tid == 0) {
        atomicAdd(t1.stats + 1, nOrig);
        atomicAdd(t1.stats + 2, ne);
        atomicMax(t1.ctr + 6, rounds);
        if (rollback) atomicAdd(t1.stats + 5, 1);
        else {
            atomicAdd(t1.stats + 3, *(volatile int*)&ctl->flips);
            atomicSub(t1.count, nOrig);
        }
        __threadfence();
        amLast = kCoop || atomicAdd(t1.ctr + 7, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    lap(4);
    if (!amLast) return;
    if (tid == 0) t1.stats[4] += *(volatile int*)(t1.ctr + 6);
    // summary bits of words that are now empty
    for (int sw = tid; sw < t1.nSummary; sw += blockDim.x) {
        unsigned sword = *(volatile unsigned*)(t1.summary + sw);
        unsigned keep = sword;
        while (sword) {
            const int b = __ffs(sword) - 1;
            sword &= sword - 1u;
            const int w = sw * 32 + b;
            if (w >= t1.nWords || *(volatile unsigned*)(t1.bits + w) == 0u) keep &= ~(1u << b);
        }
        t1.summary[sw] = keep;
    }
}

// Ring bookkeeping for all vertices after a topology upload: for each cell and ring position,
// record it in the vertex's slot for that cell.
__global__ void k_ring_index(const int* __restrict__ ring, const int* __restrict__ ringCount, int Wc, int nC,
                             int4* vcell, int4* vlast, int4* vnext, int4* vrpos, int* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nC) return;
    const int n = ringCount[c];
    const int* rg = ring + (long)c * Wc;
    for (int k = 0; k < n; ++k) {
        const int u = rg[k];
        bool found = false;
        for (int s = 0; s < 3; ++s)
            if (compRef(vcell, u, s) == c) {
                compRef(vrpos, u, s) = k;
                compRef(vlast, u, s) = rg[k == 0 ? n - 1 : k - 1];
                compRef(vnext, u, s) = rg[k + 1 == n ? 0 : k + 1];
                found = true;
            }
        if (!found) atomicOr(status, SVM_DEV_BAD_TOPOLOGY);
    }
}

__global__ void k_energy(const double2* __restrict__ ap, const double2* __restrict__ pref, double Kr, int nC,
                         double* partials, unsigned* ticket, double* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (c < nC) {
        const double da = ap[c].x - pref[c].x, dp = ap[c].y - pref[c].y;
        e = __dadd_rn(__dmul_rn(__dmul_rn(Kr, da), da), __dmul_rn(dp, dp));
    }
    const double bs = block_sum(e);
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        amLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (amLast) {
        double s = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(partials + b);
        const double total = block_sum(s);
        if (threadIdx.x == 0) { *out = total; *ticket = 0u; }
    }
}

__global__ void k_widen4(const float4* __restrict__ in, double4_32a* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3(out, i, ld3(in, i));
}

// dynamicalFeatures::computeMSD / computeOverlapFunction (src/analysis/dynamicalFeatures.cpp:17-53)
// over the first `count` cells: geodesicDistance(initial, current) per cell, the squares summed
// (NaN distances skipped) and the distances below `cutoff` counted; both divided by count.  Block
// sums in a fixed order, then the last block.
template <class PT>
__global__ void k_dynamics(const double4_32a* __restrict__ ref, const PT* __restrict__ cur, int count, double R,
                           double cutoff, double* partials, int stride, unsigned* ticket, double* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0.0, in = 0.0;
    if (c < count) {
        const double d = geodesic(ld3(ref, c), ld3(cur, c), R);
        if (!isnan(d)) sq = __dmul_rn(d, d);
        if (d < cutoff) in = 1.0;
    }
    const double bs = block_sum(sq), bo = block_sum(in);
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        partials[stride + blockIdx.x] = bo;
        __threadfence();
        amLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (amLast) {
        double s = 0.0, o = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
            s += __ldcg(partials + b);
            o += __ldcg(partials + stride + b);
        }
        const double ts = block_sum(s), to = block_sum(o);
        if (threadIdx.x == 0) {
            out[0] = ts / count;
            out[1] = to / count;
            *ticket = 0u;
        }
    }
}

// ---- self-propelled particles (sphericalSelfPropelledParticle::integrateEOMCPU,
// src/updaters/sphericalSelfPropelledParticle.cpp:16-47) on the vertex model's directors ----------
// The displacement dt (v0 n + mu F) and the move, in place, every product and sum rounded as on the
// CPU (the director n as the previous step left it).
__global__ void k_spp_move(double4_32a* __restrict__ pos, const double4_32a* __restrict__ dir,
                           const double4_32a* __restrict__ force, double dt, double mu, double v0, int nV, double R) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const D3 n = ld3(dir, v), f = ld3(force, v);
    const D3 d{__dmul_rn(dt, __dadd_rn(__dmul_rn(v0, n.x), __dmul_rn(mu, f.x))),
               __dmul_rn(dt, __dadd_rn(__dmul_rn(v0, n.y), __dmul_rn(mu, f.y))),
               __dmul_rn(dt, __dadd_rn(__dmul_rn(v0, n.z), __dmul_rn(mu, f.z)))};
    st3(pos, v, move_exact(ld3(pos, v), d, R));
}
// After the move and its T1 flips: each director projected onto the tangent plane at its vertex and
// normalised (projectToTangentPlaneAndNormalize, sphericalDomain.h:173-177), then rotated about the
// vertex's position vector, unnormalised as the reference passes it (rodriguesRotation,
// inc/functions.h:175-181), by theta = r amp, amp = sqrt(2 dt tau) and r uniform in [-1/2, 1/2):
// injected (r[v]) or from Philox counter word 3 of (vertex, step).
template <int kNoise>
__global__ void k_spp_dirs(const double4_32a* __restrict__ pos, double4_32a* __restrict__ dir,
                           const double* __restrict__ r, uint64_t seed,
                           const unsigned long long* __restrict__ stepCounter, double amp, int nV) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const D3 p = ld3(pos, v);
    D3 n = ld3(dir, v);
    const double s = __ddiv_rn(dot3(n, p), dot3(p, p));
    n = D3{__dsub_rn(n.x, __dmul_rn(s, p.x)), __dsub_rn(n.y, __dmul_rn(s, p.y)), __dsub_rn(n.z, __dmul_rn(s, p.z))};
    const double inv = f64_div(1.0, f64_sqrt(dot3(n, n)));
    n = D3{__dmul_rn(inv, n.x), __dmul_rn(inv, n.y), __dmul_rn(inv, n.z)};
    double rv;
    if (kNoise == SVM_NOISE_BUFFER) {
        rv = r[v];
    } else {
        const unsigned long long step = *stepCounter;
        const uint4 q = philox4x32_10(make_uint4((unsigned)v, (unsigned)step, (unsigned)(step >> 32), 3u),
                                      make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
        rv = u53(q.x, q.y) - 0.5;
    }
    const double theta = __dmul_rn(rv, amp);
    const double c = cos(theta), sn = sin(theta);
    const D3 cp = cross3(p, n);
    const double w = __dmul_rn(1.0 - c, dot3(p, n));
    st3(dir, v, D3{__dadd_rn(__dadd_rn(__dmul_rn(c, n.x), __dmul_rn(sn, cp.x)), __dmul_rn(w, p.x)),
                   __dadd_rn(__dadd_rn(__dmul_rn(c, n.y), __dmul_rn(sn, cp.y)), __dmul_rn(w, p.y)),
                   __dadd_rn(__dadd_rn(__dmul_rn(c, n.z), __dmul_rn(sn, cp.z)), __dmul_rn(w, p.z))});
}

// ---- vectorial Vicsek alignment (sphericalVectorialVicsek::integrateEOMCPU,
// src/updaters/sphericalVectorialVicsek.cpp:5-60) on the vertex model's directors ------------------
// After the self-propelled move and its T1 flips, from the directors before this update: a random
// unit vector (u, w: phi = 2 pi u, theta = acos(2 w - 1)) projected onto the tangent plane at the
// vertex and normalised; the target (n_v + the three vertex neighbours' n) / 4 + eta point,
// projected and normalised.  u, w injected (r[2v], r[2v + 1]) or from Philox counter word 4.
template <int kNoise>
__global__ void k_vicsek_target(const double4_32a* __restrict__ pos, const double4_32a* __restrict__ dir,
                                const int4* __restrict__ vnbr, double4_32a* __restrict__ target,
                                const double* __restrict__ r, uint64_t seed,
                                const unsigned long long* __restrict__ stepCounter, double eta, int nV) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    double u, w;
    if (kNoise == SVM_NOISE_BUFFER) {
        u = r[2 * v]; w = r[2 * v + 1];
    } else {
        const unsigned long long step = *stepCounter;
        const uint4 q = philox4x32_10(make_uint4((unsigned)v, (unsigned)step, (unsigned)(step >> 32), 4u),
                                      make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
        u = u53(q.x, q.y); w = u53(q.z, q.w);
    }
    const D3 p = ld3(pos, v);
    const double phi = __dmul_rn(2.0 * 3.141592653589793, u), theta = acos(__dsub_rn(__dmul_rn(2.0, w), 1.0));
    const double st = sin(theta);
    D3 sp{__dmul_rn(st, cos(phi)), __dmul_rn(st, sin(phi)), cos(theta)};
    const double ps = __ddiv_rn(dot3(sp, p), dot3(p, p));
    sp = D3{__dsub_rn(sp.x, __dmul_rn(ps, p.x)), __dsub_rn(sp.y, __dmul_rn(ps, p.y)), __dsub_rn(sp.z, __dmul_rn(ps, p.z))};
    const double is = f64_div(1.0, f64_sqrt(dot3(sp, sp)));
    sp = D3{__dmul_rn(sp.x, is), __dmul_rn(sp.y, is), __dmul_rn(sp.z, is)};
    const int4 nb = vnbr[v];
    D3 t = ld3(dir, v);
    const int nbs[3] = {nb.x, nb.y, nb.z};
    for (int k = 0; k < 3; ++k) {
        const D3 o = ld3(dir, nbs[k]);
        t = D3{__dadd_rn(t.x, o.x), __dadd_rn(t.y, o.y), __dadd_rn(t.z, o.z)};
    }
    const double mi = 1.0 / 4.0;  // self plus three neighbours
    t = D3{__dadd_rn(__dmul_rn(t.x, mi), __dmul_rn(sp.x, eta)), __dadd_rn(__dmul_rn(t.y, mi), __dmul_rn(sp.y, eta)),
           __dadd_rn(__dmul_rn(t.z, mi), __dmul_rn(sp.z, eta))};
    const double ts = __ddiv_rn(dot3(t, p), dot3(p, p));
    t = D3{__dsub_rn(t.x, __dmul_rn(ts, p.x)), __dsub_rn(t.y, __dmul_rn(ts, p.y)), __dsub_rn(t.z, __dmul_rn(ts, p.z))};
    const double it = f64_div(1.0, f64_sqrt(dot3(t, t)));
    st3(target, v, D3{__dmul_rn(t.x, it), __dmul_rn(t.y, it), __dmul_rn(t.z, it)});
}
// n += (dt / tau)(target - n), projected onto the tangent plane and normalised.
__global__ void k_vicsek_update(const double4_32a* __restrict__ pos, double4_32a* __restrict__ dir,
                                const double4_32a* __restrict__ target, double rate, int nV) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const D3 p = ld3(pos, v), t = ld3(target, v);
    D3 n = ld3(dir, v);
    n = D3{__dadd_rn(n.x, __dmul_rn(rate, __dsub_rn(t.x, n.x))), __dadd_rn(n.y, __dmul_rn(rate, __dsub_rn(t.y, n.y))),
           __dadd_rn(n.z, __dmul_rn(rate, __dsub_rn(t.z, n.z)))};
    const double s = __ddiv_rn(dot3(n, p), dot3(p, p));
    n = D3{__dsub_rn(n.x, __dmul_rn(s, p.x)), __dsub_rn(n.y, __dmul_rn(s, p.y)), __dsub_rn(n.z, __dmul_rn(s, p.z))};
    const double inv = f64_div(1.0, f64_sqrt(dot3(n, n)));
    st3(dir, v, D3{__dmul_rn(n.x, inv), __dmul_rn(n.y, inv), __dmul_rn(n.z, inv)});
}

// ---- launch helpers --------------------------------------------------------------------------
static ApplyArgs apply_args(svm_model* m, int bump) {
    ApplyArgs A;
    A.pos32 = m->precision == SVM_PRECISION_MIXED ? m->pos32[m->cur] : nullptr;
    A.repR = m->repR;
    A.pos = m->pos[m->cur]; A.vsph = m->vsph; A.vcell = m->vcell; A.vnbr = m->vnbr; A.vlast = m->vlast;
    A.vnext = m->vnext; A.vrpos = m->vrpos; A.ring = m->ring; A.ringCount = m->ringCount; A.corner = m->corner;
    A.Wc = m->Wc; A.nV = m->nVertices; A.nC = m->nCells; A.R = m->R; A.t1Threshold = m->t1Threshold;
    A.status = m->status; A.stepCounter = m->stepCounter; A.bumpStep = bump;
    A.ringMax = m->ringMax; A.ringMaxOut = m->ringMaxHostDev; A.barrierSpins = m->t1WaitLimit;
    A.hostOut = A.pos32 ? nullptr : m->ioHostOut;
    t1_bracket(m->t1Threshold, m->R, &A.cosLo, &A.cosHi);
    t1_sin2_bracket(m->t1Threshold, m->R, &A.s2Lo, &A.s2Hi);
    return A;
}

int launch_corners(svm_model* m, bool t1test, bool vnormReady) {
    // FP64: k_vnorm (unless the moving kernel wrote the norms), k_edges, k_corner
    PhaseTimer pt(m, SVM_PHASE_CORNERS, m->precision == SVM_PRECISION_MIXED ? 1 : (vnormReady ? 2 : 3));
    if (m->precision == SVM_PRECISION_MIXED) {
        m->cornersValid = true;
        return m->nRep > 1 ? batch_tuned_corners(m, t1test) : mixed_launch_corners(m, t1test);
    }
    if (!m->edgeC) return SVM_ERR_ARG;  // FP64 corners exist for single spheres only
    const int bv = spread_block(m, m->nVertices);
    if (!vnormReady) k_vnorm<<<blocksFor(m->nVertices, bv), bv, 0, m->stream>>>(m->pos[m->cur], m->vnorm, m->nVertices);
    k_edges<<<blocksFor(m->nVertices, bv), bv, 0, m->stream>>>(m->pos[m->cur], m->vnorm, m->vsph, m->vnbr, m->edgeC,
                                                              m->edgeArc, m->nVertices, m->R, t1test ? 1 : 0,
                                                              m->t1Threshold, m->t1);
    // both corner kernels write the same values; the three-thread one is faster below ~100k vertices
    if (m->nVertices < kCornerSlotsBelow)
        k_corner_s<<<(m->nVertices + kCornerVerts - 1) / kCornerVerts, 3 * kCornerVerts, 0, m->stream>>>(
            m->pos[m->cur], m->vcell, m->vlast, m->vnext, m->vrpos, m->vnbr, m->edgeC, m->edgeArc, m->corner, m->Wc,
            m->nVertices, m->R);
    else
        k_corner<<<blocksFor(m->nVertices), kBlock, 0, m->stream>>>(m->pos[m->cur], m->vcell, m->vlast, m->vnext,
                                                                   m->vrpos, m->vnbr, m->edgeC, m->edgeArc, m->corner,
                                                                   m->Wc, m->nVertices, m->R);
    m->cornersValid = true;
    return check_launch();
}

int max_block_cells_batch() {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, (const void*)k_cells<float4>) != cudaSuccess) return 256;
    return a.maxThreadsPerBlock / 32 * 32;
}

static int launch_cells_batch(svm_model* m) {
    const int bs = m->blkCells;
    k_cells<float4><<<(m->nCells + bs - 1) / bs, bs, 0, m->stream>>>(
        m->pos32[m->cur], m->ring, m->ringCount, m->corner, m->Wc, m->nCells, m->R, m->repR, m->cellPos32, nullptr,
        m->ap, nullptr, nullptr, nullptr, nullptr, m->pref, m->dap32);
    return check_launch();
}

static int launch_cells(svm_model* m) {
    const bool mixed = m->precision == SVM_PRECISION_MIXED;
    const bool batch = m->nRep > 1;
    {
        PhaseTimer pt(m, SVM_PHASE_CELLS, batch ? 2 : 1);
        if (batch) {
            if (int rc = batch_tuned_cells(m, launch_cells_batch)) return rc;
            if (int rc = launch_rep_check(m)) return rc;
        } else if (mixed) {
            k_cells<float4><<<blocksFor(m->nCells), kBlock, 0, m->stream>>>(
                m->pos32[m->cur], m->ring, m->ringCount, m->corner, m->Wc, m->nCells, m->R, m->repR, m->cellPos32,
                nullptr, m->ap, m->partials, m->ticket, m->scalars, m->fallbackFlag, m->pref, m->dap32);
        } else {
            k_cells<double4_32a><<<blocksFor(m->nCells), kBlock, 0, m->stream>>>(
                m->pos[m->cur], m->ring, m->ringCount, m->corner, m->Wc, m->nCells, m->R, nullptr, m->cellPos,
                m->cellSph, m->ap, m->partials, m->ticket, m->scalars, m->fallbackFlag);
        }
    }
    PhaseTimer pt(m, SVM_PHASE_FALLBACK);
    const int nb = blocksFor(m->nCells);
    if (m->Wc <= 32) {
        const int nf = (m->nCells + kFanCells - 1) / kFanCells;
        if (mixed)
            k_fallback_fan<float4><<<nf, kFanThreads, 0, m->stream>>>(
                m->pos32[m->cur], m->ring, m->ringCount, m->cellPos32, m->Wc, m->nCells, m->R, m->fallbackFlag,
                batch ? m->repFlag : nullptr, m->repR, m->ap, m->pref, m->dap32);
        else
            k_fallback_fan<double4_32a><<<nf, kFanThreads, 0, m->stream>>>(
                m->pos[m->cur], m->ring, m->ringCount, m->cellPos, m->Wc, m->nCells, m->R, m->fallbackFlag, nullptr,
                nullptr, m->ap);
    } else if (mixed)
        k_fallback<float4><<<nb, kBlock, 0, m->stream>>>(m->pos32[m->cur], m->ring, m->ringCount, m->cellPos32, m->Wc,
                                                         m->nCells, m->R, m->fallbackFlag, batch ? m->repFlag : nullptr,
                                                         m->repR, m->ap, m->pref, m->dap32);
    else
        k_fallback<double4_32a><<<nb, kBlock, 0, m->stream>>>(m->pos[m->cur], m->ring, m->ringCount, m->cellPos, m->Wc,
                                                              m->nCells, m->R, m->fallbackFlag, nullptr, nullptr, m->ap);
    return check_launch();
}

int launch_geometry(svm_model* m) {
    int rc = SVM_OK;
    if (!m->cornersValid) rc = launch_corners(m, false);
    if (rc) return rc;
    return launch_cells(m);
}

// Blocks of a single sphere's parallel T1 pass: one, or a cooperative grid of about one block per
// 3000 vertices (from 20000 vertices on, at most the co-resident count), or the count set by
// svm_model_set_t1_blocks.
static int t1_coop_blocks(svm_model* m) {
    // co-resident blocks of k_t1_parallel<true>, per device (computed on the model's device, which
    // is current while its calls run); atomics, as host threads may drive models concurrently
    constexpr int kMaxDevices = 64;
    static std::atomic<int> maxCoopOf[kMaxDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    int maxCoop = dev >= 0 && dev < kMaxDevices ? maxCoopOf[dev].load(std::memory_order_relaxed) : 0;
    if (maxCoop == 0) {
        int sms = 0, perSm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_t1_parallel<true>, kCoopThreads, 0);
        maxCoop = std::max(1, sms * perSm);
        if (dev >= 0 && dev < kMaxDevices) maxCoopOf[dev].store(maxCoop, std::memory_order_relaxed);
    }
    int n = m->t1Blocks;
    if (n == 0) n = m->nVertices < 20000 ? 1 : std::max(8, std::min(152, m->nVertices / 3000));
    return std::min(n, maxCoop);
}

// Copies the first ringCount[c] entries of every ring from stride Wc to stride Wn (the rest -1).
__global__ void k_regrid_rings(const int* __restrict__ ring, int Wc, const int* __restrict__ ringCount, int nC,
                               int* __restrict__ out, int Wn) {
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= (long)nC * Wn) return;
    const int c = (int)(e / Wn), k = (int)(e % Wn);
    out[e] = k < ringCount[c] ? ring[(long)c * Wc + k] : -1;
}

// growCellVerticesList (sphericalVertexModel.cpp:733-758): the rings re-laid out at capacity Wn
// (rounded up to a multiple of 4, which keeps the 16-entry flip path), with the corner and undo
// arrays that share their stride.  The width of the storage changes no result; captured graphs,
// which hold the old arrays, are rebuilt on their next use.
int grow_rings(svm_model* m, int Wn) {
    Wn = (Wn + 3) & ~3;
    if (Wn <= m->Wc) return SVM_OK;
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    const long nC = m->nCells;
    int *ring = nullptr, *undoRings = nullptr;
    double2* corner = nullptr;
    if (cudaMalloc(&ring, sizeof(int) * nC * Wn) != cudaSuccess ||
        cudaMalloc(&corner, sizeof(double2) * nC * Wn) != cudaSuccess ||
        cudaMalloc(&undoRings, sizeof(int) * (size_t)m->t1.undoCap * 4 * Wn) != cudaSuccess) {
        cudaFree(ring); cudaFree(corner); cudaFree(undoRings);
        cudaGetLastError();
        return SVM_ERR_CUDA;
    }
    k_regrid_rings<<<blocksFor(nC * Wn), kBlock, 0, m->stream>>>(m->ring, m->Wc, m->ringCount, m->nCells, ring, Wn);
    if (check_launch() || cudaStreamSynchronize(m->stream) != cudaSuccess) {
        cudaFree(ring); cudaFree(corner); cudaFree(undoRings);
        return SVM_ERR_CUDA;
    }
    cudaFree(m->ring); cudaFree(m->corner); cudaFree(m->t1.undoRings);
    m->ring = ring; m->corner = corner; m->t1.undoRings = undoRings;
    m->Wc = Wn;
    m->cornersValid = false;
    m->paramsVersion++;
    m->ringGrowths++;
    return SVM_OK;
}

// Before a T1 pass launched outside a capture: grows the ring capacity when ringHeadroom or fewer
// slots are free in the largest ring.  The host first waits for the pass before last, so the
// maximum it reads lags at most two passes; a reading close to the capacity is confirmed after a
// synchronisation.  (Graph launches check between replays instead.)
int ensure_ring_headroom(svm_model* m) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(m->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return SVM_OK;
    cudaEvent_t& ev = m->passEv[m->passSlot];
    if (ev && cudaEventSynchronize(ev) != cudaSuccess) return SVM_ERR_CUDA;
    volatile int* h = m->ringMaxHost;
    if (*h + m->ringHeadroom < m->Wc) return SVM_OK;
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    const int mx = *h;
    if (mx + m->ringHeadroom < m->Wc) return SVM_OK;
    return grow_rings(m, mx + m->ringHeadroom + 8);
}
// Marks the end of a pass launched outside a capture (the wait of ensure_ring_headroom two passes on).
static int mark_pass(svm_model* m) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(m->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return SVM_OK;
    cudaEvent_t& ev = m->passEv[m->passSlot];
    if (!ev && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) { ev = nullptr; return SVM_ERR_CUDA; }
    if (cudaEventRecord(ev, m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    m->passSlot ^= 1;
    return SVM_OK;
}

int launch_t1_apply(svm_model* m, int bump) {
    if (int rc = ensure_ring_headroom(m)) return rc;
    PhaseTimer pt(m, SVM_PHASE_T1APPLY, 3);
    // touched-cell count (ctr[5]), per-pass round maximum (ctr[6]), block ticket (ctr[7]) and the
    // cooperative pass's counters and barrier (t1.ctl, after them)
    if (cudaMemsetAsync(m->t1.ctr + 5, 0, (3 + kT1CtlInts) * sizeof(int), m->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    const bool batch = m->nRep > 1;
    const int nSeg = batch ? m->nRep : 1;
    const int coop = batch ? 1 : t1_coop_blocks(m);
    if (coop > 1) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(coop);
        cfg.blockDim = dim3(kCoopThreads);
        cfg.stream = m->stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const int* noSeg = nullptr;
        if (cudaLaunchKernelEx(&cfg, k_t1_parallel<true>, apply_args(m, bump), m->t1, noSeg, kListPad,
                               m->t1.undoCap) != cudaSuccess)
            return SVM_ERR_CUDA;
    } else {
        k_t1_parallel<false><<<nSeg, batch ? kParThreadsBatch : kParThreads, 0, m->stream>>>(
            apply_args(m, bump), m->t1, batch ? m->repVertOff : nullptr, batch ? kListPadBatch : kListPad,
            m->t1.undoCap / nSeg);
    }
    k_t1_apply<<<1, kApplyThreads, 0, m->stream>>>(apply_args(m, bump), m->t1);
    k_t1_patch<<<2 * m->sms, 256, 0, m->stream>>>(apply_args(m, bump), m->t1);
    if (int rc = check_launch()) return rc;
    return mark_pass(m);
}

// The T1 edge test on its own (k_t1_test: the decisions of the test fused into the corner
// kernels), for a state whose corners are not needed before the positions change again.
int launch_t1_test(svm_model* m) {
    PhaseTimer pt(m, SVM_PHASE_CORNERS);
    double lo, hi, s2lo, s2hi;
    t1_bracket(m->t1Threshold, m->R, &lo, &hi);
    t1_sin2_bracket(m->t1Threshold, m->R, &s2lo, &s2hi);
    k_t1_test<<<blocksFor(m->nVertices), kBlock, 0, m->stream>>>(
        m->pos[m->cur], m->precision == SVM_PRECISION_MIXED ? m->pos32[m->cur] : nullptr, m->repR, m->vnbr,
        m->nVertices, m->R, m->t1Threshold, lo, hi, s2lo, s2hi, m->t1);
    return check_launch();
}

// One fused Brownian timestep (see the file header).  With `deferCorners` the moved state gets
// only the T1 test and flips, and its corners are left invalid: the next step computes them (for
// callers that replace the positions between steps, whose corners would otherwise be computed
// twice).  Positions, topology and every later value are the same either way.
static int bd_step(svm_model* m, double T, double dt, double mu, int noiseMode, const double* noise, uint64_t seed,
                   bool deferCorners = false) {
    int rc = SVM_OK;
    if (m->nRep > 1 && !capturing(m->stream) && (rc = update_rep_noise(m, dt, mu))) return rc;
    rc = launch_geometry(m);
    if (rc) return rc;
    const double fp = dt * mu;
    const double np = sqrt(2.0 * fp * T);
    const int nxt = 1 - m->cur;
    {
    PhaseTimer pt(m, SVM_PHASE_FORCE);
    if (m->precision == SVM_PRECISION_MIXED && m->nRep > 1)
        rc = batch_tuned_force_bd(m, T, dt, mu, noiseMode, noise, seed, nxt);
    else if (m->precision == SVM_PRECISION_MIXED)
        rc = mixed_launch_force_bd(m, T, dt, mu, noiseMode, noise, seed, nxt);
    else
        rc = launch_force_bd_fp64(m, np, fp, noiseMode, noise, seed, nxt);
    }
    if (rc || (rc = check_launch())) return rc;
    m->cur = nxt;
    if (deferCorners) {
        m->cornersValid = false;
        if (!m->restricted && (rc = launch_t1_test(m))) return rc;
        rc = launch_t1_apply(m, 1);
        m->cornersValid = false;  // the patch of touched cells leaves the others stale
        return rc;
    }
    // corners of the moved state, with the T1 edge test fused in
    rc = launch_corners(m, !m->restricted);
    if (rc) return rc;
    return launch_t1_apply(m, 1);
}

}  // namespace svm

// ================================ C ABI ===================================================
extern "C" {

const char* svm_status_string(int s) {
    switch (s) {
        case SVM_OK: return "ok";
        case SVM_ERR_ARG: return "invalid argument";
        case SVM_ERR_CUDA: return "CUDA error";
        case SVM_ERR_HULL: return "convex hull failed";
        case SVM_ERR_DEVICE: return "device status set";
        case SVM_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown";
    }
}

int svm_device_count(int* count) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); n = 0; }
    if (count) *count = n;
    return n > 0 ? SVM_OK : SVM_ERR_NO_DEVICE;
}

int svm_topology_from_points(const double* pts, int n, svm_topology** out) {
    if (!pts || n < 4 || !out) return SVM_ERR_ARG;
    std::vector<int> tris;
    svm_topology* t = new svm_topology();
    if (!svm::convexHullTriangles(pts, n, tris) || !svm::topologyFromTriangles(pts, n, tris, t->t)) {
        delete t;
        return SVM_ERR_HULL;
    }
    *out = t;
    return SVM_OK;
}

int svm_topology_from_triangles(const double* pts, int n, const int* tri, int ntri, svm_topology** out) {
    if (!pts || !tri || n < 4 || ntri != 2 * n - 4 || !out) return SVM_ERR_ARG;
    std::vector<int> tris(tri, tri + 3 * (size_t)ntri);
    svm_topology* t = new svm_topology();
    if (!svm::topologyFromTriangles(pts, n, tris, t->t)) { delete t; return SVM_ERR_HULL; }
    *out = t;
    return SVM_OK;
}

int svm_topology_sizes(const svm_topology* t, int* nC, int* nV, int* maxRing) {
    if (!t) return SVM_ERR_ARG;
    if (nC) *nC = t->t.nCells;
    if (nV) *nV = t->t.nVertices;
    if (maxRing) *maxRing = t->t.maxRing;
    return SVM_OK;
}

int svm_topology_get(const svm_topology* t, double* vp, int* rings, int stride, unsigned* counts, int* vc, int* vn) {
    if (!t) return SVM_ERR_ARG;
    const svm::Topology& T = t->t;
    if (rings && stride < T.maxRing) return SVM_ERR_ARG;
    if (vp) std::memcpy(vp, T.vertexPos.data(), sizeof(double) * T.vertexPos.size());
    if (vc) std::memcpy(vc, T.vertexCells.data(), sizeof(int) * T.vertexCells.size());
    if (vn) std::memcpy(vn, T.vertexNeighbors.data(), sizeof(int) * T.vertexNeighbors.size());
    for (int c = 0; c < T.nCells; ++c) {
        const int b = T.ringOffsets[c], e = T.ringOffsets[c + 1];
        if (counts) counts[c] = (unsigned)(e - b);
        if (rings)
            for (int k = 0; k < stride; ++k) rings[(size_t)c * stride + k] = k < e - b ? T.ringVertices[b + k] : -1;
    }
    return SVM_OK;
}

void svm_topology_free(svm_topology* t) { delete t; }

#define SVM_CUDA(x)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (x);                                                                \
        if (e_ != cudaSuccess) {                                                             \
            std::fprintf(stderr, "libsvm: %s failed: %s\n", #x, cudaGetErrorString(e_));     \
            return SVM_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

int svm_model_create(int nCells, int nVertices, int Wc, double radius, void* stream, svm_model** out) {
    if (nCells < 4 || nVertices != 2 * nCells - 4 || Wc < 3 || Wc > 64 || !(radius > 0) || !out) return SVM_ERR_ARG;
    return svm::model_alloc(nCells, nVertices, Wc, &radius, 1, stream, out);
}

}  // extern "C"

// Allocation of a model (one sphere, or nRep replicas concatenated: replica r's radius radius[r]).
int svm::model_alloc(int nCells, int nVertices, int Wc, const double* radius, int nRep, void* stream,
                     svm_model** out) {
    int ndev = 0;
    if (svm_device_count(&ndev) != SVM_OK) return SVM_ERR_NO_DEVICE;
    svm_model* m = new svm_model();
    m->nCells = nCells; m->nVertices = nVertices; m->Wc = Wc; m->R = radius[0]; m->nRep = nRep;
    {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
            m->sms = sms;
    }
    if (stream) { m->stream = (cudaStream_t)stream; }
    else {
        if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) { delete m; return SVM_ERR_CUDA; }
        m->ownStream = true;
    }
    const size_t nV = nVertices, nC = nCells;
    bool ok = true;
    auto alloc = [&](void** p, size_t bytes) { if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false; if (ok) cudaMemset(*p, 0, bytes); };
    alloc((void**)&m->pos[0], nV * sizeof(double4_32a));
    alloc((void**)&m->pos[1], nV * sizeof(double4_32a));
    alloc((void**)&m->vsph, nV * sizeof(double4_32a));
    alloc((void**)&m->vnorm, nV * sizeof(double));
    if (nRep == 1) alloc((void**)&m->dir, nV * sizeof(double4_32a));
    if (nRep == 1) {  // the FP64 corner pass's edge terms (batches run in the mixed form only)
        alloc((void**)&m->edgeC, 3 * (size_t)nV * sizeof(double4_32a));
        alloc((void**)&m->edgeArc, 3 * (size_t)nV * sizeof(double));
    }
    alloc((void**)&m->vcell, nV * sizeof(int4));
    alloc((void**)&m->vnbr, nV * sizeof(int4));
    alloc((void**)&m->vlast, nV * sizeof(int4));
    alloc((void**)&m->vnext, nV * sizeof(int4));
    alloc((void**)&m->vrpos, nV * sizeof(int4));
    alloc((void**)&m->ring, nC * Wc * sizeof(int));
    alloc((void**)&m->ringCount, nC * sizeof(int));
    alloc((void**)&m->corner, nC * Wc * sizeof(double2));
    alloc((void**)&m->cellPos, nC * sizeof(double4_32a));
    alloc((void**)&m->cellSph, nC * sizeof(double4_32a));
    alloc((void**)&m->ap, nC * sizeof(double2));
    alloc((void**)&m->pref, nC * sizeof(double2));
    alloc((void**)&m->force, nV * sizeof(double4_32a));
    alloc((void**)&m->vel, nV * sizeof(double4_32a));
    alloc((void**)&m->noiseBuf, 3 * nV * sizeof(double));
    alloc((void**)&m->dispBuf, 3 * nV * sizeof(double));
    m->maxPartialBlocks = svm::blocksFor((long)std::max(nV, nC)) + 8;
    alloc((void**)&m->partials, (size_t)m->maxPartialBlocks * 8 * sizeof(double));
    alloc((void**)&m->ticket, 8 * sizeof(unsigned));
    alloc((void**)&m->scalars, 16 * sizeof(double));
    alloc((void**)&m->fallbackFlag, 2 * sizeof(int));  // [0] this pass's flag, [1] passes that took it
    alloc((void**)&m->status, sizeof(int));
    alloc((void**)&m->stepCounter, sizeof(unsigned long long));
    m->t1.nWords = (int)((3 * nV + 31) / 32);
    m->t1.nSummary = (m->t1.nWords + 31) / 32;
    m->t1.flipLogCap = 1 << 16;
    m->t1.touchedCap = 4 * 65536;
    m->t1.cap = (int)(3 * nV / 2 + (nRep > 1 ? svm::kListPadBatch * (size_t)nRep : svm::kListPad));
    m->t1.undoCap = std::max(65536, 256 * nRep);
    alloc((void**)&m->t1.bits, (size_t)m->t1.nSummary * 32 * sizeof(unsigned));
    alloc((void**)&m->t1.summary, (size_t)m->t1.nSummary * sizeof(unsigned));
    alloc((void**)&m->t1.count, sizeof(int));
    alloc((void**)&m->t1.flipLog, 4 * (size_t)m->t1.flipLogCap * sizeof(int));
    alloc((void**)&m->t1.pass, sizeof(int));
    alloc((void**)&m->t1.listA, (size_t)m->t1.cap * sizeof(int));
    alloc((void**)&m->t1.listB, (size_t)m->t1.cap * sizeof(int));
    alloc((void**)&m->t1.listOrig, (size_t)m->t1.cap * sizeof(int));
    alloc((void**)&m->t1.fp, (size_t)m->t1.cap * svm::kFootprint * sizeof(int));
    alloc((void**)&m->t1.comList, (size_t)m->t1.cap * svm::kFootprint * sizeof(int));
    alloc((void**)&m->t1.resV, nV * sizeof(int));
    alloc((void**)&m->t1.resC, nC * sizeof(int));
    alloc((void**)&m->t1.comV, nV * sizeof(int));
    alloc((void**)&m->t1.comC, nC * sizeof(int));
    alloc((void**)&m->t1.undo, (size_t)m->t1.undoCap * sizeof(svm::UndoEntry));
    alloc((void**)&m->t1.undoRings, (size_t)m->t1.undoCap * 4 * Wc * sizeof(int));
    alloc((void**)&m->t1.ctr, (8 + svm::kT1CtlInts) * sizeof(int));
    if (ok) m->t1.ctl = reinterpret_cast<svm::T1Ctl*>(m->t1.ctr + 8);
    alloc((void**)&m->t1.stats, 8 * sizeof(int));
    alloc((void**)&m->t1.flipCount, sizeof(int));
    alloc((void**)&m->t1.touched, (size_t)m->t1.touchedCap * sizeof(int));
    alloc((void**)&m->repR, nRep * sizeof(double));
    alloc((void**)&m->repNp, nRep * sizeof(float));
    alloc((void**)&m->repCellOff, (nRep + 1) * sizeof(int));
    alloc((void**)&m->repVertOff, (nRep + 1) * sizeof(int));
    alloc((void**)&m->repFlag, nRep * sizeof(int));
    alloc((void**)&m->repScal, 3 * nRep * sizeof(double));
    alloc((void**)&m->ringMax, sizeof(int));
    if (ok && cudaHostAlloc((void**)&m->ringMaxHost, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
        m->ringMaxHost = nullptr;
        ok = false;
    }
    if (ok) {
        *m->ringMaxHost = 0;
        ok = cudaHostGetDevicePointer((void**)&m->ringMaxHostDev, m->ringMaxHost, 0) == cudaSuccess;
    }
    if (!ok) { svm_model_destroy(m); return SVM_ERR_CUDA; }
    cudaMemcpy(m->repR, radius, nRep * sizeof(double), cudaMemcpyHostToDevice);
    m->repT.assign(nRep, 0.0);
    cudaMemset(m->t1.resV, 0x7f, nV * sizeof(int));   // kResFree
    cudaMemset(m->t1.resC, 0x7f, nC * sizeof(int));
    cudaMemset(m->t1.comV, 0xff, nV * sizeof(int));   // -1
    cudaMemset(m->t1.comC, 0xff, nC * sizeof(int));
    std::vector<double2> pref(nC, make_double2(1.0, 3.8));
    cudaMemcpy(m->pref, pref.data(), nC * sizeof(double2), cudaMemcpyHostToDevice);
    if (cudaDeviceSynchronize() != cudaSuccess || zig_init() != SVM_OK) { svm_model_destroy(m); return SVM_ERR_CUDA; }
    *out = m;
    return SVM_OK;
}

extern "C" {

int svm_model_destroy(svm_model* m) {
    if (!m) return SVM_ERR_ARG;
    if (m->stream) cudaStreamSynchronize(m->stream);
    for (svm_fire* F : m->fires) svm::fire_detach(F);
    void* ptrs[] = {m->pos[0], m->pos[1], m->vsph, m->vnorm, m->dir, m->dirTarget, m->cellRef, m->edgeC, m->edgeArc, m->vcell, m->vnbr, m->vlast, m->vnext, m->vrpos, m->ring,
                    m->ringCount, m->corner, m->cellPos, m->cellSph, m->ap, m->pref, m->force, m->vel, m->noiseBuf,
                    m->dispBuf, m->partials, m->ticket, m->scalars, m->fallbackFlag, m->status, m->stepCounter,
                    m->t1.bits, m->t1.summary, m->t1.count, m->t1.flipLog, m->t1.flipCount, m->t1.touched,
                    m->t1.pass, m->t1.listA, m->t1.listB, m->t1.listOrig, m->t1.fp, m->t1.comList, m->t1.resV,
                    m->t1.resC, m->t1.comV, m->t1.comC, m->t1.undo, m->t1.undoRings, m->t1.ctr, m->t1.stats,
                    m->pos32[0], m->pos32[1], m->cellPos32, m->force32, m->dap32, m->repR, m->repNp, m->repCellOff,
                    m->repVertOff, m->t1.clocks,
                    m->repFlag, m->repScal, m->dotPartials, m->ringMax};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (m->ringMaxHost) cudaFreeHost(m->ringMaxHost);
    for (cudaEvent_t e : m->passEv)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : m->runEv)
        if (e) cudaEventDestroy(e);
    if (m->bdGraph) cudaGraphExecDestroy(m->bdGraph);
    for (auto& g : m->ioGraph)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (m->ioEnergy) cudaFreeHost(m->ioEnergy);
    svm::batch_release(m);
    for (auto& v : m->profEvents) for (cudaEvent_t e : v) cudaEventDestroy(e);
    if (m->ownStream && m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SVM_OK;
}

__global__ void k_aos_to_d4(const double* __restrict__ in, double4_32a* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_double4_32a(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.0);
}
__global__ void k_d4_to_aos(const double4_32a* __restrict__ in, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { const double4_32a q = in[i]; out[3 * i] = q.x; out[3 * i + 1] = q.y; out[3 * i + 2] = q.z; }
}

// Host AoS double[3n] -> device double4 through the staging buffer (a pinned caller buffer is
// copied by DMA without a host-side repack).
static int upload_vec(svm_model* m, const double* in, double4_32a* dst, int n) {
    SVM_CUDA(cudaMemcpyAsync(m->dispBuf, in, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, m->stream));
    k_aos_to_d4<<<svm::blocksFor(n), svm::kBlock, 0, m->stream>>>(m->dispBuf, dst, n);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

static int upload_positions(svm_model* m, const double* in) {
    int rc = upload_vec(m, in, m->pos[m->cur], m->nVertices);
    if (!rc && m->precision == SVM_PRECISION_MIXED) {
        // dispBuf still holds the AoS copy; round it to the FP32 positions
        if (svm::mixed_upload_positions(m, m->dispBuf)) return SVM_ERR_CUDA;
        SVM_CUDA(cudaStreamSynchronize(m->stream));
    }
    m->cornersValid = false;
    return rc;
}

int svm_model_set_topology(svm_model* m, const double* vp, const int* rings, int stride, const unsigned* counts,
                           const int* vc, const int* vn) {
    if (!m || !vp || !rings || !counts || !vc || !vn || stride < 3) return SVM_ERR_ARG;
    int maxCount = 0;
    for (int c = 0; c < m->nCells; ++c) maxCount = std::max(maxCount, (int)counts[c]);
    if (maxCount + m->ringHeadroom >= m->Wc) {  // room for the rings to grow (growCellVerticesList)
        const int rc = svm::grow_rings(m, maxCount + m->ringHeadroom + 8);
        if (rc) return rc;
    }
    const int nC = m->nCells, nV = m->nVertices, Wc = m->Wc;
    std::vector<int> rg((size_t)nC * Wc, -1), cnt(nC);
    for (int c = 0; c < nC; ++c) {
        if ((int)counts[c] > Wc || (int)counts[c] > stride || counts[c] < 3) return SVM_ERR_ARG;
        cnt[c] = (int)counts[c];
        for (int k = 0; k < cnt[c]; ++k) {
            const int u = rings[(size_t)c * stride + k];
            if (u < 0 || u >= nV) return SVM_ERR_ARG;
            rg[(size_t)c * Wc + k] = u;
        }
    }
    std::vector<int4> vcell(nV), vnbr(nV);
    for (int v = 0; v < nV; ++v) {
        for (int s = 0; s < 3; ++s)
            if (vc[3 * v + s] < 0 || vc[3 * v + s] >= nC || vn[3 * v + s] < 0 || vn[3 * v + s] >= nV) return SVM_ERR_ARG;
        vcell[v] = make_int4(vc[3 * v], vc[3 * v + 1], vc[3 * v + 2], -1);
        vnbr[v] = make_int4(vn[3 * v], vn[3 * v + 1], vn[3 * v + 2], -1);
    }
    SVM_CUDA(cudaMemcpyAsync(m->ring, rg.data(), sizeof(int) * rg.size(), cudaMemcpyHostToDevice, m->stream));
    SVM_CUDA(cudaMemcpyAsync(m->ringCount, cnt.data(), sizeof(int) * nC, cudaMemcpyHostToDevice, m->stream));
    SVM_CUDA(cudaMemcpyAsync(m->vcell, vcell.data(), sizeof(int4) * nV, cudaMemcpyHostToDevice, m->stream));
    SVM_CUDA(cudaMemcpyAsync(m->vnbr, vnbr.data(), sizeof(int4) * nV, cudaMemcpyHostToDevice, m->stream));
    // a new state: status bits of the old one no longer apply, and this upload's checks set their own
    SVM_CUDA(cudaMemsetAsync(m->status, 0, sizeof(int), m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));  // no pass may still write the host-visible maximum
    SVM_CUDA(cudaMemcpy(m->ringMax, &maxCount, sizeof(int), cudaMemcpyHostToDevice));
    *m->ringMaxHost = maxCount;
    k_ring_index<<<svm::blocksFor(nC), svm::kBlock, 0, m->stream>>>(m->ring, m->ringCount, Wc, nC, m->vcell, m->vlast,
                                                                    m->vnext, m->vrpos, m->status);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    int rc = upload_positions(m, vp);
    if (rc) return rc;
    int st = 0;
    SVM_CUDA(cudaMemcpy(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost));
    return st ? SVM_ERR_DEVICE : SVM_OK;
}

int svm_model_set_preferred_parameters(svm_model* m, double a0, double p0) {
    if (!m) return SVM_ERR_ARG;
    std::vector<double2> pref(m->nCells, make_double2(a0, p0));
    SVM_CUDA(cudaMemcpyAsync(m->pref, pref.data(), sizeof(double2) * m->nCells, cudaMemcpyHostToDevice, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

int svm_model_set_preferred_array(svm_model* m, const double* a0p0) {
    if (!m || !a0p0) return SVM_ERR_ARG;
    SVM_CUDA(cudaMemcpyAsync(m->pref, a0p0, sizeof(double2) * m->nCells, cudaMemcpyHostToDevice, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

int svm_model_set_scalar_model_parameter(svm_model* m, double kr) {
    if (!m) return SVM_ERR_ARG;
    m->Kr = kr; m->paramsVersion++;
    return SVM_OK;
}
int svm_model_set_t1_threshold(svm_model* m, double t) {
    if (!m) return SVM_ERR_ARG;
    m->t1Threshold = t; m->paramsVersion++;
    return SVM_OK;
}
int svm_model_set_restricted_motion(svm_model* m, int r) {
    if (!m) return SVM_ERR_ARG;
    m->restricted = r != 0; m->paramsVersion++;
    return SVM_OK;
}

int svm_model_compute_geometry(svm_model* m) {
    if (!m) return SVM_ERR_ARG;
    m->cornersValid = false;  // corners follow the current state; recompute them
    return svm::launch_geometry(m);
}

int svm_model_compute_forces(svm_model* m) {
    if (!m) return SVM_ERR_ARG;
    int rc = svm_model_compute_geometry(m);
    if (rc) return rc;
    svm::PhaseTimer pt(m, SVM_PHASE_FORCE);
    if (m->precision == SVM_PRECISION_MIXED) return svm::mixed_launch_force(m);
    return svm::launch_force_fp64(m);
}

int svm_model_compute_energy(svm_model* m, double* e) {
    if (!m || !e) return SVM_ERR_ARG;
    k_energy<<<svm::blocksFor(m->nCells), svm::kBlock, 0, m->stream>>>(m->ap, m->pref, m->Kr, m->nCells,
                                                                         m->partials + m->maxPartialBlocks,
                                                                         m->ticket + 1, m->scalars + 2);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    SVM_CUDA(cudaMemcpyAsync(e, m->scalars + 2, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

int svm_model_enforce_topology(svm_model* m) {
    if (!m) return SVM_ERR_ARG;
    if (svm::launch_t1_test(m)) return SVM_ERR_CUDA;
    // the patch of touched cells writes corners; all of them are recomputed before their next use
    int rc = svm::launch_t1_apply(m, 0);
    m->cornersValid = false;
    return rc;
}

int svm_model_move_particles(svm_model* m, const double* disp, double scale) {
    if (!m || !disp) return SVM_ERR_ARG;
    {
    svm::PhaseTimer pt(m, SVM_PHASE_MOVE);
    if (m->precision == SVM_PRECISION_MIXED) {
        if (svm::mixed_launch_move(m, disp, scale)) return SVM_ERR_CUDA;
    } else {
        k_move<<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(m->pos[m->cur], disp, scale, m->nVertices, m->R);
    }
    }
    if (svm::check_launch()) return SVM_ERR_CUDA;
    m->cornersValid = false;
    if (!m->restricted) return svm_model_enforce_topology(m);
    return SVM_OK;
}

int svm_model_move_particles_host(svm_model* m, const double* disp, double scale) {
    if (!m || !disp) return SVM_ERR_ARG;
    SVM_CUDA(cudaMemcpyAsync(m->dispBuf, disp, sizeof(double) * 3 * m->nVertices, cudaMemcpyHostToDevice, m->stream));
    return svm_model_move_particles(m, m->dispBuf, scale);
}

static int get_vec4(svm_model* m, const double4_32a* src, int n, double* out) {
    double* stage = n <= m->nVertices ? m->dispBuf : nullptr;
    if (!stage) return SVM_ERR_ARG;
    k_d4_to_aos<<<svm::blocksFor(n), svm::kBlock, 0, m->stream>>>(src, stage, n);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    SVM_CUDA(cudaMemcpyAsync(out, stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

// FP32 device vectors (mixed form) -> host AoS double[3n], widened exactly
static int get_vec4f(svm_model* m, const float4* src, int n, double* out) {
    if (n > m->nVertices) return SVM_ERR_ARG;
    if (svm::mixed_download(m, src, n, m->dispBuf)) return SVM_ERR_CUDA;
    SVM_CUDA(cudaMemcpyAsync(out, m->dispBuf, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

static bool mixed(const svm_model* m) { return m->precision == SVM_PRECISION_MIXED; }

int svm_model_get_positions(svm_model* m, double* out) {
    if (!m || !out) return SVM_ERR_ARG;
    return mixed(m) ? get_vec4f(m, m->pos32[m->cur], m->nVertices, out) : get_vec4(m, m->pos[m->cur], m->nVertices, out);
}
int svm_model_set_positions(svm_model* m, const double* in) { if (!m || !in) return SVM_ERR_ARG; return upload_positions(m, in); }
int svm_model_get_forces(svm_model* m, double* out) {
    if (!m || !out) return SVM_ERR_ARG;
    return mixed(m) ? get_vec4f(m, m->force32, m->nVertices, out) : get_vec4(m, m->force, m->nVertices, out);
}
int svm_model_get_velocities(svm_model* m, double* out) { if (!m || !out) return SVM_ERR_ARG; return get_vec4(m, m->vel, m->nVertices, out); }
int svm_model_get_cell_positions(svm_model* m, double* out) {
    if (!m || !out) return SVM_ERR_ARG;
    return mixed(m) ? get_vec4f(m, m->cellPos32, m->nCells, out) : get_vec4(m, m->cellPos, m->nCells, out);
}

int svm_model_set_velocities(svm_model* m, const double* in) {
    if (!m || !in) return SVM_ERR_ARG;
    return upload_vec(m, in, m->vel, m->nVertices);
}

int svm_model_get_area_perimeter(svm_model* m, double* out) {
    if (!m || !out) return SVM_ERR_ARG;
    SVM_CUDA(cudaMemcpyAsync(out, m->ap, sizeof(double2) * m->nCells, cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

int svm_model_set_t1_wait_limit(svm_model* m, int polls) {
    if (!m || polls < 0) return SVM_ERR_ARG;
    m->t1WaitLimit = polls;
    m->paramsVersion++;  // captured graphs hold the old limit
    return SVM_OK;
}

int svm_model_set_ring_headroom(svm_model* m, int slots) {
    if (!m || slots < 0 || slots > 64) return SVM_ERR_ARG;
    m->ringHeadroom = slots;
    return SVM_OK;
}

int svm_model_ring_info(svm_model* m, int* out3) {
    if (!m || !out3) return SVM_ERR_ARG;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    out3[0] = m->Wc;
    out3[1] = *(volatile int*)m->ringMaxHost;
    out3[2] = m->ringGrowths;
    return SVM_OK;
}

int svm_model_get_rings(svm_model* m, int* rings, int stride, unsigned* counts) {
    if (!m || !rings || !counts) return SVM_ERR_ARG;
    std::vector<int> rg((size_t)m->nCells * m->Wc), cnt(m->nCells);
    SVM_CUDA(cudaMemcpyAsync(rg.data(), m->ring, sizeof(int) * rg.size(), cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaMemcpyAsync(cnt.data(), m->ringCount, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    for (int c = 0; c < m->nCells; ++c) {
        if (cnt[c] > stride) return SVM_ERR_ARG;
        counts[c] = (unsigned)cnt[c];
        for (int k = 0; k < stride; ++k) rings[(size_t)c * stride + k] = k < cnt[c] ? rg[(size_t)c * m->Wc + k] : -1;
    }
    return SVM_OK;
}

static int get_int4x3(svm_model* m, const int4* src, int* out) {
    std::vector<int4> h(m->nVertices);
    SVM_CUDA(cudaMemcpyAsync(h.data(), src, sizeof(int4) * m->nVertices, cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    for (int i = 0; i < m->nVertices; ++i) { out[3 * i] = h[i].x; out[3 * i + 1] = h[i].y; out[3 * i + 2] = h[i].z; }
    return SVM_OK;
}
int svm_model_get_vertex_cells(svm_model* m, int* out) { if (!m || !out) return SVM_ERR_ARG; return get_int4x3(m, m->vcell, out); }
int svm_model_get_vertex_neighbors(svm_model* m, int* out) { if (!m || !out) return SVM_ERR_ARG; return get_int4x3(m, m->vnbr, out); }

int svm_model_status(svm_model* m, int* st) {
    if (!m || !st) return SVM_ERR_ARG;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    SVM_CUDA(cudaMemcpy(st, m->status, sizeof(int), cudaMemcpyDeviceToHost));
    SVM_CUDA(cudaMemset(m->status, 0, sizeof(int)));
    return SVM_OK;
}

int svm_model_area_check(svm_model* m, double* total, double* excess, int* taken) {
    if (!m) return SVM_ERR_ARG;
    double sc[2];
    int f = 0;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    SVM_CUDA(cudaMemcpy(sc, m->scalars, sizeof(sc), cudaMemcpyDeviceToHost));
    SVM_CUDA(cudaMemcpy(&f, m->fallbackFlag, sizeof(int), cudaMemcpyDeviceToHost));
    if (total) *total = sc[0];
    if (excess) *excess = sc[1];
    if (taken) *taken = f;
    return SVM_OK;
}

int svm_model_fallback_count(svm_model* m, int* count) {
    if (!m || !count) return SVM_ERR_ARG;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    SVM_CUDA(cudaMemcpy(count, m->fallbackFlag + 1, sizeof(int), cudaMemcpyDeviceToHost));
    SVM_CUDA(cudaMemset(m->fallbackFlag + 1, 0, sizeof(int)));
    return SVM_OK;
}

int svm_model_take_flips(svm_model* m, int* pairs, int cap, int* count) {
    if (!m || !count) return SVM_ERR_ARG;
    int n = 0;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    SVM_CUDA(cudaMemcpy(&n, m->t1.flipCount, sizeof(int), cudaMemcpyDeviceToHost));
    *count = n;
    const int k = std::min(n, m->t1.flipLogCap);
    if (pairs && k > 0) {
        std::vector<int4> e(k);
        SVM_CUDA(cudaMemcpy(e.data(), m->t1.flipLog, sizeof(int4) * k, cudaMemcpyDeviceToHost));
        // entries of a rolled-back parallel pass carry pass -1 (the flips were undone and replayed)
        e.erase(std::remove_if(e.begin(), e.end(), [](const int4& a) { return a.x < 0; }), e.end());
        // the CPU order: pass by pass, ascending edge position within a pass
        std::stable_sort(e.begin(), e.end(), [](const int4& a, const int4& b) {
            return a.x != b.x ? a.x < b.x : a.y < b.y;
        });
        *count = (int)e.size() + (n - k);
        for (int i = 0; i < std::min((int)e.size(), cap); ++i) { pairs[2 * i] = e[i].z; pairs[2 * i + 1] = e[i].w; }
    }
    SVM_CUDA(cudaMemset(m->t1.flipCount, 0, sizeof(int)));
    return SVM_OK;
}

int svm_model_profile(svm_model* m, int enable) {
    if (!m) return SVM_ERR_ARG;
    if (m->prof) svm::profile_drain(m);
    m->prof = enable != 0;
    m->profMask = (enable & SVM_PROFILE_ONLY) ? (enable & ((1 << SVM_PHASE_COUNT) - 1)) : 0xff;
    for (int ph = 0; ph < SVM_PHASE_COUNT; ++ph) { m->profMs[ph] = 0; m->profLaunches[ph] = 0; }
    return SVM_OK;
}

int svm_model_profile_read(svm_model* m, double* ms, int* launches) {
    if (!m) return SVM_ERR_ARG;
    svm::profile_drain(m);
    for (int ph = 0; ph < SVM_PHASE_COUNT; ++ph) {
        if (ms) ms[ph] = m->profMs[ph];
        if (launches) launches[ph] = m->profLaunches[ph];
        m->profMs[ph] = 0;
        m->profLaunches[ph] = 0;
    }
    return SVM_OK;
}

int svm_model_t1_stats(svm_model* m, int* st) {
    if (!m || !st) return SVM_ERR_ARG;
    int h[8];
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    SVM_CUDA(cudaMemcpy(h, m->t1.stats, sizeof(h), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 6; ++i) st[i] = h[i];
    SVM_CUDA(cudaMemset(m->t1.stats, 0, 6 * sizeof(int)));
    return SVM_OK;
}

int svm_model_set_t1_blocks(svm_model* m, int blocks) {
    if (!m || blocks < 0) return SVM_ERR_ARG;
    m->t1Blocks = blocks;
    m->paramsVersion++;  // captured graphs hold the old launch
    return SVM_OK;
}

int svm_model_t1_clocks(svm_model* m, int enable, unsigned long long* cycles5) {
    if (!m) return SVM_ERR_ARG;
    if (cycles5 && m->t1.clocks) {
        SVM_CUDA(cudaStreamSynchronize(m->stream));
        SVM_CUDA(cudaMemcpy(cycles5, m->t1.clocks, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    }
    if (enable && !m->t1.clocks) {
        SVM_CUDA(cudaMalloc(&m->t1.clocks, 8 * sizeof(unsigned long long)));
    }
    if (!enable && m->t1.clocks) {
        SVM_CUDA(cudaStreamSynchronize(m->stream));
        cudaFree(m->t1.clocks);
        m->t1.clocks = nullptr;
    }
    if (m->t1.clocks) SVM_CUDA(cudaMemset(m->t1.clocks, 0, 8 * sizeof(unsigned long long)));
    m->paramsVersion++;  // captured graphs hold the old pointer
    return SVM_OK;
}

int svm_model_synchronize(svm_model* m) {
    if (!m) return SVM_ERR_ARG;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

int svm_model_stream(svm_model* m, void** s) {
    if (!m || !s) return SVM_ERR_ARG;
    *s = (void*)m->stream;
    return SVM_OK;
}

int svm_model_device_positions(svm_model* m, void** p) {
    if (!m || !p) return SVM_ERR_ARG;
    *p = m->precision == SVM_PRECISION_MIXED ? (void*)m->pos32[m->cur] : (void*)m->pos[m->cur];
    return SVM_OK;
}

int svm_brownian_step(svm_model* m, double T, double dt, double mu, int mode, const double* noise, uint64_t seed) {
    if (!m || (mode == SVM_NOISE_BUFFER && !noise) || (mode != SVM_NOISE_BUFFER && mode != SVM_NOISE_PHILOX)) return SVM_ERR_ARG;
    return svm::bd_step(m, T, dt, mu, mode, noise, seed);
}

// One Brownian step with host input and output in a single stream sequence and one
// synchronisation: positions H2D (optional), the step (Philox noise), the energy of the geometry
// the step's forces used (what computeEnergy returns after a timestep, sphericalVertexModel.cpp:
// 150-160) and the new positions D2H (optional).
namespace svm {
static bool pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeHost;
}
}  // namespace svm

static int step_io_sequence(svm_model* m, double T, double dt, double mu, uint64_t seed, const double* posIn,
                            double* posOut, double* energyOut, double* hostOut);
// The device address of a mapped page-locked output array for the FP64 forms' host-buffer step, else
// null (pageable memory, or the mixed form, whose output goes through a conversion and a copy).
// Resolved outside any stream capture.
static double* io_mapped_out(svm_model* m, double* posOut) {
    if (!posOut || m->precision == SVM_PRECISION_MIXED) return nullptr;
    void* dp = nullptr;
    if (cudaHostGetDevicePointer(&dp, posOut, 0) == cudaSuccess) return (double*)dp;
    cudaGetLastError();
    return nullptr;
}

int svm_brownian_step_io(svm_model* m, double T, double dt, double mu, uint64_t seed, const double* posIn,
                         double* posOut, double* energyOut) {
    if (!m) return SVM_ERR_ARG;
    // With both position buffers page-locked (and no per-phase profiling) the whole sequence, the
    // upload included, is one graph launch: captured once per position-buffer role and reused while
    // the parameters, buffers and form stay the same.  The energy lands in a page-locked slot of the
    // model and is copied out after the synchronisation.
    if (posIn && posOut && m->nRep == 1 && !m->prof && svm::pinned(posIn) && svm::pinned(posOut)) {
        if (!m->ioEnergy && cudaMallocHost((void**)&m->ioEnergy, sizeof(double)) != cudaSuccess) {
            m->ioEnergy = nullptr;
            return SVM_ERR_CUDA;
        }
        // the ring-capacity check of a T1 pass launched outside a capture (a growth recaptures)
        if (!m->restricted) {
            if (int rc = svm::ensure_ring_headroom(m)) return rc;
        }
        double* hostOut = io_mapped_out(m, posOut);
        auto& g = m->ioGraph[m->cur];
        const bool reuse = g.exec && g.T == T && g.dt == dt && g.mu == mu && g.seed == seed && g.in == posIn &&
                           g.out == posOut && g.outDev == hostOut && g.version == m->paramsVersion &&
                           g.precision == m->precision;
        const int cur0 = m->cur;
        if (!reuse) {
            if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
            cudaGraph_t graph;
            SVM_CUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
            const int rc = step_io_sequence(m, T, dt, mu, seed, posIn, posOut, m->ioEnergy, hostOut);
            cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
            m->cur = cur0;
            if (rc || ce != cudaSuccess) { cudaGetLastError(); return rc ? rc : SVM_ERR_CUDA; }
            ce = cudaGraphInstantiate(&g.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) { g.exec = nullptr; return SVM_ERR_CUDA; }
            g.T = T; g.dt = dt; g.mu = mu; g.seed = seed; g.in = posIn; g.out = posOut; g.outDev = hostOut;
            g.version = m->paramsVersion; g.precision = m->precision;
        }
        SVM_CUDA(cudaGraphLaunch(g.exec, m->stream));
        // the host-side state the sequence leaves: buffers swapped, corners left to the next step
        m->cur = 1 - cur0;
        m->cornersValid = false;
        SVM_CUDA(cudaStreamSynchronize(m->stream));
        if (energyOut) *energyOut = *m->ioEnergy;
        return SVM_OK;
    }
    const int rc = step_io_sequence(m, T, dt, mu, seed, posIn, posOut, energyOut, io_mapped_out(m, posOut));
    if (rc) return rc;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

// The launches of one host-io step, in stream order (no synchronisation).
static int step_io_sequence(svm_model* m, double T, double dt, double mu, uint64_t seed, const double* posIn,
                            double* posOut, double* energyOut, double* hostOut) {
    const bool mixedForm = m->precision == SVM_PRECISION_MIXED;
    if (posIn) {
        SVM_CUDA(cudaMemcpyAsync(m->dispBuf, posIn, sizeof(double) * 3 * m->nVertices, cudaMemcpyHostToDevice, m->stream));
        if (mixedForm) {
            if (svm::mixed_upload_positions(m, m->dispBuf)) return SVM_ERR_CUDA;
        } else {
            k_aos_to_d4<<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(m->dispBuf, m->pos[m->cur], m->nVertices);
            if (svm::check_launch()) return SVM_ERR_CUDA;
        }
        m->cornersValid = false;
    }
    // with a mapped output array (hostOut, io_mapped_out) the force kernel and the T1 patch write the
    // moved positions into it directly, the force kernel's stores hidden under its FP64 work, so no
    // copy follows the step
    m->ioHostOut = hostOut;
    // a caller that passes positions in is likely to replace them again before the next step
    int rc = svm::bd_step(m, T, dt, mu, SVM_NOISE_PHILOX, nullptr, seed, posIn != nullptr);
    m->ioHostOut = nullptr;
    if (rc) return rc;
    if (energyOut) {
        k_energy<<<svm::blocksFor(m->nCells), svm::kBlock, 0, m->stream>>>(m->ap, m->pref, m->Kr, m->nCells,
                                                                             m->partials + m->maxPartialBlocks,
                                                                             m->ticket + 1, m->scalars + 2);
        if (svm::check_launch()) return SVM_ERR_CUDA;
        SVM_CUDA(cudaMemcpyAsync(energyOut, m->scalars + 2, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    }
    if (posOut && !hostOut) {
        if (mixedForm) {
            if (svm::mixed_download(m, m->pos32[m->cur], m->nVertices, m->dispBuf)) return SVM_ERR_CUDA;
        } else {
            k_d4_to_aos<<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(m->pos[m->cur], m->dispBuf,
                                                                                    m->nVertices);
            if (svm::check_launch()) return SVM_ERR_CUDA;
        }
        SVM_CUDA(cudaMemcpyAsync(posOut, m->dispBuf, sizeof(double) * 3 * m->nVertices, cudaMemcpyDeviceToHost, m->stream));
    }
    return SVM_OK;
}

int svm_model_set_dynamics_reference(svm_model* m) {
    if (!m || m->nRep > 1) return SVM_ERR_ARG;
    if (!m->cellRef && cudaMalloc((void**)&m->cellRef, m->nCells * sizeof(double4_32a)) != cudaSuccess) {
        m->cellRef = nullptr;
        return SVM_ERR_CUDA;
    }
    if (m->precision == SVM_PRECISION_MIXED)
        k_widen4<<<svm::blocksFor(m->nCells), svm::kBlock, 0, m->stream>>>(m->cellPos32, m->cellRef, m->nCells);
    else
        SVM_CUDA(cudaMemcpyAsync(m->cellRef, m->cellPos, m->nCells * sizeof(double4_32a), cudaMemcpyDeviceToDevice,
                                 m->stream));
    if (svm::check_launch()) return SVM_ERR_CUDA;
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    return SVM_OK;
}

int svm_model_dynamics(svm_model* m, double fraction, double cutoff, double* msd, double* overlap) {
    if (!m || !m->cellRef || !(fraction > 0.0) || fraction > 1.0) return SVM_ERR_ARG;
    const int count = fraction < 1.0 ? (int)std::floor(m->nCells * fraction) : m->nCells;
    if (count < 1) return SVM_ERR_ARG;
    const int nb = svm::blocksFor(count);
    double* part = m->partials + 2 * m->maxPartialBlocks;
    if (m->precision == SVM_PRECISION_MIXED)
        k_dynamics<float4><<<nb, svm::kBlock, 0, m->stream>>>(m->cellRef, m->cellPos32, count, m->R, cutoff, part,
                                                             m->maxPartialBlocks, m->ticket + 2, m->scalars + 4);
    else
        k_dynamics<double4_32a><<<nb, svm::kBlock, 0, m->stream>>>(m->cellRef, m->cellPos, count, m->R, cutoff, part,
                                                                  m->maxPartialBlocks, m->ticket + 2, m->scalars + 4);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    double r[2];
    SVM_CUDA(cudaMemcpyAsync(r, m->scalars + 4, sizeof(r), cudaMemcpyDeviceToHost, m->stream));
    SVM_CUDA(cudaStreamSynchronize(m->stream));
    if (msd) *msd = r[0];
    if (overlap) *overlap = r[1];
    return SVM_OK;
}

int svm_model_set_directors(svm_model* m, const double* in) {
    if (!m || !in || !m->dir) return SVM_ERR_ARG;
    return upload_vec(m, in, m->dir, m->nVertices);
}
int svm_model_get_directors(svm_model* m, double* out) {
    if (!m || !out || !m->dir) return SVM_ERR_ARG;
    return get_vec4(m, m->dir, m->nVertices, out);
}

int svm_spp_step(svm_model* m, double dt, double mu, double v0, double tau, int noiseMode, const double* uniforms,
                 uint64_t seed) {
    if (!m || !m->dir || m->nRep > 1 || m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    if (noiseMode == SVM_NOISE_BUFFER && !uniforms) return SVM_ERR_ARG;
    if (noiseMode == SVM_NOISE_BUFFER)
        SVM_CUDA(cudaMemcpyAsync(m->noiseBuf, uniforms, sizeof(double) * m->nVertices, cudaMemcpyHostToDevice,
                                 m->stream));
    int rc = svm::launch_geometry(m);
    if (rc || (rc = svm::launch_force_fp64(m))) return rc;
    k_spp_move<<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(m->pos[m->cur], m->dir, m->force, dt, mu,
                                                                            v0, m->nVertices, m->R);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    m->cornersValid = false;
    // moveParticles: the T1 pass unless restricted, as in the Brownian step
    if ((rc = svm::launch_corners(m, !m->restricted)) || (rc = svm::launch_t1_apply(m, 1))) return rc;
    const double amp = sqrt(2.0 * dt * tau);
    if (noiseMode == SVM_NOISE_BUFFER)
        k_spp_dirs<SVM_NOISE_BUFFER><<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(
            m->pos[m->cur], m->dir, m->noiseBuf, seed, m->stepCounter, amp, m->nVertices);
    else
        k_spp_dirs<SVM_NOISE_PHILOX><<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(
            m->pos[m->cur], m->dir, nullptr, seed, m->stepCounter, amp, m->nVertices);
    return svm::check_launch();
}

int svm_vicsek_step(svm_model* m, double dt, double mu, double v0, double eta, double tau, int noiseMode,
                    const double* uniforms, uint64_t seed) {
    if (!m || !m->dir || m->nRep > 1 || m->precision == SVM_PRECISION_MIXED || !(tau != 0.0)) return SVM_ERR_ARG;
    if (noiseMode == SVM_NOISE_BUFFER && !uniforms) return SVM_ERR_ARG;
    if (!m->dirTarget) SVM_CUDA(cudaMalloc(&m->dirTarget, m->nVertices * sizeof(double4_32a)));
    if (noiseMode == SVM_NOISE_BUFFER)
        SVM_CUDA(cudaMemcpyAsync(m->noiseBuf, uniforms, sizeof(double) * 2 * m->nVertices, cudaMemcpyHostToDevice,
                                 m->stream));
    int rc = svm::launch_geometry(m);
    if (rc || (rc = svm::launch_force_fp64(m))) return rc;
    k_spp_move<<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(m->pos[m->cur], m->dir, m->force, dt, mu,
                                                                            v0, m->nVertices, m->R);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    m->cornersValid = false;
    if ((rc = svm::launch_corners(m, !m->restricted)) || (rc = svm::launch_t1_apply(m, 1))) return rc;
    if (noiseMode == SVM_NOISE_BUFFER)
        k_vicsek_target<SVM_NOISE_BUFFER><<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(
            m->pos[m->cur], m->dir, m->vnbr, m->dirTarget, m->noiseBuf, seed, m->stepCounter, eta, m->nVertices);
    else
        k_vicsek_target<SVM_NOISE_PHILOX><<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(
            m->pos[m->cur], m->dir, m->vnbr, m->dirTarget, nullptr, seed, m->stepCounter, eta, m->nVertices);
    if (svm::check_launch()) return SVM_ERR_CUDA;
    k_vicsek_update<<<svm::blocksFor(m->nVertices), svm::kBlock, 0, m->stream>>>(m->pos[m->cur], m->dir, m->dirTarget,
                                                                                 dt / tau, m->nVertices);
    return svm::check_launch();
}

int svm_brownian_step_host_noise(svm_model* m, double T, double dt, double mu, const double* noise) {
    if (!m || !noise) return SVM_ERR_ARG;
    SVM_CUDA(cudaMemcpyAsync(m->noiseBuf, noise, sizeof(double) * 3 * m->nVertices, cudaMemcpyHostToDevice, m->stream));
    return svm::bd_step(m, T, dt, mu, SVM_NOISE_BUFFER, m->noiseBuf, 0);
}

int svm_brownian_run(svm_model* m, double T, double dt, double mu, uint64_t seed, int nSteps) {
    if (!m || nSteps < 0) return SVM_ERR_ARG;
    int rc = svm::update_rep_noise(m, dt, mu);  // a batch's noise amplitudes, outside the capture
    if (rc) return rc;
    // while a batch's autotuner samples, steps run one by one with their kernels timed
    while (nSteps > 0 && m->nRep > 1 && svm::batch_tuning(m)) {
        if ((rc = svm::bd_step(m, T, dt, mu, SVM_NOISE_PHILOX, nullptr, seed))) return rc;
        --nSteps;
    }
    if (nSteps == 0) return SVM_OK;
    svm::batch_tuner_untimed(m, nSteps);
    for (cudaEvent_t& e : m->runEv)
        if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { e = nullptr; return SVM_ERR_CUDA; }
    // Chunks of up to 8 steps (4 replays of a captured pair of steps).  The host stays at most two
    // chunks ahead of the device, so that the ring-capacity check before each chunk reads a recent
    // maximum; when it grows the rings, the graph (which holds the old arrays) is captured again.
    for (int chunk = 0; nSteps > 1; ++chunk) {
        if (chunk >= 2) SVM_CUDA(cudaEventSynchronize(m->runEv[chunk % 2]));
        if ((rc = svm::ensure_ring_headroom(m))) return rc;
        const bool reuse = m->bdGraph && m->bdT == T && m->bdDt == dt && m->bdMu == mu && m->bdSeed == seed &&
                           m->bdGraphCur == m->cur && m->bdGraphVersion == m->paramsVersion;
        if (chunk == 0 || !reuse || !m->cornersValid) {
            rc = svm::launch_geometry(m);  // make corners valid outside the capture
            if (rc) return rc;
        }
        if (!reuse) {
            if (m->bdGraph) { cudaGraphExecDestroy(m->bdGraph); m->bdGraph = nullptr; }
            // a pair of steps returns the position buffers to their starting roles
            cudaGraph_t g;
            const int cur0 = m->cur;
            SVM_CUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
            int r1 = svm::bd_step(m, T, dt, mu, SVM_NOISE_PHILOX, nullptr, seed);
            int r2 = r1 ? r1 : svm::bd_step(m, T, dt, mu, SVM_NOISE_PHILOX, nullptr, seed);
            cudaError_t ce = cudaStreamEndCapture(m->stream, &g);
            m->cur = cur0;
            if (r2 || ce != cudaSuccess) { cudaGetLastError(); return SVM_ERR_CUDA; }
            ce = cudaGraphInstantiate(&m->bdGraph, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) { m->bdGraph = nullptr; return SVM_ERR_CUDA; }
            m->bdT = T; m->bdDt = dt; m->bdMu = mu; m->bdSeed = seed;
            m->bdGraphCur = m->cur; m->bdGraphVersion = m->paramsVersion;
        }
        const int pairs = std::min(nSteps / 2, 4);
        for (int i = 0; i < pairs; ++i) SVM_CUDA(cudaGraphLaunch(m->bdGraph, m->stream));
        m->cornersValid = true;  // a replayed pair leaves the moved state's corners
        SVM_CUDA(cudaEventRecord(m->runEv[chunk % 2], m->stream));
        nSteps -= 2 * pairs;
    }
    if (nSteps == 1) {
        rc = svm::bd_step(m, T, dt, mu, SVM_NOISE_PHILOX, nullptr, seed);
        if (rc) return rc;
    }
    return SVM_OK;
}

}  // extern "C"
