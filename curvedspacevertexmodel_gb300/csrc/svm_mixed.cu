// Mixed-precision form of the Brownian step (SVM_PRECISION_MIXED): FP32 positions, forces and
// integration; the included angles, the spherical-excess areas (angle sums), the energy
// accumulation and the renormalisation onto the sphere in FP64.
//
// The FP64 form evaluates the reference's closed-form gradients in spherical coordinates
// (sphericalDomain.h:248-411), whose denominators 1 - s^2 cancel for short arcs; in FP32 they
// would lose all digits at N = 100k (arcs of ~0.007 rad).  The FP32 forces here are the same
// gradients written in raw position differences (exact for nearby FP32 points), which keep full
// FP32 relative accuracy down to the shortest edges:
//   geodesic d(v, u):   grad_v d = -P_a(u - v) / |P_a(u - v)|,  a = v / |v|, P_a = 1 - a a^T
//   signed triangle area A = R^2 E(a, b, c), tan(E / 2) = N / D (Van Oosterom and Strackee, 1983),
//     N = a . (b x c) = a . (beta x gamma),  D = 1 + a.b + b.c + c.a = 4 - |beta|^2 - |gamma|^2 + beta.gamma,
//     beta = (u - v) / |v|, gamma = (w - v) / |v|,  b x c = a x gamma + beta x a + beta x gamma,
//     grad_v A = R P_a [ 2 (D (b x c) - N (beta + gamma)) / (N^2 + D^2) ].
// The signed area matches the reference's gradient of the unsigned area times sign(det(v1, v2, v3))
// (sphericalDomain.h:395-402).
#include <algorithm>
#include "svm_internal.cuh"

namespace svm {
int check_launch();
}

namespace {
using namespace svm;

constexpr int kB = 256;
inline int blocksFor(long n) { return (int)((n + kB - 1) / kB); }

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float4 p) { return F3{p.x, p.y, p.z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 crossf(F3 a, F3 b) { return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ F3 unit(F3 a) { return (1.0f / sqrtf(dotf(a, a))) * a; }

// Unit tangent at a pointing away from the neighbour at a + d (gradient of the geodesic distance
// at any radius).  d is the raw difference of the two FP32 positions: for nearby points it is
// exact (Sterbenz), so short edges keep full relative accuracy, unlike differences of normalised
// vectors.
__device__ __forceinline__ F3 grad_geo32(F3 a, F3 d) {
    const F3 t = d - dotf(d, a) * a;
    return (-1.0f / sqrtf(dotf(t, t))) * t;
}
// Gradient w.r.t. v = R a of the signed spherical triangle area R^2 E(a, a + beta, a + gamma),
// with beta and gamma the raw position differences divided by |v|.
__device__ __forceinline__ F3 grad_tri32(F3 a, F3 beta, F3 gamma, float R) {
    const F3 bg = crossf(beta, gamma);
    const F3 bxc = crossf(a, gamma) + crossf(beta, a) + bg;
    const float N = dotf(a, bg);
    const float D = 4.0f - dotf(beta, beta) - dotf(gamma, gamma) + dotf(beta, gamma);
    const float w = 2.0f / (N * N + D * D);
    const F3 g = w * (D * bxc - N * (beta + gamma));
    return R * (g - dotf(g, a) * a);
}

struct Args32 {
    const float4* pos;
    const int4* vcell;
    const int4* vlast;
    const int4* vnext;
    const float4* cellPos;
    const float2* dap;     // per cell (A - A0, P - P0)
    const double* repR;    // per-replica radius, indexed by pos[v].w
    float Kr;
};

__device__ __forceinline__ int comp(const int4& a, int s) { return s == 0 ? a.x : (s == 1 ? a.y : a.z); }

// Per-vertex force of the quadratic model (the sum of sphericalVertexModel.cpp:380-417) in FP32.
__device__ __forceinline__ F3 vertex_force32(const Args32& A, int v, float R) {
    const F3 P = f3(A.pos[v]);
    const float inv = 1.0f / sqrtf(dotf(P, P));
    const F3 a = inv * P;
    const int4 cells = A.vcell[v], lasts = A.vlast[v], nexts = A.vnext[v];
    F3 f{0.f, 0.f, 0.f};
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int c = comp(cells, s);
        const F3 dc = f3(A.cellPos[c]) - P;
        const F3 dl = f3(A.pos[comp(lasts, s)]) - P, dx = f3(A.pos[comp(nexts, s)]) - P;
        const float2 d = A.dap[c];
        const float dA = d.x, dP = d.y;
        const float pp = 2.0f * dP, aa = 2.0f * A.Kr * dA;
        const F3 bl = inv * dl, bc = inv * dc, bx = inv * dx;
        const F3 fs = (-pp) * (grad_geo32(a, dl) + grad_geo32(a, dx)) +
                      (-aa) * (grad_tri32(a, bl, bc, R) + grad_tri32(a, bc, bx, R));
        if (!isnan(fs.x)) f = f + fs;
    }
    return f;
}

// p <- R (p + P_p d) / |p + P_p d| (sphericalDomain::move): the tangential projection of the FP32
// displacement in FP32, then p + d and the renormalisation onto the sphere in FP64, rounded to
// FP32 (w, the replica, carried over).
__device__ __forceinline__ float4 move_fp64(float4 p, F3 d, double R) {
    const F3 pf = f3(p);
    const F3 dt = d - (dotf(d, pf) / dotf(pf, pf)) * pf;
    const double qx = sf::widen(p.x) + sf::widen(dt.x), qy = sf::widen(p.y) + sf::widen(dt.y),
                 qz = sf::widen(p.z) + sf::widen(dt.z);
    const double k = R * rsqrt(qx * qx + qy * qy + qz * qz);
    return make_float4(sf::narrow(k * qx), sf::narrow(k * qy), sf::narrow(k * qz), p.w);
}

// Philox4x32-10 (Salmon et al., SC'11), as in the FP64 form.
__device__ __forceinline__ uint4 philox(uint4 ctr, uint2 key) {
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
__device__ __forceinline__ float u24(unsigned a) { return ((float)(a >> 8) + 0.5f) * 0x1.0p-24f; }
// three standard normals for (vertex, step): Box-Muller on one Philox draw
__device__ __forceinline__ F3 normals32(uint64_t seed, unsigned long long step, int v) {
    const uint4 r = philox(make_uint4((unsigned)v, (unsigned)step, (unsigned)(step >> 32), 2u),
                           make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const float a = sqrtf(-2.0f * logf(u24(r.x))), b = sqrtf(-2.0f * logf(u24(r.z)));
    float s0, c0;
    sincospif(2.0f * u24(r.y), &s0, &c0);
    return F3{a * c0, a * s0, b * cospif(2.0f * u24(r.w))};
}

__global__ void k32_corners(const float4* __restrict__ pos, const int4* __restrict__ vcell,
                            const int4* __restrict__ vlast, const int4* __restrict__ vnext,
                            const int4* __restrict__ vrpos, const int4* __restrict__ vnbr,
                            double2* __restrict__ corner, int Wc, int nV, const double* __restrict__ repR,
                            int t1test, float t1Threshold, T1Scratch t1) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const float4 p = pos[v];
    const float R = sf::narrow(repR[rep_of(p)]);
    const D3 pd = ld3(pos, v);
    const int4 cells = vcell[v], lasts = vlast[v], nexts = vnext[v], rp = vrpos[v], nb = vnbr[v];
    // per neighbour: FP64 cross product with p and its norm (for the included angles), FP32 arc
    D3 U[3], C[3];
    double nC[3];
    float arc[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float4 q = pos[comp(nb, j)];
        U[j] = D3{sf::widen(q.x), sf::widen(q.y), sf::widen(q.z)};
        C[j] = cross3e(pd, U[j]);
        nC[j] = f64_sqrt(dot3e(C[j], C[j]));
        arc[j] = arc32(q, p, R);
    }
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int jl = nbr_slot(nb, comp(lasts, s)), jx = nbr_slot(nb, comp(nexts, s));
        double2 cr;
        if (jl >= 0 && jx >= 0) {
            cr = make_double2(sf::widen(pick3(arc, jl)), included_angle_pre<true>(pick3(C, jx), pick3(C, jl),
                                                                               pick3(nC, jx), pick3(nC, jl), pick3(U, jl)));
        } else {  // inconsistent lists: evaluate directly
            const int L = comp(lasts, s), X = comp(nexts, s);
            cr = make_double2(sf::widen(arc32(pos[L], p, R)), included_angle_clamped(ld3(pos, L), pd, ld3(pos, X)));
        }
        corner[(long)comp(cells, s) * Wc + comp(rp, s)] = cr;
    }
    if (t1test) {
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            const int u = comp(nb, s);
            if (v < u && arc[s] < t1Threshold) {
                const int q = 3 * v + s;
                atomicOr(&t1.bits[q >> 5], 1u << (q & 31));
                atomicOr(&t1.summary[q >> 10], 1u << ((q >> 5) & 31));
                atomicAdd(t1.count, 1);
            }
        }
    }
}

__global__ void k32_force(Args32 A, int nV, float4* __restrict__ force) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const F3 f = vertex_force32(A, v, sf::narrow(A.repR[rep_of(A.pos[v])]));
    force[v] = make_float4(f.x, f.y, f.z, 0.f);
}

// Noise amplitude: `repNp[replica]` for a batch of replicas, else `np`.
template <int kNoise>
__global__ void k32_force_bd(Args32 A, int nV, float4* __restrict__ force, float4* __restrict__ posNext,
                             const double* __restrict__ noise, uint64_t seed,
                             const unsigned long long* __restrict__ stepCounter, float np,
                             const float* __restrict__ repNp, float fp) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const float4 p = A.pos[v];
    const int rep = rep_of(p);
    const double R = A.repR[rep];
    const F3 f = vertex_force32(A, v, sf::narrow(R));
    force[v] = make_float4(f.x, f.y, f.z, 0.f);
    F3 xi;
    if (kNoise == SVM_NOISE_BUFFER) xi = F3{sf::narrow(noise[3 * v]), sf::narrow(noise[3 * v + 1]), sf::narrow(noise[3 * v + 2])};
    else xi = normals32(seed, *stepCounter, v);
    const float a = repNp ? repNp[rep] : np;
    posNext[v] = move_fp64(p, a * xi + fp * f, R);
}

__global__ void k32_move(float4* __restrict__ pos, const double* __restrict__ disp, double scale, int nV,
                         const double* __restrict__ repR) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const F3 d{(float)(scale * disp[3 * v]), (float)(scale * disp[3 * v + 1]), (float)(scale * disp[3 * v + 2])};
    const float4 p = pos[v];
    pos[v] = move_fp64(p, d, repR[rep_of(p)]);
}

__global__ void k_d4_to_f4(const double4_32a* __restrict__ in, float4* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3(out, i, ld3(in, i));
}
__global__ void k_f4_to_d4(const float4* __restrict__ in, double4_32a* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3(out, i, ld3(in, i));
}
__global__ void k_aos_to_f4(const double* __restrict__ in, float4* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3_keep(out, i, D3{in[3 * i], in[3 * i + 1], in[3 * i + 2]});
}
__global__ void k_f4_to_aos(const float4* __restrict__ in, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { const D3 p = ld3(in, i); out[3 * i] = p.x; out[3 * i + 1] = p.y; out[3 * i + 2] = p.z; }
}

Args32 args32(svm_model* m, int buf) {
    Args32 A;
    A.pos = m->pos32[buf]; A.vcell = m->vcell; A.vlast = m->vlast; A.vnext = m->vnext; A.cellPos = m->cellPos32;
    A.dap = m->dap32; A.repR = m->repR; A.Kr = (float)m->Kr;
    return A;
}

}  // namespace

namespace svm {

int mixed_launch_corners(svm_model* m, bool t1test) {
    const int bs = m->blkCorners;
    k32_corners<<<(m->nVertices + bs - 1) / bs, bs, 0, m->stream>>>(m->pos32[m->cur], m->vcell, m->vlast, m->vnext,
                                                                  m->vrpos, m->vnbr, m->corner, m->Wc, m->nVertices,
                                                                  m->repR, t1test ? 1 : 0, (float)m->t1Threshold, m->t1);
    return check_launch();
}

int mixed_launch_force(svm_model* m) {
    k32_force<<<blocksFor(m->nVertices), kB, 0, m->stream>>>(args32(m, m->cur), m->nVertices, m->force32);
    return check_launch();
}

int mixed_launch_force_bd(svm_model* m, double T, double dt, double mu, int noiseMode, const double* noise,
                          uint64_t seed, int nxt) {
    const double fp = dt * mu, np = sqrt(2.0 * fp * T);
    const float* repNp = m->nRep > 1 ? m->repNp : nullptr;
    const int bs = m->blkForce, nb = (m->nVertices + bs - 1) / bs;
    if (noiseMode == SVM_NOISE_BUFFER)
        k32_force_bd<SVM_NOISE_BUFFER><<<nb, bs, 0, m->stream>>>(args32(m, m->cur), m->nVertices, m->force32,
                                                                m->pos32[nxt], noise, seed, m->stepCounter, (float)np,
                                                                repNp, (float)fp);
    else
        k32_force_bd<SVM_NOISE_PHILOX><<<nb, bs, 0, m->stream>>>(args32(m, m->cur), m->nVertices, m->force32,
                                                                m->pos32[nxt], noise, seed, m->stepCounter, (float)np,
                                                                repNp, (float)fp);
    return check_launch();
}

// largest block size (a multiple of 32) the batch's tuned kernels can launch with
static int max_block(const void* f) {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, f) != cudaSuccess) return 256;
    return a.maxThreadsPerBlock / 32 * 32;
}
int mixed_max_block_corners() { return max_block((const void*)k32_corners); }
int mixed_max_block_force() {
    return std::min(max_block((const void*)k32_force_bd<SVM_NOISE_PHILOX>),
                    max_block((const void*)k32_force_bd<SVM_NOISE_BUFFER>));
}

int mixed_launch_move(svm_model* m, const double* disp, double scale) {
    k32_move<<<blocksFor(m->nVertices), kB, 0, m->stream>>>(m->pos32[m->cur], disp, scale, m->nVertices, m->repR);
    return check_launch();
}

int mixed_upload_positions(svm_model* m, const double* deviceAos) {
    k_aos_to_f4<<<blocksFor(m->nVertices), kB, 0, m->stream>>>(deviceAos, m->pos32[m->cur], m->nVertices);
    return check_launch();
}

int mixed_download(svm_model* m, const float4* src, int n, double* deviceAos) {
    k_f4_to_aos<<<blocksFor(n), kB, 0, m->stream>>>(src, deviceAos, n);
    return check_launch();
}

}  // namespace svm

extern "C" int svm_model_set_precision(svm_model* m, int precision) {
    if (!m || precision < SVM_PRECISION_FP64 || precision > SVM_PRECISION_FP64_VECTOR) return SVM_ERR_ARG;
    if (m->nRep > 1 && precision != SVM_PRECISION_MIXED) return SVM_ERR_ARG;  // batches run mixed
    if (precision == m->precision) return SVM_OK;
    const bool toMixed = precision == SVM_PRECISION_MIXED, fromMixed = m->precision == SVM_PRECISION_MIXED;
    const size_t nV = m->nVertices, nC = m->nCells;
    if (toMixed) {
        if (!m->pos32[0]) {
            bool ok = cudaMalloc(&m->pos32[0], nV * sizeof(float4)) == cudaSuccess &&
                      cudaMalloc(&m->pos32[1], nV * sizeof(float4)) == cudaSuccess &&
                      cudaMalloc(&m->cellPos32, nC * sizeof(float4)) == cudaSuccess &&
                      cudaMalloc(&m->force32, nV * sizeof(float4)) == cudaSuccess &&
                      cudaMalloc(&m->dap32, nC * sizeof(float2)) == cudaSuccess;
            if (!ok) return SVM_ERR_CUDA;
            cudaMemsetAsync(m->force32, 0, nV * sizeof(float4), m->stream);
        }
        k_d4_to_f4<<<blocksFor(nV), kB, 0, m->stream>>>(m->pos[m->cur], m->pos32[m->cur], (int)nV);
    } else if (fromMixed) {
        k_f4_to_d4<<<blocksFor(nV), kB, 0, m->stream>>>(m->pos32[m->cur], m->pos[m->cur], (int)nV);
    }
    if (svm::check_launch()) return SVM_ERR_CUDA;
    m->precision = precision;
    m->cornersValid = false;
    m->paramsVersion++;
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}
