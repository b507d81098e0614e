// FIRE energy minimisation over velocity Verlet with every decision on the device.
//
// Restates energyMinimizerFIRE::minimize / fireStepCPU (src/updaters/energyMinimizerFIRE.cpp:
// 122-200) and velocityVerlet::integrateEOMCPU (src/updaters/velocityVerlet.cpp:6-38).  One
// iteration is
//   k_fire_vv1     per vertex: the previous iteration's FIRE velocity update, then
//                  disp = dt v + dt^2/2 F, v += dt/2 F / m, move onto the sphere (in place), and
//                  the moved vertex's norm for the corner pass
//   corners + T1   unless motion is restricted: k_edges (edge terms and the T1 length test),
//                  k_corner or k_corner_s, then the T1 pass (k_t1_parallel, k_t1_apply, k_t1_patch)
//   geometry       k_cells, k_fallback_fan (the corners too when motion is restricted)
//   k_fire_force   per vertex: F, v += dt/2 F / m, block partials of F.v, F.F, v.v, max |F|^2;
//                  the last block reduces them in a fixed order and runs the FIRE control
//                  (power test, dt / alpha adaptation, stopping test)
// The host launches captured batches of iterations and reads only the `done` flag between them.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>
#include "svm_internal.cuh"
#include "svm_force.cuh"

using namespace svm;

struct FireState {
    double dt, alpha, alphaUsed, scaling, power, forceNorm, velNorm, maxF2, rmsOverN, maxForce;
    double dtMin, dtMax, dtInc, dtDec, alphaStart, alphaDec, alphaMin, cutoff;
    int nMin, nSince, iterations, maxIterations, criterion, done, pending, zeroV;
};

struct svm_fire {
    svm_model* m = nullptr;
    FireState* d = nullptr;
    FireState h{};
    double* partials = nullptr;
    unsigned* ticket = nullptr;
    int nBlocks = 0;
    cudaGraphExec_t graph = nullptr;
    int graphCriterion = -1;
    int graphIters = 0;
    int graphCur = -1;
    unsigned graphVersion = ~0u;
};

namespace {

constexpr int kB = 256;

// Block sum (bmax: maximum) in a fixed order, valid in thread 0.  Warps from `live` on hold zeros and
// skip their shuffles (their +0.0 leaves the sum's bits unchanged).
__device__ double bsum(double v, double* sh, int live = 32) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < live)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    __syncthreads();
    return r;
}
__device__ double bmax(double v, double* sh, int live = 32) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < live)
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sh[w]);
    __syncthreads();
    return r;
}

__device__ __forceinline__ D3 move_exact_f(D3 p, D3 v, double R) {
    const double vp = __dadd_rn(__dadd_rn(__dmul_rn(v.x, p.x), __dmul_rn(v.y, p.y)), __dmul_rn(v.z, p.z));
    const double pp = __dadd_rn(__dadd_rn(__dmul_rn(p.x, p.x), __dmul_rn(p.y, p.y)), __dmul_rn(p.z, p.z));
    const double s = f64_div(vp, pp);
    D3 q{__dadd_rn(p.x, __dsub_rn(v.x, __dmul_rn(s, p.x))), __dadd_rn(p.y, __dsub_rn(v.y, __dmul_rn(s, p.y))),
         __dadd_rn(p.z, __dsub_rn(v.z, __dmul_rn(s, p.z)))};
    const double qq = __dadd_rn(__dadd_rn(__dmul_rn(q.x, q.x), __dmul_rn(q.y, q.y)), __dmul_rn(q.z, q.z));
    const double inv = f64_div(1.0, f64_sqrt(qq));
    return D3{__dmul_rn(R, __dmul_rn(inv, q.x)), __dmul_rn(R, __dmul_rn(inv, q.y)), __dmul_rn(R, __dmul_rn(inv, q.z))};
}

// FIRE velocity update of fireStepCPU (energyMinimizerFIRE.cpp:146-149, 168-172).
__device__ __forceinline__ D3 fire_velocity(const FireState& S, D3 v, D3 f) {
    if (S.zeroV) return D3{0.0, 0.0, 0.0};
    const double a1 = 1.0 - S.alphaUsed, as = S.alphaUsed * S.scaling;
    return D3{__dadd_rn(__dmul_rn(a1, v.x), __dmul_rn(as, f.x)), __dadd_rn(__dmul_rn(a1, v.y), __dmul_rn(as, f.y)),
              __dadd_rn(__dmul_rn(a1, v.z), __dmul_rn(as, f.z))};
}

// velocityVerlet::integrateEOMCPU's first loop for one vertex (velocityVerlet.cpp:14-20: unit
// masses, the model's masses being 1): disp = dt v + (dt^2 / 2) F, v += (dt / 2) F, then the move
// onto the sphere (moveParticles).  Products rounded before the sums, as on the CPU.
__device__ __forceinline__ void vv_drift(double4_32a* __restrict__ pos, double4_32a* __restrict__ vel,
                                         double* __restrict__ vnorm, int i, D3 v, D3 f, double dt, double R) {
    const double hv = (0.5 / 1.0) * dt, h2 = 0.5 * dt * dt;
    const D3 d{__dadd_rn(__dmul_rn(dt, v.x), __dmul_rn(h2, f.x)), __dadd_rn(__dmul_rn(dt, v.y), __dmul_rn(h2, f.y)),
               __dadd_rn(__dmul_rn(dt, v.z), __dmul_rn(h2, f.z))};
    v = D3{__dadd_rn(v.x, __dmul_rn(hv, f.x)), __dadd_rn(v.y, __dmul_rn(hv, f.y)), __dadd_rn(v.z, __dmul_rn(hv, f.z))};
    st3(vel, i, v);
    const D3 q = move_exact_f(ld3(pos, i), d, R);
    st3(pos, i, q);
    vnorm[i] = pos_norm(q);  // k_vnorm's value, for the corner pass that follows
}
// gpu_update_velocity (velocityVerlet.cu): v += (dt / 2) F / m with unit masses.
__device__ __forceinline__ D3 vv_kick(D3 v, D3 f, double dt) {
    const double hv = (0.5 / 1.0) * dt;
    return D3{__dadd_rn(v.x, __dmul_rn(hv, f.x)), __dadd_rn(v.y, __dmul_rn(hv, f.y)), __dadd_rn(v.z, __dmul_rn(hv, f.z))};
}

// The iteration's first kernel.  It leaves the pending flag as it is: the control of every iteration
// (k_fire_force's last block) sets it again before this kernel next reads it, and after the last
// iteration k_fire_finish applies the update it stands for.  Once FIRE has stopped, the positions
// stay and only their norms are written (the corner pass of a batch's remaining iterations reads them).
__global__ void k_fire_vv1(const FireState* __restrict__ Sp, double4_32a* __restrict__ pos,
                           double4_32a* __restrict__ vel, const double4_32a* __restrict__ force,
                           double* __restrict__ vnorm, int nV, double R) {
    const FireState S = *Sp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    if (S.done) {
        vnorm[i] = pos_norm(ld3(pos, i));
        return;
    }
    const D3 f = ld3(force, i);
    D3 v = ld3(vel, i);
    if (S.pending) v = fire_velocity(S, v, f);
    vv_drift(pos, vel, vnorm, i, v, f, S.dt, R);
}

// The standalone velocity-Verlet drift: vv_drift with the caller's dt.
__global__ void k_vv_drift(double4_32a* __restrict__ pos, double4_32a* __restrict__ vel,
                           const double4_32a* __restrict__ force, double* __restrict__ vnorm, int nV, double dt,
                           double R) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    vv_drift(pos, vel, vnorm, i, ld3(vel, i), ld3(force, i), dt, R);
}
__global__ void k_vv_half(double4_32a* __restrict__ vel, const double4_32a* __restrict__ force, int nV, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    st3(vel, i, vv_kick(ld3(vel, i), ld3(force, i), dt));
}

// F.v, F.F and v.v of one vertex, each a dot product accumulated in component order.
__device__ __forceinline__ void fire_dots(D3 f, D3 v, double& P, double& FF, double& VV) {
    P = __dadd_rn(__dadd_rn(__dmul_rn(f.x, v.x), __dmul_rn(f.y, v.y)), __dmul_rn(f.z, v.z));
    FF = __dadd_rn(__dadd_rn(__dmul_rn(f.x, f.x), __dmul_rn(f.y, f.y)), __dmul_rn(f.z, f.z));
    VV = __dadd_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), __dmul_rn(v.z, v.z));
}

// The block partials of (F.v, F.F, v.v, max F.F), then, in the last block to finish, their sums in a
// fixed order.  kControl: the last block runs fireStepCPU's control on them (energyMinimizerFIRE.cpp:
// 138-172: scaling, power test, dt / alpha adaptation; the velocity update is left pending for the
// next vertex kernel); kCount: also minimize's iteration count and stopping test (cpp:187-191).
// Without kControl the four totals go to out4.  Every thread of the block calls it.
template <bool kControl, bool kCount>
__device__ void fire_reduce_tail(FireState* __restrict__ Sp, double P, double FF, double VV, int nV,
                                 double* __restrict__ partials, unsigned* __restrict__ ticket, double* __restrict__ out4,
                                 double* sh, bool& amLast) {
    constexpr int kLive = kSlotVerts / 32;  // the warps of the block's vertex threads
    const double bP = bsum(P, sh, kLive), bF = bsum(FF, sh, kLive), bV = bsum(VV, sh, kLive), bM = bmax(FF, sh, kLive);
    if (threadIdx.x == 0) {
        double* q = partials + 4 * blockIdx.x;
        q[0] = bP; q[1] = bF; q[2] = bV; q[3] = bM;
        __threadfence();
        amLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!amLast) return;
    double sP = 0.0, sF = 0.0, sV = 0.0, sM = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        sP += __ldcg(partials + 4 * b); sF += __ldcg(partials + 4 * b + 1);
        sV += __ldcg(partials + 4 * b + 2); sM = fmax(sM, __ldcg(partials + 4 * b + 3));
    }
    const double tP = bsum(sP, sh), tF = bsum(sF, sh), tV = bsum(sV, sh), tM = bmax(sM, sh);
    if (threadIdx.x != 0) return;
    *ticket = 0u;
    if (!kControl) {
        out4[0] = tP; out4[1] = tF; out4[2] = tV; out4[3] = tM;
        return;
    }
    FireState S = *Sp;
    S.power = tP; S.forceNorm = tF; S.velNorm = tV; S.maxF2 = tM;
    S.rmsOverN = sqrt(tF) / (double)nV;
    S.maxForce = sqrt(tM);
    S.scaling = tF > 0. ? sqrt(tV / tF) : 0.0;
    S.alphaUsed = S.alpha;
    S.zeroV = tP > 0 ? 0 : 1;
    if (tP > 0) {
        if (S.nSince > S.nMin) {
            S.dt = fmin(S.dt * S.dtInc, S.dtMax);
            S.alpha = S.alpha * S.alphaDec;
            S.alpha = fmax(S.alpha, S.alphaMin);
        }
        S.nSince += 1;
    } else {
        S.nSince = 0;
        S.dt = S.dt * S.dtDec;
        S.dt = fmax(S.dt, S.dtMin);
        S.alpha = S.alphaStart;
    }
    S.pending = 1;
    if (kCount) {
        S.iterations += 1;
        const double crit = S.criterion == SVM_FIRE_MAX_FORCE ? S.maxForce : S.rmsOverN;
        if (S.iterations >= S.maxIterations || !(crit > S.cutoff)) S.done = 1;
    }
    *Sp = S;
}

// Blocks of 3 kSlotVerts threads: three per vertex for the force (one per cell slot), then the
// first kSlotVerts threads finish their vertex.  One instantiation per force form: the vector form
// alone fits 78 registers without spill, so four blocks per SM (a 40k-vertex sphere's 625 blocks in
// 1.03 waves of them instead of 1.37 waves of three; measured 0.171 against 0.172 ms per FIRE
// iteration at 20k cells).
template <int kForm>
__global__ void __launch_bounds__(3 * kSlotVerts, kForm == kFormVector ? 4 : kSlotMinBlocks)
    k_fire_force(ForceArgs A, FireState* __restrict__ Sp, int nV, double4_32a* __restrict__ force,
                 double4_32a* __restrict__ vel, double* __restrict__ partials, unsigned* __restrict__ ticket) {
    __shared__ double sh[32];
    __shared__ bool amLast;
    __shared__ SlotShared slots;
    if (Sp->done) return;
    const double dt = Sp->dt;
    const D3 fv = block_slot_force<kForm>(A, nV, slots);
    const int i = blockIdx.x * kSlotVerts + threadIdx.x;
    double P = 0.0, FF = 0.0, VV = 0.0;
    if (threadIdx.x < kSlotVerts && i < nV) {
        const D3 f = fv;
        st3(force, i, f);
        const D3 v = vv_kick(ld3(vel, i), f, dt);
        st3(vel, i, v);
        fire_dots(f, v, P, FF, VV);
    }
    fire_reduce_tail<true, true>(Sp, P, FF, VV, nV, partials, ticket, nullptr, sh, amLast);
}

// fireStep (energyMinimizerFIRE.h:56, fireStepCPU cpp:122-174) on the current forces and
// velocities: the sums and the control, in blocks of 3 kSlotVerts threads whose first kSlotVerts
// hold one vertex each, which is k_fire_force's layout, so the sums are bitwise those of a
// minimize iteration.  With kControl false: the four totals to out4 (gpu_dVec_dot_products).
template <bool kControl>
__global__ void __launch_bounds__(3 * kSlotVerts) k_fire_sums(FireState* __restrict__ Sp, int nV,
                                                              const double4_32a* __restrict__ force,
                                                              const double4_32a* __restrict__ vel,
                                                              double* __restrict__ partials,
                                                              unsigned* __restrict__ ticket, double* __restrict__ out4) {
    __shared__ double sh[32];
    __shared__ bool amLast;
    const int i = blockIdx.x * kSlotVerts + threadIdx.x;
    double P = 0.0, FF = 0.0, VV = 0.0;
    if (threadIdx.x < kSlotVerts && i < nV) fire_dots(ld3(force, i), ld3(vel, i), P, FF, VV);
    fire_reduce_tail<kControl, false>(Sp, P, FF, VV, nV, partials, ticket, out4, sh, amLast);
}

// Applies a pending FIRE velocity update (after the loop ends).
__global__ void k_fire_finish(FireState* __restrict__ Sp, double4_32a* __restrict__ vel,
                              const double4_32a* __restrict__ force, int nV) {
    const FireState S = *Sp;
    if (!S.pending) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    st3(vel, i, fire_velocity(S, ld3(vel, i), ld3(force, i)));
}
__global__ void k_fire_clear_pending(FireState* Sp) { Sp->pending = 0; }

ForceArgs fargs(svm_model* m) { return force_args(m, m->cur); }

int fire_iteration(svm_fire* F) {
    svm_model* m = F->m;
    const int bs = spread_block(m, m->nVertices), nb = (m->nVertices + bs - 1) / bs;
    {
        PhaseTimer pt(m, SVM_PHASE_MOVE);
        k_fire_vv1<<<nb, bs, 0, m->stream>>>(F->d, m->pos[m->cur], m->vel, m->force, m->vnorm, m->nVertices, m->R);
    }
    m->cornersValid = false;
    int rc;
    if (!m->restricted) {
        rc = launch_corners(m, true, /*vnormReady=*/true);
        if (rc) return rc;
        rc = launch_t1_apply(m, 0);
        if (rc) return rc;
    }
    rc = launch_geometry(m);
    if (rc) return rc;
    PhaseTimer pt(m, SVM_PHASE_FORCE);
    const int nf = (m->nVertices + kSlotVerts - 1) / kSlotVerts;
    if (m->precision == SVM_PRECISION_FP64_VECTOR)
        k_fire_force<kFormVector><<<nf, 3 * kSlotVerts, 0, m->stream>>>(fargs(m), F->d, m->nVertices, m->force, m->vel,
                                                                        F->partials, F->ticket);
    else
        k_fire_force<kFormReference><<<nf, 3 * kSlotVerts, 0, m->stream>>>(fargs(m), F->d, m->nVertices, m->force,
                                                                           m->vel, F->partials, F->ticket);
    return check_launch();
}

}  // namespace

namespace svm {
void fire_detach(svm_fire* F) { F->m = nullptr; }
}  // namespace svm

extern "C" {

int svm_fire_create(svm_model* m, double dt, double alphaStart, double dtMax, double dtInc, double dtDec,
                    double alphaDec, int nMin, double forceCutoff, double alphaMin, int maxIterations, svm_fire** out) {
    if (!m || !out || !(dt > 0) || maxIterations < 0) return SVM_ERR_ARG;
    svm_fire* F = new svm_fire();
    F->m = m;
    m->fires.push_back(F);
    FireState& S = F->h;
    S = FireState{};
    S.dt = dt; S.dtMin = dt * .01; S.alphaStart = alphaStart; S.alpha = alphaStart; S.dtMax = dtMax;
    S.dtInc = dtInc; S.dtDec = dtDec; S.alphaDec = alphaDec; S.nMin = nMin; S.cutoff = forceCutoff;
    S.alphaMin = alphaMin; S.maxIterations = maxIterations; S.rmsOverN = 100.; S.maxForce = 100.;
    F->nBlocks = (m->nVertices + kSlotVerts - 1) / kSlotVerts;  // blocks of k_fire_force
    bool ok = cudaMalloc(&F->d, sizeof(FireState)) == cudaSuccess &&
              cudaMalloc(&F->partials, sizeof(double) * 4 * (F->nBlocks + 1)) == cudaSuccess &&
              cudaMalloc(&F->ticket, sizeof(unsigned)) == cudaSuccess;
    if (!ok) { svm_fire_destroy(F); return SVM_ERR_CUDA; }
    cudaMemsetAsync(F->ticket, 0, sizeof(unsigned), m->stream);
    cudaMemcpyAsync(F->d, &S, sizeof(FireState), cudaMemcpyHostToDevice, m->stream);
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) { svm_fire_destroy(F); return SVM_ERR_CUDA; }
    *out = F;
    return SVM_OK;
}

int svm_fire_destroy(svm_fire* F) {
    if (!F) return SVM_ERR_ARG;
    if (F->m) {
        auto& v = F->m->fires;
        v.erase(std::remove(v.begin(), v.end(), F), v.end());
        if (F->m->stream) cudaStreamSynchronize(F->m->stream);
    }
    if (F->graph) cudaGraphExecDestroy(F->graph);
    if (F->d) cudaFree(F->d);
    if (F->partials) cudaFree(F->partials);
    if (F->ticket) cudaFree(F->ticket);
    delete F;
    return SVM_OK;
}

int svm_fire_minimize(svm_fire* F, int criterion, int* iterations, double* value) {
    if (!F || !F->m) return SVM_ERR_ARG;
    svm_model* m = F->m;
    if (m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;  // FIRE runs in the FP64 forms
    FireState S;
    if (cudaMemcpyAsync(&S, F->d, sizeof(FireState), cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    const int it0 = S.iterations;
    S.criterion = criterion;
    S.done = S.iterations >= S.maxIterations ? 1 : 0;
    S.rmsOverN = 110.0; S.maxForce = 110.0;  // minimize() restarts the stopping test (cpp:187)
    cudaMemcpyAsync(F->d, &S, sizeof(FireState), cudaMemcpyHostToDevice, m->stream);
    int rc = svm_model_compute_forces(m);  // sim->computeForces() before the loop (cpp:186)
    if (rc) return rc;
    // iterations in captured batches; kernels of a batch after convergence return at once
    const int batch = 32;
    auto ensure_graph = [&]() -> int {
        if (F->graph && F->graphCriterion == criterion && F->graphIters == batch && F->graphCur == m->cur &&
            F->graphVersion == m->paramsVersion)
            return SVM_OK;
        if (F->graph) { cudaGraphExecDestroy(F->graph); F->graph = nullptr; }
        cudaGraph_t g;
        if (cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return SVM_ERR_CUDA;
        int r = SVM_OK;
        for (int k = 0; k < batch && !r; ++k) r = fire_iteration(F);
        cudaError_t ce = cudaStreamEndCapture(m->stream, &g);
        if (r || ce != cudaSuccess) { cudaGetLastError(); return SVM_ERR_CUDA; }
        ce = cudaGraphInstantiate(&F->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) { F->graph = nullptr; return SVM_ERR_CUDA; }
        F->graphCriterion = criterion;
        F->graphIters = batch;
        F->graphCur = m->cur;
        F->graphVersion = m->paramsVersion;
        return SVM_OK;
    };
    int* doneHost = nullptr;
    cudaMallocHost(&doneHost, sizeof(int));
    while (true) {
        // the ring capacity is checked between batches (the host waits for each batch anyway)
        if (!m->restricted && (rc = ensure_ring_headroom(m))) { cudaFreeHost(doneHost); return rc; }
        if ((rc = ensure_graph())) { cudaFreeHost(doneHost); return rc; }
        if (cudaGraphLaunch(F->graph, m->stream) != cudaSuccess) { cudaFreeHost(doneHost); return SVM_ERR_CUDA; }
        cudaMemcpyAsync(doneHost, &F->d->done, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
        if (cudaStreamSynchronize(m->stream) != cudaSuccess) { cudaFreeHost(doneHost); return SVM_ERR_CUDA; }
        if (*doneHost) break;
    }
    cudaFreeHost(doneHost);
    const int nb = (m->nVertices + kB - 1) / kB;
    k_fire_finish<<<nb, kB, 0, m->stream>>>(F->d, m->vel, m->force, m->nVertices);
    k_fire_clear_pending<<<1, 1, 0, m->stream>>>(F->d);
    if (check_launch()) return SVM_ERR_CUDA;
    if (cudaMemcpyAsync(&S, F->d, sizeof(FireState), cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    F->h = S;
    if (iterations) *iterations = S.iterations - it0;
    if (value) *value = criterion == SVM_FIRE_MAX_FORCE ? S.maxForce : S.rmsOverN;
    return SVM_OK;
}

// ---- per-phase entry points (the reference's fireStep, velocityVerlet and dot-product launchers)

int svm_fire_step(svm_fire* F) {
    if (!F || !F->m) return SVM_ERR_ARG;
    svm_model* m = F->m;
    if (m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    const int nb = (m->nVertices + kSlotVerts - 1) / kSlotVerts;
    k_fire_sums<true><<<nb, 3 * kSlotVerts, 0, m->stream>>>(F->d, m->nVertices, m->force, m->vel, F->partials,
                                                            F->ticket, nullptr);
    k_fire_finish<<<(m->nVertices + kB - 1) / kB, kB, 0, m->stream>>>(F->d, m->vel, m->force, m->nVertices);
    k_fire_clear_pending<<<1, 1, 0, m->stream>>>(F->d);
    return check_launch();
}

int svm_vv_half(svm_model* m, double dt) {
    if (!m || !(dt == dt) || m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    k_vv_half<<<(m->nVertices + kB - 1) / kB, kB, 0, m->stream>>>(m->vel, m->force, m->nVertices, dt);
    return check_launch();
}

int svm_velocity_verlet_step(svm_model* m, double dt, int nSteps) {
    if (!m || !(dt == dt) || nSteps < 0 || m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    const int bs = spread_block(m, m->nVertices), nb = (m->nVertices + bs - 1) / bs;
    for (int k = 0; k < nSteps; ++k) {
        {
            PhaseTimer pt(m, SVM_PHASE_MOVE);
            k_vv_drift<<<nb, bs, 0, m->stream>>>(m->pos[m->cur], m->vel, m->force, m->vnorm, m->nVertices, dt, m->R);
        }
        m->cornersValid = false;
        int rc;
        if (!m->restricted) {  // moveParticles -> enforceTopology (sphericalVertexModel.cpp:111-148)
            rc = launch_corners(m, true, /*vnormReady=*/true);
            if (rc) return rc;
            rc = launch_t1_apply(m, 0);
            if (rc) return rc;
        }
        rc = launch_geometry(m);  // sim->computeForces(): geometry, then forces
        if (rc) return rc;
        {
            PhaseTimer pt(m, SVM_PHASE_FORCE);
            rc = launch_force_fp64(m);
            if (rc) return rc;
        }
        k_vv_half<<<nb, bs, 0, m->stream>>>(m->vel, m->force, m->nVertices, dt);
        if (check_launch()) return SVM_ERR_CUDA;
    }
    return SVM_OK;
}

int svm_reduce_dots(svm_model* m, double* out4) {
    if (!m || !out4 || m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    const int nb = (m->nVertices + kSlotVerts - 1) / kSlotVerts;
    if (!m->dotPartials && cudaMalloc(&m->dotPartials, sizeof(double) * 4 * (size_t)(nb + 1)) != cudaSuccess)
        return SVM_ERR_CUDA;
    k_fire_sums<false><<<nb, 3 * kSlotVerts, 0, m->stream>>>(nullptr, m->nVertices, m->force, m->vel, m->dotPartials,
                                                             m->ticket + 3, m->scalars + 8);
    if (check_launch()) return SVM_ERR_CUDA;
    double r[4];
    if (cudaMemcpyAsync(r, m->scalars + 8, sizeof(r), cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    out4[0] = r[0]; out4[1] = r[1]; out4[2] = r[2]; out4[3] = sqrt(r[3]);
    return SVM_OK;
}

int svm_fire_set_max_iterations(svm_fire* F, int maxIterations) {
    if (!F || !F->m || maxIterations < 0) return SVM_ERR_ARG;
    svm_model* m = F->m;
    FireState S;
    if (cudaMemcpyAsync(&S, F->d, sizeof(FireState), cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    S.maxIterations = maxIterations;
    F->h.maxIterations = maxIterations;
    if (cudaMemcpyAsync(F->d, &S, sizeof(FireState), cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    return SVM_OK;
}

int svm_fire_state(svm_fire* F, double* s7) {
    if (!F || !F->m || !s7) return SVM_ERR_ARG;
    FireState S;
    if (cudaMemcpyAsync(&S, F->d, sizeof(FireState), cudaMemcpyDeviceToHost, F->m->stream) != cudaSuccess ||
        cudaStreamSynchronize(F->m->stream) != cudaSuccess) return SVM_ERR_CUDA;
    s7[0] = S.dt; s7[1] = S.alpha; s7[2] = S.power; s7[3] = S.rmsOverN; s7[4] = S.maxForce;
    s7[5] = S.nSince; s7[6] = S.iterations;
    return SVM_OK;
}

}  // extern "C"
