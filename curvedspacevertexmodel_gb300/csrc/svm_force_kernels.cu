// The FP64 force kernels of the plain form: computeForce (sphericalVertexModel.cpp:356-420) alone
// and fused with the Brownian displacement and the move (brownianDynamics.cpp:37-44,
// sphericalDomain.h:203-209).  Kept in its own translation unit so that its contraction setting
// can differ from the geometry's; it is built without FMA contraction like the rest (the force's
// rounding then differs from the CPU's only through acos), and the displacement and the move spell
// out every product and sum with __dmul_rn / __dadd_rn.
#include <mutex>

#include "svm_force.cuh"

namespace svm {
int check_launch();
}

namespace {
// The ziggurat table of this device, built once by k_zig_init (zig_init) from r alone:
// v = r f(r) + sqrt(pi/2) erfc(r / sqrt 2), then f(x_{i+1}) = v / x_i + f(x_i).
__device__ svm::ZigTable gZig;

__global__ void k_zig_init() {
    const double r = svm::kZigR, fr = exp(-0.5 * r * r);
    const double v = r * fr + sqrt(0.5 * svm::kPI) * erfc(r / sqrt(2.0));
    gZig.x[0] = v / fr;
    gZig.f[0] = 0.0;
    gZig.x[1] = r;
    gZig.f[1] = fr;
    for (int i = 1; i < 255; ++i) {
        const double f1 = v / gZig.x[i] + gZig.f[i];
        gZig.f[i + 1] = f1;
        gZig.x[i + 1] = sqrt(-2.0 * log(f1));
    }
    gZig.x[256] = 0.0;
    gZig.f[256] = 1.0;
}
}  // namespace

namespace {
using namespace svm;

// Blocks of 3 kSlotVerts threads, three per vertex (one per cell slot), kSlotVerts vertices each.
__global__ void __launch_bounds__(3 * kSlotVerts, kSlotMinBlocks) k_force(ForceArgs A, int nV,
                                                                         double4_32a* __restrict__ force) {
    __shared__ SlotShared sh;
    const D3 f = block_slot_force(A, nV, sh);
    const int v = blockIdx.x * kSlotVerts + threadIdx.x;
    if (threadIdx.x >= kSlotVerts || v >= nV) return;
    st3(force, v, f);
}

// Fused Brownian step for one vertex: force, displacement, move; reads `A.pos`, writes posNext (and
// hostOut, when non-null).  (Writing the moved vertex's norm here as well, which would spare the
// corner pass its k_vnorm, made this FP64-bound kernel as much slower as the corner pass got faster.)
template <int kNoise>
__global__ void __launch_bounds__(3 * kSlotVerts, kSlotMinBlocks) k_force_bd(
                                                             ForceArgs A, int nV, double4_32a* __restrict__ force,
                                                             double4_32a* __restrict__ posNext,
                                                             const double* __restrict__ noise, uint64_t seed,
                                                             const unsigned long long* __restrict__ stepCounter,
                                                             double np, double fp, const ZigTable* __restrict__ zig,
                                                             double* __restrict__ hostOut) {
    __shared__ SlotShared sh;
    const D3 f = block_slot_force(A, nV, sh);
    const int v = blockIdx.x * kSlotVerts + threadIdx.x;
    if (threadIdx.x >= kSlotVerts || v >= nV) return;
    st3(force, v, f);
    D3 xi;
    if (kNoise == SVM_NOISE_BUFFER) xi = D3{noise[3 * v], noise[3 * v + 1], noise[3 * v + 2]};
    else xi = philox_normals3(zig, seed, *stepCounter, v);
    const D3 d{bd_disp(xi.x, np, f.x, fp), bd_disp(xi.y, np, f.y, fp), bd_disp(xi.z, np, f.z, fp)};
    const D3 q = move_exact(ld3(A.pos, v), d, A.R);
    st3(posNext, v, q);
    // a host-buffer step's output, straight into the caller's mapped page-locked array (AoS)
    if (hostOut) { hostOut[3 * v] = q.x; hostOut[3 * v + 1] = q.y; hostOut[3 * v + 2] = q.z; }
}

}  // namespace

namespace svm {

int launch_force_fp64(svm_model* m) {
    const int nb = (m->nVertices + kSlotVerts - 1) / kSlotVerts;
    k_force<<<nb, 3 * kSlotVerts, 0, m->stream>>>(force_args(m, m->cur), m->nVertices, m->force);
    return check_launch();
}

// Builds this device's ziggurat table once (outside any stream capture: called at model creation).
static ZigTable* gZigAddr[64] = {};  // per device, once built
int zig_init() {
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SVM_ERR_CUDA;
    std::lock_guard<std::mutex> lock(mu);
    if (gZigAddr[dev]) return SVM_OK;
    ZigTable* addr = nullptr;
    if (cudaGetSymbolAddress((void**)&addr, gZig) != cudaSuccess) return SVM_ERR_CUDA;
    k_zig_init<<<1, 1>>>();
    if (check_launch() || cudaDeviceSynchronize() != cudaSuccess) return SVM_ERR_CUDA;
    gZigAddr[dev] = addr;
    return SVM_OK;
}

int launch_force_bd_fp64(svm_model* m, double np, double fp, int noiseMode, const double* noise, uint64_t seed,
                         int nxt) {
    const int nb = (m->nVertices + kSlotVerts - 1) / kSlotVerts;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || !gZigAddr[dev]) return SVM_ERR_CUDA;
    const ZigTable* zig = gZigAddr[dev];
    if (noiseMode == SVM_NOISE_BUFFER)
        k_force_bd<SVM_NOISE_BUFFER><<<nb, 3 * kSlotVerts, 0, m->stream>>>(
            force_args(m, m->cur), m->nVertices, m->force, m->pos[nxt], noise, seed, m->stepCounter, np, fp, zig,
            m->ioHostOut);
    else
        k_force_bd<SVM_NOISE_PHILOX><<<nb, 3 * kSlotVerts, 0, m->stream>>>(
            force_args(m, m->cur), m->nVertices, m->force, m->pos[nxt], noise, seed, m->stepCounter, np, fp, zig,
            m->ioHostOut);
    return check_launch();
}

}  // namespace svm
