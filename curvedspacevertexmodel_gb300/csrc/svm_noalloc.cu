// Allocation-free energy reduction (svm_energy_noalloc in include/svm.h).
//
// Some callers cannot call cudaMalloc: hosts whose device memory is handed in full to their own
// pool allocator (a raw cudaMalloc there fails or fragments the pool), and per-step code that
// must not pay cudaMalloc's implicit device-wide synchronisation.  This entry point computes the
// model energy sum_c Kr (A - A0)^2 + (P - P0)^2 from caller-owned device arrays without
// allocating: the per-block partial sums and the completion ticket live in one file-scope device
// array of fixed size, shared by every call on a device.
//
// Limits and rules:
//   * nCells <= SVM_NOALLOC_MAX_CELLS (8192 blocks of 256 cells); larger inputs are rejected.
//   * The array keeps the last call's contents; the ticket that must start at zero is cleared on
//     the caller's stream before each launch.
//   * Calls that overlap on the GPU (e.g. on two streams at once) race on the shared array.
//   * The first call on a device looks up the array's device address with cudaGetSymbolAddress
//     (with that device current) and caches it; make that first call before any stream capture.
#include <mutex>
#include "svm_internal.cuh"

namespace {

constexpr int kNaBlock = 256;
constexpr int kNaMaxBlocks = SVM_NOALLOC_MAX_CELLS / kNaBlock;
constexpr int kNaMaxDevices = 64;

// [0, kNaMaxBlocks): per-block partial sums; [kNaMaxBlocks]: completion ticket (as unsigned).
static __device__ __align__(256) double g_noallocScratch[kNaMaxBlocks + 32];

std::mutex g_noallocMutex;
double* g_noallocScratchPtr[kNaMaxDevices] = {nullptr};

__device__ double na_block_sum(double v, double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    __syncthreads();
    return r;
}

__global__ void k_energy_noalloc(const double2* __restrict__ ap, const double2* __restrict__ pref, double Kr, int nC,
                                 double* scratch, double* __restrict__ out) {
    __shared__ double sh[32];
    __shared__ bool amLast;
    unsigned* ticket = reinterpret_cast<unsigned*>(scratch + kNaMaxBlocks);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (c < nC) {
        const double da = ap[c].x - pref[c].x, dp = ap[c].y - pref[c].y;
        e = __dadd_rn(__dmul_rn(__dmul_rn(Kr, da), da), __dmul_rn(dp, dp));
    }
    const double bs = na_block_sum(e, sh);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = bs;
        __threadfence();
        amLast = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!amLast) return;
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(scratch + b);
    const double total = na_block_sum(s, sh);
    if (threadIdx.x == 0) {
        *out = total;
        *ticket = 0u;
    }
}

// Device address of the scratch array for the current device, looked up once per device.
int noalloc_scratch(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return SVM_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocScratchPtr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noallocScratch) != cudaSuccess || !p) return SVM_ERR_CUDA;
        g_noallocScratchPtr[dev] = static_cast<double*>(p);
    }
    *out = g_noallocScratchPtr[dev];
    return SVM_OK;
}

}  // namespace

extern "C" int svm_energy_noalloc(const double* areaPerimeter, const double* preference, double kr, int nCells,
                                  double* energy, void* stream) {
    if (!areaPerimeter || !preference || !energy || nCells <= 0 || nCells > SVM_NOALLOC_MAX_CELLS) return SVM_ERR_ARG;
    double* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != SVM_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(scratch + kNaMaxBlocks, 0, sizeof(unsigned), s) != cudaSuccess) return SVM_ERR_CUDA;
    const int blocks = (nCells + kNaBlock - 1) / kNaBlock;
    k_energy_noalloc<<<blocks, kNaBlock, 0, s>>>(reinterpret_cast<const double2*>(areaPerimeter),
                                                 reinterpret_cast<const double2*>(preference), kr, nCells, scratch,
                                                 energy);
    return cudaGetLastError() == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}
