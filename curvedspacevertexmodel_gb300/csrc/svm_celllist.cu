// Cell list of points on (or near) the sphere: hyperrectangularCellList on the GPU.
//
// Restates setGridSize and computeCPU of src/utilities/hyperrectangularCellList.cpp:27-51,
// 165-214: a cubic grid over [-r, r]^3 with floor(2r / a) cells per side made even,
// h = 2r / cells, bin_d = floor((x_d + r) / h), flat index x + y n + z n^2
// (inc/indexer.h:170-176).  The reference GPU kernel (hyperrectangularCellList.cu:14-51) fills
// slots in atomic order; here the slots of a bin are put in ascending point index, as the CPU
// loop leaves them, so the table is deterministic.  Kernels:
//   k_cl_clear   zero the counts of the bins the previous call used (not the whole grid)
//   k_cl_bin     bin each point, take a provisional slot with an atomic
//   k_cl_order   rank each point among its bin's entries by index, write the final slot
//   k_cl_nmax    Nmax = max(Nmax, largest occupancy), the grow-only width of the reference
#include <cmath>
#include <cstdio>
#include <vector>
#include "svm_internal.cuh"

using namespace svm;

struct svm_cell_list {
    double a = 1.0, radius = 1.0, h = 1.0;
    int nside = 0, cap = 0, nPoints = 0;
    long total = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    unsigned* counts = nullptr;   // [total]
    int* tmp = nullptr;           // [total * cap] provisional slots
    int* slots = nullptr;         // [total * cap] ordered slots
    int* binOf = nullptr;         // [nPoints]
    int* scalars = nullptr;       // [0] max occupancy this call, [1] Nmax (grow-only), [2] overflow, [3] out of grid
    bool first = true;
};

namespace {
constexpr int kB = 256;

__device__ __forceinline__ int bin_of(double x, double y, double z, double r, double h, int n, int* bad) {
    int bx = (int)floor((x + r) / h), by = (int)floor((y + r) / h), bz = (int)floor((z + r) / h);
    if (bx < 0 || by < 0 || bz < 0 || bx >= n || by >= n || bz >= n) {
        atomicExch(bad, 1);
        bx = min(max(bx, 0), n - 1); by = min(max(by, 0), n - 1); bz = min(max(bz, 0), n - 1);
    }
    return bx + by * n + bz * n * n;
}

__global__ void k_cl_clear(const int* __restrict__ binOf, unsigned* counts, int np) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np && binOf[i] >= 0) counts[binOf[i]] = 0u;
}

template <typename P>
__global__ void k_cl_bin(P pts, int np, double r, double h, int n, int cap, int* __restrict__ binOf,
                         unsigned* __restrict__ counts, int* __restrict__ tmp, int* __restrict__ scalars) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    double x, y, z;
    pts(i, x, y, z);
    const int b = bin_of(x, y, z, r, h, n, scalars + 3);
    binOf[i] = b;
    const unsigned s = atomicAdd(counts + b, 1u);
    if ((int)s < cap) tmp[(long)b * cap + s] = i;
    else atomicExch(scalars + 2, 1);
    atomicMax(scalars, (int)s + 1);
}

__global__ void k_cl_order(const int* __restrict__ binOf, const unsigned* __restrict__ counts,
                           const int* __restrict__ tmp, int* __restrict__ slots, int np, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int b = binOf[i];
    const int c = min((int)counts[b], cap);
    const int* t = tmp + (long)b * cap;
    int rank = 0;
    bool present = false;
    for (int k = 0; k < c; ++k) {
        const int j = t[k];
        rank += j < i;
        present |= j == i;
    }
    if (present) slots[(long)b * cap + rank] = i;
}

__global__ void k_cl_nmax(int* scalars) {
    scalars[1] = max(scalars[1], scalars[0]);
}

struct ModelPoints {
    const double4_32a* p;
    __device__ void operator()(int i, double& x, double& y, double& z) const { const double4_32a q = p[i]; x = q.x; y = q.y; z = q.z; }
};
struct ModelPoints32 {
    const float4* p;
    __device__ void operator()(int i, double& x, double& y, double& z) const { const float4 q = p[i]; x = q.x; y = q.y; z = q.z; }
};
struct AosPoints {
    const double* p;
    __device__ void operator()(int i, double& x, double& y, double& z) const { x = p[3 * i]; y = p[3 * i + 1]; z = p[3 * i + 2]; }
};

template <typename P>
int compute(svm_cell_list* cl, P pts, int np) {
    if (np != cl->nPoints) return SVM_ERR_ARG;
    const int nb = (np + kB - 1) / kB;
    k_cl_clear<<<nb, kB, 0, cl->stream>>>(cl->binOf, cl->counts, np);
    cudaMemsetAsync(cl->scalars, 0, sizeof(int), cl->stream);      // occupancy of this call
    cudaMemsetAsync(cl->scalars + 2, 0, 2 * sizeof(int), cl->stream);  // this call's error flags
    k_cl_bin<<<nb, kB, 0, cl->stream>>>(pts, np, cl->radius, cl->h, cl->nside, cl->cap, cl->binOf, cl->counts, cl->tmp,
                                        cl->scalars);
    k_cl_order<<<nb, kB, 0, cl->stream>>>(cl->binOf, cl->counts, cl->tmp, cl->slots, np, cl->cap);
    k_cl_nmax<<<1, 1, 0, cl->stream>>>(cl->scalars);
    return check_launch();
}
}  // namespace

extern "C" {

int svm_cell_list_create(double a, double radius, int nPoints, int cap, void* stream, svm_cell_list** out) {
    if (!(a > 0) || !(radius > 0) || nPoints <= 0 || cap < 2 || !out) return SVM_ERR_ARG;
    svm_cell_list* cl = new svm_cell_list();
    cl->a = a; cl->radius = radius; cl->nPoints = nPoints; cl->cap = cap;
    const double b = 2. * radius;  // setGridSize (hyperrectangularCellList.cpp:31-41)
    unsigned n = (unsigned)std::floor(b / a);
    if (n % 2 == 1) n -= 1;
    if (n == 0) { delete cl; return SVM_ERR_ARG; }
    cl->nside = (int)n;
    cl->h = b / n;
    cl->total = (long)n * n * n;
    if (stream) cl->stream = (cudaStream_t)stream;
    else { cudaStreamCreateWithFlags(&cl->stream, cudaStreamNonBlocking); cl->ownStream = true; }
    bool ok = cudaMalloc(&cl->counts, sizeof(unsigned) * cl->total) == cudaSuccess &&
              cudaMalloc(&cl->tmp, sizeof(int) * cl->total * cap) == cudaSuccess &&
              cudaMalloc(&cl->slots, sizeof(int) * cl->total * cap) == cudaSuccess &&
              cudaMalloc(&cl->binOf, sizeof(int) * nPoints) == cudaSuccess &&
              cudaMalloc(&cl->scalars, sizeof(int) * 4) == cudaSuccess;
    if (!ok) { svm_cell_list_destroy(cl); return SVM_ERR_CUDA; }
    cudaMemsetAsync(cl->counts, 0, sizeof(unsigned) * cl->total, cl->stream);
    cudaMemsetAsync(cl->binOf, 0xff, sizeof(int) * nPoints, cl->stream);
    const int init[4] = {0, 2, 0, 0};  // Nmax starts at 2 (hyperrectangularCellList.cpp:17,47)
    cudaMemcpyAsync(cl->scalars, init, sizeof(init), cudaMemcpyHostToDevice, cl->stream);
    if (cudaStreamSynchronize(cl->stream) != cudaSuccess) { svm_cell_list_destroy(cl); return SVM_ERR_CUDA; }
    *out = cl;
    return SVM_OK;
}

int svm_cell_list_destroy(svm_cell_list* cl) {
    if (!cl) return SVM_ERR_ARG;
    if (cl->stream) cudaStreamSynchronize(cl->stream);
    void* ptrs[] = {cl->counts, cl->tmp, cl->slots, cl->binOf, cl->scalars};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (cl->ownStream && cl->stream) cudaStreamDestroy(cl->stream);
    delete cl;
    return SVM_OK;
}

int svm_cell_list_compute_model(svm_cell_list* cl, svm_model* m) {
    if (!cl || !m) return SVM_ERR_ARG;
    if (cl->stream != m->stream) {
        // order after the model's pending work
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        cudaEventRecord(e, m->stream);
        cudaStreamWaitEvent(cl->stream, e, 0);
        cudaEventDestroy(e);
    }
    if (m->precision == SVM_PRECISION_MIXED) return compute(cl, ModelPoints32{m->pos32[m->cur]}, m->nVertices);
    return compute(cl, ModelPoints{m->pos[m->cur]}, m->nVertices);
}

int svm_cell_list_compute(svm_cell_list* cl, const double* pts, int n) {
    if (!cl || !pts) return SVM_ERR_ARG;
    return compute(cl, AosPoints{pts}, n);
}

int svm_cell_list_get(svm_cell_list* cl, int* nside, int* nmax, unsigned* counts, int* slots, long cap) {
    if (!cl) return SVM_ERR_ARG;
    int sc[4];
    if (cudaMemcpyAsync(sc, cl->scalars, sizeof(sc), cudaMemcpyDeviceToHost, cl->stream) != cudaSuccess ||
        cudaStreamSynchronize(cl->stream) != cudaSuccess) return SVM_ERR_CUDA;
    if (nside) *nside = cl->nside;
    if (nmax) *nmax = sc[1];
    if (sc[2] || sc[3]) return SVM_ERR_DEVICE;  // a bin overflowed its slots, or a point left the grid
    const int Nmax = sc[1];
    if (counts) {
        if (cudaMemcpy(counts, cl->counts, sizeof(unsigned) * cl->total, cudaMemcpyDeviceToHost) != cudaSuccess) return SVM_ERR_CUDA;
    }
    if (slots) {
        if (cap < cl->total * Nmax) return SVM_ERR_ARG;
        std::vector<unsigned> cnt(cl->total);
        std::vector<int> s((size_t)cl->total * cl->cap);
        if (cudaMemcpy(cnt.data(), cl->counts, sizeof(unsigned) * cl->total, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(s.data(), cl->slots, sizeof(int) * s.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
            return SVM_ERR_CUDA;
        for (long b = 0; b < cl->total; ++b)
            for (int k = 0; k < Nmax; ++k)
                slots[b * Nmax + k] = (k < (int)cnt[b] && k < cl->cap) ? s[(size_t)b * cl->cap + k] : -1;
    }
    return SVM_OK;
}

int svm_cell_list_bins(svm_cell_list* cl, int* binOfPoint) {
    if (!cl || !binOfPoint) return SVM_ERR_ARG;
    if (cudaMemcpyAsync(binOfPoint, cl->binOf, sizeof(int) * cl->nPoints, cudaMemcpyDeviceToHost, cl->stream) != cudaSuccess ||
        cudaStreamSynchronize(cl->stream) != cudaSuccess) return SVM_ERR_CUDA;
    return SVM_OK;
}

}  // extern "C"
