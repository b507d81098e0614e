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
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
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
    int occ = 0;
    if (i < np) {
        double x, y, z;
        pts(i, x, y, z);
        const int b = bin_of(x, y, z, r, h, n, scalars + 3);
        binOf[i] = b;
        const unsigned s = atomicAdd(counts + b, 1u);
        if ((int)s < cap) tmp[(long)b * cap + s] = i;
        else atomicExch(scalars + 2, 1);
        occ = (int)s + 1;
    }
    // one atomic per warp: a per-point atomic on this one word serialises in L2
    occ = __reduce_max_sync(0xffffffffu, occ);
    if ((threadIdx.x & 31) == 0 && occ > 0) atomicMax(scalars, occ);
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

// A bin took more points than it has slots: give every bin `cap` slots, as the reference's cell
// list widens its Nmax and bins again (hyperrectangularCellList.cpp:165-214).  The counts of the
// overflowing call stay valid for the next call's incremental clear.
int cl_grow(svm_cell_list* cl, int cap) {
    if (cudaStreamSynchronize(cl->stream) != cudaSuccess) return SVM_ERR_CUDA;
    cudaFree(cl->tmp); cudaFree(cl->slots);
    cl->tmp = nullptr; cl->slots = nullptr;
    if (cudaMalloc(&cl->tmp, sizeof(int) * cl->total * cap) != cudaSuccess ||
        cudaMalloc(&cl->slots, sizeof(int) * cl->total * cap) != cudaSuccess)
        return SVM_ERR_CUDA;
    cl->cap = cap;
    return SVM_OK;
}
// neighborList (src/utilities/neighborList.cpp:6-18, 96-151; kernels neighborList.cu:108-357): per
// point, over the adjacent bins of its (clamped) bin in the mask's order and each bin's points in
// slot order, every other point whose minimum-image displacement (periodic box of side 2 radius,
// periodicBoundaryConditions.h:124-132) is shorter than `range`; the first nmax are stored, the
// rest of each row is zero, and the count is kept whole (the host grows nmax and recomputes when a
// count exceeds it).
//
// FP64 issues at a sixty-fourth of the FP32 rate here, so a candidate is first classified in FP32
// and only neighbours (and the rare borderline candidate) see FP64:
//   phase 1, a thread per point: scan the candidates with FP32 copies of the positions.  With E
//     a bound on |d32 - d64| per component (coordinates within the grid, |x| <= radius, rounded
//     to FP32 and subtracted: E = radius 2^-21 covers both roundings with a factor of two), a
//     candidate whose |d32| components all stay below radius - 2E cannot wrap in FP64, and then
//       dd32 > thrHi (> ((range + 2E)(1 + 2^-20))^2)  => |d64| > range      => not a neighbour
//       dd32 < thrLo (< ((range - 2E)(1 - 2^-20))^2)  => |d64| < range      => a neighbour
//     (dd32's own rounding is below 3 2^-24 relative, inside the 2^-20 factors).  Any other
//     candidate takes the reference's FP64 test in place.  Neighbours are queued in order in
//     shared memory (kNlQueue per thread; the scan resumes where it stopped when a queue fills).
//   phase 2, the warp: the queued neighbours of its 32 points are dealt over the lanes, and each
//     lane computes one neighbour's displacement, squared length and root in FP64 exactly as the
//     reference does, and stores them at the owner's next row position.
// The minimum-image loops run at most kWrapIters times: points inside the grid need one, and a
// point outside it is an error the host reports (the cell list's flag).
constexpr int kNlQueue = 16;
constexpr int kWrapIters = 8;
constexpr unsigned kNlWrapped = 0x80000000u;  // queue flag: the displacement wrapped

struct NlParams {
    int np, cap, nside, K, nmax;
    double h, radius, range, range2Hi;
    float wrapLim, thrLo, thrHi;
};

__device__ __forceinline__ bool min_image(double& d, double radius) {
    bool w = false;
    for (int i = 0; i < kWrapIters && d < -radius; ++i) { d += 2. * radius; w = true; }
    for (int i = 0; i < kWrapIters && d > radius; ++i) { d -= 2. * radius; w = true; }
    return w;
}

template <typename P>
__global__ void k_nl_pack(P pts, int np, float4* __restrict__ p32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    double x, y, z;
    pts(i, x, y, z);
    p32[i] = make_float4((float)x, (float)y, (float)z, 0.f);
}

template <typename P>
__global__ void __launch_bounds__(kB, 6) k_nl(P pts, const float4* __restrict__ p32, NlParams prm,
                                          const unsigned* __restrict__ counts, const int* __restrict__ slots,
                                          const int* __restrict__ mask, unsigned* __restrict__ npp,
                                          int* __restrict__ idx, double* __restrict__ vec,
                                          double* __restrict__ dist, int* __restrict__ maxCount) {
    __shared__ unsigned queue[kNlQueue * kB];
    const int lane = threadIdx.x & 31, wbase = threadIdx.x & ~31;
    const int pp = blockIdx.x * kB + threadIdx.x;
    const bool active = pp < prm.np;
    float t32[3] = {0.f, 0.f, 0.f};
    int c[3] = {0, 0, 0};
    if (active) {
        double t[3];
        pts(pp, t[0], t[1], t[2]);
        const float4 f = p32[pp];
        t32[0] = f.x; t32[1] = f.y; t32[2] = f.z;
        for (int d = 0; d < 3; ++d) c[d] = max(0, min(prm.nside - 1, (int)floor((t[d] + prm.radius) / prm.h)));
    }
    auto cell_at = [&](int k) {
        int nb[3];
        for (int d = 0; d < 3; ++d) {
            nb[d] = (c[d] + mask[3 * k + d]) % prm.nside;
            if (nb[d] < 0) nb[d] += prm.nside;
        }
        return nb[0] + (long)nb[1] * prm.nside + (long)nb[2] * prm.nside * prm.nside;
    };
    // the next bin's count is loaded one bin ahead, off the scan's dependent-load chain
    int cc = 0, p1 = 0, n = 0, count = 0, stored = 0;
    long cell = 0, cellNext = 0;
    unsigned nNext = 0;
    if (active) { cellNext = cell_at(0); nNext = counts[cellNext]; }
    bool more = active;
    while (__any_sync(0xffffffffu, more)) {
        int nq = 0;
        // ---- phase 1: queue up to kNlQueue neighbours of this thread's point, in scan order
        while (more && nq < kNlQueue) {
            if (p1 >= n) {
                if (cc >= prm.K) { more = false; break; }
                cell = cellNext;
                n = min((int)nNext, prm.cap);
                p1 = 0;
                if (++cc < prm.K) { cellNext = cell_at(cc); nNext = counts[cellNext]; }
                continue;
            }
            const int j = slots[cell * prm.cap + p1];
            ++p1;
            if (j == pp) continue;
            const float4 q = p32[j];
            const float d0 = t32[0] - q.x, d1 = t32[1] - q.y, d2 = t32[2] - q.z;
            int verdict = 0;  // 1 neighbour, -1 not, 0 decide in FP64
            if (fabsf(d0) <= prm.wrapLim && fabsf(d1) <= prm.wrapLim && fabsf(d2) <= prm.wrapLim) {
                const float dd32 = d0 * d0 + d1 * d1 + d2 * d2;
                verdict = dd32 > prm.thrHi ? -1 : (dd32 < prm.thrLo ? 1 : 0);
            }
            unsigned entry = (unsigned)j;
            if (verdict == 0) {  // the reference's test, in FP64 (rare: the point is reloaded)
                double t[3], qd[3], disp[3];
                pts(pp, t[0], t[1], t[2]);
                pts(j, qd[0], qd[1], qd[2]);
                bool w = false;
                for (int d = 0; d < 3; ++d) {
                    disp[d] = t[d] - qd[d];
                    w |= min_image(disp[d], prm.radius);
                }
                const double dd = disp[0] * disp[0] + disp[1] * disp[1] + disp[2] * disp[2];
                verdict = (dd > prm.range2Hi || sqrt(dd) >= prm.range) ? -1 : 1;
                if (w) entry |= kNlWrapped;
            }
            if (verdict < 0) continue;
            if (count < prm.nmax) queue[nq++ * kB + threadIdx.x] = entry;
            ++count;
        }
        // ---- phase 2: the warp's queued neighbours over its lanes, in FP64
        int incl = nq;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int excl = incl - nq, total = __shfl_sync(0xffffffffu, incl, 31);
        for (int base = 0; base < total; base += 32) {
            const int g = base + lane;
            int owner = 0;  // the last lane whose queue starts at or before g
            for (int step = 16; step > 0; step >>= 1) {
                const int e = __shfl_sync(0xffffffffu, excl, owner + step);
                if (e <= g) owner += step;
            }
            const int k = g - __shfl_sync(0xffffffffu, excl, owner);
            const int row = __shfl_sync(0xffffffffu, stored, owner) + k;
            if (g < total) {
                const unsigned entry = queue[k * kB + wbase + owner];
                const int j = (int)(entry & ~kNlWrapped);
                const int po = blockIdx.x * kB + wbase + owner;
                double a[3], b[3], disp[3];
                pts(po, a[0], a[1], a[2]);
                pts(j, b[0], b[1], b[2]);
                for (int d = 0; d < 3; ++d) disp[d] = a[d] - b[d];
                if (entry & kNlWrapped)
                    for (int d = 0; d < 3; ++d) min_image(disp[d], prm.radius);
                const double dd = disp[0] * disp[0] + disp[1] * disp[1] + disp[2] * disp[2];
                const long at = (long)po * prm.nmax + row;
                idx[at] = j;
                vec[3 * at] = disp[0]; vec[3 * at + 1] = disp[1]; vec[3 * at + 2] = disp[2];
                dist[at] = sqrt(dd);
            }
        }
        stored += nq;
    }
    // ---- the rest of each row is zero (resetNeighbors), written a row at a time by the warp
    for (int o = 0; o < 32; ++o) {
        const int s = __shfl_sync(0xffffffffu, stored, o);
        const int po = blockIdx.x * kB + wbase + o;
        if (po >= prm.np) break;
        for (int k = s + lane; k < prm.nmax; k += 32) {
            const long at = (long)po * prm.nmax + k;
            idx[at] = 0;
            vec[3 * at] = 0.; vec[3 * at + 1] = 0.; vec[3 * at + 2] = 0.;
            dist[at] = 0.;
        }
    }
    if (active) npp[pp] = (unsigned)count;
    count = __reduce_max_sync(0xffffffffu, count);  // one atomic per warp on the shared word
    if (lane == 0 && count > 0) atomicMax(maxCount, count);
}
}  // namespace

struct svm_neighbor_list {
    svm_cell_list* cl = nullptr;
    double range = 1.0, radius = 1.0;
    int nPoints = 0, nmax = 4, K = 0;   // Nmax starts at 4 (neighborList.cpp:17)
    int* mask = nullptr;                // [3 K] adjacent-bin offsets
    unsigned* npp = nullptr;            // [nPoints]
    int* idx = nullptr;                 // [nPoints * nmax]
    double* vec = nullptr;              // [nPoints * nmax * 3]
    double* dist = nullptr;             // [nPoints * nmax]
    int* maxCount = nullptr;
    float4* p32 = nullptr;              // [nPoints] FP32 copies for the candidate scan
};

namespace {
int nl_alloc(svm_neighbor_list* nl) {
    cudaFree(nl->idx); cudaFree(nl->vec); cudaFree(nl->dist);
    nl->idx = nullptr; nl->vec = nullptr; nl->dist = nullptr;
    const size_t e = (size_t)nl->nPoints * nl->nmax;
    if (cudaMalloc(&nl->idx, sizeof(int) * e) != cudaSuccess || cudaMalloc(&nl->vec, sizeof(double) * 3 * e) != cudaSuccess ||
        cudaMalloc(&nl->dist, sizeof(double) * e) != cudaSuccess)
        return SVM_ERR_CUDA;
    return SVM_OK;
}

// The scan's FP32 thresholds for points within [-radius, radius]^3, rounded outward.
void nl_thresholds(NlParams& p) {
    const double E = p.radius * 0x1p-21;
    auto down = [](double v) { float f = (float)v; if ((double)f > v) f = std::nextafter(f, -INFINITY); return f; };
    auto up = [](double v) { float f = (float)v; if ((double)f < v) f = std::nextafter(f, INFINITY); return f; };
    p.wrapLim = p.radius > 2 * E ? down(p.radius - 2 * E) : -1.f;
    const double hi = (p.range + 2 * E) * (1 + 0x1p-20), lo = (p.range - 2 * E) * (1 - 0x1p-20);
    p.thrHi = up(hi * hi);
    p.thrLo = lo > 0 ? down(lo * lo) : -1.f;
}

template <typename P>
int nl_compute(svm_neighbor_list* nl, P pts, int np) {
    if (np != nl->nPoints) return SVM_ERR_ARG;
    svm_cell_list* cl = nl->cl;
    const size_t nb = (np + kB - 1) / kB;
    k_nl_pack<<<nb, kB, 0, cl->stream>>>(pts, np, nl->p32);
    for (int pass = 0; pass < 64; ++pass) {   // a third pass at most: slots widened, then nmax grown
        NlParams prm;
        prm.np = np; prm.cap = cl->cap; prm.nside = cl->nside; prm.K = nl->K; prm.nmax = nl->nmax;
        prm.h = cl->h; prm.radius = cl->radius; prm.range = nl->range;
        prm.range2Hi = nl->range * nl->range * (1.0 + 0x1p-48);
        nl_thresholds(prm);
        cudaMemsetAsync(nl->maxCount, 0, sizeof(int), cl->stream);
        k_nl<<<nb, kB, 0, cl->stream>>>(pts, nl->p32, prm, cl->counts, cl->slots, nl->mask, nl->npp, nl->idx, nl->vec,
                                        nl->dist, nl->maxCount);
        if (check_launch()) return SVM_ERR_CUDA;
        int mc = 0, sc[4];
        if (cudaMemcpyAsync(&mc, nl->maxCount, sizeof(int), cudaMemcpyDeviceToHost, cl->stream) != cudaSuccess ||
            cudaMemcpyAsync(sc, cl->scalars, sizeof(sc), cudaMemcpyDeviceToHost, cl->stream) != cudaSuccess ||
            cudaStreamSynchronize(cl->stream) != cudaSuccess)
            return SVM_ERR_CUDA;
        if (sc[3]) return SVM_ERR_DEVICE;  // a point lay outside the grid (or was not finite)
        if (sc[2]) {                       // a bin overflowed its slots: widen them, bin again
            if (cl_grow(cl, sc[0]) || compute(cl, pts, np)) return SVM_ERR_CUDA;
            continue;
        }
        if (mc <= nl->nmax) return SVM_OK;
        nl->nmax = mc;  // grow-only, then recompute
        if (nl_alloc(nl)) return SVM_ERR_CUDA;
    }
    return SVM_ERR_DEVICE;
}
}  // namespace

namespace svm {
int cell_list_bin(svm_cell_list* cl, const double* pts, int n, CellGrid* view) {
    if (!cl || !pts || !view || n != cl->nPoints) return SVM_ERR_ARG;
    for (int pass = 0; pass < 8; ++pass) {
        if (compute(cl, AosPoints{pts}, n)) return SVM_ERR_CUDA;
        int sc[4];
        if (cudaMemcpyAsync(sc, cl->scalars, sizeof(sc), cudaMemcpyDeviceToHost, cl->stream) != cudaSuccess ||
            cudaStreamSynchronize(cl->stream) != cudaSuccess)
            return SVM_ERR_CUDA;
        if (sc[3]) return SVM_ERR_DEVICE;
        if (sc[2]) { if (cl_grow(cl, sc[0])) return SVM_ERR_CUDA; continue; }
        *view = CellGrid{cl->counts, cl->slots, cl->cap, cl->nside, cl->h, cl->radius};
        return SVM_OK;
    }
    return SVM_ERR_DEVICE;
}
}  // namespace svm

extern "C" {

int svm_neighbor_list_create(double range, double radius, int subGridReduction, int nPoints, int slotCapacity,
                             void* stream, svm_neighbor_list** out) {
    if (!(range > 0) || !(radius > 0) || subGridReduction < 1 || nPoints <= 0 || !out) return SVM_ERR_ARG;
    svm_neighbor_list* nl = new svm_neighbor_list();
    nl->range = range; nl->radius = radius; nl->nPoints = nPoints;
    int rc = svm_cell_list_create(range * (1. / (double)subGridReduction), radius, nPoints, slotCapacity, stream, &nl->cl);
    if (rc) { delete nl; return rc; }
    // computeAdjacentCells (hyperrectangularCellList.cpp:219-262): offsets in iVecIterate order
    // (x fastest) whose nearest corner lies within `width` bins
    const int width = subGridReduction;
    const double h = nl->cl->h;
    std::vector<int> mask;
    for (int z = -width; z <= width; ++z)
        for (int y = -width; y <= width; ++y)
            for (int x = -width; x <= width; ++x) {
                const int g[3] = {x, y, z};
                double rmin = 0.0;
                for (int d = 0; d < 3; ++d) {
                    const double t = h * (std::max(std::abs(g[d]) - 1., 0.0));
                    rmin += t * t;
                }
                rmin = std::sqrt(rmin);
                if (rmin < h * width + 1e-6) { mask.push_back(x); mask.push_back(y); mask.push_back(z); }
            }
    nl->K = (int)mask.size() / 3;
    bool ok = cudaMalloc(&nl->mask, sizeof(int) * mask.size()) == cudaSuccess &&
              cudaMalloc(&nl->npp, sizeof(unsigned) * nPoints) == cudaSuccess &&
              cudaMalloc(&nl->maxCount, sizeof(int)) == cudaSuccess &&
              cudaMalloc(&nl->p32, sizeof(float4) * nPoints) == cudaSuccess && nl_alloc(nl) == SVM_OK;
    if (ok) ok = cudaMemcpy(nl->mask, mask.data(), sizeof(int) * mask.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) { svm_neighbor_list_destroy(nl); return SVM_ERR_CUDA; }
    *out = nl;
    return SVM_OK;
}

int svm_neighbor_list_destroy(svm_neighbor_list* nl) {
    if (!nl) return SVM_ERR_ARG;
    if (nl->cl) svm_cell_list_destroy(nl->cl);
    void* ptrs[] = {nl->mask, nl->npp, nl->idx, nl->vec, nl->dist, nl->maxCount, nl->p32};
    for (void* p : ptrs) if (p) cudaFree(p);
    delete nl;
    return SVM_OK;
}

int svm_neighbor_list_compute(svm_neighbor_list* nl, const double* pts, int n) {
    if (!nl || !pts) return SVM_ERR_ARG;
    int rc = svm_cell_list_compute(nl->cl, pts, n);
    return rc ? rc : nl_compute(nl, AosPoints{pts}, n);
}

int svm_neighbor_list_compute_model(svm_neighbor_list* nl, svm_model* m) {
    if (!nl || !m) return SVM_ERR_ARG;
    int rc = svm_cell_list_compute_model(nl->cl, m);
    if (rc) return rc;
    if (m->precision == SVM_PRECISION_MIXED) return nl_compute(nl, ModelPoints32{m->pos32[m->cur]}, m->nVertices);
    return nl_compute(nl, ModelPoints{m->pos[m->cur]}, m->nVertices);
}

int svm_neighbor_list_get(svm_neighbor_list* nl, int* nmax, unsigned* npp, int* idx, double* vec, double* dist,
                          long capacity) {
    if (!nl) return SVM_ERR_ARG;
    if (nmax) *nmax = nl->nmax;
    const size_t e = (size_t)nl->nPoints * nl->nmax;
    if ((idx || vec || dist) && (long)e > capacity) return SVM_ERR_ARG;
    cudaStream_t s = nl->cl->stream;
    if (npp && cudaMemcpyAsync(npp, nl->npp, sizeof(unsigned) * nl->nPoints, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return SVM_ERR_CUDA;
    if (idx && cudaMemcpyAsync(idx, nl->idx, sizeof(int) * e, cudaMemcpyDeviceToHost, s) != cudaSuccess) return SVM_ERR_CUDA;
    if (vec && cudaMemcpyAsync(vec, nl->vec, sizeof(double) * 3 * e, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return SVM_ERR_CUDA;
    if (dist && cudaMemcpyAsync(dist, nl->dist, sizeof(double) * e, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return SVM_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

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
