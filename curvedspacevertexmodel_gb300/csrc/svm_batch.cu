// Batches of independent replicas (svm_batch_* in include/svm.h).
//
// A batch is one model whose arrays hold every replica's cells and vertices back to back (replica
// r owns cells [cellOff[r], cellOff[r+1]) and vertices [vertOff[r], vertOff[r+1]); rings and the
// vertex lists use global indices).  All per-element kernels of a step therefore run once over all
// replicas; what differs per replica is read through the vertex's replica index, stored in the w
// component of its FP32 position: the radius, the noise amplitude sqrt(2 dt mu T_r), and the
// area check |sum_c A_c - 4 pi R_r^2| > 1e-6 (sphericalVertexModel.cpp:304-310), evaluated per
// replica by one block each.  Replica r's T1 flips are the ones the single-sphere loop would do:
// the flagged edges of different replicas share no vertex or cell, and within a replica the
// global scan order is the replica's own order.
//
// Batches run the mixed-precision form.  Their per-element kernels (corners, cells, force) take
// their block size from a KernelTuner each (the reference's kernelTuner, src/utilities/
// kernelTuner.cpp) when autotuning is on; the result of a step does not depend on block sizes.
#include <algorithm>
#include <memory>
#include "svm_internal.cuh"
#include "svm_tuner.h"

namespace {
using namespace svm;

constexpr int kRB = 256;

__device__ double rep_block_sum(double v) {
    __shared__ double ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) ws[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += ws[w];
    __syncthreads();
    return r;
}

// one block per replica: total area, excess over 4 pi R^2, fallback flag
__global__ void k_rep_check(const double2* __restrict__ ap, const int* __restrict__ cellOff,
                            const double* __restrict__ repR, int* __restrict__ repFlag, double* __restrict__ repScal) {
    const int r = blockIdx.x;
    double s = 0.0;
    for (int c = cellOff[r] + threadIdx.x; c < cellOff[r + 1]; c += blockDim.x) s += ap[c].x;
    const double total = rep_block_sum(s);
    if (threadIdx.x == 0) {
        const double R = repR[r];
        const double excess = total - 4.0 * kPI * R * R;
        repScal[3 * r] = total;
        repScal[3 * r + 1] = excess;
        repFlag[r] = fabs(excess) > 1e-6 ? 1 : 0;
    }
}

// one block per replica: sum_c Kr (A - A0)^2 + (P - P0)^2 (sphericalVertexModel.cpp:150-160)
__global__ void k_rep_energy(const double2* __restrict__ ap, const double2* __restrict__ pref, double Kr,
                             const int* __restrict__ cellOff, double* __restrict__ repScal) {
    const int r = blockIdx.x;
    double s = 0.0;
    for (int c = cellOff[r] + threadIdx.x; c < cellOff[r + 1]; c += blockDim.x) {
        const double da = ap[c].x - pref[c].x, dp = ap[c].y - pref[c].y;
        s += Kr * da * da + dp * dp;
    }
    const double e = rep_block_sum(s);
    if (threadIdx.x == 0) repScal[3 * r + 2] = e;
}

// w of every vertex's FP32 positions (both buffers) = its replica
__global__ void k_set_rep(float4* __restrict__ p0, float4* __restrict__ p1, const int* __restrict__ vertOff) {
    const int r = blockIdx.x;
    for (int v = vertOff[r] + threadIdx.x; v < vertOff[r + 1]; v += blockDim.x) {
        p0[v].w = (float)r;
        p1[v].w = (float)r;
    }
}

// one tuner per kernel family, each over the block sizes lo, lo+step, ... up to the smaller of hi
// and the largest block the kernel can launch with (its register use)
struct BatchTuners {
    KernelTuner corners, cells, force;
    cudaEvent_t start = nullptr, stop = nullptr;
    BatchTuners(int lo, int hi, int step, int samples, int period)
        : corners(lo, std::max(lo, std::min(hi, mixed_max_block_corners())), step, samples, period),
          cells(lo, std::max(lo, std::min(hi, max_block_cells_batch())), step, samples, period),
          force(lo, std::max(lo, std::min(hi, mixed_max_block_force())), step, samples, period) {}
    ~BatchTuners() {
        if (start) cudaEventDestroy(start);
        if (stop) cudaEventDestroy(stop);
    }
    bool timing() const { return corners.timing() || cells.timing() || force.timing(); }
};

}  // namespace

namespace svm {

int launch_rep_check(svm_model* m) {
    k_rep_check<<<m->nRep, kRB, 0, m->stream>>>(m->ap, m->repCellOff, m->repR, m->repFlag, m->repScal);
    return check_launch();
}

// Uploads sqrt(2 dt mu T_r) when dt, mu or the temperatures changed (not during a capture: the
// graph reads the table when it runs).
int update_rep_noise(svm_model* m, double dt, double mu) {
    if (m->nRep <= 1) return SVM_OK;
    if (m->repNpDt == dt && m->repNpMu == mu && m->repNpVersion == m->repTVersion) return SVM_OK;
    std::vector<float> np(m->nRep);
    const double fp = dt * mu;  // same expression as the single-sphere step's amplitude
    for (int r = 0; r < m->nRep; ++r) np[r] = (float)sqrt(2.0 * fp * m->repT[r]);
    if (cudaMemcpyAsync(m->repNp, np.data(), sizeof(float) * m->nRep, cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    m->repNpDt = dt; m->repNpMu = mu; m->repNpVersion = m->repTVersion;
    return SVM_OK;
}

void batch_release(svm_model* m) {
    delete static_cast<BatchTuners*>(m->tuners);
    m->tuners = nullptr;
}

// Times one launch of a tuned kernel family when its tuner is sampling; applies the tuner's next
// block size.  Outside autotuning (or during a capture) it only runs the launch.
template <class F>
static int tuned(svm_model* m, KernelTuner BatchTuners::*which, int svm_model::*blk, F launch) {
    BatchTuners* T = static_cast<BatchTuners*>(m->tuners);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(m->stream, &cs);
    if (!T || cs != cudaStreamCaptureStatusNone) return launch();
    KernelTuner& t = T->*which;
    const bool timed = t.timing();
    if (timed && !T->start &&
        (cudaEventCreate(&T->start) != cudaSuccess || cudaEventCreate(&T->stop) != cudaSuccess))
        return SVM_ERR_CUDA;
    if (timed) cudaEventRecord(T->start, m->stream);
    const int rc = launch();
    if (rc) return rc;
    float ms = 0.f;
    if (timed && (cudaEventRecord(T->stop, m->stream) != cudaSuccess || cudaEventSynchronize(T->stop) != cudaSuccess ||
                  cudaEventElapsedTime(&ms, T->start, T->stop) != cudaSuccess))
        return SVM_ERR_CUDA;
    t.call(ms);
    if (m->*blk != t.parameter()) {
        m->*blk = t.parameter();
        m->paramsVersion++;  // captured graphs hold the old block size
    }
    return SVM_OK;
}

int batch_tuned_corners(svm_model* m, bool t1test) {
    return tuned(m, &BatchTuners::corners, &svm_model::blkCorners, [&] { return mixed_launch_corners(m, t1test); });
}
int batch_tuned_cells(svm_model* m, int (*launch)(svm_model*)) {
    return tuned(m, &BatchTuners::cells, &svm_model::blkCells, [&] { return launch(m); });
}
int batch_tuned_force_bd(svm_model* m, double T, double dt, double mu, int noiseMode, const double* noise,
                         uint64_t seed, int nxt) {
    return tuned(m, &BatchTuners::force, &svm_model::blkForce,
                 [&] { return mixed_launch_force_bd(m, T, dt, mu, noiseMode, noise, seed, nxt); });
}
bool batch_tuning(svm_model* m) {
    const BatchTuners* T = static_cast<const BatchTuners*>(m->tuners);
    return T && T->timing();
}
// graph-replayed steps are untimed calls of each tuner (they count toward the rescan period)
void batch_tuner_untimed(svm_model* m, int calls) {
    BatchTuners* T = static_cast<BatchTuners*>(m->tuners);
    if (!T) return;
    for (int i = 0; i < calls && !T->timing(); ++i) {
        T->corners.call(0.f);
        T->cells.call(0.f);
        T->force.call(0.f);
    }
}

}  // namespace svm

extern "C" {

int svm_batch_create(int nReplicas, const int* nCells, const int* nVertices, int Wc, const double* radius,
                     void* stream, svm_model** out) {
    if (nReplicas < 1 || !nCells || !nVertices || !radius || !out || Wc < 3 || Wc > 64) return SVM_ERR_ARG;
    std::vector<int> cOff(nReplicas + 1, 0), vOff(nReplicas + 1, 0);
    for (int r = 0; r < nReplicas; ++r) {
        if (nCells[r] < 4 || nVertices[r] != 2 * nCells[r] - 4 || !(radius[r] > 0)) return SVM_ERR_ARG;
        if ((long)cOff[r] + nCells[r] > (1L << 30)) return SVM_ERR_ARG;
        cOff[r + 1] = cOff[r] + nCells[r];
        vOff[r + 1] = vOff[r] + nVertices[r];
    }
    if (nReplicas > (1 << 24)) return SVM_ERR_ARG;  // replica index exact in the FP32 w component
    svm_model* m = nullptr;
    int rc = svm::model_alloc(cOff[nReplicas], vOff[nReplicas], Wc, radius, nReplicas, stream, &m);
    if (rc) return rc;
    m->hRepCellOff = cOff;
    m->hRepVertOff = vOff;
    if ((rc = svm_model_set_precision(m, SVM_PRECISION_MIXED))) { svm_model_destroy(m); return rc; }
    bool ok = cudaMemcpy(m->repCellOff, cOff.data(), sizeof(int) * (nReplicas + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(m->repVertOff, vOff.data(), sizeof(int) * (nReplicas + 1), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
        k_set_rep<<<nReplicas, kRB, 0, m->stream>>>(m->pos32[0], m->pos32[1], m->repVertOff);
        ok = cudaStreamSynchronize(m->stream) == cudaSuccess;
    }
    if (!ok) { svm_model_destroy(m); return SVM_ERR_CUDA; }
    *out = m;
    return SVM_OK;
}

int svm_batch_replicas(svm_model* m, int* nReplicas) {
    if (!m || !nReplicas) return SVM_ERR_ARG;
    *nReplicas = m->nRep;
    return SVM_OK;
}

int svm_batch_offsets(svm_model* m, int* cellOffsets, int* vertexOffsets) {
    if (!m) return SVM_ERR_ARG;
    for (int r = 0; r <= m->nRep; ++r) {
        if (cellOffsets) cellOffsets[r] = m->nRep > 1 ? m->hRepCellOff[r] : (r ? m->nCells : 0);
        if (vertexOffsets) vertexOffsets[r] = m->nRep > 1 ? m->hRepVertOff[r] : (r ? m->nVertices : 0);
    }
    return SVM_OK;
}

int svm_batch_set_temperatures(svm_model* m, const double* T) {
    if (!m || !T || m->nRep < 2) return SVM_ERR_ARG;
    for (int r = 0; r < m->nRep; ++r)
        if (!(T[r] >= 0)) return SVM_ERR_ARG;
    m->repT.assign(T, T + m->nRep);
    m->repTVersion++;
    return SVM_OK;
}

int svm_batch_energies(svm_model* m, double* energies) {
    if (!m || !energies || m->nRep < 2) return SVM_ERR_ARG;
    k_rep_energy<<<m->nRep, kRB, 0, m->stream>>>(m->ap, m->pref, m->Kr, m->repCellOff, m->repScal);
    if (check_launch()) return SVM_ERR_CUDA;
    std::vector<double> sc(3 * m->nRep);
    if (cudaMemcpyAsync(sc.data(), m->repScal, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, m->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    for (int r = 0; r < m->nRep; ++r) energies[r] = sc[3 * r + 2];
    return SVM_OK;
}

int svm_batch_area_check(svm_model* m, double* totals, double* excess, int* fallbackTaken) {
    if (!m || m->nRep < 2) return SVM_ERR_ARG;
    std::vector<double> sc(3 * m->nRep);
    std::vector<int> fl(m->nRep);
    if (cudaMemcpyAsync(sc.data(), m->repScal, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, m->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(fl.data(), m->repFlag, sizeof(int) * m->nRep, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    for (int r = 0; r < m->nRep; ++r) {
        if (totals) totals[r] = sc[3 * r];
        if (excess) excess[r] = sc[3 * r + 1];
        if (fallbackTaken) fallbackTaken[r] = fl[r];
    }
    return SVM_OK;
}

int svm_batch_autotune(svm_model* m, int lo, int hi, int step, int nSamples, int period) {
    if (!m || m->nRep < 2) return SVM_ERR_ARG;
    batch_release(m);
    if (lo <= 0) {  // off: back to the default block size
        m->blkCorners = m->blkCells = m->blkForce = 256;
        m->paramsVersion++;
        return SVM_OK;
    }
    if (lo < 32 || hi > 1024 || step <= 0 || hi < lo || lo % 32 || step % 32 || nSamples < 1 || period < 0)
        return SVM_ERR_ARG;
    m->tuners = new BatchTuners(lo, hi, step, nSamples, period);
    m->blkCorners = m->blkCells = m->blkForce = lo;
    m->paramsVersion++;
    return SVM_OK;
}

int svm_batch_block_sizes(svm_model* m, int* sizes3, int* samplingComplete) {
    if (!m || !sizes3) return SVM_ERR_ARG;
    sizes3[0] = m->blkCorners; sizes3[1] = m->blkCells; sizes3[2] = m->blkForce;
    if (samplingComplete) {
        const BatchTuners* T = static_cast<const BatchTuners*>(m->tuners);
        *samplingComplete = !T || (T->corners.samplingComplete() && T->cells.samplingComplete() &&
                                   T->force.samplingComplete());
    }
    return SVM_OK;
}

}  // extern "C"
