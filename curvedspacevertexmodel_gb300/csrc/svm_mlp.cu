// Learned warm start for FIRE (svm_mlp_* in include/svm.h): a per-vertex MLP 24 -> 64 -> 64 -> 2
// (ReLU hidden layers, BF16 weights, FP32 accumulation) that reads the local tangent-frame
// geometry of a vertex and predicts its displacement to the relaxed state.  No counterpart in the
// reference.
//
// Features of vertex v (FP32, from the FP64 model state after geometry and forces):
//   frame: n = v/|v|, e1 = unit tangent projection of (nbr0 - v), e2 = n x e1;
//   [0..5]   offsets to the three neighbours (vnbr slots) in (e1, e2);
//   [6..11]  offsets to the three adjacent cells' centroids (vcell slots) in (e1, e2);
//   [12..17] (A - A0, P - P0) of the three cells;
//   [18..20] (ring size - 6) of the three cells;
//   [21..22] the force in (e1, e2);  [23] |force|.
// Output: the displacement in (e1, e2), in units of the network's output scale.
//
// Parameters (FP32 master copy, kParams floats): W1[64][24], b1[64], W2[64][64], b2[64],
// W3[2][64], b3[2], row-major (out, in).  The forward pass uses their BF16 roundings; gradients
// are taken with respect to those (straight-through) and applied to the master copy by Adam.
//
// Training runs one thread per sample in blocks of kTB samples: the forward activations and the
// backward deltas are staged in shared memory, and each block writes its partial gradient sums
// (products summed over its samples in a fixed order); a second kernel sums the block partials in
// block order, so gradients are deterministic.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <cstdio>
#include <random>
#include <vector>
#include <cuda_bf16.h>
#include "svm_internal.cuh"

namespace {
using namespace svm;

constexpr int kIn = 24, kH = 64, kOut = 2;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kOut * kH, kParams = oB3 + kOut;
constexpr int kTB = 128;       // samples per training block
constexpr int kPad = kH + 1;   // shared-memory row stride of the activations (bank-conflict free)

__device__ __forceinline__ int c3(const int4& a, int s) { return s == 0 ? a.x : (s == 1 ? a.y : a.z); }

struct FeatArgs {
    const double4_32a* pos;
    const int4* vnbr;
    const int4* vcell;
    const double4_32a* cellPos;
    const double2* ap;
    const double2* pref;
    const int* ringCount;
    const double4_32a* force;
};

// features and tangent frame of vertex v
__device__ void vertex_features(const FeatArgs& A, int v, float* x, D3& e1, D3& e2, D3& p) {
    p = ld3(A.pos, v);
    const D3 n = scl3(1.0 / sqrt(dot3(p, p)), p);
    const int4 nb = A.vnbr[v], cells = A.vcell[v];
    D3 d0 = sub3(ld3(A.pos, nb.x), p);
    d0 = sub3(d0, scl3(dot3(d0, n), n));
    e1 = scl3(1.0 / sqrt(dot3(d0, d0)), d0);
    e2 = cross3(n, e1);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const D3 d = sub3(ld3(A.pos, c3(nb, s)), p);
        x[2 * s] = (float)dot3(d, e1);
        x[2 * s + 1] = (float)dot3(d, e2);
        const int c = c3(cells, s);
        const D3 dc = sub3(ld3(A.cellPos, c), p);
        x[6 + 2 * s] = (float)dot3(dc, e1);
        x[7 + 2 * s] = (float)dot3(dc, e2);
        const double2 apc = A.ap[c], pr = A.pref[c];
        x[12 + 2 * s] = (float)(apc.x - pr.x);
        x[13 + 2 * s] = (float)(apc.y - pr.y);
        x[18 + s] = (float)(A.ringCount[c] - 6);
    }
    const D3 f = ld3(A.force, v);
    x[21] = (float)dot3(f, e1);
    x[22] = (float)dot3(f, e2);
    x[23] = (float)sqrt(dot3(f, f));
}

__global__ void k_features(FeatArgs A, int nV, float* __restrict__ X, double* __restrict__ frames) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    float x[kIn];
    D3 e1, e2, p;
    vertex_features(A, v, x, e1, e2, p);
    for (int k = 0; k < kIn; ++k) X[(long)v * kIn + k] = x[k];
    if (frames) {
        double* fr = frames + 6L * v;
        fr[0] = e1.x; fr[1] = e1.y; fr[2] = e1.z; fr[3] = e2.x; fr[4] = e2.y; fr[5] = e2.z;
    }
}

// BF16 weights -> FP32 in shared memory
__device__ void load_weights(const __nv_bfloat16* __restrict__ wb, float* w) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = __bfloat162float(wb[i]);
    __syncthreads();
}

// y = W3 relu(W2 relu(W1 x + b1) + b2) + b3 for one sample, activations into h1, h2 (may be null)
__device__ void forward1(const float* w, const float* x, float* y, float* h1, float* h2) {
    float a1[kH];
#pragma unroll 4
    for (int j = 0; j < kH; ++j) {
        float s = w[oB1 + j];
        for (int k = 0; k < kIn; ++k) s = fmaf(w[oW1 + j * kIn + k], x[k], s);
        a1[j] = fmaxf(s, 0.f);
        if (h1) h1[j] = a1[j];
    }
    float o0 = w[oB3], o1 = w[oB3 + 1];
    for (int j = 0; j < kH; ++j) {
        float s = w[oB2 + j];
        for (int k = 0; k < kH; ++k) s = fmaf(w[oW2 + j * kH + k], a1[k], s);
        s = fmaxf(s, 0.f);
        if (h2) h2[j] = s;
        o0 = fmaf(w[oW3 + j], s, o0);
        o1 = fmaf(w[oW3 + kH + j], s, o1);
    }
    y[0] = o0;
    y[1] = o1;
}

// Forward + backward of one block of samples; per-block partial gradients and loss.
// Dynamic shared memory: w[kParams] | X[kTB][kIn] | H1[kTB][kPad] | H2[kTB][kPad] | D2[kTB][kPad] | DY[kTB][2]
__global__ void __launch_bounds__(kTB) k_train_block(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ X,
                                                     const float* __restrict__ Y, const int* __restrict__ order,
                                                     int first, int count, float invBatch,
                                                     float* __restrict__ partials, double* __restrict__ lossPartials) {
    extern __shared__ float sm[];
    float* w = sm;
    float* sx = w + kParams;
    float* h1 = sx + kTB * kIn;
    float* h2 = h1 + kTB * kPad;
    float* d2 = h2 + kTB * kPad;
    float* dy = d2 + kTB * kPad;
    __shared__ double lossSh[kTB / 32];
    load_weights(wb, w);
    const int t = threadIdx.x;
    const int local = blockIdx.x * kTB + t;
    const bool live = local < count;
    float x[kIn], y[kOut];
    double loss = 0.0;
    if (live) {
        const int sIdx = order ? order[first + local] : first + local;
        for (int k = 0; k < kIn; ++k) x[k] = X[(long)sIdx * kIn + k];
        forward1(w, x, y, h1 + t * kPad, h2 + t * kPad);
        const float r0 = y[0] - Y[2L * sIdx], r1 = y[1] - Y[2L * sIdx + 1];
        loss = (double)r0 * r0 + (double)r1 * r1;
        dy[2 * t] = 2.f * r0 * invBatch;
        dy[2 * t + 1] = 2.f * r1 * invBatch;
        // delta of layer 2 pre-activations
        for (int j = 0; j < kH; ++j) {
            const float g = w[oW3 + j] * dy[2 * t] + w[oW3 + kH + j] * dy[2 * t + 1];
            d2[t * kPad + j] = h2[t * kPad + j] > 0.f ? g : 0.f;
        }
    } else {
        for (int k = 0; k < kIn; ++k) x[k] = 0.f;
        for (int j = 0; j < kH; ++j) { h1[t * kPad + j] = 0.f; h2[t * kPad + j] = 0.f; d2[t * kPad + j] = 0.f; }
        dy[2 * t] = dy[2 * t + 1] = 0.f;
    }
    for (int k = 0; k < kIn; ++k) sx[t * kIn + k] = x[k];
    // block loss
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
    if ((t & 31) == 0) lossSh[t >> 5] = loss;
    __syncthreads();
    float* out = partials + (long)blockIdx.x * kParams;
    if (t == 0) {
        double l = 0.0;
        for (int i = 0; i < kTB / 32; ++i) l += lossSh[i];
        lossPartials[blockIdx.x] = l;
    }
    // dW3, db3 (needs H2 and DY)
    for (int e = t; e < kOut * kH; e += kTB) {
        const int o = e / kH, j = e % kH;
        float s = 0.f;
        for (int q = 0; q < kTB; ++q) s = fmaf(dy[2 * q + o], h2[q * kPad + j], s);
        out[oW3 + e] = s;
    }
    if (t < kOut) {
        float s = 0.f;
        for (int q = 0; q < kTB; ++q) s += dy[2 * q + t];
        out[oB3 + t] = s;
    }
    // dW2, db2 (D2 and H1)
    for (int e = t; e < kH * kH; e += kTB) {
        const int i = e / kH, j = e % kH;
        float s = 0.f;
        for (int q = 0; q < kTB; ++q) s = fmaf(d2[q * kPad + i], h1[q * kPad + j], s);
        out[oW2 + e] = s;
    }
    if (t < kH) {
        float s = 0.f;
        for (int q = 0; q < kTB; ++q) s += d2[q * kPad + t];
        out[oB2 + t] = s;
    }
    __syncthreads();
    // delta of layer 1 pre-activations, into H2's rows (H2 no longer needed)
    float* d1 = h2;
    for (int j = 0; j < kH; ++j) {
        float g = 0.f;
        for (int i = 0; i < kH; ++i) g = fmaf(w[oW2 + i * kH + j], d2[t * kPad + i], g);
        d1[t * kPad + j] = h1[t * kPad + j] > 0.f ? g : 0.f;
    }
    __syncthreads();
    // dW1, db1 (D1 and X)
    for (int e = t; e < kH * kIn; e += kTB) {
        const int i = e / kIn, k = e % kIn;
        float s = 0.f;
        for (int q = 0; q < kTB; ++q) s = fmaf(d1[q * kPad + i], sx[q * kIn + k], s);
        out[oW1 + e] = s;
    }
    if (t < kH) {
        float s = 0.f;
        for (int q = 0; q < kTB; ++q) s += d1[q * kPad + t];
        out[oB1 + t] = s;
    }
}

// grad[i] = sum over blocks (in block order) of the partials
__global__ void k_reduce_grad(const float* __restrict__ partials, int nBlocks, float* __restrict__ grad,
                              const double* __restrict__ lossPartials, double* __restrict__ loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) {
        float s = 0.f;
        for (int b = 0; b < nBlocks; ++b) s += partials[(long)b * kParams + i];
        grad[i] = s;
    }
    if (i == 0 && loss) {
        double l = 0.0;
        for (int b = 0; b < nBlocks; ++b) l += lossPartials[b];
        *loss = l;
    }
}

// Adam (Kingma and Ba, 2015) on the FP32 master weights, then the BF16 copy.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) wb[i] = __float2bfloat16_rn(w[i]);
}

__global__ void k_predict(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ X, int n,
                          float* __restrict__ Y) {
    __shared__ float w[kParams];
    load_weights(wb, w);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x[kIn], y[kOut];
    for (int k = 0; k < kIn; ++k) x[k] = X[(long)i * kIn + k];
    forward1(w, x, y, nullptr, nullptr);
    Y[2L * i] = y[0];
    Y[2L * i + 1] = y[1];
}

// Fused inference: features of the current state, the network, and the move of every vertex by
// scale * (y0 e1 + y1 e2) onto the sphere (sphericalDomain::move), written to the other buffer.
__global__ void k_warm_start(const __nv_bfloat16* __restrict__ wb, FeatArgs A, int nV, double scale, double R,
                             double4_32a* __restrict__ posOut) {
    __shared__ float w[kParams];
    load_weights(wb, w);
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    float x[kIn], y[kOut];
    D3 e1, e2, p;
    vertex_features(A, v, x, e1, e2, p);
    forward1(w, x, y, nullptr, nullptr);
    const D3 d = add3(scl3(scale * y[0], e1), scl3(scale * y[1], e2));
    st3(posOut, v, sphere_move(p, d, R));
}

size_t train_smem() {
    return sizeof(float) * (kParams + kTB * kIn + 3 * kTB * kPad + 2 * kTB);
}

}  // namespace

struct svm_mlp {
    cudaStream_t stream = nullptr;
    float* w = nullptr;       // FP32 master [kParams]
    float* m = nullptr;       // Adam moments
    float* v = nullptr;
    float* g = nullptr;       // gradient
    __nv_bfloat16* wb = nullptr;
    float* partials = nullptr;
    double* lossPartials = nullptr;
    double* loss = nullptr;
    int maxBlocks = 0;
    long adamStep = 0;
    double outScale = 1.0;
    float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
};

static int mlp_reserve(svm_mlp* M, int blocks) {
    if (blocks <= M->maxBlocks) return SVM_OK;
    if (M->partials) cudaFree(M->partials);
    if (M->lossPartials) cudaFree(M->lossPartials);
    M->partials = nullptr; M->lossPartials = nullptr;
    if (cudaMalloc(&M->partials, sizeof(float) * (size_t)blocks * kParams) != cudaSuccess ||
        cudaMalloc(&M->lossPartials, sizeof(double) * blocks) != cudaSuccess)
        return SVM_ERR_CUDA;
    M->maxBlocks = blocks;
    return SVM_OK;
}

// forward + backward over samples [first, first + count) of `order` (or of X directly); gradient
// of sum (y - t)^2 * invBatch into M->g, loss sum into M->loss
static int mlp_grad(svm_mlp* M, const float* X, const float* Y, const int* order, int first, int count,
                    float invBatch) {
    const int blocks = (count + kTB - 1) / kTB;
    int rc = mlp_reserve(M, blocks);
    if (rc) return rc;
    // the training kernel's shared memory exceeds the default 48 KB: opt in (per device)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SVM_ERR_CUDA;
    static std::once_flag once[64];
    static cudaError_t attrErr[64];
    std::call_once(once[dev], [&] {
        attrErr[dev] = cudaFuncSetAttribute(k_train_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem());
    });
    if (attrErr[dev] != cudaSuccess) return SVM_ERR_CUDA;
    k_train_block<<<blocks, kTB, train_smem(), M->stream>>>(M->wb, X, Y, order, first, count, invBatch, M->partials,
                                                          M->lossPartials);
    k_reduce_grad<<<(kParams + 255) / 256, 256, 0, M->stream>>>(M->partials, blocks, M->g, M->lossPartials, M->loss);
    return check_launch();
}

static FeatArgs feat_args(svm_model* m) {
    FeatArgs A;
    A.pos = m->pos[m->cur]; A.vnbr = m->vnbr; A.vcell = m->vcell; A.cellPos = m->cellPos; A.ap = m->ap;
    A.pref = m->pref; A.ringCount = m->ringCount; A.force = m->force;
    return A;
}

extern "C" {

int svm_mlp_create(unsigned seed, void* stream, svm_mlp** out) {
    if (!out) return SVM_ERR_ARG;
    svm_mlp* M = new svm_mlp();
    M->stream = static_cast<cudaStream_t>(stream);
    bool ok = cudaMalloc(&M->w, sizeof(float) * kParams) == cudaSuccess &&
              cudaMalloc(&M->m, sizeof(float) * kParams) == cudaSuccess &&
              cudaMalloc(&M->v, sizeof(float) * kParams) == cudaSuccess &&
              cudaMalloc(&M->g, sizeof(float) * kParams) == cudaSuccess &&
              cudaMalloc(&M->wb, sizeof(__nv_bfloat16) * kParams) == cudaSuccess &&
              cudaMalloc(&M->loss, sizeof(double)) == cudaSuccess;
    if (!ok) { svm_mlp_destroy(M); return SVM_ERR_CUDA; }
    // He-uniform initialisation from the seed, zero biases
    std::mt19937 gen(seed);
    std::vector<float> w(kParams, 0.f);
    auto fill = [&](int off, int fanOut, int fanIn) {
        std::uniform_real_distribution<float> u(-std::sqrt(6.f / fanIn), std::sqrt(6.f / fanIn));
        for (int i = 0; i < fanOut * fanIn; ++i) w[off + i] = u(gen);
    };
    fill(oW1, kH, kIn);
    fill(oW2, kH, kH);
    fill(oW3, kOut, kH);
    for (int i = oW3; i < oW3 + kOut * kH; ++i) w[i] *= 0.1f;  // small initial outputs
    int rc = svm_mlp_set_weights(M, w.data());
    if (rc) { svm_mlp_destroy(M); return rc; }
    *out = M;
    return SVM_OK;
}

int svm_mlp_destroy(svm_mlp* M) {
    if (!M) return SVM_ERR_ARG;
    if (M->stream) cudaStreamSynchronize(M->stream);
    void* ptrs[] = {M->w, M->m, M->v, M->g, M->wb, M->partials, M->lossPartials, M->loss};
    for (void* p : ptrs) if (p) cudaFree(p);
    delete M;
    return SVM_OK;
}

int svm_mlp_parameter_count(int* n) {
    if (!n) return SVM_ERR_ARG;
    *n = kParams;
    return SVM_OK;
}

int svm_mlp_set_weights(svm_mlp* M, const float* w) {
    if (!M || !w) return SVM_ERR_ARG;
    if (cudaMemcpyAsync(M->w, w, sizeof(float) * kParams, cudaMemcpyHostToDevice, M->stream) != cudaSuccess ||
        cudaMemsetAsync(M->m, 0, sizeof(float) * kParams, M->stream) != cudaSuccess ||
        cudaMemsetAsync(M->v, 0, sizeof(float) * kParams, M->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    k_to_bf16<<<(kParams + 255) / 256, 256, 0, M->stream>>>(M->w, M->wb);
    M->adamStep = 0;
    if (check_launch()) return SVM_ERR_CUDA;
    return cudaStreamSynchronize(M->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

int svm_mlp_get_weights(svm_mlp* M, float* w) {
    if (!M || !w) return SVM_ERR_ARG;
    if (cudaMemcpyAsync(w, M->w, sizeof(float) * kParams, cudaMemcpyDeviceToHost, M->stream) != cudaSuccess ||
        cudaStreamSynchronize(M->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    return SVM_OK;
}

int svm_mlp_set_output_scale(svm_mlp* M, double scale) {
    if (!M || !(scale > 0)) return SVM_ERR_ARG;
    M->outScale = scale;
    return SVM_OK;
}

int svm_mlp_features(svm_model* m, float* X, double* frames) {
    if (!m || !X || m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    k_features<<<(m->nVertices + 255) / 256, 256, 0, m->stream>>>(feat_args(m), m->nVertices, X, frames);
    if (check_launch()) return SVM_ERR_CUDA;
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

int svm_mlp_gradient(svm_mlp* M, const float* X, const float* Y, int n, float* grad, double* loss) {
    if (!M || !X || !Y || n <= 0 || !grad) return SVM_ERR_ARG;
    int rc = mlp_grad(M, X, Y, nullptr, 0, n, 1.f / n);
    if (rc) return rc;
    if (cudaMemcpyAsync(grad, M->g, sizeof(float) * kParams, cudaMemcpyDeviceToHost, M->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    double l = 0.0;
    if (cudaMemcpyAsync(&l, M->loss, sizeof(double), cudaMemcpyDeviceToHost, M->stream) != cudaSuccess ||
        cudaStreamSynchronize(M->stream) != cudaSuccess)
        return SVM_ERR_CUDA;
    if (loss) *loss = l / n;
    return SVM_OK;
}

int svm_mlp_train(svm_mlp* M, const float* X, const float* Y, const int* order, int n, int batch, float lr,
                  double* meanLoss) {
    if (!M || !X || !Y || !order || n <= 0 || batch <= 0) return SVM_ERR_ARG;
    double total = 0.0;
    for (int first = 0; first < n; first += batch) {
        const int count = std::min(batch, n - first);
        int rc = mlp_grad(M, X, Y, order, first, count, 1.f / count);
        if (rc) return rc;
        M->adamStep++;
        const float c1 = 1.f - std::pow(M->beta1, (float)M->adamStep);
        const float c2 = 1.f - std::pow(M->beta2, (float)M->adamStep);
        k_adam<<<(kParams + 255) / 256, 256, 0, M->stream>>>(M->w, M->m, M->v, M->g, M->wb, lr, M->beta1, M->beta2,
                                                            M->eps, c1, c2);
        if (check_launch()) return SVM_ERR_CUDA;
        if (meanLoss) {
            double l = 0.0;
            if (cudaMemcpyAsync(&l, M->loss, sizeof(double), cudaMemcpyDeviceToHost, M->stream) != cudaSuccess ||
                cudaStreamSynchronize(M->stream) != cudaSuccess)
                return SVM_ERR_CUDA;
            total += l;
        }
    }
    if (meanLoss) *meanLoss = total / n;
    return cudaStreamSynchronize(M->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

int svm_mlp_predict(svm_mlp* M, const float* X, int n, float* Y) {
    if (!M || !X || !Y || n <= 0) return SVM_ERR_ARG;
    k_predict<<<(n + 255) / 256, 256, 0, M->stream>>>(M->wb, X, n, Y);
    if (check_launch()) return SVM_ERR_CUDA;
    return cudaStreamSynchronize(M->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

int svm_mlp_warm_start(svm_mlp* M, svm_model* m) {
    if (!M || !m || m->precision == SVM_PRECISION_MIXED) return SVM_ERR_ARG;
    if (cudaStreamSynchronize(M->stream) != cudaSuccess) return SVM_ERR_CUDA;  // training done
    // geometry and forces of the current state feed the features
    int rc = svm_model_compute_forces(m);
    if (rc) return rc;
    const int nxt = 1 - m->cur;
    k_warm_start<<<(m->nVertices + 255) / 256, 256, 0, m->stream>>>(M->wb, feat_args(m), m->nVertices, M->outScale,
                                                                    m->R, m->pos[nxt]);
    if (check_launch()) return SVM_ERR_CUDA;
    m->cur = nxt;
    m->cornersValid = false;
    m->paramsVersion++;  // captured graphs hold the old buffer roles
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? SVM_OK : SVM_ERR_CUDA;
}

}  // extern "C"
