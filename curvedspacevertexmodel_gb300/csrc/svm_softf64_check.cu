// svm_softf64_check: the device build of svm_softf64.cuh against the hardware's correctly rounded
// FP64 instructions and conversions, on random operands.  A diagnostic entry point (no counterpart in the
// reference): the FP64 kernels' divisions and square roots go through these functions.
#include <cuda_runtime.h>
#include "svm_softf64.cuh"
#include "../../include/svm.h"

namespace {

__device__ unsigned long long splitmix(unsigned long long z) {  // splitmix64 (Steele et al. 2014)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ bool same_bits(double x, double y) { return (x != x && y != y) || sf::bits(x) == sf::bits(y); }

__global__ void k_softf64_check(unsigned long long seed, long long cases, unsigned long long* bad) {
    unsigned nb[6] = {0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cases; i += stride) {
        const unsigned long long k = seed ^ ((unsigned long long)i * 8ull);
        unsigned long long ua = splitmix(k), ub = splitmix(k + 1);
        const unsigned long long r = splitmix(k + 2);
        const int mode = (int)(r & 7);
        if (mode >= 2) {  // exponents near 1
            ua = (ua & (sf::kMant | sf::kSign)) | ((unsigned long long)(1023 + (int)((r >> 8) % 81) - 40) << 52);
            ub = (ub & (sf::kMant | sf::kSign)) | ((unsigned long long)(1023 + (int)((r >> 16) % 81) - 40) << 52);
        }
        if (mode == 3) ub = ua ^ (splitmix(k + 3) & 0xFFFF) ^ ((r >> 30) & 1 ? sf::kSign : 0);  // near cancellation
        if (mode == 4) ub &= ~0xFFFFFFull;                                                       // short significand
        if (mode == 5) { ua &= ~0xFFFFFFFFull; ub = (ub & ~sf::kMant) | (splitmix(k + 4) & 0xF); }  // b just above 2^k
        if (mode == 6) { ub = (ub | sf::kMant) ^ (splitmix(k + 5) & 0xF); ua = ub + (splitmix(k + 6) % 9) - 4; }
        const double a = sf::dbl(ua), b = sf::dbl(ub);
        nb[0] += !same_bits(sf::mul(a, b), __dmul_rn(a, b));
        nb[1] += !same_bits(sf::add(a, b), __dadd_rn(a, b));
        nb[2] += !same_bits(sf::div(a, b), __ddiv_rn(a, b));
        nb[3] += !same_bits(sf::sqrt(fabs(a)), __dsqrt_rn(fabs(a)));
        // conversions: a float from the low word of ua (any bit pattern), and a double whose 29
        // dropped bits sit at, next to or away from a rounding tie (mode 7: the largest binade)
        const float f = sf::f32of((unsigned)ua);
        nb[4] += !same_bits(sf::widen(f), (double)f);
        unsigned long long ud = ub;
        if (mode & 1) ud = (ud & ~0x1FFFFFFFull) | (0x10000000ull + (r >> 40) % 5) - 2;
        if (mode == 7) ud = (ud & ~(0x7FFull << 52)) | (1150ull << 52) | 0xFFFFFE0000000ull;
        const double dn = sf::dbl(ud);
        const float fn = sf::narrow(dn), fh = __double2float_rn(dn);
        nb[5] += !((fn != fn && fh != fh) || sf::f32bits(fn) == sf::f32bits(fh));
    }
    for (int q = 0; q < 6; ++q)
        if (nb[q]) atomicAdd(bad + q, (unsigned long long)nb[q]);
}

}  // namespace

extern "C" int svm_softf64_check(long long cases, unsigned long long seed, unsigned long long* mismatches6) {
    if (cases < 0 || !mismatches6) return SVM_ERR_ARG;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 6 * sizeof(unsigned long long)) != cudaSuccess) return SVM_ERR_CUDA;
    cudaMemset(d, 0, 6 * sizeof(unsigned long long));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    k_softf64_check<<<8 * (sms > 0 ? sms : 1), 256>>>(seed, cases, d);
    const bool ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
                    cudaMemcpy(mismatches6, d, 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(d);
    return ok ? SVM_OK : SVM_ERR_CUDA;
}
