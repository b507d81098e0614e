// A portable arccosine: the same IEEE-754 binary64 operations, in the same order, on the GPU and
// on any host CPU, so it returns the same bits everywhere.
//
// Library arccosines (CUDA's, glibc's on x86-64 or on aarch64) are not correctly rounded, and
// they differ from one another in the last bit for some arguments.  The vertex model's area,
// perimeter and T1 decisions go through acos, and its closed-form gradients divide by 1 - s^2 for
// short edges, so a one-ulp difference grows along a trajectory.  Built with this function on both
// sides (the device library compiled with -DSVM_PORTABLE_ACOS, the CPU restatement switched to it
// at run time), the GPU and CPU trajectories can be compared bit for bit.
//
// Method (Cody and Waite, "Software Manual for the Elementary Functions", 1980: argument
// reduction of asin/acos to [0, 1/2]):
//   |x| <= 1/2:  acos x = pi/2 - asin x,        asin x = x + x t P(t),  t = x^2
//   x > 1/2:     acos x = 2 asin s,             s = sqrt((1 - x) / 2)   ((1 - x) is exact)
//   x < -1/2:    acos x = pi - 2 asin s,        s = sqrt((1 + x) / 2)
// P is a degree-11 polynomial in t approximating (asin(sqrt t) - sqrt t) / t^(3/2) on [0, 1/4],
// fitted for this file by Chebyshev interpolation in 60-digit arithmetic (mpmath.chebyfit) and
// rounded to double; its relative error is below 3e-16, far below the final rounding.  pi/2 is
// carried as a double-double (hi + lo).  Maximum error 1.35 ulp over [-1, 1] (measured against a
// 60-digit acos at 75,000 points, densest near 0 and +-1); acos(1) = 0, acos(-1) = kPI, NaN
// outside [-1, 1] and for NaN.  Only +, -, * and sqrt are used, each rounded separately (explicit
// round-to-nearest intrinsics on the device, the square root on the integer pipes; the host side is
// compiled without FP contraction).
#pragma once

#if defined(__CUDACC__)
#define SVM_ACOS_HD __host__ __device__ __forceinline__
#else
#define SVM_ACOS_HD inline
#endif

#include <cmath>

#include "svm_softf64.cuh"

namespace svm_portable {

SVM_ACOS_HD double mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
SVM_ACOS_HD double add(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
SVM_ACOS_HD double sub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
SVM_ACOS_HD double root(double a) {
#if defined(__CUDA_ARCH__)
    return sf::sqrt(a);  // the IEEE square root on the integer pipes (svm_softf64.cuh): same bits
#else
    return std::sqrt(a);
#endif
}

// t P(t) by Horner's rule, highest degree first.
SVM_ACOS_HD double asin_tail(double t) {
    double p = 0.028169218060881414;
    p = add(mul(p, t), -0.010749050339697808);
    p = add(mul(p, t), 0.01603551434914882);
    p = add(mul(p, t), 0.0078029494773533175);
    p = add(mul(p, t), 0.011875494382636922);
    p = add(mul(p, t), 0.013929652902326633);
    p = add(mul(p, t), 0.017355259955786323);
    p = add(mul(p, t), 0.02237204763174451);
    p = add(mul(p, t), 0.03038194736709848);
    p = add(mul(p, t), 0.044642857103423646);
    p = add(mul(p, t), 0.07500000000020764);
    p = add(mul(p, t), 0.1666666666666665);
    return mul(t, p);
}

SVM_ACOS_HD double acos(double x) {
    const double kPio2Hi = 1.5707963267948966;      // pi/2 rounded to double
    const double kPio2Lo = 6.123233995736766e-17;   // pi/2 - kPio2Hi
    const double ax = x < 0.0 ? -x : x;
    if (!(ax <= 1.0)) return sub(x, x) / sub(x, x);  // NaN for |x| > 1 and NaN input
    // the polynomial's argument first (t = x^2, or z = (1 - |x|) / 2), so that it is evaluated once
    const bool small = ax <= 0.5;
    const double t = small ? mul(x, x) : mul(sub(1.0, ax), 0.5);
    const double r = asin_tail(t);
    if (small) return sub(kPio2Hi, sub(x, sub(kPio2Lo, mul(x, r))));
    const double s = root(t);
    if (x > 0.0) return mul(2.0, add(s, mul(s, r)));
    return mul(2.0, sub(kPio2Hi, add(s, sub(mul(s, r), kPio2Lo))));
}

}  // namespace svm_portable
