// Conservative pre-check of the T1 length test (geodesic(p1, p2) < t, sphericalVertexModel.cpp:475
// and sphericalVertexModel.cu:225-273) that issues no FP64 instruction: most edges of a vertex
// model are several times longer than the threshold, and on GB300 the FP64 pipe (2 lanes per clock
// per SM) is the scarce one.  Host and device builds evaluate the same IEEE FP32 operations, so
// tests/native/edge_filter_check.cpp checks the bound on the CPU.
#pragma once
#include "svm_softf64.cuh"

namespace svm_edge {

SF_HD float f32(unsigned u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    __builtin_memcpy(&x, &u, 4);
    return x;
#endif
}
SF_HD float fma32(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}

// x as an FP32 value built from its high word alone: sign, exponent and the top 20 mantissa bits
// (truncated towards zero, |error| < 2^-20 |x|), on the integer pipes.  Magnitudes below 2^-100
// read as 0; those of 2^128 or more, infinities and NaN read as NaN.
SF_HD float hi_word_float(double x) {
    const unsigned hi = (unsigned)(sf::bits(x) >> 32);
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned sign = hi & 0x80000000u;
    if (e < 1023 - 100) return f32(sign);
    if (e > 1023 + 127) return f32(0x7fc00000u);
    return f32(sign | ((unsigned)(e - 1023 + 127) << 23) | ((hi & 0xfffffu) << 3));
}

// True when the edge p1-p2 (points of a sphere of radius R) is certainly longer than t: its chord,
// evaluated in FP32 from hi_word_float coordinates, exceeds t (1 + 1e-3) + 1e-5 R.  Each coordinate
// is then off by less than 2^-20 R and the FP32 roundings by a few 2^-24 relative, so the exact
// chord exceeds t by more than 9e-4 t + 6e-6 R, and the arc (never shorter than the chord) does
// too: far beyond the FP64 test's rounding (relative 1e-12 at the model's shortest edges), which
// therefore reaches the same "not shorter" decision.  A coordinate, R or t out of hi_word_float's
// range makes it false (undecided).
SF_HD bool clearly_longer(double x1, double y1, double z1, double x2, double y2, double z2, double R, double t) {
    const float dx = hi_word_float(x1) - hi_word_float(x2);
    const float dy = hi_word_float(y1) - hi_word_float(y2);
    const float dz = hi_word_float(z1) - hi_word_float(z2);
    const float lim = fma32(hi_word_float(t), 1.001f, 1e-5f * hi_word_float(R));
    return fma32(dx, dx, fma32(dy, dy, dz * dz)) > lim * lim;
}

}  // namespace svm_edge
