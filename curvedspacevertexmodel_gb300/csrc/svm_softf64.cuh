// IEEE-754 binary64 arithmetic, round to nearest even, computed on the integer and FP32 pipes.
//
// GB300 issues FP64 at 2 lanes per clock per SM (a warp instruction every 16 SM cycles), and a
// double division or square root is a sequence of about eight FP64 instructions.  The functions
// here return the same bits as the hardware's correctly rounded operations (they are the IEEE
// operations, computed another way) from 64-bit integer arithmetic, so a kernel bound by FP64 issue
// can move part of its work off the FP64 pipe without changing any result.
//
// Each function handles the common case -- normal finite operands and a normal result -- itself and
// passes everything else (zeros, subnormals, infinities, NaNs, results that overflow or underflow)
// to the hardware operation, so every input gets the IEEE result.
//
// Methods:
//   mul   the 106-bit product of the significands (64x64 -> 128-bit integer multiply), rounded.
//   add   significands aligned with 10 guard bits and a sticky bit, added or subtracted,
//         renormalised (count of leading zeros), rounded.
//   div   reciprocal of the divisor: an FP32 seed refined once in FP32 (two-term seed, ~46 bits),
//         one Newton-Raphson step r <- r + r (1 - y r) in 64-bit fixed point; the quotient from the
//         reciprocal, then corrected against the exact integer remainder and rounded from it.
//   sqrt  reciprocal square root: an FP32 seed, two Newton-Raphson steps r <- r (3 - x r^2) / 2 in
//         64-bit fixed point; the root from it, corrected against the exact integer remainder.
//   widen / narrow  float <-> double by moving the fields (narrow: round to nearest even on the
//         29 dropped bits).
// (Newton-Raphson refinement of reciprocals and the final correction by an exact remainder are the
// classical methods of P. Markstein, "IA-64 and Elementary Functions", 2000, and of integer
// division by invariant integers, T. Granlund and P. Montgomery, PLDI 1994.)
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define SF_HD __host__ __device__ __forceinline__
#else
#define SF_HD inline
#endif

namespace sf {

constexpr unsigned long long kMant = 0xFFFFFFFFFFFFFull, kHid = 0x10000000000000ull, kSign = 0x8000000000000000ull;

SF_HD unsigned long long bits(double x) {
#if defined(__CUDA_ARCH__)
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long u;
    __builtin_memcpy(&u, &x, 8);
    return u;
#endif
}
SF_HD double dbl(unsigned long long u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, 8);
    return x;
#endif
}
SF_HD unsigned long long mulhi(unsigned long long a, unsigned long long b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}
SF_HD int clz64(unsigned long long x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}
// FP32 helpers of the seeds: round-to-nearest reciprocal and reciprocal square root of a float.
SF_HD float rcp32(float x) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}
SF_HD float rsqrt32(float x) {
#if defined(__CUDA_ARCH__)
    return __frsqrt_rn(x);
#else
    return 1.0f / __builtin_sqrtf(x);
#endif
}
SF_HD float fma32(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
// The hardware operations (the fallback for operands and results outside the fast paths).
SF_HD double hw_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}
SF_HD double hw_add(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    volatile double r = a + b;
    return r;
#endif
}
SF_HD double hw_div(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    volatile double r = a / b;
    return r;
#endif
}
SF_HD double hw_sqrt(double a) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a);
#else
    volatile double r = __builtin_sqrt(a);
    return r;
#endif
}

// Rounds the significand m (hidden bit at 52) with the rest `rest` (2^63 = one half of the last
// place) to nearest even and packs it with the biased exponent E (the carry of a round-up into
// bit 53 increments the exponent, up to infinity) and the sign.
SF_HD double pack(unsigned long long sign, int E, unsigned long long m, unsigned long long rest) {
    const unsigned long long up = (rest > kSign) | ((rest == kSign) & (m & 1ull));
    return dbl(sign | ((((unsigned long long)(E - 1)) << 52) + m + up));
}

SF_HD double mul(double a, double b) {
    const unsigned long long ia = bits(a), ib = bits(b);
    const unsigned ea = (unsigned)(ia >> 52) & 0x7ffu, eb = (unsigned)(ib >> 52) & 0x7ffu;
    const int E = (int)ea + (int)eb - 1023;
    if (ea - 1u < 2046u && eb - 1u < 2046u && (unsigned)(E - 1) < 2045u) {
        const unsigned long long ma = (ia & kMant) | kHid, mb = (ib & kMant) | kHid;
        const unsigned long long lo = ma * mb, hi = mulhi(ma, mb);  // product in [2^104, 2^106)
        const unsigned n = (unsigned)(hi >> 41);                    // 1: product >= 2^105
        const unsigned long long m = (hi << (12 - n)) | (lo >> (52 + n));
        return pack((ia ^ ib) & kSign, E + (int)n, m, lo << (12 - n));
    }
    return hw_mul(a, b);
}

SF_HD double add(double a, double b) {
    unsigned long long ia = bits(a), ib = bits(b);
    unsigned long long aa = ia & ~kSign, ab = ib & ~kSign;
    if (aa < ab) {
        unsigned long long t = ia; ia = ib; ib = t;
        t = aa; aa = ab; ab = t;
    }
    const unsigned ea = (unsigned)(aa >> 52), eb = (unsigned)(ab >> 52);
    if (ea - 1u < 2046u && eb - 1u < 2046u) {
        const unsigned d = ea - eb;
        const unsigned long long A = ((aa & kMant) | kHid) << 10;
        unsigned long long B = ((ab & kMant) | kHid) << 10;
        if (d) B = d < 64 ? ((B >> d) | (unsigned long long)((B << (64 - d)) != 0)) : 1ull;
        int E = (int)ea;
        unsigned long long S;
        if (!((ia ^ ib) >> 63)) {
            S = A + B;
            if (S >> 63) { S = (S >> 1) | (S & 1ull); E += 1; }
        } else {
            S = A - B;
            if (S == 0) return 0.0;
            const int lz = clz64(S) - 1;
            S <<= lz;
            E -= lz;
        }
        if ((unsigned)(E - 1) < 2046u) return pack(ia & kSign, E, S >> 10, S << 54);
    }
    return hw_add(a, b);
}

SF_HD double sub(double a, double b) { return add(a, dbl(bits(b) ^ kSign)); }

SF_HD double div(double a, double b) {
    const unsigned long long ia = bits(a), ib = bits(b);
    const unsigned ea = (unsigned)(ia >> 52) & 0x7ffu, eb = (unsigned)(ib >> 52) & 0x7ffu;
    if (ea - 1u < 2046u && eb - 1u < 2046u) {
        const unsigned long long sign = (ia ^ ib) & kSign;
        const unsigned long long ma = (ia & kMant) | kHid, mb = (ib & kMant) | kHid;
        const int n = ma >= mb ? 1 : 0;                  // quotient of the significands in [1, 2)
        const int E = (int)ea - (int)eb + 1022 + n;
        if ((unsigned)(E - 1) < 2045u) {
            if ((ib & kMant) == 0) return dbl(sign | ((((unsigned long long)(E - 1)) << 52) + ma));  // b = 2^k
            // two-term FP32 seed of 2^40 / Y, Y = mb << 11: y = yh + yl (48 leading bits, both exact)
            const unsigned long long Y = mb << 11;
            const float yh = (float)(unsigned)(Y >> 40), yl = (float)(unsigned)((Y >> 16) & 0xFFFFFFu) * 0x1p-24f;
            const float r = rcp32(yh);
            const float e = fma32(-r, yl, fma32(-r, yh, 1.0f));   // 1 - r (yh + yl)
            // R ~ 2^127 / Y in (2^63, 2^64): r (1 + e) scaled, the two terms converted separately
            const unsigned long long t = (unsigned long long)(r * 0x1p86f);   // in (2^62, 2^63]
            unsigned long long R = t >= kSign ? ~0ull : t << 1;          // 2^64 saturates to 2^64 - 1
            const long long c0 = (long long)(r * e * 0x1p87f);
            R = (unsigned long long)((long long)R + c0);
            // one Newton-Raphson step in fixed point: R += R (2^127 - Y R) / 2^127
            const unsigned long long plo = Y * R, phi = mulhi(Y, R);
            const long long eh = (long long)(kSign - phi - (plo != 0));  // top half of 2^127 - Y R
            const unsigned long long ae = (unsigned long long)(eh < 0 ? -eh : eh);
            const unsigned long long chi = mulhi(R, ae), clo = R * ae;
            const unsigned long long c = (chi << 1) | (clo >> 63);     // R |e| / 2^63
            R = eh < 0 ? R - c : R + c;
            // quotient with a guard bit: Q ~ floor(ma 2^(54 - n) / mb), then the exact remainder
            const unsigned long long Qp = mulhi(ma << 11, R);            // ~ (ma / mb) 2^63
            long long Q = (long long)(Qp >> (9 + n));
            long long rem = (long long)((ma << (54 - n)) - (unsigned long long)Q * mb);
            for (int k = 0; k < 3 && rem < 0; ++k) { Q -= 1; rem += (long long)mb; }
            for (int k = 0; k < 3 && rem >= (long long)mb; ++k) { Q += 1; rem -= (long long)mb; }
            const unsigned long long q = (unsigned long long)Q;   // in [2^53, 2^54)
            // rest of the 53-bit significand q >> 1: the guard bit, and the remainder as a sticky bit
            const unsigned long long rest = ((q & 1ull) << 63) | (unsigned long long)(rem != 0);
            return pack(sign, E, q >> 1, rest);
        }
    }
    return hw_div(a, b);
}

SF_HD double sqrt(double a) {
    const unsigned long long ia = bits(a);
    const unsigned ea = (unsigned)(ia >> 52);  // sign bit included: negatives take the fallback
    if (ea - 1u < 2046u) {
        const unsigned long long ma = (ia & kMant) | kHid;
        const int odd = (int)((ea - 1023u) & 1u);     // unbiased exponent odd: the root of 2 ma
        const int E = ((int)ea - 1023 - odd) / 2 + 1023;  // (an even difference: exact)
        // m = M / 2^52 in [1, 4); R ~ 2^63 / sqrt(m) in (2^62, 2^63]
        const unsigned long long M = ma << odd;                           // [2^52, 2^54)
        const float mf = (float)(unsigned)(M >> 29) * 0x1p-23f;        // m to 24 bits (truncated)
        const float rf = rsqrt32(mf);                                   // 1 / sqrt(m), ~2^-23
        unsigned long long R = (unsigned long long)(rf * 0x1p63f);      // 2^63 / sqrt(m) in (2^62, 2^63]
        // two Newton-Raphson steps r <- r (3 - m r^2) / 2 in fixed point (m r^2 ~ 1 at 2^62 scale)
        for (int it = 0; it < 2; ++it) {
            const unsigned long long r2 = mulhi(R, R);                  // R^2 / 2^64 = 2^62 r^2
            const unsigned long long mr2 = mulhi(M << 10, r2) << 2;    // M r2 / 2^52 = 2^62 m r^2
            const long long d = (long long)((1ull << 62) - mr2);       // 2^62 (1 - m r^2)
            const unsigned long long ad = (unsigned long long)(d < 0 ? -d : d);
            const unsigned long long cor = mulhi(R, ad) << 1;           // R (1 - m r^2) / 2, magnitude
            R = d < 0 ? R - cor : R + cor;
        }
        // root with a guard bit: S ~ sqrt(m) 2^53 = m r 2^53 = M R / 2^62, in [2^53, 2^54)
        long long S = (long long)(mulhi(M << 10, R) >> 8);
        // exact remainder of S^2 against M 2^54 (both below 2^108; their difference is small)
        long long rem = (long long)((M << 54) - (unsigned long long)S * (unsigned long long)S);
        for (int k = 0; k < 3 && rem < 0; ++k) { rem += 2 * S - 1; S -= 1; }
        for (int k = 0; k < 3 && rem > 2 * S; ++k) { S += 1; rem -= 2 * S - 1; }
        const unsigned long long s = (unsigned long long)S;
        const unsigned long long rest = ((s & 1ull) << 63) | (unsigned long long)(rem != 0);
        return pack(0ull, E, s >> 1, rest);
    }
    return hw_sqrt(a);
}

// Conversions between float and double, on the integer pipes (conversion instructions with a 64-bit
// operand issue on GB300's FP64 pipe, at its rate).  widen is exact; narrow rounds to nearest even.
// Zeros, subnormals, infinities and NaN -- and doubles outside the normal float range -- take the
// hardware conversion.
SF_HD unsigned f32bits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    unsigned u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
SF_HD float f32of(unsigned u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}
SF_HD double hw_widen(float f) {
#if defined(__CUDA_ARCH__)
    return (double)f;
#else
    volatile double r = (double)f;
    return r;
#endif
}
SF_HD float hw_narrow(double d) {
#if defined(__CUDA_ARCH__)
    return __double2float_rn(d);
#else
    volatile float r = (float)d;
    return r;
#endif
}
SF_HD double widen(float f) {
    const unsigned u = f32bits(f), e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return hw_widen(f);
    // sign, exponent rebiased by 1023 - 127, the 23 significand bits on top of the double's 52
    return dbl(((unsigned long long)(u & 0x80000000u) << 32) | ((unsigned long long)(e + 896u) << 52) |
               ((unsigned long long)(u & 0x7fffffu) << 29));
}
SF_HD float narrow(double d) {
    const unsigned long long b = bits(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 126 || e > 1023 + 127) return hw_narrow(d);
    // 23 significand bits kept, 29 rounded: to nearest, ties to even; a carry out of the
    // significand raises the exponent (up to infinity from the largest binade), as IEEE rounding does
    const unsigned m = (unsigned)((b >> 29) & 0x7fffffu), r = (unsigned)(b & 0x1fffffffu);
    unsigned f = ((unsigned)(b >> 32) & 0x80000000u) | ((unsigned)(e - 896) << 23) | m;
    if (r > 0x10000000u || (r == 0x10000000u && (m & 1u))) f += 1u;
    return f32of(f);
}

}  // namespace sf
