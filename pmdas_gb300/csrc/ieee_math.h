// ieee_math.h — reproducible single-precision helpers built only from
// IEEE-754 operations that round identically on a GB300 and on a host CPU
// (add, sub, mul, div, sqrt, fmaf, bit casts).
//
// Used by:
//   * the strict-IEEE build of the MDAS kernels (the `pow` in the leaf
//     acceptance test `powf(error / g_error, alpha) >= rnd(seed)`,
//     SDK/lib/mdas/kdgrid.cu:326, and the sRGB transfer in
//     SDK/cuda/helpers.h:35-43),
//   * the analytic integrands (concentric lens mapping, SDK/cuda/whitted.cu:186-206),
//   * and the CPU oracle, which must reproduce both bit for bit.
//
// The functions are written from the series definitions named beside each one;
// they are not CUDA's or any C library's algorithms, and they are not meant to
// be as accurate as a libm (about 1e-6 relative is enough here); they are meant
// to give the same bits on every machine that rounds IEEE binary32 correctly.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define MDAS_HD __host__ __device__ __forceinline__
#else
#define MDAS_HD static inline
#endif

MDAS_HD uint32_t mdas_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

MDAS_HD float mdas_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// Fused multiply-add with a single rounding; fmaf is correctly rounded on the
// device (fma.rn.f32) and in any conforming C library.
MDAS_HD float mdas_fma(float a, float b, float c) { return fmaf(a, b, c); }

// 2^n for integer n in [-149, 127], exact.
MDAS_HD float mdas_exp2i(int n) {
    if (n >= -126) return mdas_u2f((uint32_t)(n + 127) << 23);
    return mdas_u2f(1u << (n + 149));  // subnormal powers of two
}

// log2(x) for finite x > 0.
// x = m * 2^e with m in [sqrt(1/2), sqrt(2)); ln(m) = 2 atanh(s), s = (m-1)/(m+1),
// atanh(s) = s + s^3/3 + s^5/5 + ... (Taylor series, |s| <= 0.1716, terms to s^13).
MDAS_HD float mdas_log2f(float x) {
    int e = 0;
    if (x < 1.17549435e-38f) {  // subnormal: scale into the normal range (exact)
        x = x * 8388608.0f;     // 2^23
        e = -23;
    }
    uint32_t u = mdas_f2u(x);
    e += (int)((u >> 23) & 0xffu) - 127;
    float m = mdas_u2f((u & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > 1.41421356f) {
        m = m * 0.5f;  // exact
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 0.0769230769f;            // 1/13
    p = mdas_fma(p, s2, 0.0909090909f); // 1/11
    p = mdas_fma(p, s2, 0.111111111f);  // 1/9
    p = mdas_fma(p, s2, 0.142857143f);  // 1/7
    p = mdas_fma(p, s2, 0.2f);          // 1/5
    p = mdas_fma(p, s2, 0.333333333f);  // 1/3
    p = p * s2;
    const float two_s = s + s;
    const float ln_m = mdas_fma(two_s, p, two_s);
    const float log2_m = ln_m * 1.44269504f;  // 1/ln(2)
    return (float)e + log2_m;
}

// 2^t for finite t.  t = n + f, n = nearest integer, |f| <= 1/2;
// 2^f = e^(f ln 2) by its Taylor series to degree 8.
MDAS_HD float mdas_exp2f(float t) {
    if (!(t > -150.0f)) return 0.0f;  // also maps NaN to 0
    if (t >= 128.0f) return mdas_u2f(0x7f800000u);
    const float n = rintf(t);
    const float f = t - n;            // exact
    const float g = f * 0.693147181f; // ln(2)
    float p = 2.48015873e-5f;         // 1/8!
    p = mdas_fma(p, g, 1.98412698e-4f);  // 1/7!
    p = mdas_fma(p, g, 1.38888889e-3f);  // 1/6!
    p = mdas_fma(p, g, 8.33333333e-3f);  // 1/5!
    p = mdas_fma(p, g, 4.16666667e-2f);  // 1/4!
    p = mdas_fma(p, g, 0.166666667f);    // 1/3!
    p = mdas_fma(p, g, 0.5f);            // 1/2!
    p = mdas_fma(p, g, 1.0f);
    p = mdas_fma(p, g, 1.0f);
    const int ni = (int)n;
    if (ni >= -126) return p * mdas_exp2i(ni);
    // split the scale so that the intermediate stays normal
    return (p * mdas_exp2i(ni + 64)) * mdas_exp2i(-64);
}

// x^y for x >= 0 (the only domain MDAS needs: error ratios and colours).
MDAS_HD float mdas_powf(float x, float y) {
    if (x == 1.0f || y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return 0.0f;  // x == 0 (y > 0) and NaN
    return mdas_exp2f(y * mdas_log2f(x));
}

// sin and cos of phi in [-pi/4, pi/4] (Taylor series to degree 11 / 10).
MDAS_HD void mdas_sincos_quarter(float phi, float* s, float* c) {
    const float t2 = phi * phi;
    float ps = -2.50521084e-8f;            // -1/11!
    ps = mdas_fma(ps, t2, 2.75573192e-6f); // 1/9!
    ps = mdas_fma(ps, t2, -1.98412698e-4f);// -1/7!
    ps = mdas_fma(ps, t2, 8.33333333e-3f); // 1/5!
    ps = mdas_fma(ps, t2, -0.166666667f);  // -1/3!
    ps = ps * t2;
    *s = mdas_fma(phi, ps, phi);
    float pc = -2.75573192e-7f;            // -1/10!
    pc = mdas_fma(pc, t2, 2.48015873e-5f); // 1/8!
    pc = mdas_fma(pc, t2, -1.38888889e-3f);// -1/6!
    pc = mdas_fma(pc, t2, 4.16666667e-2f); // 1/4!
    pc = mdas_fma(pc, t2, -0.5f);          // -1/2!
    *c = mdas_fma(pc, t2, 1.0f);
}
