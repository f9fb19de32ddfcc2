/*
 * gpr_rngmath.h -- the float transcendental and rounding steps that turn raw
 * random integers into proposal values, written so that the host (g++,
 * -ffp-contract=off) and the device (nvcc, explicit _rn intrinsics) produce
 * bit-identical results.
 *
 * Why this file exists.  The reference draws proposals through
 *   random_float  : float(random_int(1000000)) / 1000000.0      (main.cu:230-232)
 *   random_normal : sqrtf(-2.0*logf(u)) * sinf(2.0*PIf*v)         (main.cu:237-241)
 *   random_geometric: ceilf(logf(random_float()) / log(r))        (main.cu:251-254)
 * The double-precision steps (k/1e6 in double, 2*pi*v in double) are emulated
 * here in FP32 with error-free transforms: the replacements were checked
 * exhaustively against the double computation for every one of the 10^6
 * possible values of k (see tests/test_rngmath.py), because native FP64 on
 * GB300 runs at roughly 1/64 of the FP32 rate.  logf and sinf are project
 * functions (not libm, not CUDA's math library): a Cody-Waite range reduction
 * followed by truncated Taylor/atanh series, each step an IEEE-specified
 * operation, so one definition gives the same bits everywhere.
 *
 * The oracle build of the reference swaps these two functions in for logf/sinf
 * inside random_normal/random_geometric only, so proposals can be compared bit
 * for bit; everywhere else the reference keeps its libm calls.
 */
#ifndef GPR_RNGMATH_H
#define GPR_RNGMATH_H

#include <stdint.h>
#include <math.h>
#include <string.h>

#ifndef GPR_HD
#if defined(__CUDACC__)
#define GPR_HD __host__ __device__ __forceinline__
#else
#define GPR_HD static inline
#endif
#endif

/* Non-contractible IEEE operations.  On the device nvcc would otherwise fuse
 * a*b+c into an FMA; the host side is compiled with -ffp-contract=off. */
#if defined(__CUDA_ARCH__)
#define GPR_FMUL(a, b) __fmul_rn((a), (b))
#define GPR_FADD(a, b) __fadd_rn((a), (b))
#define GPR_FSUB(a, b) __fsub_rn((a), (b))
#define GPR_FDIV(a, b) __fdiv_rn((a), (b))
#define GPR_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define GPR_FMUL(a, b) ((float)(a) * (float)(b))
#define GPR_FADD(a, b) ((float)(a) + (float)(b))
#define GPR_FSUB(a, b) ((float)(a) - (float)(b))
#define GPR_FDIV(a, b) ((float)(a) / (float)(b))
#define GPR_FMA(a, b, c) fmaf((a), (b), (c))
#endif

GPR_HD uint32_t gpr_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
GPR_HD float gpr_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}

/* float((double)k / 1e6) for 0 <= k <= 10^6.  The correctly rounded float
 * quotient equals the double-rounded one for every k in range, and one FMA
 * correction of k * float(1e-6) equals the correctly rounded quotient for
 * every k in range (both checked exhaustively), so no division is needed. */
GPR_HD float gpr_rng_k_over_1e6(int k) {
    const float kf = (float)k;
    const float r = 9.99999997475242708e-07f;      /* float(1e-6) */
    const float q = GPR_FMUL(kf, r);
    const float e = GPR_FMA(-q, 1000000.0f, kf);
    return GPR_FMA(e, r, q);
}

/* float(6.283185307178 * (double)v), i.e. the argument the reference passes to
 * sinf in random_normal (2.0*PIf*v with PIf = 3.141592653589, main.cu:194,240).
 * Two-term split of the double constant plus an FMA error term; exact for all
 * v = k/1e6 (exhaustive). */
GPR_HD float gpr_rng_twopi_times(float v) {
    const float Dh = 6.28318548202514648f;     /* float(2*3.141592653589)      */
    const float Dl = -1.74847144734990434e-07f; /* float(2*3.141592653589 - Dh) */
    float p = GPR_FMUL(v, Dh);
    float e = GPR_FMA(v, Dh, -p);
    float t = GPR_FMA(v, Dl, e);
    return GPR_FADD(p, t);
}

/* Natural log.  x = 2^e * m with m in [sqrt(1/2), sqrt(2)];
 * log(m) = 2 atanh(t), t = (m-1)/(m+1), |t| <= 0.1716, series to t^9;
 * e*ln2 added with a two-part (Cody-Waite) ln2.  Within 2 ulp of logf. */
GPR_HD float gpr_rng_logf(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? -INFINITY : NAN;
    if (x == INFINITY) return x;
    uint32_t b = gpr_f2u(x);
    int e = 0;
    if (b < 0x00800000u) {              /* subnormal: scale by 2^23 (exact) */
        x = GPR_FMUL(x, 8388608.0f);
        b = gpr_f2u(x);
        e = -23;
    }
    e += (int)((b >> 23) & 0xffu) - 127;
    float m = gpr_u2f((b & 0x007fffffu) | 0x3f800000u);     /* [1,2) */
    if (m > 1.41421356f) { m = GPR_FMUL(m, 0.5f); e += 1; }
    float num = GPR_FSUB(m, 1.0f);                          /* exact */
    float den = GPR_FADD(m, 1.0f);
    float t = GPR_FDIV(num, den);
    float t2 = GPR_FMUL(t, t);
    float p = GPR_FMA(t2, 0.111111111f, 0.142857143f);
    p = GPR_FMA(t2, p, 0.2f);
    p = GPR_FMA(t2, p, 0.333333333f);
    p = GPR_FMUL(p, t2);
    float tt = GPR_FMUL(t, 2.0f);                           /* exact */
    float lm = GPR_FMA(tt, p, tt);
    float fe = (float)e;
    const float ln2_hi = 0.693145751953125f;                /* 13 significant bits */
    const float ln2_lo = 1.42860682030941723212e-6f;
    return GPR_FMA(fe, ln2_hi, GPR_FMA(fe, ln2_lo, lm));
}

/* sin(y), |y| < 65536: quadrant k = rint(y*2/pi), three-part pi/2 reduction
 * with FMAs, Taylor polynomials for sin and cos on |r| <= pi/4.  The proposal
 * path only calls it on [0, 2*pi).  Larger arguments return NaN (not used). */
GPR_HD float gpr_rng_sinf(float y) {
    if (!(fabsf(y) < 65536.0f)) return NAN;
    const float PIO2_1 = 1.57079637050628662109375f;
    const float PIO2_2 = -4.37113900018624283e-08f;
    const float PIO2_3 = -1.71512451000590e-15f;
    float k = rintf(GPR_FMUL(y, 0.636619772367581343f));
    float r = GPR_FMA(-k, PIO2_1, y);
    r = GPR_FMA(-k, PIO2_2, r);
    r = GPR_FMA(-k, PIO2_3, r);
    int q = ((int)k) & 3;
    float r2 = GPR_FMUL(r, r);
    float res;
    if (q & 1) {
        float c = GPR_FMA(r2, -2.75573192e-07f, 2.48015873e-05f);
        c = GPR_FMA(r2, c, -1.38888889e-03f);
        c = GPR_FMA(r2, c, 4.16666667e-02f);
        c = GPR_FMA(r2, c, -0.5f);
        res = GPR_FMA(r2, c, 1.0f);
    } else {
        float s = GPR_FMA(r2, 2.75573192e-06f, -1.98412698e-04f);
        s = GPR_FMA(r2, s, 8.33333333e-03f);
        s = GPR_FMA(r2, s, -0.166666667f);
        s = GPR_FMUL(s, r2);
        res = GPR_FMA(r, s, r);
    }
    return (q & 2) ? -res : res;
}

#endif /* GPR_RNGMATH_H */
