/*
 * gpr_fastmath.cuh -- compact FP32 exp, log and pow for the evaluator.
 *
 * Written from the textbook methods (J.-M. Muller, "Elementary Functions:
 * Algorithms and Implementation", ch. 11; W. Cody & W. Waite, "Software
 * Manual for the Elementary Functions", 1980):
 *   exp(x) = 2^n * 2^f,  n = rint(x log2 e),  f = x log2 e - n computed with a
 *            two-part log2 e (Cody-Waite), 2^f from the hardware ex2
 *            approximation (PTX ex2.approx), 2^n applied to the exponent;
 *   log(x) = e ln2 + 2 atanh(s),  x = 2^e m,  m in [sqrt(1/2), sqrt(2)),
 *            s = (m-1)/(m+1), odd series in s;
 *   pow(a,b) = 2^(b log2|a|) with log2|a| and the product b*log2|a| carried
 *            as double-float (about 44 bits), so the result keeps FP32
 *            accuracy even when b*log2|a| is large; C99 Annex F special cases.
 * Each routine is a few dozen FP32 instructions without slow paths, so the
 * interpreter can unroll it over its K points per lane: the small code keeps
 * the kernel inside the instruction cache and the unrolling gives ILP.
 * Accuracy is measured against FP64 by tests/test_gpu_math.py.
 */
#ifndef GPR_FASTMATH_CUH
#define GPR_FASTMATH_CUH

#include <math.h>
#include <stdint.h>

namespace gpr {

__device__ __forceinline__ float gx_ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float gx_rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

/* r * 2^n for r in [0.5, 2] and integer-valued n in [-200, 200]: two exact
 * power-of-two factors (each a normal float), one final rounding, which also
 * produces correctly placed subnormals and overflow to infinity. */
__device__ __forceinline__ float gx_scale2(float r, float n) {
    const int ni = (int)n;
    const int n1 = ni >> 1;
    const int n2 = ni - n1;
    return (r * __int_as_float((n1 + 127) << 23)) * __int_as_float((n2 + 127) << 23);
}

/* The routines below are branch-free: each computes its general case on a
 * sanitised argument and selects the special values afterwards, so the
 * interpreter's unrolled lanes never diverge on them. */

/* 2^t for t = th + tl (double-float), |tl| <= ulp(th) */
__device__ __forceinline__ float gx_exp2_df(float th, float tl) {
    const float thc = fminf(fmaxf(th, -200.0f), 200.0f);   /* NaN -> -200; the result is replaced */
    const float n = rintf(thc);
    const float f = (thc - n) + tl;       /* thc - n is exact */
    const float r = gx_scale2(gx_ex2_approx(f), n);
    return (th != th) ? th : (th > -200.0f ? (th < 200.0f ? r : INFINITY) : 0.0f);
}

__device__ __forceinline__ float gx_exp(float x) {
    const float L2E_HI = 1.44269502162933349609375f;      /* float(log2 e) */
    const float L2E_LO = 1.925963033500011079e-08f;       /* log2 e - L2E_HI */
    const float th = x * L2E_HI;
    const float tl = fmaf(x, L2E_HI, -th) + x * L2E_LO;    /* exact product error + low part */
    const float r = gx_exp2_df(th, tl);
    return (x != x) ? x : r;
}

/* Split x > 0 (finite) into 2^e * m, m in [sqrt(1/2), sqrt(2)). */
__device__ __forceinline__ float gx_frexp_sqrt2(float x, int& e) {
    const bool sub = __float_as_uint(x) < 0x00800000u;      /* subnormal: scale by 2^23 (exact) */
    const uint32_t b = __float_as_uint(sub ? x * 8388608.0f : x);
    e = (int)((b >> 23) & 0xffu) - 127 - (sub ? 23 : 0);
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    const bool hi = m > 1.41421356f;
    m = hi ? m * 0.5f : m;
    e += hi ? 1 : 0;
    return m;
}

__device__ __forceinline__ float gx_log(float x) {
    const bool ok = x > 0.0f && x < INFINITY;
    const float xs = ok ? x : 1.0f;
    int e;
    const float m = gx_frexp_sqrt2(xs, e);
    const float num = m - 1.0f;                       /* exact */
    const float den = m + 1.0f;
    float q = num * gx_rcp_approx(den);
    q = fmaf(fmaf(-q, den, num), gx_rcp_approx(den), q);   /* one Newton correction */
    const float s2 = q * q;
    float p = fmaf(s2, 0.1111111119f, 0.1428571343f);
    p = fmaf(s2, p, 0.2000000030f);
    p = fmaf(s2, p, 0.3333333433f);
    const float tq = 2.0f * q;
    const float lm = fmaf(tq * s2, p, tq);
    const float fe = (float)e;
    const float r = fmaf(fe, 0.693145751953125f, fmaf(fe, 1.42860682030941723212e-6f, lm));
    return ok ? r : (x > 0.0f ? x : (x == 0.0f ? -INFINITY : __int_as_float(0x7fc00000)));
}

/* log2(x) for finite x > 0 as a double-float (hi, lo). */
__device__ __forceinline__ void gx_log2_df(float x, float& hi, float& lo) {
    int e;
    const float m = gx_frexp_sqrt2(x, e);
    const float num = m - 1.0f;                       /* exact */
    /* den = m + 1 as an exact double-float */
    const float dh = m + 1.0f;
    const float dl = (1.0f - (dh - m)) + (m - (dh - (dh - m)));   /* TwoSum(m, 1) error */
    /* q = num / den in double-float: q_hi, then the residual */
    const float r0 = gx_rcp_approx(dh);
    float qh = num * r0;
    qh = fmaf(fmaf(-qh, dh, num), r0, qh);
    float res = fmaf(-qh, dh, num);                   /* num - qh*dh, exact */
    res = fmaf(-qh, dl, res);                         /* - qh*dl */
    const float ql = res * r0;
    /* ln(m) = 2q + 2q q^2 T(q^2) */
    const float s2 = qh * qh;
    float T = fmaf(s2, 0.07692307692f, 0.09090909091f);
    T = fmaf(s2, T, 0.1111111111f);
    T = fmaf(s2, T, 0.1428571429f);
    T = fmaf(s2, T, 0.2f);
    T = fmaf(s2, T, 0.3333333333f);
    const float tail = 2.0f * qh * s2 * T + 2.0f * ql;
    /* ln(m) = 2qh + tail  ->  double-float */
    const float lnh0 = 2.0f * qh;
    float lnh = lnh0 + tail;
    float lnl = tail - (lnh - lnh0);
    /* times log2(e) = L_hi + L_lo */
    const float L_HI = 1.44269502162933349609375f;
    const float L_LO = 1.925963033500011079e-08f;
    float ph = lnh * L_HI;
    float pl = fmaf(lnh, L_HI, -ph);
    pl = fmaf(lnh, L_LO, fmaf(lnl, L_HI, pl));
    /* + e (exact integer) */
    const float fe = (float)e;
    const float sh = fe + ph;
    const float bv = sh - fe;
    const float sl = (fe - (sh - bv)) + (ph - bv) + pl;
    hi = sh + sl;
    lo = sl - (hi - sh);
}

__device__ __forceinline__ float gx_pow(float a, float b) {
    const float fa = fabsf(a);
    const bool b_int = (truncf(b) == b);
    const bool b_odd = b_int && fabsf(b) < 16777216.0f && (((int)b) & 1);
    /* the general case, 2^(b log2|a|), on a finite nonzero |a| and a finite b */
    const bool gen = fa > 0.0f && fa < INFINITY;
    const float fs = gen ? fa : 1.0f;
    const float bs = isfinite(b) ? b : 0.0f;
    float lh, ll;
    gx_log2_df(fs, lh, ll);
    const float th = bs * lh;
    const float tl = fmaf(bs, lh, -th) + bs * ll;
    float r = gx_exp2_df(th, tl);
    /* C99 Annex F special values, in order of precedence (the last select wins) */
    r = (fa == 0.0f) ? ((b < 0.0f) ? INFINITY : 0.0f) : (fa == INFINITY ? ((b < 0.0f) ? 0.0f : INFINITY) : r);
    r = ((a < 0.0f || (a == 0.0f && __float_as_uint(a) != 0u)) && b_odd) ? -r : r;
    r = (gen && a < 0.0f && !b_int) ? __int_as_float(0x7fc00000) : r;
    r = isinf(b) ? (fa == 1.0f ? 1.0f : (((fa < 1.0f) == (b < 0.0f)) ? INFINITY : 0.0f)) : r;
    r = (a != a || b != b) ? a + b : r;                /* NaN */
    return (b == 0.0f || a == 1.0f) ? 1.0f : r;
}

}  // namespace gpr

#endif /* GPR_FASTMATH_CUH */
