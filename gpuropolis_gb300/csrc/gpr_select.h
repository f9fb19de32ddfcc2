/*
 * gpr_select.h -- order-preserving keys of chain posteriors and the constant
 * scales of the initial distribution, shared by the device selection kernels
 * (gpr_resample.cu), the host library and the oracle.
 */
#ifndef GPR_SELECT_H
#define GPR_SELECT_H

#include <stdint.h>
#include <string.h>

#ifndef GPR_HD
#if defined(__CUDACC__)
#define GPR_HD __host__ __device__ __forceinline__
#else
#define GPR_HD static inline
#endif
#endif

/* Unsigned key whose order is the order of the reference's comparator
 * (main.cu:987-995): every NaN below everything else (key 0), then the IEEE
 * order of the values.  -0.0 and +0.0 get neighbouring keys; any cutoff
 * compares them alike. */
GPR_HD unsigned long long gpr_post_key(double v) {
    if (v != v) return 0ull;
    unsigned long long b;
    memcpy(&b, &v, sizeof b);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

/* The posterior a key stands for (NaN for key 0). */
GPR_HD double gpr_key_value(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    if (k == 0ull) b = 0x7ff8000000000000ull;
    double v;
    memcpy(&v, &b, sizeof v);
    return v;
}

/* powf(10, order) for the constant orders of the initial distribution,
 * C_MIN_ORDER = -4 .. C_MAX_ORDER - 1 = 3 (main.cu:30-31, 1226-1227): the
 * float nearest each power of ten. */
GPR_HD float gpr_pow10_order(int order) {
    switch (order) {
        case -4: return 1e-4f;
        case -3: return 1e-3f;
        case -2: return 1e-2f;
        case -1: return 1e-1f;
        case 0: return 1.0f;
        case 1: return 10.0f;
        case 2: return 100.0f;
        default: return 1000.0f;
    }
}

#endif /* GPR_SELECT_H */
