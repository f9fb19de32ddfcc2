/*
 * ref_shim.h -- lets the reference's main.cu compile as host C++ (g++) so the
 * reference's own per-chain code can serve as the parity oracle and as the
 * CPU baseline.  TEST INFRASTRUCTURE ONLY: nothing in the product includes it.
 *
 * build_ref.py writes a substituted copy of main.cu into oracle/_ref/src/ whose
 * line 12 (#include <cuda_runtime.h>) includes this file instead.  It provides:
 *   - empty __device__/__host__/__global__ qualifiers and a per-thread
 *     threadIdx/blockIdx/blockDim, so MH_simple_kernel (main.cu:679) runs as a
 *     plain function once per chain, the chains spread over OpenMP threads;
 *   - fdividef and the CUDART_* constants of math_constants.h (main.cu:17);
 *   - the handful of CUDA runtime calls main() makes (main.cu:1037-1051,
 *     1123-1147, 1163-1167, 1233-1234, 1251-1254) as host memory operations;
 *   - the RNG hooks used by the substituted lines: GPR_RNG_T / GPR_RNG_SEED
 *     (main.cu:207,691), the Philox stream (main.cu:215), the op-set map
 *     GPR_OPMAP / GPR_NOPS (main.cu:536,718,1133,1225).
 *
 * Compile-time knobs (all -D):
 *   GPR_REF_PL            program length (default 31, main.cu:26-27)
 *   GPR_REF_OPSET         0 = the reference's 27 ops, 1 = {CONST,A,B,+,-,*,/,log,exp,pow}
 *   GPR_REF_PHILOX        0 = reference LCG (main.cu:213-216), 1 = Philox stream
 *   GPR_REF_PROJECT_MATH  1 = logf/sinf inside random_normal/random_geometric
 *                         come from gpr_rngmath.h (bit-identical to the device)
 *   GPR_REF_RW, _RW_SD    1: constant moves are C += sd*N(0,1) (the dead
 *                         branch of main.cu:779-784 made live, P_PROPOSE_C_GEOMETRIC=0)
 *   GPR_REF_MAPD, _MAP_DELTA  1: resample chains below (max posterior - delta)
 *                         instead of the median (main.cu:1219)
 */
#ifndef GPR_REF_SHIM_H
#define GPR_REF_SHIM_H

/* System headers first: the reference defines a function-like `max` macro
 * (main.cu:186) that would break libstdc++ headers included after it. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <cmath>
#include <vector>
#include <string>
#include <iostream>
#include <algorithm>
#include <chrono>
#include <omp.h>

#include "../gpuropolis_gb300/csrc/gpr_rngmath.h"
#include "../gpuropolis_gb300/csrc/gpr_philox.h"

#ifndef GPR_REF_PL
#define GPR_REF_PL 31
#endif
#ifndef GPR_REF_OPSET
#define GPR_REF_OPSET 0
#endif
#ifndef GPR_REF_PHILOX
#define GPR_REF_PHILOX 0
#endif
#ifndef GPR_REF_PROJECT_MATH
#define GPR_REF_PROJECT_MATH 0
#endif
#ifndef GPR_REF_RW
#define GPR_REF_RW 0
#endif
#ifndef GPR_REF_RW_SD
#define GPR_REF_RW_SD 0.0
#endif
#ifndef GPR_REF_MAPD
#define GPR_REF_MAPD 0
#endif
#ifndef GPR_REF_MAP_DELTA
#define GPR_REF_MAP_DELTA 0.0
#endif

#if GPR_REF_RW
#define GPR_REF_P_GEOM 0.0
#else
#define GPR_REF_P_GEOM 1.0
#endif

/* ---- CUDA qualifiers and thread indices -------------------------------- */
#define __device__
#define __host__
#define __global__
struct gpr_ref_dim { unsigned int x, y, z; };
static thread_local gpr_ref_dim threadIdx = {0, 0, 0};
static thread_local gpr_ref_dim blockIdx = {0, 0, 0};
static thread_local gpr_ref_dim blockDim = {1, 1, 1};

static inline float fdividef(float a, float b) { return a / b; }
#define CUDART_NAN_F NAN
#define CUDART_INF_F INFINITY

/* ---- CUDA runtime calls used by main() ---------------------------------- */
typedef enum { cudaSuccess = 0 } cudaError_t;
typedef enum { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 } cudaMemcpyKind;
static inline cudaError_t cudaGetLastError(void) { return cudaSuccess; }
static inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }
static inline cudaError_t cudaGetDeviceCount(int* n) { *n = 1; return cudaSuccess; }
static inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
static inline cudaError_t cudaGetDevice(int* d) { *d = 0; return cudaSuccess; }
static inline cudaError_t cudaDeviceReset(void) { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
static inline cudaError_t cudaMallocHost(void** p, size_t n) { *p = malloc(n ? n : 1); return cudaSuccess; }
static inline cudaError_t cudaMalloc(void** p, size_t n) { *p = malloc(n ? n : 1); return cudaSuccess; }
static inline cudaError_t cudaFreeHost(void* p) { free(p); return cudaSuccess; }
static inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    if (n) memcpy(d, s, n);
    return cudaSuccess;
}

/* ---- RNG hooks ----------------------------------------------------------- */
#if GPR_REF_PHILOX
#define GPR_RNG_T gpr_philox_stream
#define GPR_RNG_SEED(rx, s, i) gpr_philox_stream_init(&(rx), (uint32_t)(s), (uint32_t)(i))
static inline int gpr_ref_philox_next(gpr_philox_stream& s) { return gpr_philox_stream_next(&s); }
#else
#define GPR_RNG_T int
#define GPR_RNG_SEED(rx, s, i) ((rx) = (s) + (i))
#endif

/* ---- op sets: index drawn by random_int -> op code of the reference enum -- */
#if GPR_REF_OPSET == 1
/* CONST, A, B, PLUS, MINUS, TIMES, DIV, LOG, EXP, POW in main.cu:53 numbering */
static const int gpr_ref_opmap_table[10] = {1, 3, 4, 5, 6, 9, 11, 13, 14, 15};
#define GPR_NOPS 10
#define GPR_OPMAP(k) (gpr_ref_opmap_table[(k)])
#else
#define GPR_NOPS NOPS
#define GPR_OPMAP(k) (k)
#endif

#endif /* GPR_REF_SHIM_H */
