/*
 * gpr_resample.cu -- selection over chain posteriors on the device.
 *
 *  - the resampling cutoff of main.cu:1215-1219 (the posterior at rank
 *    (int)(N * quantile) in the order of the reference's comparator,
 *    main.cu:987-995) or max - delta, by radix selection instead of qsort;
 *  - the re-draw of every chain strictly below the cutoff from the initial
 *    distribution (main.cu:1221-1229), driven by a counter-based stream per
 *    chain instead of the host's rand();
 *  - the candidate list of the k best chains, which replaces the external
 *    `sort -g -k3 samples.txt | tail -n k` behind tops.txt (run-all.sh:45).
 *
 * This is integer and byte work over N doubles (1 MB at 131,072 chains): one
 * pass writes an order-preserving 64-bit key per chain, one CTA radix-selects
 * over the keys (8 passes of 8 bits, L2-resident), and one thread per chain
 * re-draws or collects.
 */
#include "gpr_mh.cuh"
#include "gpr_select.h"

namespace gpr {

__global__ void post_key_kernel(const double* prior, const double* lik, int N, unsigned long long* keys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        keys[i] = gpr_post_key(prior[i] + lik[i]);
}

/* The key of rank `rank` (0-based, ascending) among keys[0..N) of segment
 * blockIdx.x (keys + blockIdx.x * N; one segment per dataset of a batched
 * handle), into out[blockIdx.x].  One CTA per segment: per 8-bit digit, a
 * shared histogram of the keys that match the digits fixed so far, then warp
 * 0 finds the bin that holds the rank. */
__global__ void __launch_bounds__(1024) select_rank_kernel(const unsigned long long* keys, int N, int rank,
                                                           unsigned long long* out) {
    keys += (size_t)blockIdx.x * (size_t)N;
    out += blockIdx.x;
    __shared__ unsigned int hist[256];
    __shared__ unsigned long long s_prefix;
    __shared__ int s_rank;
    unsigned long long prefix = 0ull, mask = 0ull;
    int r = rank;
#pragma unroll 1
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const unsigned long long k = keys[i];
            if ((k & mask) == prefix) atomicAdd(&hist[(unsigned)(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            unsigned c[8];
            unsigned s = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) { c[j] = hist[lane * 8 + j]; s += c[j]; }
            unsigned incl = s;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned t = __shfl_up_sync(FULLMASK, incl, o);
                if (lane >= o) incl += t;
            }
            const unsigned excl = incl - s;
            if (excl <= (unsigned)r && (unsigned)r < incl) {
                unsigned cum = excl;
#pragma unroll 1
                for (int j = 0; j < 8; ++j) {
                    if ((unsigned)r < cum + c[j]) {
                        s_prefix = prefix | ((unsigned long long)(lane * 8 + j) << shift);
                        s_rank = r - (int)cum;
                        break;
                    }
                    cum += c[j];
                }
            }
        }
        __syncthreads();
        prefix = s_prefix;
        r = s_rank;
        mask |= 0xffull << shift;
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = prefix;
}

/* Re-draw chains whose posterior is strictly below the cutoff, in the
 * reference's order (all PL ops, then all PL constants; main.cu:1224-1228):
 * op = ops[random_int(n_ops - 1)], constant = 10^(random_int(8) - 4) *
 * random_normal().  Draws come from the Philox stream keyed by
 * (seed, (chain + chain_offset) | 2^31): with the offset of a handle's first
 * chain in a population spread over several handles or GPUs, every chain of
 * the population has its own stream.  seg_len > 0: chain c compares with the cutoff of
 * its segment, sel_key[c / seg_len]. */
__global__ void redraw_kernel(const __grid_constant__ KParams p, const unsigned long long* sel_key, int seg_len,
                              int map_delta, double delta, uint32_t seed, uint32_t chain_offset, Magic mag_ops1,
                              Magic mag_order, int* n_redrawn) {
    const int chain = blockIdx.x * blockDim.x + threadIdx.x;
    if (chain >= p.N) return;
    double cutoff = gpr_key_value(sel_key[seg_len > 0 ? chain / seg_len : 0]);
    if (map_delta) cutoff -= delta;
    if (!(p.prior[chain] + p.lik[chain] < cutoff)) return;
    Rng r;
    r.s = 0u; r.key0 = seed; r.key1 = ((uint32_t)chain + chain_offset) | 0x80000000u; r.blk = 0xffffffffu; r.drawn = 0u;
    r.w0 = r.w1 = r.w2 = r.w3 = 0u;
    const size_t N = (size_t)p.N;
#pragma unroll 1
    for (int i = 0; i < p.PL; ++i) p.P[(size_t)i * N + chain] = p.opmap[random_int<1>(r, p.nops - 1, mag_ops1)];
#pragma unroll 1
    for (int i = 0; i < p.PL; ++i) {
        const int order = random_int<1>(r, 8, mag_order) - 4;
        p.C[(size_t)i * N + chain] = __fmul_rn(gpr_pow10_order(order), random_normal<1>(r, p));
    }
    atomicAdd(n_redrawn, 1);
}

/* Chains whose key is >= kmin (NaN never), appended in any order. */
__global__ void collect_kernel(const unsigned long long* keys, int N, unsigned long long kmin, int* out, int cap,
                               int* count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        if (k != 0ull && k >= kmin) {
            const int j = atomicAdd(count, 1);
            if (j < cap) out[j] = i;
        }
    }
}

/* The smallest chain whose key equals *k. */
__global__ void first_index_kernel(const unsigned long long* keys, int N, const unsigned long long* k, int* out) {
    const unsigned long long want = *k;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        if (keys[i] == want) atomicMin(out, i);
}

static int grid_for(int n, int threads) {
    int b = (n + threads - 1) / threads;
    return b < 1 ? 1 : (b > 4096 ? 4096 : b);
}

cudaError_t launch_select(const KParams& p, int rank, unsigned long long* keys, unsigned long long* out,
                          cudaStream_t st, int segments) {
    if (segments < 1 || p.N % segments) return cudaErrorInvalidValue;
    post_key_kernel<<<grid_for(p.N, 256), 256, 0, st>>>(p.prior, p.lik, p.N, keys);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    select_rank_kernel<<<segments, 1024, 0, st>>>(keys, p.N / segments, rank, out);
    return cudaGetLastError();
}

cudaError_t launch_redraw(const KParams& p, const unsigned long long* sel_key, int seg_len, int map_delta,
                          double delta, uint32_t seed, Magic mag_ops1, Magic mag_order, int* n_redrawn,
                          cudaStream_t st, uint32_t chain_offset) {
    redraw_kernel<<<(p.N + 127) / 128, 128, 0, st>>>(p, sel_key, seg_len, map_delta, delta, seed, chain_offset,
                                                       mag_ops1, mag_order, n_redrawn);
    return cudaGetLastError();
}

cudaError_t launch_collect(const unsigned long long* keys, int N, unsigned long long kmin, int* out, int cap,
                           int* count, cudaStream_t st) {
    collect_kernel<<<grid_for(N, 256), 256, 0, st>>>(keys, N, kmin, out, cap, count);
    return cudaGetLastError();
}

cudaError_t launch_first_index(const unsigned long long* keys, int N, const unsigned long long* k, int* out,
                               cudaStream_t st) {
    first_index_kernel<<<grid_for(N, 256), 256, 0, st>>>(keys, N, k, out);
    return cudaGetLastError();
}

}  // namespace gpr
