/* The phase-timed instantiations of the MH kernels (PROF = true) for the
 * single-dataset, one-variable, LCG layouts with heavy ops unrolled: a
 * diagnostics build that adds clock64 reads at phase boundaries
 * (gpr_debug_phase_profile).  The product kernels carry none of it. */
#include "gpr_pipe.cuh"

namespace gpr {
template __global__ void mh_block_kernel<4, true, 0, false, false, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, false, false, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, false, true, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<8, true, 0, false, false, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<8, false, 0, false, false, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, false, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, true, 1, false, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<8, true, 0, false, false, 1, false, true>(const __grid_constant__ KParams p);

static const void* pipe_prof(int K, int onepass, int rng, int stream) {
    if (rng != 0) return nullptr;
    if (K == 4 && !onepass) return stream ? (const void*)mh_pipe_kernel<4, false, 0, false, true, 1, false, true>
                                          : (const void*)mh_pipe_kernel<4, false, 0, false, false, 1, false, true>;
    if (K == 8 && onepass && !stream) return (const void*)mh_pipe_kernel<8, true, 0, false, false, 1, false, true>;
    return nullptr;
}

const void* mh_kernel_prof(int K, int onepass, int rng, int stream) {
    if (rng != 0) return nullptr;
    if (K == 4 && stream) return onepass ? nullptr : (const void*)mh_block_kernel<4, false, 0, false, true, 1, false, true>;
    if (stream) return nullptr;
    if (K == 4) return onepass ? (const void*)mh_block_kernel<4, true, 0, false, false, 1, false, true>
                               : (const void*)mh_block_kernel<4, false, 0, false, false, 1, false, true>;
    if (K == 8) return onepass ? (const void*)mh_block_kernel<8, true, 0, false, false, 1, false, true>
                               : (const void*)mh_block_kernel<8, false, 0, false, false, 1, false, true>;
    return nullptr;
}

const void* prof_kernel(const LaunchCfg& lc) {
    return lc.pipe ? pipe_prof(lc.K, lc.onepass, 0, lc.stream) : mh_kernel_prof(lc.K, lc.onepass, 0, lc.stream);
}

cudaError_t launch_mh_block_prof(const KParams& p, const LaunchCfg& lc, cudaStream_t st) {
    if (p.nv == 3 || p.nds > 0 || lc.rolled || !p.phase) return cudaErrorInvalidValue;
    const void* f = lc.pipe ? pipe_prof(lc.K, lc.onepass, p.rng_mode, lc.stream)
                            : mh_kernel_prof(lc.K, lc.onepass, p.rng_mode, lc.stream);
    if (!f) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lc.smem_bytes);
    if (e != cudaSuccess) return e;
    /* the instrumented kernel may hold more registers: size the grid for it */
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, lc.warps_per_cta * 32, lc.smem_bytes);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int dev = 0, nsm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    long long ctas = (long long)nsm * per_sm;
    const int per_cta = lc.pipe ? 2 * lc.warps_per_cta : lc.warps_per_cta;
    const long long need = (p.N + per_cta - 1) / per_cta;
    if (ctas > need) ctas = need;
    if (ctas > lc.ctas) ctas = lc.ctas;   /* p.part holds rows for lc.ctas CTAs */
    KParams pp = p;
    pp.lockstep = lc.lockstep;
    void* args[] = {(void*)&pp};
    return cudaLaunchKernel(f, dim3((unsigned)ctas), dim3(lc.warps_per_cta * 32), args, lc.smem_bytes, st);
}
}  // namespace gpr
