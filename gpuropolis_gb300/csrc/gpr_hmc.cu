/*
 * gpr_hmc.cu -- instantiations and launchers of the adjoint kernel
 * (gpr_loglik_grad) and of the MH kernel with Hamiltonian constant moves
 * (gpr_hmc.cuh).  Four points per lane; the thread-local tape holds up to
 * 130 instructions (PROGRAM_LENGTH <= 63) or 258 (PROGRAM_LENGTH <= 127); the
 * dataset is staged per CTA or, when too large, read from device memory.
 */
#include "gpr_hmc.cuh"

namespace gpr {


size_t grad_smem_bytes(const KParams& p, int warps_per_cta, int stream) {
    return 16 + (stream ? 0 : align16((size_t)data_arrays(p) * p.nd_pad * 4)) +
           (size_t)warps_per_cta * grad_warp_bytes(p.PL, p.max_instr);
}

bool grad_supported(const KParams& p) { return p.max_instr <= 258 && p.levels <= GPR_ASTK_MAX; }

template <int MAXI, int NV>
static const void* grad_kernel_nv(int stream) {
    return stream ? (const void*)loglik_grad_kernel<GPR_HMC_K, MAXI, true, NV>
                  : (const void*)loglik_grad_kernel<GPR_HMC_K, MAXI, false, NV>;
}

template <int MAXI>
static const void* grad_kernel_t(int stream, int nv) {
    return nv == 3 ? grad_kernel_v3(MAXI, stream) : grad_kernel_nv<MAXI, 1>(stream);
}

cudaError_t launch_loglik_grad(const KParams& p, double* grad, double* lik, int stream, cudaStream_t st) {
    if (!grad_supported(p)) return cudaErrorInvalidValue;
    if (p.nds > 0) stream = 1;   /* batched data are read per chain from device memory */
    const int wpc = 4;
    const size_t smem = grad_smem_bytes(p, wpc, stream);
    const void* f = p.max_instr <= 130 ? grad_kernel_t<130>(stream, p.nv) : grad_kernel_t<258>(stream, p.nv);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    KParams pp = p;
    void* args[] = {(void*)&pp, (void*)&grad, (void*)&lik};
    return cudaLaunchKernel(f, dim3((p.N + wpc - 1) / wpc), dim3(wpc * 32), args, smem, st);
}

template <int MAXI, int RNG, int NV>
static const void* hmc_kernel_t(int stream) {
    return stream ? (const void*)mh_hmc_kernel<GPR_HMC_K, MAXI, RNG, true, NV>
                  : (const void*)mh_hmc_kernel<GPR_HMC_K, MAXI, RNG, false, NV>;
}

static const void* hmc_kernel(const KParams& p, int stream) {
    if (p.nv == 3) return hmc_kernel_v3(p, stream);
    if (p.max_instr <= 130) return p.rng_mode ? hmc_kernel_t<130, 1, 1>(stream) : hmc_kernel_t<130, 0, 1>(stream);
    return p.rng_mode ? hmc_kernel_t<258, 1, 1>(stream) : hmc_kernel_t<258, 0, 1>(stream);
}

/* The shared-memory share of the L1/shared array: the rest is L1, where the
 * thread-local tapes live.  carveout 0 leaves the driver's default. */
static cudaError_t set_carveout(const void* f, int carveout) {
    return cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
                                carveout > 0 ? carveout : -1);
}

cudaError_t hmc_occupancy(const KParams& p, int warps_per_cta, size_t smem, int carveout, int stream,
                          int* ctas_per_sm) {
    if (!grad_supported(p)) return cudaErrorInvalidValue;
    const void* f = hmc_kernel(p, stream);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = set_carveout(f, carveout);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, f, warps_per_cta * 32, smem);
}

cudaError_t launch_hmc_block(const KParams& p, const LaunchCfg& lc, cudaStream_t st) {
    if (!grad_supported(p) || (p.nds > 0 && !lc.stream)) return cudaErrorInvalidValue;
    const void* f = hmc_kernel(p, lc.stream);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lc.smem_bytes);
    if (e == cudaSuccess) e = set_carveout(f, lc.carveout);
    if (e != cudaSuccess) return e;
    KParams pp = p;
    void* args[] = {(void*)&pp};
    return cudaLaunchKernel(f, dim3(lc.ctas), dim3(lc.warps_per_cta * 32), args, lc.smem_bytes, st);
}

}  // namespace gpr
