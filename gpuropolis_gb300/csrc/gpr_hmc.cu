/*
 * gpr_hmc.cu -- instantiations and launchers of the adjoint kernel
 * (gpr_loglik_grad) and of the MH kernel with Hamiltonian constant moves
 * (gpr_hmc.cuh).
 */
#include "gpr_hmc.cuh"

namespace gpr {

#define GPR_HMC_K 1

size_t grad_smem_bytes(const KParams& p, int warps_per_cta) {
    return 16 + align16((size_t)3 * p.nd_pad * 4) +
           (size_t)warps_per_cta * grad_warp_bytes(p.PL, p.max_instr, p.levels, GPR_HMC_K);
}

cudaError_t launch_loglik_grad(const KParams& p, double* grad, double* lik, cudaStream_t st) {
    const int wpc = 4;
    const size_t smem = grad_smem_bytes(p, wpc);
    const void* f = (const void*)loglik_grad_kernel<GPR_HMC_K>;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    loglik_grad_kernel<GPR_HMC_K><<<(p.N + wpc - 1) / wpc, wpc * 32, smem, st>>>(p, grad, lik);
    return cudaGetLastError();
}

static const void* hmc_kernel(int rng) {
    return rng ? (const void*)mh_hmc_kernel<GPR_HMC_K, 1> : (const void*)mh_hmc_kernel<GPR_HMC_K, 0>;
}

cudaError_t hmc_occupancy(const KParams& p, int warps_per_cta, size_t smem, int* ctas_per_sm) {
    const void* f = hmc_kernel(p.rng_mode);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, f, warps_per_cta * 32, smem);
}

cudaError_t launch_hmc_block(const KParams& p, const LaunchCfg& lc, cudaStream_t st) {
    const void* f = hmc_kernel(p.rng_mode);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lc.smem_bytes);
    if (e != cudaSuccess) return e;
    KParams pp = p;
    void* args[] = {(void*)&pp};
    return cudaLaunchKernel(f, dim3(lc.ctas), dim3(lc.warps_per_cta * 32), args, lc.smem_bytes, st);
}

}  // namespace gpr
