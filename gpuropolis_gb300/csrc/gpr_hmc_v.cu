/*
 * gpr_hmc_v.cu -- the adjoint and Hamiltonian-move kernels for data with three
 * input variables (x1, x2, x3); a translation unit of its own so that they
 * compile in parallel with the univariate ones (gpr_hmc.cu).
 */
#include "gpr_hmc.cuh"

namespace gpr {

const void* grad_kernel_v3(int maxi, int stream) {
    if (maxi <= 130)
        return stream ? (const void*)loglik_grad_kernel<GPR_HMC_K, 130, true, 3>
                      : (const void*)loglik_grad_kernel<GPR_HMC_K, 130, false, 3>;
    return stream ? (const void*)loglik_grad_kernel<GPR_HMC_K, 258, true, 3>
                  : (const void*)loglik_grad_kernel<GPR_HMC_K, 258, false, 3>;
}

template <int MAXI, int RNG>
static const void* pick(int stream) {
    return stream ? (const void*)mh_hmc_kernel<GPR_HMC_K, MAXI, RNG, true, 3>
                  : (const void*)mh_hmc_kernel<GPR_HMC_K, MAXI, RNG, false, 3>;
}

const void* hmc_kernel_v3(const KParams& p, int stream) {
    if (p.max_instr <= 130) return p.rng_mode ? pick<130, 1>(stream) : pick<130, 0>(stream);
    return p.rng_mode ? pick<258, 1>(stream) : pick<258, 0>(stream);
}

}  // namespace gpr
