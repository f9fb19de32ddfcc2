/* Instantiations of the MH block kernel for K = 8 points per lane, dataset read from shared memory in passes
 * (a translation unit of its own so the kernels compile in parallel). */
#include "gpr_mh.cuh"

namespace gpr {
template __global__ void mh_block_kernel<8, false, 0, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<8, false, 1, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<8, false, 0, true, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<8, false, 1, true, false, 1, false>(const __grid_constant__ KParams p);
const void* mh_kernel_k8m(int rng, int rolled) {
    if (rolled) return rng ? (const void*)mh_block_kernel<8, false, 1, true, false, 1, false> : (const void*)mh_block_kernel<8, false, 0, true, false, 1, false>;
    return rng ? (const void*)mh_block_kernel<8, false, 1, false, false, 1, false> : (const void*)mh_block_kernel<8, false, 0, false, false, 1, false>;
}
}  // namespace gpr
