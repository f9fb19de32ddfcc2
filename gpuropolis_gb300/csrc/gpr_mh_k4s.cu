/* Instantiations of the MH block kernel that read the dataset from device
 * memory instead of staging it (K = 4 points per lane, in passes): the layout
 * for datasets too large for shared memory (a translation unit of its own so
 * the kernels compile in parallel). */
#include "gpr_mh.cuh"

namespace gpr {
template __global__ void mh_block_kernel<4, false, 0, false, true, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, false, true, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, true, true, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, true, true, 1, false>(const __grid_constant__ KParams p);
const void* mh_kernel_k4s(int rng, int rolled) {
    if (rolled) return rng ? (const void*)mh_block_kernel<4, false, 1, true, true, 1, false> : (const void*)mh_block_kernel<4, false, 0, true, true, 1, false>;
    return rng ? (const void*)mh_block_kernel<4, false, 1, false, true, 1, false> : (const void*)mh_block_kernel<4, false, 0, false, true, 1, false>;
}
}  // namespace gpr
