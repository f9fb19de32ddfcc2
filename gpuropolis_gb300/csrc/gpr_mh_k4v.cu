/* Instantiations of the MH block kernel for data with three input variables
 * (x1, x2, x3): K = 4 points per lane in passes, dataset staged or streamed
 * (a translation unit of its own so the kernels compile in parallel). */
#include "gpr_mh.cuh"

namespace gpr {
template __global__ void mh_block_kernel<4, false, 0, false, false, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, false, false, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, true, false, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, true, false, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, false, true, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, false, true, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, true, true, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, true, true, 3, false>(const __grid_constant__ KParams p);
const void* mh_kernel_k4v(int rng, int rolled, int stream) {
    if (stream) {
        if (rolled) return rng ? (const void*)mh_block_kernel<4, false, 1, true, true, 3, false> : (const void*)mh_block_kernel<4, false, 0, true, true, 3, false>;
        return rng ? (const void*)mh_block_kernel<4, false, 1, false, true, 3, false> : (const void*)mh_block_kernel<4, false, 0, false, true, 3, false>;
    }
    if (rolled) return rng ? (const void*)mh_block_kernel<4, false, 1, true, false, 3, false> : (const void*)mh_block_kernel<4, false, 0, true, false, 3, false>;
    return rng ? (const void*)mh_block_kernel<4, false, 1, false, false, 3, false> : (const void*)mh_block_kernel<4, false, 0, false, false, 3, false>;
}
}  // namespace gpr
