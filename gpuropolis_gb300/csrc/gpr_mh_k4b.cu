/* Instantiations of the MH block kernel for batched data (one input variable): many
 * datasets in one launch, K = 4 points per lane in passes, each chain group's
 * dataset staged per group or streamed (a translation unit of its own so the
 * kernels compile in parallel). */
#include "gpr_mh.cuh"

namespace gpr {
template __global__ void mh_block_kernel<4, false, 0, false, false, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, false, false, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, true, false, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, true, false, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, false, true, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, false, true, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 0, true, true, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_block_kernel<4, false, 1, true, true, 1, true>(const __grid_constant__ KParams p);
const void* mh_kernel_k4b(int rng, int rolled, int stream) {
    if (stream) {
        if (rolled) return rng ? (const void*)mh_block_kernel<4, false, 1, true, true, 1, true> : (const void*)mh_block_kernel<4, false, 0, true, true, 1, true>;
        return rng ? (const void*)mh_block_kernel<4, false, 1, false, true, 1, true> : (const void*)mh_block_kernel<4, false, 0, false, true, 1, true>;
    }
    if (rolled) return rng ? (const void*)mh_block_kernel<4, false, 1, true, false, 1, true> : (const void*)mh_block_kernel<4, false, 0, true, false, 1, true>;
    return rng ? (const void*)mh_block_kernel<4, false, 1, false, false, 1, true> : (const void*)mh_block_kernel<4, false, 0, false, false, 1, true>;
}
}  // namespace gpr
