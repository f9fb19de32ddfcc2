/* Instantiations of the pipelined MH kernel, one input variable, K = 8
 * points per lane, data staged: in registers (one pass) or in passes (a
 * translation unit of its own so the kernels compile in parallel). */
#include "gpr_pipe.cuh"

namespace gpr {
template __global__ void mh_pipe_kernel<8, true, 0, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<8, true, 1, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<8, false, 0, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<8, false, 1, false, false, 1, false>(const __grid_constant__ KParams p);
const void* pipe_kernel_k8(int rng, int rolled, int onepass) {
    if (rolled) return nullptr;
    if (onepass) return rng ? (const void*)mh_pipe_kernel<8, true, 1, false, false, 1, false>
                            : (const void*)mh_pipe_kernel<8, true, 0, false, false, 1, false>;
    return rng ? (const void*)mh_pipe_kernel<8, false, 1, false, false, 1, false>
               : (const void*)mh_pipe_kernel<8, false, 0, false, false, 1, false>;
}
}  // namespace gpr
