/* Instantiations of the pipelined MH kernel for three input variables (K = 4
 * in passes, staged or streamed; a translation unit of its own so the
 * kernels compile in parallel). */
#include "gpr_pipe.cuh"

namespace gpr {
template __global__ void mh_pipe_kernel<4, false, 0, false, false, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, false, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, true, 3, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, true, 3, false>(const __grid_constant__ KParams p);
const void* pipe_kernel_k4v(int rng, int rolled, int stream) {
    if (rolled) return nullptr;
    if (stream) return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, true, 3, false>
                           : (const void*)mh_pipe_kernel<4, false, 0, false, true, 3, false>;
    return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, false, 3, false>
               : (const void*)mh_pipe_kernel<4, false, 0, false, false, 3, false>;
}
}  // namespace gpr
