/* Instantiations of the pipelined MH kernel, one input variable, K = 4
 * points per lane: data in registers (one pass), staged in passes, or
 * streamed from device memory (a translation unit of its own so the kernels
 * compile in parallel). */
#include "gpr_pipe.cuh"

namespace gpr {
template __global__ void mh_pipe_kernel<4, true, 0, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, true, 1, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, false, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, true, 1, false>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, true, 1, false>(const __grid_constant__ KParams p);
const void* pipe_kernel_k4(int rng, int rolled, int onepass, int stream) {
    if (rolled) return nullptr;
    if (stream) {
        if (onepass) return nullptr;
        return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, true, 1, false>
                   : (const void*)mh_pipe_kernel<4, false, 0, false, true, 1, false>;
    }
    if (onepass) return rng ? (const void*)mh_pipe_kernel<4, true, 1, false, false, 1, false>
                            : (const void*)mh_pipe_kernel<4, true, 0, false, false, 1, false>;
    return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, false, 1, false>
               : (const void*)mh_pipe_kernel<4, false, 0, false, false, 1, false>;
}
}  // namespace gpr
