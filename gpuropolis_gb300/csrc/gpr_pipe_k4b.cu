/* Instantiations of the pipelined MH kernel for batched datasets, one or
 * three input variables (K = 4 in passes, staged per chain group or streamed;
 * a translation unit of its own so the kernels compile in parallel). */
#include "gpr_pipe.cuh"

namespace gpr {
template __global__ void mh_pipe_kernel<4, false, 0, false, false, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, false, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, true, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, true, 1, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, false, 3, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, false, 3, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 0, false, true, 3, true>(const __grid_constant__ KParams p);
template __global__ void mh_pipe_kernel<4, false, 1, false, true, 3, true>(const __grid_constant__ KParams p);
const void* pipe_kernel_k4b(int rng, int rolled, int stream, int nv) {
    if (rolled) return nullptr;
    if (nv == 3) {
        if (stream) return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, true, 3, true>
                               : (const void*)mh_pipe_kernel<4, false, 0, false, true, 3, true>;
        return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, false, 3, true>
                   : (const void*)mh_pipe_kernel<4, false, 0, false, false, 3, true>;
    }
    if (stream) return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, true, 1, true>
                           : (const void*)mh_pipe_kernel<4, false, 0, false, true, 1, true>;
    return rng ? (const void*)mh_pipe_kernel<4, false, 1, false, false, 1, true>
               : (const void*)mh_pipe_kernel<4, false, 0, false, false, 1, true>;
}
}  // namespace gpr
