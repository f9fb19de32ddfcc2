/*
 * gpr_kernels.cu -- host-side launch helpers of the MH block kernels
 * (gpr_mh.cuh, instantiated in gpr_mh_k*.cu) and the diagnostics kernel that
 * evaluates compiled programs point by point for the parity tests.
 */
#include "gpr_pipe.cuh"

namespace gpr {

/* ------------------------------------------------------------------------ */
size_t mh_smem_bytes(const KParams& p, int K, int warps_per_cta, int stream) {
    return 16 + (stream ? 0 : align16((size_t)data_arrays(p) * p.nd_pad * 4)) +
           (size_t)warps_per_cta * warp_smem_bytes(p.PL, p.max_instr, p.levels, K);
}

int pipe_part_stride(int nd) {
    const int nch = (nd + GPR_CHUNK_POINTS - 1) / GPR_CHUNK_POINTS;
    return nch <= GPR_PIPE_CHUNKS ? 0 : nch;
}

size_t pipe_smem_bytes(const KParams& p, int K, int warps_per_cta, int stream) {
    return 16 + (stream ? 0 : align16((size_t)data_arrays(p) * p.nd_pad * 4)) +
           (size_t)warps_per_cta * pipe_warp_bytes(p.PL, p.max_instr, p.levels, K) +
           (pipe_part_stride(p.nd) == 0 ? pipe_board_bytes() : 0);
}

static const void* pick_pipe(int K, int onepass, int rng, int rolled, int stream, int nv, int batched) {
    if (batched) return (K == 4 && !onepass) ? pipe_kernel_k4b(rng, rolled, stream, nv) : nullptr;
    if (nv == 3) return (K == 4 && !onepass) ? pipe_kernel_k4v(rng, rolled, stream) : nullptr;
    if (K == 4) return pipe_kernel_k4(rng, rolled, onepass, stream);
    if (K == 8) return stream ? nullptr : pipe_kernel_k8(rng, rolled, onepass);
    return nullptr;
}

static const void* pick_kernel(int K, int onepass, int rng, int rolled, int stream, int nv, int batched, int pipe) {
    if (pipe) return pick_pipe(K, onepass, rng, rolled, stream, nv, batched);
    if (batched) {
        if (K != 4 || onepass) return nullptr;
        return nv == 3 ? mh_kernel_k4bv(rng, rolled, stream) : mh_kernel_k4b(rng, rolled, stream);
    }
    if (nv == 3) return (K == 4 && !onepass) ? mh_kernel_k4v(rng, rolled, stream) : nullptr;
    if (stream) return (K == 4 && !onepass) ? mh_kernel_k4s(rng, rolled) : nullptr;
    if (K == 4) return onepass ? mh_kernel_k4(rng, rolled) : mh_kernel_k4m(rng, rolled);
    if (K == 8) return onepass ? mh_kernel_k8(rng, rolled) : mh_kernel_k8m(rng, rolled);
    return nullptr;
}

void fill_lcg_jump_table(KParams& p) {
    uint32_t a = 1103515245u, c = 12345u;
    for (int b = 0; b < 20; ++b) {
        p.lcgA[b] = a; p.lcgC[b] = c;
        c = a * c + c;   /* the map composed with itself: 2^(b+1) steps */
        a = a * a;
    }
}

cudaError_t mh_occupancy(const KParams& p, const LaunchCfg& lc, int* ctas_per_sm) {
    const void* f = pick_kernel(lc.K, lc.onepass, p.rng_mode, lc.rolled, lc.stream, p.nv, p.nds > 0, lc.pipe);
    if (!f) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lc.smem_bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, f, lc.warps_per_cta * 32, lc.smem_bytes);
}

cudaError_t launch_mh_block(const KParams& p, const LaunchCfg& lc, cudaStream_t st) {
    const void* f = pick_kernel(lc.K, lc.onepass, p.rng_mode, lc.rolled, lc.stream, p.nv, p.nds > 0, lc.pipe);
    if (!f) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lc.smem_bytes);
    if (e != cudaSuccess) return e;
    KParams pp = p;
    pp.lockstep = lc.lockstep;
    void* args[] = {(void*)&pp};
    return cudaLaunchKernel(f, dim3(lc.ctas), dim3(lc.warps_per_cta * 32), args, lc.smem_bytes, st);
}

/* ------------------------------------------------------------------------ */
/* Diagnostics kernel: one warp per chain, values of the compiled program at
 * nx points, plus its length and node count. */
__global__ void __launch_bounds__(128) eval_values_kernel(const __grid_constant__ KParams p, const float* xs, int nx,
                                                          float* out, float* length, int* count) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const size_t wbytes = warp_smem_bytes(p.PL, p.max_instr, p.levels, 1);
    WarpSmem ws = carve_warp<1>(smem + (size_t)warp * wbytes, p.PL, p.max_instr, p.levels);
    const int chain = blockIdx.x * (blockDim.x >> 5) + warp;
    if (chain >= p.N) return;
    for (int i = lane; i < p.PL; i += 32) {
        int o = p.P[(size_t)i * p.N + chain];
        ws.ops[0][i] = (uint8_t)((o >= 0 && o < OP_NALL) ? o : 255);
        ws.Cs[0][i] = p.C[(size_t)i * p.N + chain];
    }
    __syncwarp();
    CompileOut co = compile_parallel<3>(ws.ops[0], p.PL, ws.prog[0], compile_scratch(ws.stk, p.PL), lane);
    if (lane == 0) {
        length[chain] = co.length;
        count[chain] = co.count;
    }
    __syncwarp();
    build_eval_program(ws.prog[0], ws.Cs[0], co.ninstr, ws.eprog, lane);
    __syncwarp();
    for (int b = 0; b < nx; b += 32) {
        float x[3][1], acc[1];
        int i = b + lane;
        const bool in = i < nx;
        x[0][0] = in ? xs[i] : 0.0f;
        x[1][0] = (in && p.nv == 3) ? xs[nx + i] : 0.0f;    /* multivariate: xs holds x1 | x2 | x3 */
        x[2][0] = (in && p.nv == 3) ? xs[2 * nx + i] : 0.0f;
        run_program<1, false, 3>(ws.eprog, x, acc, ws.stk, ws.scr, lane);
        if (i < nx) out[(size_t)chain * nx + i] = acc[0];
    }
}

cudaError_t launch_eval_values(const KParams& p, const float* xs, int nx, float* out,
                               float* length, int* count, cudaStream_t st) {
    const int wpc = 4;
    size_t smem = (size_t)wpc * warp_smem_bytes(p.PL, p.max_instr, p.levels, 1);
    cudaError_t e = cudaFuncSetAttribute((const void*)eval_values_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = (p.N + wpc - 1) / wpc;
    eval_values_kernel<<<blocks, wpc * 32, smem, st>>>(p, xs, nx, out, length, count);
    return cudaGetLastError();
}

/* Diagnostics: the evaluator's exp (op 0), log (1), pow (2) elementwise. */
__global__ void math_kernel(int op, const float* a, const float* b, float* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r;
    if (op == 0) r = gx_exp(a[i]);
    else if (op == 1) r = gx_log(a[i]);
    else r = gx_pow(a[i], b[i]);
    out[i] = r;
}

/* Diagnostics: four independent chains of adds per thread, FP64 (on every
 * lane, or on lane 0 of each warp only) or FP32, to time the issue cost of
 * FP64 arithmetic against FP32 on the device. */
template <typename T>
__global__ void fp_add_kernel(T* out, int iters, int lane0_only) {
    T a = (T)(threadIdx.x & 31) * (T)1e-3, b = a + (T)1, c = a + (T)2, d = a + (T)3;
    if (!lane0_only || (threadIdx.x & 31) == 0) {
#pragma unroll 4
        for (int i = 0; i < iters; ++i) {
            a = a + (T)1.000001; b = b + (T)1.000002; c = c + (T)1.000003; d = d + (T)1.000004;
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a + b + c + d;
}

cudaError_t time_fp_adds(int iters, float* ms_d32, float* ms_d1, float* ms_f32) {
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = nsm * 8, threads = 256;
    double* d = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if ((e = cudaMalloc(&d, (size_t)blocks * threads * sizeof(double))) != cudaSuccess) return e;
    if ((e = cudaEventCreate(&e0)) == cudaSuccess) e = cudaEventCreate(&e1);
    float* outs[3] = {ms_d32, ms_d1, ms_f32};
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep)      /* the first round warms up */
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
            e = cudaEventRecord(e0);
            if (k < 2) fp_add_kernel<double><<<blocks, threads>>>(d, iters, k);
            else fp_add_kernel<float><<<blocks, threads>>>((float*)d, iters, 0);
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(e1);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(outs[k], e0, e1);
        }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    return e;
}

cudaError_t launch_math(int op, const float* a, const float* b, float* out, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    math_kernel<<<(n + 255) / 256, 256, 0, st>>>(op, a, b, out, n);
    return cudaGetLastError();
}

}  // namespace gpr
