// peak_probe.cu -- measured FP32 FMA throughput of this GPU (roofline
// denominator for the validator, which runs on the FP32 CUDA cores).
#include <cuda_runtime.h>

#include "../../include/mrpop.h"

namespace {

// 8 independent FMA chains per thread; out keeps the result alive.
__global__ void __launch_bounds__(256) fma_loop(float *out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-7f + i;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int r = 0; r < 16; r++)
#pragma unroll
            for (int i = 0; i < 8; i++) x[i] = __fmaf_rn(x[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    if (s == 1234.5f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" mrpop_status mrpop_fp32_peak_probe(int blocks, int iters, float *scratch, double *flops_out,
                                              void *stream) {
    if (blocks < 1 || iters < 1 || !scratch || !flops_out) return MRPOP_ERR_INVALID_ARGUMENT;
    fma_loop<<<blocks, 256, 0, (cudaStream_t)stream>>>(scratch, iters, 0.999999f, 1e-7f);
    *flops_out = 2.0 * 8 * 16 * (double)iters * 256.0 * blocks;
    return cudaGetLastError() == cudaSuccess ? MRPOP_OK : MRPOP_ERR_CUDA;
}
