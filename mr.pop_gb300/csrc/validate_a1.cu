// validate_a1.cu -- validator instantiations for 1 arm(s).
#include "launch.h"

namespace mrpop {

template <>
cudaError_t launch_validate_arms<1>(const EdgeParams &p, size_t smem_bytes, cudaStream_t stream) {
    static int max_blocks[3] = {0, 0, 0};
    static size_t max_blocks_smem[3] = {0, 0, 0};
    const int spl = p.g > 32 ? 2 : 1;
    const void *fn = spl == 2 ? (const void *)validate_kernel<1, 2> : (const void *)validate_kernel<1, 1>;
    cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (err != cudaSuccess) return err;
    if (max_blocks_smem[spl] != smem_bytes) {
        int nb = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * kWarpsPerBlock, smem_bytes);
        if (err != cudaSuccess) return err;
        max_blocks[spl] = nb > 0 ? nb : 1;
        max_blocks_smem[spl] = smem_bytes;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long need = (p.n_edges + kWarpsPerBlock - 1) / kWarpsPerBlock;
    long long grid = (long long)sms * max_blocks[spl];
    if (need < grid) grid = need;
    if (grid < 1) grid = 1;
    if (spl == 2)
        validate_kernel<1, 2><<<(unsigned)grid, 32 * kWarpsPerBlock, smem_bytes, stream>>>(p);
    else
        validate_kernel<1, 1><<<(unsigned)grid, 32 * kWarpsPerBlock, smem_bytes, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace mrpop
