// validate_a5.cu -- validator kernel instantiations for 5 arm(s).
#include "launch.h"

namespace mrpop {

namespace {

template <int SPL>
const void *kernel_fn(KernelKind kind) {
    switch (kind) {
    case kBroad: return (const void *)broad_kernel<5, SPL>;
    case kNarrow: return (const void *)narrow_kernel<5, SPL>;
    default: return (const void *)validate_kernel<5, SPL>;
    }
}

}  // namespace

template <>
cudaError_t launch_validate_arms<5>(KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream) {
    static int max_blocks[3][3] = {};
    static size_t max_blocks_smem[3][3] = {};
    const int spl = p.g > 32 ? 2 : 1;
    const void *fn = spl == 2 ? kernel_fn<2>(kind) : kernel_fn<1>(kind);
    cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (err != cudaSuccess) return err;
    if (max_blocks_smem[kind][spl] != smem_bytes) {
        int nb = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * kWarpsPerBlock, smem_bytes);
        if (err != cudaSuccess) return err;
        max_blocks[kind][spl] = nb > 0 ? nb : 1;
        max_blocks_smem[kind][spl] = smem_bytes;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long need = (p.n_edges + kWarpsPerBlock - 1) / kWarpsPerBlock;
    long long grid = (long long)sms * max_blocks[kind][spl];
    if (need < grid) grid = need;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&p};
    return cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(32 * kWarpsPerBlock), args, smem_bytes, stream);
}

}  // namespace mrpop
