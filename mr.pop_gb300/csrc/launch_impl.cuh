// launch_impl.cuh -- host launchers of the kernels for one arm count A,
// included by validate_a{1..5}.cu (one translation unit per arm count, so the
// instantiations compile in parallel).
#pragma once
#include <mutex>

#include "launch.h"

namespace mrpop {

// seg: segment-round variant of the split kernels (segmented rules)
template <int A, int SPL>
const void *kernel_fn(KernelKind kind, bool seg) {
    switch (kind) {
    case kBroad: return seg ? (const void *)broad_kernel<A, SPL, true> : (const void *)broad_kernel<A, SPL, false>;
    case kNarrow: return seg ? (const void *)narrow_kernel<A, SPL, true> : (const void *)narrow_kernel<A, SPL, false>;
    default: return (const void *)validate_kernel<A, SPL>;
    }
}

template <int A, int SPL>
const void *batch_fn(bool narrow) {
    return narrow ? (const void *)batch_kernel<A, SPL, true> : (const void *)batch_kernel<A, SPL, false>;
}

// Persistent grid: SMs x resident CTAs at this shared-memory size (cached per
// kernel), no more CTAs than tiles of kWarpsPerBlock edges.  The kernel's
// shared-memory attribute only grows, so a launch racing with another host
// thread's never finds it below its own size; the cache is guarded.
template <int A>
cudaError_t launch_validate_impl(KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream) {
    static std::mutex mu;
    static int max_blocks[3][3][2] = {};
    static size_t max_blocks_smem[3][3][2] = {};
    static size_t set_bytes[3][3][2] = {};
    const int spl = p.g > 32 ? 2 : 1;
    const int seg = p.rule != 0 ? 1 : 0;
    const void *fn = spl == 2 ? kernel_fn<A, 2>(kind, seg) : kernel_fn<A, 1>(kind, seg);
    std::unique_lock<std::mutex> lk(mu);
    cudaError_t err = cudaSuccess;
    if (smem_bytes > set_bytes[kind][spl][seg]) {
        err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
        if (err != cudaSuccess) return err;
        set_bytes[kind][spl][seg] = smem_bytes;
    }
    if (max_blocks_smem[kind][spl][seg] != smem_bytes) {
        int nb = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * kWarpsPerBlock, smem_bytes);
        if (err != cudaSuccess) return err;
        max_blocks[kind][spl][seg] = nb > 0 ? nb : 1;
        max_blocks_smem[kind][spl][seg] = smem_bytes;
    }
    const int per_sm = max_blocks[kind][spl][seg];
    lk.unlock();
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long need = (p.n_edges + kWarpsPerBlock - 1) / kWarpsPerBlock;
    long long grid = (long long)sms * per_sm;
    if (need < grid) grid = need;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&p};
    return cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(32 * kWarpsPerBlock), args, smem_bytes, stream);
}

// Batch kernels: the shared-memory attribute is raised (never lowered) when a
// batch is created, so every batch created so far stays launchable; launches
// themselves (and graph capture) do not touch it.
template <int A>
cudaError_t batch_occupancy_impl(bool narrow, int spl, size_t smem_bytes, int *blocks_per_sm) {
    static std::mutex mu;
    static size_t set_bytes[2][3] = {};
    const void *fn = spl == 2 ? batch_fn<A, 2>(narrow) : batch_fn<A, 1>(narrow);
    std::lock_guard<std::mutex> lk(mu);
    if (smem_bytes > set_bytes[narrow][spl]) {
        const cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
        if (err != cudaSuccess) return err;
        set_bytes[narrow][spl] = smem_bytes;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, 32 * kWarpsPerBlock, smem_bytes);
}

template <int A>
cudaError_t launch_batch_impl(bool narrow, int spl, const BatchParams &b, size_t smem_bytes, int grid,
                              cudaStream_t stream) {
    const void *fn = spl == 2 ? batch_fn<A, 2>(narrow) : batch_fn<A, 1>(narrow);
    void *args[] = {(void *)&b};
    return cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(32 * kWarpsPerBlock), args, smem_bytes, stream);
}

}  // namespace mrpop

// Defines the per-arm-count entry points declared in launch.h.
#define MRPOP_DEFINE_ARM_LAUNCHERS(A)                                                                       \
    namespace mrpop {                                                                                   \
    template <>                                                                                         \
    cudaError_t launch_validate_arms<A>(KernelKind kind, const EdgeParams &p, size_t smem_bytes,       \
                                        cudaStream_t stream) {                                          \
        return launch_validate_impl<A>(kind, p, smem_bytes, stream);                                    \
    }                                                                                                   \
    template <>                                                                                         \
    cudaError_t batch_occupancy_arms<A>(bool narrow, int spl, size_t smem_bytes, int *blocks_per_sm) {  \
        return batch_occupancy_impl<A>(narrow, spl, smem_bytes, blocks_per_sm);                         \
    }                                                                                                   \
    template <>                                                                                         \
    cudaError_t launch_batch_arms<A>(bool narrow, int spl, const BatchParams &b, size_t smem_bytes,     \
                                     int grid, cudaStream_t stream) {                                   \
        return launch_batch_impl<A>(narrow, spl, b, smem_bytes, grid, stream);                          \
    }                                                                                                   \
    }
