// launch_impl.cuh -- host launchers of the kernels for one arm count A,
// included by validate_a{1..5}.cu (one translation unit per arm count, so the
// instantiations compile in parallel).
#pragma once
#include <mutex>

#include "launch.h"

namespace mrpop {

namespace {

// Per-kernel launch state of this translation unit (internal linkage, so that
// two builds of the library loaded into one process never share it): the
// largest dynamic shared-memory size the kernel's attribute allows, and the
// resident CTAs per SM at the last size asked.  Guarded by launch_mu.
struct LaunchState {
    const void *fn = nullptr;
    size_t attr_bytes = 0;
    size_t occ_bytes = 0;
    int occ_blocks = 0;
};
std::mutex launch_mu;
LaunchState launch_states[64];

LaunchState *launch_state(const void *fn) {
    for (LaunchState &s : launch_states) {
        if (s.fn == fn) return &s;
        if (!s.fn) {
            s.fn = fn;
            return &s;
        }
    }
    return nullptr;
}

// Raises the kernel's dynamic shared-memory attribute to smem_bytes if it is
// lower (it only grows, so launches racing on other threads stay valid), and
// returns the resident CTAs per SM at that size when blocks_per_sm is given.
cudaError_t prepare_kernel(const void *fn, size_t smem_bytes, int *blocks_per_sm, int threads = 32 * kWarpsPerBlock) {
    std::lock_guard<std::mutex> lk(launch_mu);
    LaunchState *st = launch_state(fn);
    if (!st || smem_bytes > st->attr_bytes) {
        const cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
        if (err != cudaSuccess) return err;
        if (st) st->attr_bytes = smem_bytes;
    }
    if (!blocks_per_sm) return cudaSuccess;
    if (!st || st->occ_bytes != smem_bytes || st->occ_blocks == 0) {
        int nb = 0;
        const cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem_bytes);
        if (err != cudaSuccess) return err;
        *blocks_per_sm = nb > 0 ? nb : 1;
        if (st) {
            st->occ_blocks = *blocks_per_sm;
            st->occ_bytes = smem_bytes;
        }
        return cudaSuccess;
    }
    *blocks_per_sm = st->occ_blocks;
    return cudaSuccess;
}

}  // namespace

// seg: segment-round variant of the split kernels (segmented rules)
template <int A, int SPL>
const void *kernel_fn(KernelKind kind, bool seg) {
    switch (kind) {
    case kBroad: return seg ? (const void *)broad_kernel<A, SPL, true> : (const void *)broad_kernel<A, SPL, false>;
    case kNarrow: return seg ? (const void *)narrow_kernel<A, SPL, true> : (const void *)narrow_kernel<A, SPL, false>;
    case kFusedPair: return (const void *)pair_kernel<A>;
    case kArmwise: return (const void *)armwise_kernel<A, SPL>;
    default: return (const void *)validate_kernel<A, SPL>;
    }
}

template <int A, int SPL>
const void *batch_fn(int mode, bool seg) {
    if (mode == kBatchArmwise) return (const void *)batch_armwise_kernel<A, SPL>;
    if (!seg) {
        switch (mode) {
        case kBatchBroad: return (const void *)batch_kernel<A, SPL, kBatchBroad, false>;
        case kBatchNarrow: return (const void *)batch_kernel<A, SPL, kBatchNarrow, false>;
        default: return (const void *)batch_kernel<A, SPL, kBatchFused, false>;
        }
    }
    switch (mode) {
    case kBatchBroad: return (const void *)batch_kernel<A, SPL, kBatchBroad, true>;
    case kBatchNarrow: return (const void *)batch_kernel<A, SPL, kBatchNarrow, true>;
    default: return (const void *)batch_kernel<A, SPL, kBatchFused, true>;
    }
}

// Persistent grid: SMs x resident CTAs at this shared-memory size, no more
// CTAs than edges / kWarpsPerBlock.
template <int A>
cudaError_t launch_validate_impl(KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream) {
    if (kind == kArmwise) {
        // A warps per CTA, one edge per CTA at a time; only while every edge
        // of the call has a CTA of its own (a second round of edges would
        // double the call's time: then the pair or one-warp kernel)
        const size_t arm_smem =
            smem_bytes - (size_t)kWarpsPerBlock * sizeof(WarpScratch) + (size_t)A * sizeof(WarpScratch);
        const void *fn = p.g > 32 ? (const void *)armwise_kernel<A, 2> : (const void *)armwise_kernel<A, 1>;
        int per_sm = 0, dev = 0, sms = 0;
        const cudaError_t err = prepare_kernel(fn, arm_smem, &per_sm, 32 * A);
        if (err != cudaSuccess) return err;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long resident = (long long)sms * (per_sm > 0 ? per_sm : 1);
        if (p.n_edges <= resident) {
            void *args[] = {(void *)&p};
            return cudaLaunchKernel(fn, dim3((unsigned)(p.n_edges > 0 ? p.n_edges : 1)), dim3(32 * A), args, arm_smem,
                                    stream);
        }
        kind = p.g > 32 ? kFusedPair : kFused;
    }
    const int spl = p.g > 32 ? 2 : 1;
    const bool seg = p.rule != 0;
    const void *fn = spl == 2 ? kernel_fn<A, 2>(kind, seg) : kernel_fn<A, 1>(kind, seg);
    int per_sm = 0;
    const cudaError_t err = prepare_kernel(fn, smem_bytes, &per_sm);
    if (err != cudaSuccess) return err;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_cta = kind == kFusedPair ? kWarpsPerBlock / 2 : kWarpsPerBlock;  // edges in flight per CTA
    const long long need = (p.n_edges + per_cta - 1) / per_cta;
    long long grid = (long long)sms * per_sm;
    if (need < grid) grid = need;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&p};
    if (kind != kNarrow)
        return cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(32 * kWarpsPerBlock), args, smem_bytes, stream);
    // the narrow kernel follows the broad one as a programmatic dependent: its
    // CTAs start (and stage the scene) while the broad kernel's last warps
    // finish, and wait for it in griddepcontrol.wait
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(32 * kWarpsPerBlock);
    cfg.dynamicSmemBytes = smem_bytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

// Batch kernels: the attribute is raised when a batch is created (or tuned),
// so launches (and graph capture) do not touch it.  A CTA may have fewer warps
// than kWarpsPerBlock (the kernel indexes its per-warp scratch by warp).
// The arm-per-warp batch kernel runs A warps per CTA whatever `warps` says:
// its CTA size and shared memory (callers give the size for `warps` warps).
inline void armwise_shape(int A, size_t &smem_bytes, int &warps) {
    smem_bytes = smem_bytes - (size_t)warps * sizeof(WarpScratch) + (size_t)A * sizeof(WarpScratch);
    warps = A;
}

template <int A>
cudaError_t batch_occupancy_impl(int mode, bool seg, int spl, size_t smem_bytes, int warps, int *blocks_per_sm) {
    if (mode == kBatchArmwise) armwise_shape(A, smem_bytes, warps);
    const void *fn = spl == 2 ? batch_fn<A, 2>(mode, seg) : batch_fn<A, 1>(mode, seg);
    cudaError_t err = prepare_kernel(fn, smem_bytes, nullptr);
    if (err != cudaSuccess) return err;
    int nb = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * warps, smem_bytes);
    if (err == cudaSuccess) *blocks_per_sm = nb > 0 ? nb : 1;
    return err;
}

template <int A>
cudaError_t launch_batch_impl(int mode, bool seg, int spl, const BatchParams &b, size_t smem_bytes, int grid,
                              int warps, cudaStream_t stream) {
    if (mode == kBatchArmwise) armwise_shape(A, smem_bytes, warps);
    const void *fn = spl == 2 ? batch_fn<A, 2>(mode, seg) : batch_fn<A, 1>(mode, seg);
    void *args[] = {(void *)&b};
    return cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(32 * warps), args, smem_bytes, stream);
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
    cudaError_t batch_occupancy_arms<A>(int mode, bool seg, int spl, size_t smem_bytes, int warps,     \
                                        int *blocks_per_sm) {                                           \
        return batch_occupancy_impl<A>(mode, seg, spl, smem_bytes, warps, blocks_per_sm);               \
    }                                                                                                   \
    template <>                                                                                         \
    cudaError_t launch_batch_arms<A>(int mode, bool seg, int spl, const BatchParams &b,                \
                                     size_t smem_bytes, int grid, int warps, cudaStream_t stream) {    \
        return launch_batch_impl<A>(mode, seg, spl, b, smem_bytes, grid, warps, stream);                \
    }                                                                                                   \
    }
