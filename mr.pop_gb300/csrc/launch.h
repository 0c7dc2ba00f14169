// launch.h -- host-side launch interface between the C ABI and the kernel
// instantiations (one translation unit per arm count, compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include "edge_kernel.cuh"

namespace mrpop {

// Which kernel to launch.
enum KernelKind { kFused = 0, kBroad = 1, kNarrow = 2 };

// Launch a validator kernel for `arms` arms (1..5).  smem_bytes: dynamic
// shared memory (staged scene + per-warp scratch).  Returns the launch error.
cudaError_t launch_validate(int arms, KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream);

template <int A>
cudaError_t launch_validate_arms(KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream);

}  // namespace mrpop
