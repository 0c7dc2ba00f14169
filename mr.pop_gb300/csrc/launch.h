// launch.h -- host-side launch interface between the C ABI and the kernel
// instantiations (one translation unit per arm count, compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include "edge_kernel.cuh"

namespace mrpop {

// Launch the validator for `arms` arms (1..5).  smem_bytes: dynamic shared
// memory (staged scene + per-warp scratch).  Returns the launch error.
cudaError_t launch_validate(int arms, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream);

template <int A>
cudaError_t launch_validate_arms(const EdgeParams &p, size_t smem_bytes, cudaStream_t stream);

// Blocks of `validate_kernel<A, SPL>` that fit on one SM with smem_bytes.
int validate_occupancy(int arms, int spl, size_t smem_bytes);

}  // namespace mrpop
