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

#include "../../include/mrpop.h"

namespace mrpop {

// Argument checks, parameter block and launch(es) behind every validate entry
// point (api.cu).  ext_scratch: device scratch for the single-segment
// pipeline, or nullptr to use the library's stream-ordered pool.
mrpop_status run_validator(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0,
                           const float *q1, int64_t n_edges, int g, int rule, float range, uint32_t flags,
                           int arm, uint8_t *valid, int32_t *first_hit, int32_t *n_seg_out, double *flops,
                           cudaStream_t stream, void *ext_scratch);

// Records msg as the calling thread's last error and returns st.
mrpop_status fail_status(mrpop_status st, const char *msg);

}  // namespace mrpop
