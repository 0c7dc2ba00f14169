// launch.h -- host-side launch interface between the C ABI and the kernel
// instantiations (one translation unit per arm count, compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include "edge_kernel.cuh"

namespace mrpop {

// Which kernel to launch.
// kFusedPair: the fused kernel with two warps per edge (granularity above 32);
// timed as kFused.
// kArmwise: the fused kernel with one warp per arm; timed as kFused.
enum KernelKind { kFused = 0, kBroad = 1, kNarrow = 2, kFusedPair = 3, kArmwise = 4 };

// Launch a validator kernel for `arms` arms (1..5).  smem_bytes: dynamic
// shared memory (staged scene + per-warp scratch).  Returns the launch error.
cudaError_t launch_validate(int arms, KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream);

template <int A>
cudaError_t launch_validate_arms(KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream);

// Batch kernels (BatchParams: the instances of one arm count, samples per
// lane and segmentation kind; mode = kBatchBroad / kBatchNarrow / kBatchFused,
// seg = segmented instances): resident CTAs per SM at a shared-memory size
// and CTA size (warps of 32 threads, 1..kWarpsPerBlock), and a launch on
// `grid` CTAs of `warps` warps.  The dispatchers switch on the arm count
// (api.cu).
cudaError_t batch_occupancy(int arms, int mode, bool seg, int spl, size_t smem_bytes, int warps, int *blocks_per_sm);
cudaError_t launch_batch(int arms, int mode, bool seg, int spl, const BatchParams &b, size_t smem_bytes, int grid,
                         int warps, cudaStream_t stream);
template <int A>
cudaError_t batch_occupancy_arms(int mode, bool seg, int spl, size_t smem_bytes, int warps, int *blocks_per_sm);
template <int A>
cudaError_t launch_batch_arms(int mode, bool seg, int spl, const BatchParams &b, size_t smem_bytes, int grid,
                              int warps, cudaStream_t stream);

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

// Argument checks and the parameter block of one validate call (run_validator
// and the batch path).  A = arm count of the check, smem = dynamic shared
// memory of its kernels.  n_edges == 0 passes.
mrpop_status make_params(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0, const float *q1,
                         int64_t n_edges, int g, int rule, float range, uint32_t flags, int arm, uint8_t *valid,
                         int32_t *first_hit, int32_t *n_seg_out, double *flops, EdgeParams &p, int &A,
                         size_t &smem);

// Shared-memory scratch of one warp (the per-CTA dynamic size is the staged
// scene plus this times the warps per CTA).
size_t warp_scratch_bytes();

// Scratch of the single-segment pipeline (staged flags, candidate masks and
// reference-sphere bounds): its size, and its slices in p.  Two work counters
// in a 128-byte head (every edge's flag words start on an L2 line), then per
// edge: 32 * spl samples x {env, self} flag words, {env, self} candidate
// masks, A arms' reference-sphere bounds and the segment state.
constexpr size_t kSplitScratchHead = 128;
constexpr size_t split_scratch_bytes(int64_t n_edges, int g, int A) {
    return kSplitScratchHead +
           (size_t)n_edges * (32 * (g > 32 ? 2 : 1) * 2 * sizeof(uint64_t) + 2 * sizeof(uint64_t) +
                              (size_t)A * kRefSpheres * sizeof(float4) + 2 * sizeof(int32_t));
}
void set_split_scratch(EdgeParams &p, void *scratch, int64_t n_edges, int g, int A);

// The dRRT / AO-x planner (drrt.cu) with any validator (validate_many, if
// not null, takes the groups of checks of the roadmap rounds in one call);
// device_nn: tree searches as a kernel on the current device, else on the host.
using check_many_fn = int (*)(void *ctx, const mrpop_check_call *calls, int n_calls);
mrpop_status drrt_run(int arms, mrpop_check_fn validate, check_many_fn validate_many, void *ctx, bool device_nn,
                      const float *start, const float *goals, int num_goals, const mrpop_drrt_settings *settings,
                      float *path_out, int64_t max_waypoints, mrpop_drrt_solution_fn on_solution, void *solution_ctx,
                      mrpop_drrt_result *out);

// Arm count of a robot set (0 for null).
int robotset_arms(const mrpop_robotset *robots);

// Records msg as the calling thread's last error and returns st.
mrpop_status fail_status(mrpop_status st, const char *msg);
// The fused-edge limit of run_validator (mrpop_set_fused_edges); returns the previous one.
int64_t set_fused_edges(int64_t max_edges);

}  // namespace mrpop
