// no_alloc.cu -- single-segment edge validation without any device allocation.
//
// The ordinary entry points take the split pipeline's scratch (every sample's
// flag words and every edge's candidate masks) from a stream-ordered memory
// pool.  Some callers cannot allow that: a serving process that reserves its
// whole device-memory budget when it starts and admits work against it (an
// allocation inside a call could fail, or change the budget it accounts for),
// or a planner loop that must not enter the allocator while it runs.  This file
// gives them mrpop_validate_edges_noalloc, which runs the same two kernels with
// their scratch in a fixed array that lives in the library's own device memory.
//
// The array: kNoAllocBytes bytes per device (MRPOP_NOALLOC_MAX_EDGES edges at
// the largest granularity), held by every GPU that loads the library until
// the process exits.  Every call uses the same array, so calls that overlap on
// the GPU (for example on two streams at once) race on it and must be ordered
// by the caller.  The array keeps the previous call's contents; nothing in it
// needs to start at zero, because each call's first kernel writes every word of
// scratch that its second kernel reads.
#include <cuda_runtime.h>

#include <mutex>

#include "launch.h"

namespace {

// The scratch of the largest call allowed: MRPOP_NOALLOC_MAX_EDGES edges at
// granularity 64 with 5 arms (the same size function the pool path uses).
constexpr size_t kNoAllocBytes = mrpop::split_scratch_bytes(MRPOP_NOALLOC_MAX_EDGES, 64, mrpop::kMaxArms);
static_assert(kNoAllocBytes >= mrpop::split_scratch_bytes(MRPOP_NOALLOC_MAX_EDGES, 32, mrpop::kMaxArms),
              "the array must hold the largest call at every granularity");

// Host code must not use this name as a device address (on the host it is only
// a stand-in); the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the array on the current device, looked up once per
// device (with that device current) on the first call there.  The cached
// address belongs to that device's primary context: after cudaDeviceReset
// (which also invalidates every scene and robot-set handle) it is stale, so
// the library is not to be used across a reset.
mrpop_status scratch_address(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return mrpop::fail_status(MRPOP_ERR_CUDA, "validate_edges_noalloc: no usable current device");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return mrpop::fail_status(MRPOP_ERR_CUDA, "validate_edges_noalloc: cudaGetSymbolAddress failed");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return MRPOP_OK;
}

}  // namespace

extern "C" mrpop_status mrpop_validate_edges_noalloc(const mrpop_scene *scene, const mrpop_robotset *robots,
                                                     const float *q0, const float *q1, int64_t n_edges,
                                                     int granularity, uint32_t flags, int arm, uint8_t *valid,
                                                     int32_t *first_hit, void *stream) {
    if (n_edges > MRPOP_NOALLOC_MAX_EDGES)
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT,
                                  "validate_edges_noalloc: n_edges exceeds MRPOP_NOALLOC_MAX_EDGES (16384); split "
                                  "the batch or use mrpop_validate_edges");
    if (!valid || !first_hit)
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "validate_edges_noalloc: null output pointer");
    if (n_edges <= 0)
        return n_edges == 0 ? MRPOP_OK
                            : mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "validate_edges_noalloc: n_edges < 0");
    void *scratch = nullptr;
    const mrpop_status st = scratch_address(&scratch);
    if (st != MRPOP_OK) return st;
    return mrpop::run_validator(scene, robots, q0, q1, n_edges, granularity, MRPOP_RULE_PLAIN, 0.0f, flags, arm,
                                valid, first_hit, nullptr, nullptr, (cudaStream_t)stream, scratch);
}
