// batch.cu -- many independent validate calls (planning instances of
// different arm counts, edge counts, granularities, scenes and segmentation
// rules) in one persistent launch per kernel variant and round, replayable as
// one CUDA graph.
//
// Instances are grouped by (arm count, samples per lane, segmented), the
// template parameters of the kernels.  Each group gets a device array of
// parameter blocks, a chunk table (up to `chunk` edges of one instance per
// chunk, instances in order) and work counters; batch_kernel<A, SPL, MODE,
// SEG> hands chunks to CTAs and edges to warps.  A group's run is a broad and
// a narrow launch (each after its counter reset); a segmented group runs them
// for kSegRounds rounds and then the fused kernel.  The captured graph runs
// each group on its own branch so small groups overlap.
//
// Launch shape, per group: the chunk size (edges a CTA takes at a time), and
// per kernel the warps per CTA (each warp one edge at a time, one lane per
// sample; fewer warps per CTA put more scene copies -- and fewer warps -- on
// an SM) and the grid.  mrpop_batch_tune picks all three by timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "launch.h"

struct mrpop_batch {
    struct Group {
        int arms = 0, spl = 1;
        bool seg = false;  // segmented instances (connect, B-spline, shortcut)
        int64_t n_items = 0;
        mrpop::EdgeParams *d_items = nullptr;
        int4 *d_chunks = nullptr;
        int n_chunks = 0;
        unsigned long long *d_work = nullptr;  // chunk counters of the broad, narrow and fused launches
        size_t scene_bytes = 0;       // largest staged scene of the group's instances
        std::vector<int64_t> edges;   // per instance
        int chunk = 0;                // edges per chunk
        int warps[3] = {0, 0, 0};     // warps per CTA of the broad / narrow / fused launch
        int grid[3] = {0, 0, 0};      // CTAs of the broad / narrow / fused launch
        size_t smem(int mode) const { return scene_bytes + (size_t)warps[mode] * mrpop::warp_scratch_bytes(); }
    };
    int device = 0;
    std::vector<Group> groups;
    void *d_scratch = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaStream_t> branch;  // capture-time branch streams
};

namespace {

constexpr int kChunkEdges = 96;
constexpr int kTuneChunks[] = {24, 48, 96, 192};
constexpr int kTuneWarps[] = {2, 3, 4, 6};

mrpop_status cuda_status(cudaError_t e, const char *what) {
    return mrpop::fail_status(MRPOP_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
}

void release(mrpop_batch *b) {
    for (auto &g : b->groups) {
        cudaFree(g.d_items);
        cudaFree(g.d_chunks);
        cudaFree(g.d_work);
    }
    cudaFree(b->d_scratch);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (cudaStream_t s : b->branch) cudaStreamDestroy(s);
    delete b;
}

// One kernel of a group (mode kBatchBroad / kBatchNarrow / kBatchFused; seg0:
// the round, or the first segment of the fused launch): its chunk counter is
// zeroed first (in stream order).
cudaError_t launch_group(const mrpop_batch::Group &g, int mode, int grid, int seg0, cudaStream_t s) {
    mrpop::BatchParams p;
    p.items = g.d_items;
    p.chunks = g.d_chunks;
    p.n_chunks = g.n_chunks;
    p.seg0 = seg0;
    p.work = g.d_work + mode;
    cudaError_t err = cudaMemsetAsync(p.work, 0, sizeof(unsigned long long), s);
    if (err == cudaSuccess) err = mrpop::launch_batch(g.arms, mode, g.seg, g.spl, p, g.smem(mode), grid, g.warps[mode], s);
    return err;
}

// The chunk table of a group for a chunk size (synchronous upload; the table
// grows when it needs more room).
cudaError_t set_chunks(mrpop_batch::Group &g, int chunk) {
    std::vector<int4> chunks;
    for (size_t i = 0; i < g.edges.size(); i++)
        for (int64_t e0 = 0; e0 < g.edges[i]; e0 += chunk)
            chunks.push_back(make_int4((int)i, (int)e0, (int)std::min<int64_t>(chunk, g.edges[i] - e0), 0));
    if ((int)chunks.size() > g.n_chunks || !g.d_chunks) {
        cudaFree(g.d_chunks);
        g.d_chunks = nullptr;
        const cudaError_t err = cudaMalloc(&g.d_chunks, chunks.size() * sizeof(int4));
        if (err != cudaSuccess) return err;
    }
    g.n_chunks = (int)chunks.size();
    g.chunk = chunk;
    return cudaMemcpy(g.d_chunks, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice);
}

// The largest grid of a group's kernel at its warps per CTA: SMs x resident
// CTAs, at most the chunk count.
cudaError_t max_grid(const mrpop_batch::Group &g, int mode, int warps, int sms, int *out) {
    int nb = 0;
    const size_t smem = g.scene_bytes + (size_t)warps * mrpop::warp_scratch_bytes();
    const cudaError_t err = mrpop::batch_occupancy(g.arms, mode, g.seg, g.spl, smem, warps, &nb);
    *out = (int)std::max(1LL, std::min<long long>((long long)sms * std::max(nb, 1), g.n_chunks));
    return err;
}

// A group's whole run: broad and narrow, in segment rounds for a segmented
// group, then the fused kernel for the edges with segments left.
cudaError_t run_group(const mrpop_batch::Group &g, cudaStream_t s) {
    cudaError_t err = cudaSuccess;
    const int rounds = g.seg ? mrpop::kSegRounds : 1;
    for (int r = 0; r < rounds && err == cudaSuccess; r++) {
        err = launch_group(g, mrpop::kBatchBroad, g.grid[0], r, s);
        if (err == cudaSuccess) err = launch_group(g, mrpop::kBatchNarrow, g.grid[1], r, s);
    }
    if (err == cudaSuccess && g.seg) err = launch_group(g, mrpop::kBatchFused, g.grid[2], mrpop::kSegRounds, s);
    return err;
}

}  // namespace

extern "C" {

mrpop_status mrpop_batch_create(const mrpop_batch_item *items, int64_t n_items, mrpop_batch **out) {
    if (!out) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_create: null out");
    *out = nullptr;
    if (n_items < 0 || (n_items > 0 && !items))
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_create: bad item list");
    mrpop_batch *b = new (std::nothrow) mrpop_batch();
    if (!b) return mrpop::fail_status(MRPOP_ERR_OUT_OF_MEMORY, "batch_create: host allocation");
    cudaGetDevice(&b->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);

    // parameter blocks, grouped by (arms, samples per lane)
    struct Entry {
        mrpop::EdgeParams p;
        int arms, spl;
        bool seg;
        size_t smem, scratch;
    };
    std::vector<Entry> ent;
    size_t scratch_total = 0;
    for (int64_t i = 0; i < n_items; i++) {
        const mrpop_batch_item &it = items[i];
        Entry e;
        const mrpop_status st =
            mrpop::make_params(it.scene, it.robots, it.q0, it.q1, it.n_edges, it.granularity, it.rule, it.range,
                               it.flags, it.arm, it.valid, it.first_hit, nullptr, nullptr, e.p, e.arms, e.smem);
        if (st != MRPOP_OK) {
            release(b);
            return mrpop::fail_status(st, ("batch_create: item " + std::to_string(i) + ": " + mrpop_last_error()).c_str());
        }
        if (it.n_edges == 0) continue;
        e.spl = it.granularity > 32 ? 2 : 1;
        e.seg = it.rule != MRPOP_RULE_PLAIN;
        e.scratch = (mrpop::split_scratch_bytes(it.n_edges, it.granularity, e.arms) + 255) & ~(size_t)255;
        scratch_total += e.scratch;
        ent.push_back(e);
    }
    cudaError_t err = cudaSuccess;
    if (scratch_total) err = cudaMalloc(&b->d_scratch, scratch_total);
    if (err != cudaSuccess) {
        release(b);
        return cuda_status(err, "batch_create: scratch");
    }
    size_t off = 0;
    for (Entry &e : ent) {
        mrpop::set_split_scratch(e.p, (char *)b->d_scratch + off, e.p.n_edges, e.p.g, e.arms);
        off += e.scratch;
    }
    for (int key = 0; key < 4 * MRPOP_MAX_ARMS; key++) {
        {
            const int arms = 1 + key / 4, spl = 1 + key % 2;
            const bool seg = (key / 2) % 2 == 1;
            mrpop_batch::Group g;
            g.arms = arms;
            g.spl = spl;
            g.seg = seg;
            std::vector<mrpop::EdgeParams> ps;
            for (const Entry &e : ent) {
                if (e.arms != arms || e.spl != spl || e.seg != seg) continue;
                if (e.p.n_edges > INT32_MAX) {
                    release(b);
                    return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_create: an item has 2^31 edges or more");
                }
                ps.push_back(e.p);
                g.edges.push_back(e.p.n_edges);
                g.scene_bytes = std::max(g.scene_bytes, e.smem - (size_t)mrpop::kWarpsPerBlock * mrpop::warp_scratch_bytes());
            }
            if (ps.empty()) continue;
            g.n_items = (int64_t)ps.size();
            err = cudaMalloc(&g.d_items, ps.size() * sizeof(mrpop::EdgeParams));
            if (err == cudaSuccess) err = cudaMalloc(&g.d_work, 3 * sizeof(unsigned long long));
            if (err == cudaSuccess)
                err = cudaMemcpy(g.d_items, ps.data(), ps.size() * sizeof(mrpop::EdgeParams), cudaMemcpyHostToDevice);
            if (err == cudaSuccess) err = set_chunks(g, kChunkEdges);
            for (int k = 0; k < (seg ? 3 : 2) && err == cudaSuccess; k++) {
                g.warps[k] = mrpop::kWarpsPerBlock;
                err = max_grid(g, k, g.warps[k], sms, &g.grid[k]);
            }
            b->groups.push_back(g);
            if (err != cudaSuccess) {
                release(b);
                return cuda_status(err, "batch_create: group set-up");
            }
        }
    }
    *out = b;
    return MRPOP_OK;
}

mrpop_status mrpop_batch_run(mrpop_batch *b, void *stream) {
    if (!b) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_run: null batch");
    const cudaStream_t s = (cudaStream_t)stream;
    for (const auto &g : b->groups) {
        const cudaError_t err = run_group(g, s);
        if (err != cudaSuccess) return cuda_status(err, "batch_run: launch");
    }
    return MRPOP_OK;
}

// Launch-shape tuner.  Per group, for each chunk size (edges per chunk) and
// each kernel of the split pipeline, every warps-per-CTA choice with every
// grid (multiples of the SM count up to the resident maximum at that CTA
// size, and that maximum) is timed over three launches; the group keeps the
// chunk size whose best broad + narrow times sum lowest, with those shapes.
// The narrow kernel reads the broad kernel's output, so each narrow timing
// follows a broad launch.  A segmented group is tuned on its first round and
// its fused kernel keeps the default shape at the largest grid.  Synchronous;
// not for use during capture.  It launches on the items' own buffers (see
// mrpop.h).
mrpop_status mrpop_batch_tune(mrpop_batch *b, void *stream) {
    if (!b) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_tune: null batch");
    const cudaStream_t s = (cudaStream_t)stream;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return cuda_status(cudaGetLastError(), "batch_tune: events");
    cudaError_t err = cudaSuccess;
    auto time3 = [&](mrpop_batch::Group &g, int k, float *out) {
        float tot = 0.0f;
        for (int r = 0; r < 3 && err == cudaSuccess; r++) {
            if (k == 1) err = launch_group(g, mrpop::kBatchBroad, g.grid[0], 0, s);
            if (err == cudaSuccess) err = cudaEventRecord(e0, s);
            if (err == cudaSuccess) err = launch_group(g, k, g.grid[k], 0, s);
            if (err == cudaSuccess) err = cudaEventRecord(e1, s);
            if (err == cudaSuccess) err = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
            tot += ms;
        }
        *out = tot;
    };
    for (auto &g : b->groups) {
        float best_sum = 1e30f;
        int best_chunk = g.chunk, best_w[2] = {g.warps[0], g.warps[1]}, best_g[2] = {g.grid[0], g.grid[1]};
        int last_chunks = -1;
        for (int chunk : kTuneChunks) {
            if (err != cudaSuccess) break;
            err = set_chunks(g, chunk);
            if (err != cudaSuccess || g.n_chunks == last_chunks) continue;  // same table as the last size
            last_chunks = g.n_chunks;
            float sum = 0.0f;
            int cw[2], cg[2];
            for (int k = 0; k < 2 && err == cudaSuccess; k++) {
                float best = 1e30f;
                cw[k] = g.warps[k];
                cg[k] = g.grid[k];
                for (int w : kTuneWarps) {
                    int mg = 0;
                    err = max_grid(g, k, w, sms, &mg);
                    if (err != cudaSuccess) break;
                    std::vector<int> cand;
                    for (int m = 1; (long long)m * sms <= mg; m++) cand.push_back(m * sms);
                    cand.push_back(mg);
                    std::sort(cand.begin(), cand.end());
                    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
                    for (int grid : cand) {
                        g.warps[k] = w;
                        g.grid[k] = grid;
                        float t = 0.0f;
                        time3(g, k, &t);
                        if (err != cudaSuccess) break;
                        if (t < best) {
                            best = t;
                            cw[k] = w;
                            cg[k] = grid;
                        }
                    }
                    if (err != cudaSuccess) break;
                }
                g.warps[k] = cw[k];  // the narrow kernel is timed behind the best broad shape
                g.grid[k] = cg[k];
                sum += best;
            }
            if (err == cudaSuccess && sum < best_sum) {
                best_sum = sum;
                best_chunk = chunk;
                best_w[0] = cw[0];
                best_w[1] = cw[1];
                best_g[0] = cg[0];
                best_g[1] = cg[1];
            }
        }
        if (err == cudaSuccess) err = set_chunks(g, best_chunk);
        g.warps[0] = best_w[0];
        g.warps[1] = best_w[1];
        g.grid[0] = best_g[0];
        g.grid[1] = best_g[1];
        if (g.seg && err == cudaSuccess) {
            g.warps[2] = mrpop::kWarpsPerBlock;
            err = max_grid(g, 2, g.warps[2], sms, &g.grid[2]);
        }
        if (err != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return cuda_status(err, "batch_tune");
    return MRPOP_OK;
}

// Captures one run into a CUDA graph: each group's launches on a branch of
// their own, joined at the end.  Replaces an earlier capture.
mrpop_status mrpop_batch_capture(mrpop_batch *b) {
    if (!b) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_capture: null batch");
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    cudaError_t err = cudaSuccess;
    while (b->branch.size() < b->groups.size() + 1 && err == cudaSuccess) {
        cudaStream_t s;
        err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (err == cudaSuccess) b->branch.push_back(s);
    }
    if (err != cudaSuccess) return cuda_status(err, "batch_capture: streams");
    cudaStream_t origin = b->branch[0];
    std::vector<cudaEvent_t> ev(b->groups.size() + 1, nullptr);
    for (auto &e : ev)
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaGraph_t graph = nullptr;
    if (err == cudaSuccess) err = cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        cudaError_t cerr = cudaEventRecord(ev[0], origin);
        for (size_t i = 0; i < b->groups.size() && cerr == cudaSuccess; i++) {
            cudaStream_t s = b->branch[i + 1];
            cerr = cudaStreamWaitEvent(s, ev[0], 0);
            if (cerr == cudaSuccess) cerr = run_group(b->groups[i], s);
            if (cerr == cudaSuccess) cerr = cudaEventRecord(ev[i + 1], s);
            if (cerr == cudaSuccess) cerr = cudaStreamWaitEvent(origin, ev[i + 1], 0);
        }
        err = cudaStreamEndCapture(origin, &graph);
        if (err == cudaSuccess) err = cerr;
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&b->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (err != cudaSuccess) {
        b->exec = nullptr;
        return cuda_status(err, "batch_capture");
    }
    return MRPOP_OK;
}

mrpop_status mrpop_batch_launch(mrpop_batch *b, void *stream) {
    if (!b) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_launch: null batch");
    if (!b->exec) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_launch: no captured graph");
    const cudaError_t err = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
    if (err != cudaSuccess) return cuda_status(err, "batch_launch");
    return MRPOP_OK;
}

mrpop_status mrpop_batch_info(const mrpop_batch *b, int64_t *n_groups, int32_t *grids, int64_t max_groups) {
    if (!b || !n_groups) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_info: null argument");
    *n_groups = (int64_t)b->groups.size();
    for (int64_t i = 0; grids && i < max_groups && i < (int64_t)b->groups.size(); i++) {
        const auto &g = b->groups[i];
        grids[5 * i + 0] = g.arms;
        grids[5 * i + 1] = g.spl;
        grids[5 * i + 2] = g.seg ? 1 : 0;
        grids[5 * i + 3] = g.grid[0];
        grids[5 * i + 4] = g.grid[1];
    }
    return MRPOP_OK;
}

mrpop_status mrpop_batch_shapes(const mrpop_batch *b, int64_t *n_groups, int32_t *out, int64_t max_groups) {
    if (!b || !n_groups) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_shapes: null argument");
    *n_groups = (int64_t)b->groups.size();
    for (int64_t i = 0; out && i < max_groups && i < (int64_t)b->groups.size(); i++) {
        const auto &g = b->groups[i];
        int32_t *o = out + MRPOP_BATCH_SHAPE_INTS * i;
        const int32_t v[MRPOP_BATCH_SHAPE_INTS] = {g.arms, g.spl, g.seg ? 1 : 0, g.chunk, g.n_chunks,
                                                   g.warps[0], g.grid[0], g.warps[1], g.grid[1],
                                                   g.warps[2], g.grid[2], 0};
        for (int k = 0; k < MRPOP_BATCH_SHAPE_INTS; k++) o[k] = v[k];
    }
    return MRPOP_OK;
}

mrpop_status mrpop_batch_set_shape(mrpop_batch *b, int64_t group, int32_t chunk_edges, const int32_t *warps,
                                   const int32_t *grids) {
    if (!b || group < 0 || group >= (int64_t)b->groups.size() || !warps || !grids)
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_set_shape: bad argument");
    auto &g = b->groups[(size_t)group];
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);  // the captured graph used the old shape
        b->exec = nullptr;
    }
    if (chunk_edges > 0 && chunk_edges != g.chunk) {
        const cudaError_t err = set_chunks(g, chunk_edges);
        if (err != cudaSuccess) return cuda_status(err, "batch_set_shape: chunks");
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    for (int k = 0; k < 3; k++) {
        if (k == 2 && !g.seg) continue;
        if (warps[k] > 0) {
            if (warps[k] > mrpop::kWarpsPerBlock)
                return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "batch_set_shape: too many warps per CTA");
            g.warps[k] = warps[k];
        }
        int mg = 0;
        const cudaError_t err = max_grid(g, k, g.warps[k], sms, &mg);
        if (err != cudaSuccess) return cuda_status(err, "batch_set_shape: occupancy");
        g.grid[k] = grids[k] > 0 ? std::min(grids[k], mg) : mg;
    }
    return MRPOP_OK;
}

mrpop_status mrpop_batch_destroy(mrpop_batch *b) {
    if (b) release(b);
    return MRPOP_OK;
}

}  // extern "C"
