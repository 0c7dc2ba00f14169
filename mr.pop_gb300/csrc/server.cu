// server.cu -- continuous-batching validation service for many concurrent
// planning queries on one GPU.
//
// The reference runs one planning query per process: dRRT::solve owns the GPU,
// allocates its state and validates one edge per block of its own kernels
// (pop_planner.cu:220-737, 973).  Serving many queries at once needs three
// things that it does not have, and this file provides them:
//   - admission by device-memory footprint: a query opens a session, which
//     reserves the scratch of its largest step inside one arena allocated when
//     the server starts; a session that does not fit waits until others close;
//   - co-batching: the steps that sessions submit (extend, connect, B-spline or
//     shortcut edge sets) are gathered by one worker thread into waves, and
//     every wave runs as one set of persistent batch launches (batch_kernel,
//     the kernels of the mrpop_batch_* entry points) over all of its steps;
//   - overlap: waves go to a ring of streams, so a wave is formed and launched
//     while earlier ones are still on the GPU, and their kernels share the SMs
//     at their tails.  A step's results are those of the same call made alone.
// Completion comes back through a host function enqueued behind each wave;
// it only takes the lock, marks the wave's steps done and wakes the waiters.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "launch.h"

namespace {

constexpr int kChunkEdges = 96;    // largest chunk (the batch entry points' chunk)
// A wave is cut into chunks of kWarpsPerBlock..kChunkEdges edges, sized so
// that it has about kWaveCtasPerSm chunks per SM: a planner step of a few
// dozen edges then spreads over several CTAs instead of running through one
// CTA's warps in turn.
constexpr int kWaveCtasPerSm = 3;
// Groups of at most this many edges in a wave (mrpop_server_config.fused_edges)
// run as one fused launch -- broad and narrow phase per edge in one warp, from
// segment 0 -- instead of the split kernels (1 launch instead of 2, or of
// 2 * kSegRounds + 1 for segmented rules): launch latency and the serial
// dependency between the split kernels dominate small waves.
constexpr int64_t kFusedEdgesDefault = 4096;
// Groups of 3 to 5 arms with at most this many edges in a wave run the
// arm-per-warp kernel (a CTA of A warps per edge; about as many edges as its
// CTAs resident on the device at 5 arms).
constexpr int64_t kArmwiseEdges = 456;
// Work counters per group and wave: one per launch (split rounds + fused
// tail), zeroed together with the parameter upload so that no launch needs a
// memset of its own.
constexpr int kCountersPerGroup = 2 * mrpop::kSegRounds + 1;
constexpr int kGroupKeys = 4 * MRPOP_MAX_ARMS;
constexpr size_t kAlign = 256;

size_t round_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

int64_t host_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

}  // namespace

struct mrpop_session;

struct mrpop_server {
    // One step: a validate call with its scratch in its session's arena block.
    struct Step {
        mrpop_session *session = nullptr;
        mrpop::EdgeParams p{};
        int arms = 1, spl = 1;
        bool seg = false;
        size_t smem = 0;
        int n_chunks = 0;
        int64_t t_submit = 0;  // host clock, ns
    };
    // A ring slot: stream, device tables (work counters, parameter blocks and
    // chunk lists of one wave) and their page-locked host mirror.
    struct Slot {
        cudaStream_t stream = nullptr;
        char *d_tab = nullptr;
        char *h_tab = nullptr;
        bool busy = false;
        int64_t t_launch = 0;  // host clock when the wave was formed, ns
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // before the wave's first command, after its last
        int64_t device_ns = 0;                     // ev0 to ev1 of the last finished wave
        std::vector<Step> steps;
    };

    int device = 0;
    int sms = 0;
    mrpop_server_config cfg{};
    char *d_arena = nullptr;
    std::map<size_t, size_t> free_blocks;  // offset -> size, first fit
    size_t in_use = 0;
    char *h_arena = nullptr;               // page-locked host arena of the sessions' buffers
    std::map<size_t, size_t> free_host;
    size_t host_in_use = 0;
    std::vector<Slot> slots;
    size_t tab_params_off = 0, tab_chunks_off = 0, tab_bytes = 0;

    std::mutex mu;
    std::condition_variable work_cv;  // the worker: a step pending, a slot freed, or stop
    std::condition_variable room_cv;  // admission: blocks freed
    std::deque<Step> pending;
    std::atomic<int64_t> n_pending{0};  // pending.size(), read by the dispatcher without the lock
    bool stop = false;
    std::thread worker;
    mrpop_server_stats stats{};
    std::atomic<int64_t> launches{0};  // kernels enqueued (the worker adds, stats readers load)
    std::map<uint64_t, int> occupancy;  // resident CTAs per SM by kernel and shared-memory size (worker only)
};

struct mrpop_session {
    mrpop_server *server = nullptr;
    int arms = 0;
    int64_t max_edges = 0;
    int max_g = 0;
    size_t offset = 0, bytes = 0;
    size_t host_off = 0, host_bytes = 0;
    float *h_q0 = nullptr, *h_q1 = nullptr;
    uint8_t *h_valid = nullptr;
    int32_t *h_first = nullptr;
    // guarded by server->mu
    std::condition_variable done_cv;  // this session's steps done
    int in_flight = 0;                // steps submitted and not yet retired
    mrpop_status result = MRPOP_OK;
    std::string error;
};

namespace {

mrpop_status fail(mrpop_status st, const std::string &msg) { return mrpop::fail_status(st, msg.c_str()); }

// First-fit allocation in an arena's free list; returns false if no block is large enough.
bool arena_take(std::map<size_t, size_t> &free_list, size_t &in_use, size_t bytes, size_t *off) {
    for (auto it = free_list.begin(); it != free_list.end(); ++it) {
        if (it->second < bytes) continue;
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t at = it->first + bytes;
        free_list.erase(it);
        if (rest) free_list[at] = rest;
        in_use += bytes;
        return true;
    }
    return false;
}

void arena_give(std::map<size_t, size_t> &free_list, size_t &in_use, size_t off, size_t bytes) {
    auto it = free_list.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_list.end() && it->first + it->second == next->first) {
        it->second += next->second;
        free_list.erase(next);
    }
    if (it != free_list.begin()) {
        auto prev = std::prev(it);
        if (prev->first + prev->second == it->first) {
            prev->second += it->second;
            free_list.erase(it);
        }
    }
    in_use -= bytes;
}

// A session's device and host blocks, both or neither (caller holds the lock).
bool take_blocks(mrpop_server *s, mrpop_session *ss) {
    if (!arena_take(s->free_blocks, s->in_use, ss->bytes, &ss->offset)) return false;
    if (!arena_take(s->free_host, s->host_in_use, ss->host_bytes, &ss->host_off)) {
        arena_give(s->free_blocks, s->in_use, ss->offset, ss->bytes);
        return false;
    }
    return true;
}

// One kernel of a group of the wave (its counter was zeroed by the wave's
// upload).  The grid is the resident maximum, at most the chunk count; the
// resident CTAs per SM are looked up once per kernel and shared-memory size
// (the look-up also raises the kernel's shared-memory limit).
cudaError_t launch_one(mrpop_server *s, int arms, bool seg, int spl, size_t smem, int mode, int seg0,
                       const mrpop::EdgeParams *items, const int4 *chunks, int n_chunks, unsigned long long *work,
                       cudaStream_t stream) {
    mrpop::BatchParams b;
    b.items = items;
    b.chunks = chunks;
    b.n_chunks = n_chunks;
    b.seg0 = seg0;
    b.work = work;
    const uint64_t key = ((uint64_t)smem << 16) | (uint64_t)(arms << 8 | mode << 4 | (seg ? 2 : 0) | (spl - 1));
    auto it = s->occupancy.find(key);
    if (it == s->occupancy.end()) {
        int nb = 0;
        const cudaError_t err = mrpop::batch_occupancy(arms, mode, seg, spl, smem, mrpop::kWarpsPerBlock, &nb);
        if (err != cudaSuccess) return err;
        it = s->occupancy.emplace(key, std::max(nb, 1)).first;
    }
    const int grid = (int)std::max(1LL, std::min<long long>((long long)s->sms * it->second, n_chunks));
    s->launches++;
    return mrpop::launch_batch(arms, mode, seg, spl, b, smem, grid, mrpop::kWarpsPerBlock, stream);
}

// Builds the wave's tables in the slot, uploads them and launches every group.
cudaError_t launch_wave(mrpop_server *s, mrpop_server::Slot &slot) {
    auto *h_work = reinterpret_cast<unsigned long long *>(slot.h_tab);
    auto *h_params = reinterpret_cast<mrpop::EdgeParams *>(slot.h_tab + s->tab_params_off);
    auto *h_chunks = reinterpret_cast<int4 *>(slot.h_tab + s->tab_chunks_off);
    auto *d_work = reinterpret_cast<unsigned long long *>(slot.d_tab);
    auto *d_params = reinterpret_cast<mrpop::EdgeParams *>(slot.d_tab + s->tab_params_off);
    auto *d_chunks = reinterpret_cast<int4 *>(slot.d_tab + s->tab_chunks_off);
    std::memset(h_work, 0, s->tab_params_off);

    struct Range {
        int p0 = 0, np = 0, c0 = 0, nc = 0;
        int64_t edges = 0;
        size_t smem = 0;
        bool armwise = false;
    };
    // chunk size of this wave (a multiple of the warps per CTA)
    int64_t total = 0;
    for (const auto &st : slot.steps) total += st.p.n_edges;
    const int64_t target = (int64_t)s->sms * kWaveCtasPerSm;
    int chunk = (int)std::min<int64_t>(kChunkEdges, std::max<int64_t>(mrpop::kWarpsPerBlock, (total + target - 1) / target));
    chunk = (chunk + mrpop::kWarpsPerBlock - 1) / mrpop::kWarpsPerBlock * mrpop::kWarpsPerBlock;
    for (;;) {
        int64_t n = 0;
        for (const auto &st : slot.steps) n += (st.p.n_edges + chunk - 1) / chunk;
        if (n <= s->cfg.max_wave_chunks || chunk >= kChunkEdges) break;
        chunk = std::min(kChunkEdges, chunk + mrpop::kWarpsPerBlock);
    }
    // chunks of every group at the wave's chunk size (they fit the table)
    int64_t left = 0;
    for (const auto &st : slot.steps) left += (st.p.n_edges + chunk - 1) / chunk;
    Range ranges[kGroupKeys];
    int np = 0, nc = 0;
    for (int key = 0; key < kGroupKeys; key++) {
        const int arms = 1 + key / 4, spl = 1 + key % 2;
        const bool seg = (key / 2) % 2 == 1;
        Range &r = ranges[key];
        r.p0 = np;
        r.c0 = nc;
        int64_t edges = 0, at_chunk = 0;
        for (const auto &st : slot.steps)
            if (st.arms == arms && st.spl == spl && st.seg == seg) {
                edges += st.p.n_edges;
                at_chunk += (st.p.n_edges + chunk - 1) / chunk;
            }
        left -= at_chunk;
        // a small group of 3 to 5 arms runs one warp per arm, one edge per
        // CTA: its chunks are single edges, if the table has room for them
        r.armwise = arms >= 3 && edges <= kArmwiseEdges && edges <= s->cfg.fused_edges &&
                    nc + edges + left <= s->cfg.max_wave_chunks;
        const int cs = r.armwise ? 1 : chunk;
        for (const auto &st : slot.steps) {
            if (st.arms != arms || st.spl != spl || st.seg != seg) continue;
            const int item = np - r.p0;
            h_params[np++] = st.p;
            for (int64_t e0 = 0; e0 < st.p.n_edges; e0 += cs)
                h_chunks[nc++] = make_int4(item, (int)e0, (int)std::min<int64_t>(cs, st.p.n_edges - e0), 0);
            r.smem = std::max(r.smem, st.smem);
            r.edges += st.p.n_edges;
        }
        r.np = np - r.p0;
        r.nc = nc - r.c0;
    }
    // work counters (zero) and parameter blocks in one copy, chunk lists in another
    cudaError_t err = cudaEventRecord(slot.ev0, slot.stream);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_work, h_work, s->tab_params_off + (size_t)np * sizeof(mrpop::EdgeParams),
                                      cudaMemcpyHostToDevice, slot.stream);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(d_chunks, h_chunks, (size_t)nc * sizeof(int4), cudaMemcpyHostToDevice, slot.stream);
    for (int key = 0; key < kGroupKeys && err == cudaSuccess; key++) {
        const Range &r = ranges[key];
        if (!r.np) continue;
        const int arms = 1 + key / 4, spl = 1 + key % 2;
        const bool seg = (key / 2) % 2 == 1;
        unsigned long long *work = d_work + (size_t)kCountersPerGroup * key;
        const mrpop::EdgeParams *items = d_params + r.p0;
        const int4 *chunks = d_chunks + r.c0;
        if (r.armwise) {
            err = launch_one(s, arms, seg, spl, r.smem, mrpop::kBatchArmwise, 0, items, chunks, r.nc, work, slot.stream);
            continue;
        }
        if (r.edges <= s->cfg.fused_edges) {
            err = launch_one(s, arms, seg, spl, r.smem, mrpop::kBatchFused, 0, items, chunks, r.nc, work, slot.stream);
            continue;
        }
        const int rounds = seg ? mrpop::kSegRounds : 1;
        for (int rd = 0; rd < rounds && err == cudaSuccess; rd++) {
            err = launch_one(s, arms, seg, spl, r.smem, mrpop::kBatchBroad, rd, items, chunks, r.nc, work + 2 * rd,
                             slot.stream);
            if (err == cudaSuccess)
                err = launch_one(s, arms, seg, spl, r.smem, mrpop::kBatchNarrow, rd, items, chunks, r.nc,
                                 work + 2 * rd + 1, slot.stream);
        }
        if (err == cudaSuccess && seg)
            err = launch_one(s, arms, seg, spl, r.smem, mrpop::kBatchFused, mrpop::kSegRounds, items, chunks, r.nc,
                             work + 2 * rounds, slot.stream);
    }
    return err;
}

// Moves pending steps (FIFO, while the wave's tables have room) into a free
// slot (caller holds the lock).
void form_wave(mrpop_server *s, mrpop_server::Slot &slot) {
    int items = 0;
    int64_t chunks = 0;
    while (!s->pending.empty()) {
        const auto &st = s->pending.front();
        if (items + 1 > s->cfg.max_wave_steps || chunks + st.n_chunks > s->cfg.max_wave_chunks) break;
        items++;
        chunks += st.n_chunks;
        slot.steps.push_back(st);
        s->pending.pop_front();
    }
    s->n_pending.store((int64_t)s->pending.size(), std::memory_order_relaxed);
    slot.busy = true;
    slot.t_launch = host_ns();
    for (const auto &st : slot.steps) s->stats.queue_ns += slot.t_launch - st.t_submit;
    s->stats.waves++;
    s->stats.steps += items;
    s->stats.max_wave_steps = std::max<int64_t>(s->stats.max_wave_steps, items);
    int in_flight = 0;
    for (auto &sl : s->slots) in_flight += sl.busy ? 1 : 0;
    s->stats.max_waves_in_flight = std::max<int64_t>(s->stats.max_waves_in_flight, in_flight);
}

// Marks a finished (or failed) wave's steps done and frees its slot (caller
// holds the lock).
void retire_wave(mrpop_server *s, mrpop_server::Slot &slot, cudaError_t err) {
    s->stats.flight_ns += (host_ns() - slot.t_launch) * (int64_t)slot.steps.size();
    const std::string msg = err == cudaSuccess ? std::string() : std::string("server: wave failed: ") + cudaGetErrorString(err);
    for (auto &st : slot.steps) {
        if (err != cudaSuccess) {
            st.session->result = MRPOP_ERR_CUDA;
            st.session->error = msg;
        }
        if (--st.session->in_flight == 0) st.session->done_cv.notify_one();
    }
    slot.steps.clear();
    slot.busy = false;
}

// The dispatcher: forms a wave from the pending steps whenever a slot is
// free, and retires each wave when the event after its last command has
// completed.  While any wave is in flight it polls those events (one host
// core, completions seen within microseconds); with none in flight and
// nothing pending it sleeps until a step is submitted.  The slots are this
// thread's alone; the lock guards the queue, the sessions' flags and the
// statistics.
void worker_loop(mrpop_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        // poll the waves in flight, without the lock
        bool any_busy = false, any_free = false;
        mrpop_server::Slot *done[64];
        cudaError_t done_err[64];
        int n_done = 0;
        for (auto &sl : s->slots) {
            if (!sl.busy) {
                any_free = true;
                continue;
            }
            const cudaError_t q = cudaEventQuery(sl.ev1);
            if (q == cudaErrorNotReady) {
                any_busy = true;
                continue;
            }
            float ms = 0.0f;
            if (q == cudaSuccess && cudaEventElapsedTime(&ms, sl.ev0, sl.ev1) == cudaSuccess)
                sl.device_ns = (int64_t)(ms * 1e6);
            done[n_done] = &sl;
            done_err[n_done++] = q;
            any_free = true;
        }
        const bool launchable = any_free && s->n_pending.load(std::memory_order_relaxed) > 0;
        if (!n_done && !launchable) {
            if (any_busy) {
                std::this_thread::yield();
                continue;
            }
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop && s->pending.empty()) break;
            s->work_cv.wait(lk, [&] { return s->stop || !s->pending.empty(); });
            continue;
        }
        std::unique_lock<std::mutex> lk(s->mu);
        for (int i = 0; i < n_done; i++) {
            s->stats.device_ns += done[i]->device_ns;
            retire_wave(s, *done[i], done_err[i]);
        }
        // launch: one wave per free slot while steps are pending
        for (auto &sl : s->slots) {
            if (s->pending.empty()) break;
            if (sl.busy) continue;
            form_wave(s, sl);
            lk.unlock();
            cudaError_t err = launch_wave(s, sl);
            if (err == cudaSuccess) err = cudaEventRecord(sl.ev1, sl.stream);
            if (err != cudaSuccess) cudaStreamSynchronize(sl.stream);  // what was enqueued, before failing the steps
            lk.lock();
            if (err != cudaSuccess) retire_wave(s, sl, err);
        }
    }
}

void destroy_server(mrpop_server *s) {
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->work_cv.notify_all();
        s->worker.join();
    }
    for (auto &sl : s->slots) {
        if (sl.stream) {
            cudaStreamSynchronize(sl.stream);
            cudaStreamDestroy(sl.stream);
        }
        if (sl.ev0) cudaEventDestroy(sl.ev0);
        if (sl.ev1) cudaEventDestroy(sl.ev1);
        cudaFree(sl.d_tab);
        cudaFreeHost(sl.h_tab);
    }
    cudaFree(s->d_arena);
    cudaFreeHost(s->h_arena);
    delete s;
}

}  // namespace

extern "C" {

mrpop_status mrpop_server_create(const mrpop_server_config *cfg, mrpop_server **out) {
    if (!out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "server_create: null out");
    *out = nullptr;
    mrpop_server_config c{};
    if (cfg) c = *cfg;
    if (c.budget_bytes <= 0) c.budget_bytes = (int64_t)1 << 30;
    if (c.streams <= 0) c.streams = 4;
    if (c.max_wave_steps <= 0) c.max_wave_steps = 1024;
    if (c.max_wave_chunks <= 0) c.max_wave_chunks = 16384;
    if (c.host_bytes <= 0) c.host_bytes = (int64_t)256 << 20;
    if (c.fused_edges == 0) c.fused_edges = kFusedEdgesDefault;
    if (c.streams > 16 || c.max_wave_steps > (1 << 20) || c.max_wave_chunks > (1 << 24))
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "server_create: streams <= 16, max_wave_steps <= 2^20, "
                                                "max_wave_chunks <= 2^24");
    auto *s = new (std::nothrow) mrpop_server();
    if (!s) return fail(MRPOP_ERR_OUT_OF_MEMORY, "server_create: host allocation");
    s->cfg = c;
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    const size_t arena = round_up((size_t)c.budget_bytes);
    cudaError_t err = cudaMalloc(&s->d_arena, arena);
    if (err != cudaSuccess) {
        delete s;
        return fail(MRPOP_ERR_OUT_OF_MEMORY, std::string("server_create: arena: ") + cudaGetErrorString(err));
    }
    s->free_blocks[0] = arena;
    s->stats.budget_bytes = (int64_t)arena;
    const size_t harena = round_up((size_t)c.host_bytes);
    err = cudaHostAlloc(&s->h_arena, harena, cudaHostAllocDefault);
    if (err != cudaSuccess) {
        cudaFree(s->d_arena);
        delete s;
        return fail(MRPOP_ERR_OUT_OF_MEMORY, std::string("server_create: host arena: ") + cudaGetErrorString(err));
    }
    s->free_host[0] = harena;
    s->tab_params_off = round_up(kGroupKeys * kCountersPerGroup * sizeof(unsigned long long));
    s->tab_chunks_off = round_up(s->tab_params_off + (size_t)c.max_wave_steps * sizeof(mrpop::EdgeParams));
    s->tab_bytes = round_up(s->tab_chunks_off + (size_t)c.max_wave_chunks * sizeof(int4));
    s->slots.resize(c.streams);
    for (auto &sl : s->slots) {
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaEventCreate(&sl.ev0);
        if (err == cudaSuccess) err = cudaEventCreate(&sl.ev1);
        if (err == cudaSuccess) err = cudaMalloc(&sl.d_tab, s->tab_bytes);
        if (err == cudaSuccess) err = cudaHostAlloc(&sl.h_tab, s->tab_bytes, cudaHostAllocDefault);
        sl.steps.reserve(c.max_wave_steps);
    }
    if (err != cudaSuccess) {
        destroy_server(s);
        return fail(MRPOP_ERR_CUDA, std::string("server_create: slots: ") + cudaGetErrorString(err));
    }
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return MRPOP_OK;
}

mrpop_status mrpop_server_destroy(mrpop_server *s) {
    if (s) destroy_server(s);
    return MRPOP_OK;
}

mrpop_status mrpop_server_get_stats(mrpop_server *s, mrpop_server_stats *out) {
    if (!s || !out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "server_stats: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->bytes_in_use = (int64_t)s->in_use;
    out->kernel_launches = s->launches.load();
    return MRPOP_OK;
}

mrpop_status mrpop_session_open(mrpop_server *s, int arms, int64_t max_edges, int max_granularity,
                                int64_t timeout_ms, mrpop_session **out) {
    if (!s || !out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_open: null argument");
    *out = nullptr;
    if (arms < 1 || arms > MRPOP_MAX_ARMS || max_edges < 1 || max_granularity < 1 ||
        max_granularity > MRPOP_MAX_GRANULARITY)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_open: arms 1..5, max_edges >= 1, max_granularity 1..64");
    const int64_t max_chunks = (max_edges + kChunkEdges - 1) / kChunkEdges;
    if (max_chunks > s->cfg.max_wave_chunks || max_edges > INT32_MAX)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_open: max_edges exceeds one wave's chunk table");
    // scratch of max_edges edges at the largest arm count and granularity, and
    // room for the per-item header and alignment of a multi-item submission
    const size_t bytes =
        round_up(mrpop::split_scratch_bytes(max_edges, max_granularity, arms) + 2 * MRPOP_SESSION_MAX_ITEMS * kAlign);
    const size_t qbytes = round_up((size_t)max_edges * 7 * arms * sizeof(float));
    const size_t host_bytes = 2 * qbytes + round_up((size_t)max_edges) + round_up((size_t)max_edges * sizeof(int32_t));
    if ((int64_t)bytes > s->stats.budget_bytes || host_bytes > round_up((size_t)s->cfg.host_bytes))
        return fail(MRPOP_ERR_OUT_OF_MEMORY, "session_open: the session's scratch exceeds the server's budget");
    auto *ss = new (std::nothrow) mrpop_session();
    if (!ss) return fail(MRPOP_ERR_OUT_OF_MEMORY, "session_open: host allocation");
    ss->server = s;
    ss->arms = arms;
    ss->max_edges = max_edges;
    ss->max_g = max_granularity;
    ss->bytes = bytes;
    ss->host_bytes = host_bytes;
    std::unique_lock<std::mutex> lk(s->mu);
    bool waited = false;
    if (!take_blocks(s, ss)) {
        waited = true;
        bool ok = false;
        const auto fits = [&] { return take_blocks(s, ss); };
        if (timeout_ms < 0) {
            s->room_cv.wait(lk, fits);
            ok = true;
        } else if (timeout_ms > 0) {
            ok = s->room_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), fits);
        }
        if (!ok) {
            s->stats.admission_timeouts++;
            lk.unlock();
            delete ss;
            return fail(MRPOP_ERR_OUT_OF_MEMORY, "session_open: no room in the server's budget before the timeout");
        }
    }
    char *h = s->h_arena + ss->host_off;
    ss->h_q0 = reinterpret_cast<float *>(h);
    ss->h_q1 = reinterpret_cast<float *>(h + qbytes);
    ss->h_valid = reinterpret_cast<uint8_t *>(h + 2 * qbytes);
    ss->h_first = reinterpret_cast<int32_t *>(h + 2 * qbytes + round_up((size_t)max_edges));
    s->stats.sessions++;
    if (waited) s->stats.admission_waits++;
    s->stats.peak_bytes_in_use = std::max<int64_t>(s->stats.peak_bytes_in_use, (int64_t)s->in_use);
    *out = ss;
    return MRPOP_OK;
}

mrpop_status mrpop_session_submit_many(mrpop_session *ss, const mrpop_batch_item *items, int n) {
    if (!ss || (!items && n)) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: null argument");
    if (n < 0 || n > MRPOP_SESSION_MAX_ITEMS)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: at most MRPOP_SESSION_MAX_ITEMS steps at once");
    mrpop_server *s = ss->server;
    mrpop_server::Step steps[MRPOP_SESSION_MAX_ITEMS];
    int n_steps = 0;
    int64_t edges = 0;
    size_t off = 0;  // scratch offset in the session's block
    for (int k = 0; k < n; k++) {
        const mrpop_batch_item *it = &items[k];
        mrpop_server::Step &st = steps[n_steps];
        st = mrpop_server::Step{};
        st.session = ss;
        int A = 0;
        const mrpop_status r = mrpop::make_params(it->scene, it->robots, it->q0, it->q1, it->n_edges, it->granularity,
                                                  it->rule, it->range, it->flags, it->arm, it->valid, it->first_hit,
                                                  nullptr, nullptr, st.p, A, st.smem);
        if (r != MRPOP_OK) return r;
        if (it->n_edges > ss->max_edges || it->granularity > ss->max_g || A > ss->arms)
            return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: step larger than the session was opened for");
        edges += it->n_edges;
        if (it->n_edges == 0) continue;
        const size_t need = mrpop::split_scratch_bytes(it->n_edges, it->granularity, A);
        if (off + need > ss->bytes)
            return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: the steps' scratch exceeds the session's");
        st.arms = A;
        st.spl = it->granularity > 32 ? 2 : 1;
        st.seg = it->rule != MRPOP_RULE_PLAIN;
        st.n_chunks = (int)((it->n_edges + kChunkEdges - 1) / kChunkEdges);
        mrpop::set_split_scratch(st.p, s->d_arena + ss->offset + off, it->n_edges, it->granularity, A);
        off = round_up(off + need);
        n_steps++;
    }
    if (edges > ss->max_edges)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: the steps' edges exceed the session's max_edges");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (ss->in_flight) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: the previous step is not done");
        ss->result = MRPOP_OK;
        ss->error.clear();
        if (!n_steps) return MRPOP_OK;
        ss->in_flight = n_steps;
        const int64_t now = host_ns();
        for (int k = 0; k < n_steps; k++) {
            steps[k].t_submit = now;
            s->pending.push_back(steps[k]);
        }
        s->n_pending.store((int64_t)s->pending.size(), std::memory_order_relaxed);
    }
    s->work_cv.notify_one();
    return MRPOP_OK;
}

mrpop_status mrpop_session_submit(mrpop_session *ss, const mrpop_batch_item *it) {
    if (!it) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_submit: null argument");
    return mrpop_session_submit_many(ss, it, 1);
}

mrpop_status mrpop_session_wait(mrpop_session *ss, int64_t timeout_ms) {
    if (!ss) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_wait: null session");
    mrpop_server *s = ss->server;
    std::unique_lock<std::mutex> lk(s->mu);
    if (timeout_ms < 0) {
        ss->done_cv.wait(lk, [&] { return ss->in_flight == 0; });
    } else if (!ss->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return ss->in_flight == 0; })) {
        return fail(MRPOP_ERR_DEVICE_TIMEOUT, "session_wait: the step is still running");
    }
    if (ss->result != MRPOP_OK) return fail(ss->result, ss->error);
    return MRPOP_OK;
}

mrpop_status mrpop_session_close(mrpop_session *ss) {
    if (!ss) return MRPOP_OK;
    mrpop_server *s = ss->server;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        ss->done_cv.wait(lk, [&] { return ss->in_flight == 0; });
        arena_give(s->free_blocks, s->in_use, ss->offset, ss->bytes);
        arena_give(s->free_host, s->host_in_use, ss->host_off, ss->host_bytes);
    }
    s->room_cv.notify_all();
    delete ss;
    return MRPOP_OK;
}

mrpop_status mrpop_session_host_buffers(mrpop_session *ss, float **q0, float **q1, uint8_t **valid,
                                        int32_t **first_hit) {
    if (!ss) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_host_buffers: null session");
    if (q0) *q0 = ss->h_q0;
    if (q1) *q1 = ss->h_q1;
    if (valid) *valid = ss->h_valid;
    if (first_hit) *first_hit = ss->h_first;
    return MRPOP_OK;
}

}  // extern "C"

namespace {

// The planner's validator for a session: the step's edges go through the
// session's host buffers, which the kernels read and write in place.
struct SessionValidator {
    mrpop_session *ss;
    const mrpop_scene *scene;
    const mrpop_robotset *robots;
    uint32_t flags;
    int dof;
};

int session_validate(void *ctx, const float *q0, const float *q1, int64_t n, int g, int rule, float range,
                     uint8_t *valid, int32_t *first_hit) {
    auto *v = static_cast<SessionValidator *>(ctx);
    mrpop_session *ss = v->ss;
    if (n > ss->max_edges) return MRPOP_ERR_INVALID_ARGUMENT;
    std::memcpy(ss->h_q0, q0, (size_t)n * v->dof * sizeof(float));
    std::memcpy(ss->h_q1, q1, (size_t)n * v->dof * sizeof(float));
    mrpop_batch_item it{};
    it.scene = v->scene;
    it.robots = v->robots;
    it.q0 = ss->h_q0;
    it.q1 = ss->h_q1;
    it.n_edges = n;
    it.granularity = g;
    it.flags = v->flags;
    it.arm = -1;
    it.valid = ss->h_valid;
    it.first_hit = ss->h_first;
    it.rule = rule;
    it.range = range;
    mrpop_status st = mrpop_session_submit(ss, &it);
    if (st == MRPOP_OK) st = mrpop_session_wait(ss, -1);
    if (st != MRPOP_OK) return st;
    std::memcpy(valid, ss->h_valid, (size_t)n);
    std::memcpy(first_hit, ss->h_first, (size_t)n * sizeof(int32_t));
    return MRPOP_OK;
}

}  // namespace

extern "C" mrpop_status mrpop_session_plan(mrpop_session *ss, const mrpop_scene *scene, const mrpop_robotset *robots,
                                           uint32_t flags, const float *start, const float *goal,
                                           const mrpop_plan_settings *settings, float *path_out,
                                           int64_t max_waypoints, mrpop_plan_result *out) {
    if (!ss || !settings) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_plan: null argument");
    if (std::max(settings->batch, settings->shortcut_pairs) > ss->max_edges || settings->granularity > ss->max_g)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_plan: the session is smaller than the plan's steps");
    if (mrpop::robotset_arms(robots) != ss->arms)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_plan: the robot set's arm count differs from the session's");
    SessionValidator v{ss, scene, robots, flags, 7 * ss->arms};
    return mrpop_plan(ss->arms, start, goal, settings, session_validate, &v, path_out, max_waypoints, out);
}

namespace {

// Validation of the dRRT planner's checks through a session: each call is cut
// into steps of at most the session's edge count, each submitted and waited
// for in turn (single-arm roadmap checks use 7 floats per configuration).
struct SessionChecker {
    mrpop_session *ss;
    const mrpop_scene *scene;
    const mrpop_robotset *robots;
};

int session_check(void *ctx, const float *q0, const float *q1, int64_t n, int g, int rule, float range,
                  uint32_t flags, int arm, uint8_t *valid, int32_t *first_hit) {
    auto *c = static_cast<SessionChecker *>(ctx);
    mrpop_session *ss = c->ss;
    const int dof = 7 * (arm >= 0 ? 1 : ss->arms);
    for (int64_t e0 = 0; e0 < n; e0 += ss->max_edges) {
        const int64_t m = std::min<int64_t>(ss->max_edges, n - e0);
        std::memcpy(ss->h_q0, q0 + e0 * dof, (size_t)m * dof * sizeof(float));
        std::memcpy(ss->h_q1, q1 + e0 * dof, (size_t)m * dof * sizeof(float));
        mrpop_batch_item it{};
        it.scene = c->scene;
        it.robots = c->robots;
        it.q0 = ss->h_q0;
        it.q1 = ss->h_q1;
        it.n_edges = m;
        it.granularity = g;
        it.flags = flags;
        it.arm = arm;
        it.valid = ss->h_valid;
        it.first_hit = ss->h_first;
        it.rule = rule;
        it.range = range;
        mrpop_status st = mrpop_session_submit(ss, &it);
        if (st == MRPOP_OK) st = mrpop_session_wait(ss, -1);
        if (st != MRPOP_OK) return st;
        std::memcpy(valid + e0, ss->h_valid, (size_t)m);
        std::memcpy(first_hit + e0, ss->h_first, (size_t)m * sizeof(int32_t));
    }
    return MRPOP_OK;
}

// A group of the planner's checks: as many as fit the session's buffers
// (edges, endpoint floats, MRPOP_SESSION_MAX_ITEMS) are packed into them and
// submitted together; a check larger than the session goes alone, in steps.
int session_check_many(void *ctx, const mrpop_check_call *calls, int n) {
    auto *c = static_cast<SessionChecker *>(ctx);
    mrpop_session *ss = c->ss;
    const int64_t qcap = ss->max_edges * 7 * ss->arms;
    int i = 0;
    while (i < n) {
        if (calls[i].n_edges > ss->max_edges) {
            const mrpop_check_call &f = calls[i];
            const int rc = session_check(ctx, f.q0, f.q1, f.n_edges, f.granularity, f.rule, f.range, f.flags, f.arm,
                                         f.valid, f.first_hit);
            if (rc) return rc;
            i++;
            continue;
        }
        mrpop_batch_item items[MRPOP_SESSION_MAX_ITEMS];
        int64_t e_off[MRPOP_SESSION_MAX_ITEMS];
        int64_t e_at = 0, q_at = 0;
        int k = 0, j = i;
        for (; j < n && k < MRPOP_SESSION_MAX_ITEMS; j++, k++) {
            const mrpop_check_call &f = calls[j];
            const int dof = 7 * (f.arm >= 0 ? 1 : ss->arms);
            if (f.n_edges > ss->max_edges || e_at + f.n_edges > ss->max_edges || q_at + f.n_edges * dof > qcap) break;
            std::memcpy(ss->h_q0 + q_at, f.q0, (size_t)f.n_edges * dof * sizeof(float));
            std::memcpy(ss->h_q1 + q_at, f.q1, (size_t)f.n_edges * dof * sizeof(float));
            mrpop_batch_item &it = items[k];
            it = mrpop_batch_item{};
            it.scene = c->scene;
            it.robots = c->robots;
            it.q0 = ss->h_q0 + q_at;
            it.q1 = ss->h_q1 + q_at;
            it.n_edges = f.n_edges;
            it.granularity = f.granularity;
            it.flags = f.flags;
            it.arm = f.arm;
            it.valid = ss->h_valid + e_at;
            it.first_hit = ss->h_first + e_at;
            it.rule = f.rule;
            it.range = f.range;
            e_off[k] = e_at;
            e_at += f.n_edges;
            q_at += f.n_edges * dof;
        }
        mrpop_status st = mrpop_session_submit_many(ss, items, k);
        if (st == MRPOP_OK) st = mrpop_session_wait(ss, -1);
        if (st != MRPOP_OK) return st;
        for (int m = 0; m < k; m++) {
            const mrpop_check_call &f = calls[i + m];
            std::memcpy(f.valid, ss->h_valid + e_off[m], (size_t)f.n_edges);
            std::memcpy(f.first_hit, ss->h_first + e_off[m], (size_t)f.n_edges * sizeof(int32_t));
        }
        i = j;
    }
    return MRPOP_OK;
}

}  // namespace

extern "C" mrpop_status mrpop_session_drrt(mrpop_session *ss, const mrpop_scene *scene, const mrpop_robotset *robots,
                                           const float *start, const float *goals, int num_goals,
                                           const mrpop_drrt_settings *settings, float *path_out,
                                           int64_t max_waypoints, mrpop_drrt_solution_fn on_solution,
                                           void *solution_ctx, mrpop_drrt_result *out) {
    if (!ss || !settings) return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_drrt: null argument");
    if (settings->granularity > ss->max_g)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_drrt: the session's granularity is below the settings'");
    if (mrpop::robotset_arms(robots) != ss->arms)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "session_drrt: the robot set's arm count differs from the session's");
    SessionChecker c{ss, scene, robots};
    return mrpop::drrt_run(ss->arms, session_check, session_check_many, &c, true, start, goals, num_goals, settings, path_out,
                           max_waypoints, on_solution, solution_ctx, out);
}
