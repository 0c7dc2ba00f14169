// drrt.cu -- the reference's dRRT / AO-x planner on the batched validator.
//
// The reference (dRRT::solve, src/planning/pop_planner.cu:739-1030) runs its
// planner as persistent kernels: a cooperative roadmap kernel
// (build_roadmap, pop_planner.cu:173-218 -> roadmap_interior.cuh:36-341) and
// rrtc<Robot> with 300 blocks of 4g threads (pop_planner.cu:220-737), each
// block validating one edge at a time.  Here the host steps every block's
// attempt of an iteration together, and each kind of edge check of the
// iteration is one batched call into the validator:
//   roadmap round   per arm: every block's 230 samples node-checked in one
//                   call (single-arm form, g = 1: the reference checks the
//                   node as g identical samples, all of which reach the
//                   detailed phase, so the verdict is the same), then every
//                   (old node, new node) pair within `range` in one call
//   rrtc iteration  every block's extend edge (self only) in one call, then
//                   every new node's connect edge (connect segmentation) in one
//   simplification  all B-spline candidate edges of a step in one call, and
//                   all shortcut pairs (i, i+2 .. i+16) in one call before the
//                   shortcut dynamic programme runs on the host
// Nearest-neighbour searches over the trees (pop_planner.cu:472-507, 630-663)
// run as one kernel launch per tree and query chunk, over device copies of
// the trees that grow as nodes are added.
//
// Where the reference's blocks race (atomicAdd node indices, the
// atomicCAS(solved) winner), attempts are taken in block order within an
// iteration; the rest follows the reference step for step, including its
// quirks: a new node's cost is its parent's cost plus the distance to the
// random sample (pop_planner.cu:531), a connect node's cost adds only
// 1/n_ext of the connect distance (:717), the first-pass relaunch loop
// (:958-984), the PHS transform (:290-341, 398-442), and the path from the
// goal to the start (path_processing.cu:11-70).
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "launch.h"

namespace {

using Clock = std::chrono::steady_clock;
int64_t ns_since(Clock::time_point t0) {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
}

// Panda joint limits as q = u * s_m + s_a (Robots.hh:13-23).
constexpr float kSm[7] = {5.9342f, 3.6652f, 5.9342f, 3.2289f, 5.9342f, 3.9095999999999997f, 5.9342f};
constexpr float kSa[7] = {-2.9671f, -1.8326f, -2.9671f, -3.1416f, -2.9671f, -0.0873f, -2.9671f};
constexpr int kRoadmapIters = 230;        // ROADMAP_BUILD_ITER (roadmap_interior.cuh:20)
constexpr int kMaxRoadmap = 100000;       // MAX_ROADMAP_SIZE (roadmap_interior.cuh:21)
constexpr float kExistSq = 1e-5f;         // a node "already exists" within this squared distance (:526)
constexpr int kShortcutSpan = 16;         // the simplify kernel's 16 blocks (pop_planner.cu:911)
constexpr int kNNChunk = 16;              // queries per nearest-neighbour job (one grid row of blocks)

// splitmix64 (Steele, Lea, Flood 2014) streams; uniform() is in (0, 1).
struct Rng {
    uint64_t s = 0;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return ((float)(next() >> 40) + 0.5f) * 0x1.0p-24f; }
};

Rng rng_stream(uint64_t seed, uint64_t kind, uint64_t index) {
    Rng r{seed ^ (kind * 0xD1B54A32D192ED03ull) ^ ((index + 1) * 0xA0761D6478BD642Full)};
    r.next();
    return r;
}

// The reference's distance arithmetic (utils.cuh:123-144): ans += d * d, which
// its compiler fuses; written as fmaf so host and device round alike.
inline float sq_l2(const float *a, const float *b, int dim) {
    float s = 0.0f;
    for (int i = 0; i < dim; i++) {
        const float d = a[i] - b[i];
        s = fmaf(d, d, s);
    }
    return s;
}
inline float l2(const float *a, const float *b, int dim) { return sqrtf(sq_l2(a, b, dim)); }

// compute_angle (utils.cuh:63-95): the angle at c1 between c2 - c1 and c3 - c1.
float angle_at(const float *c1, const float *c2, const float *c3, int dim) {
    float v[7], w[7];
    for (int t = 0; t < dim; t++) {
        v[t] = c2[t] - c1[t];
        w[t] = c3[t] - c1[t];
    }
    float dot = 0.0f, vn = 0.0f, wn = 0.0f;
    for (int t = 0; t < dim; t++) dot = fmaf(v[t], w[t], dot);
    for (int t = 0; t < dim; t++) {
        vn = fmaf(v[t], v[t], vn);
        wn = fmaf(w[t], w[t], wn);
    }
    vn = sqrtf(vn);
    wn = sqrtf(wn);
    if (vn < 1e-8f || wn < 1e-8f) return 0.0f;
    float c = dot / (vn * wn);
    c = fminf(1.0f, fmaxf(-1.0f, c));
    return acosf(c);
}

// ---------------------------------------------------------------------------
// Per-arm roadmap: nodes, sorted adjacency lists, union-find components.
// ---------------------------------------------------------------------------
struct Roadmap {
    std::vector<float> q;  // [n][7]
    std::vector<std::vector<int>> adj;
    std::vector<int> uf;
    int64_t edges = 0;
    int size() const { return (int)adj.size(); }
    const float *node(int i) const { return &q[(size_t)i * 7]; }
    int add(const float *x) {
        q.insert(q.end(), x, x + 7);
        adj.emplace_back();
        uf.push_back(size() - 1);
        return size() - 1;
    }
    int find(int x) {
        while (uf[x] != x) {
            uf[x] = uf[uf[x]];
            x = uf[x];
        }
        return x;
    }
    void link(int a, int b) {  // a < b: b is the newer node
        adj[a].push_back(b);
        adj[b].push_back(a);
        edges++;
        const int ra = find(a), rb = find(b);
        if (ra != rb) uf[std::max(ra, rb)] = std::min(ra, rb);
    }
};

// ---------------------------------------------------------------------------
// Trees: host master copy plus a device copy for the nearest-neighbour kernel
// (rows of dim + 1 floats: the configuration, then the node's cost).
// ---------------------------------------------------------------------------
struct Tree {
    int dim = 0, arms = 0;
    std::vector<float> q, cost, rows;
    std::vector<int> parent, rid;  // rid [n][arms]: roadmap vertex of each arm, -1 for connect nodes
    std::unordered_map<uint64_t, std::vector<int>> by_ids;
    std::vector<int> connect_nodes;
    // device copy: rows [0, dirty_from) are current there
    float *d_rows = nullptr;
    size_t d_bytes = 0;
    int64_t dirty_from = 0;

    int64_t size() const { return (int64_t)parent.size(); }
    const float *node(int64_t i) const { return &q[(size_t)i * dim]; }
    static uint64_t key(const int *ids, int arms) {
        uint64_t h = 0xCBF29CE484222325ull;
        for (int a = 0; a < arms; a++) {
            h ^= (uint64_t)(uint32_t)ids[a];
            h *= 0x100000001B3ull;
        }
        return h;
    }
    void clear() {
        q.clear();
        cost.clear();
        rows.clear();
        parent.clear();
        rid.clear();
        by_ids.clear();
        connect_nodes.clear();
        dirty_from = 0;
    }
    int add(const float *x, int par, float c, const int *ids) {
        const int i = (int)size();
        q.insert(q.end(), x, x + dim);
        cost.push_back(c);
        rows.insert(rows.end(), x, x + dim);
        rows.push_back(c);
        parent.push_back(par < 0 ? i : par);
        if (ids) {
            rid.insert(rid.end(), ids, ids + arms);
            by_ids[key(ids, arms)].push_back(i);
        } else {
            rid.insert(rid.end(), (size_t)arms, -1);
            connect_nodes.push_back(i);
        }
        return i;
    }
    void set_cost(int i, float c) {
        cost[i] = c;
        rows[(size_t)i * (dim + 1) + dim] = c;
        dirty_from = std::min<int64_t>(dirty_from, i);
    }
    // An existing node within the reference's 1e-5 squared distance of x
    // (pop_planner.cu:522-528), looked up by roadmap-vertex tuple and among
    // the connect nodes; -1 if none.
    int existing(const float *x, const int *ids) const {
        auto it = by_ids.find(key(ids, arms));
        if (it != by_ids.end())
            for (int i : it->second)
                if (sq_l2(node(i), x, dim) <= kExistSq) return i;
        for (int i : connect_nodes)
            if (sq_l2(node(i), x, dim) <= kExistSq) return i;
        return -1;
    }
    // One copy of the rows added or re-costed since the last one.
    cudaError_t sync_device(cudaStream_t s) {
        const int64_t n = size();
        const size_t row = (size_t)(dim + 1) * sizeof(float);
        if ((size_t)n * row > d_bytes) {
            size_t bytes = std::max<size_t>(d_bytes * 2, (size_t)65536 * row);
            while (bytes < (size_t)n * row) bytes *= 2;
            float *nr = nullptr;
            const cudaError_t e = cudaMalloc(&nr, bytes);
            if (e != cudaSuccess) return e;
            if (d_rows) cudaFree(d_rows);
            d_rows = nr;
            d_bytes = bytes;
            dirty_from = 0;
        }
        cudaError_t e = cudaSuccess;
        if (n > dirty_from)
            e = cudaMemcpyAsync(d_rows + dirty_from * (dim + 1), &rows[(size_t)dirty_from * (dim + 1)],
                                (size_t)(n - dirty_from) * (dim + 1) * sizeof(float), cudaMemcpyHostToDevice, s);
        dirty_from = n;
        return e;
    }
};

// ---------------------------------------------------------------------------
// Nearest-neighbour kernel: for each query, the lowest (squared distance,
// index) among the nodes that pass the query's filter.
//   mode 0 (extend search): node cost < bound      (pop_planner.cu:479)
//   mode 1 (connect search): sqrt(distance) < bound (pop_planner.cu:642)
// One thread per node (held in registers); queries in shared memory.
// ---------------------------------------------------------------------------
constexpr int kNNMaxJobs = 64;

// One launch for the query chunks of both trees: job j = (tree, first query,
// queries); blockIdx.y is the job, blockIdx.x a block of 256 nodes.
struct NNLaunch {
    const float *rows[2];  // per tree [n][dim + 1]: configuration, cost
    long long n[2];
    const float *qx, *qb;  // every job's queries [.][dim] and bounds [.]
    unsigned long long *best;
    int mode;
    int tree[kNNMaxJobs], q0[kNNMaxJobs], nq[kNNMaxJobs];
};

// A thread holds kNNNodes nodes; the query rows are read from shared memory as
// float4.  The searches are latency-bound (trees of a few thousand nodes leave
// most of the device idle), so queries go in jobs of kNNChunk, each job a row
// of blocks: more blocks, fewer queries per thread.
constexpr int kNNNodes = 1;

template <int DIM>
__global__ void __launch_bounds__(256) tree_nn_kernel(const __grid_constant__ NNLaunch L) {
    constexpr int DIMP = (DIM + 3) / 4 * 4;  // query row stride (float4 loads)
    __shared__ __align__(16) float sx[kNNChunk * DIMP];
    __shared__ float sb[kNNChunk];
    __shared__ unsigned long long red[8][kNNChunk];
    const int job = blockIdx.y, t = L.tree[job], nq = L.nq[job];
    const long long n = L.n[t];
    const long long i0 = (long long)blockIdx.x * blockDim.x * kNNNodes + threadIdx.x;
    if ((long long)blockIdx.x * blockDim.x * kNNNodes >= n) return;  // whole block past this tree's nodes
    const float *qx = L.qx + (size_t)L.q0[job] * DIM, *qb = L.qb + L.q0[job];
    for (int j = threadIdx.x; j < nq * DIMP; j += blockDim.x) {
        const int q = j / DIMP, d = j - q * DIMP;
        sx[j] = d < DIM ? qx[q * DIM + d] : 0.0f;
    }
    for (int j = threadIdx.x; j < nq; j += blockDim.x) sb[j] = qb[j];
    __syncthreads();
    float x[kNNNodes][DIM], c[kNNNodes];
    bool have[kNNNodes];
#pragma unroll
    for (int m = 0; m < kNNNodes; m++) {
        const long long i = i0 + (long long)m * blockDim.x;
        have[m] = i < n;
        const float *row = L.rows[t] + (size_t)(have[m] ? i : 0) * (DIM + 1);
#pragma unroll
        for (int d = 0; d < DIM; d++) x[m][d] = have[m] ? row[d] : 0.0f;
        c[m] = have[m] ? row[DIM] : 0.0f;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float4 *sx4 = reinterpret_cast<const float4 *>(sx);
    for (int q = 0; q < nq; q++) {
        float s[kNNNodes];
#pragma unroll
        for (int m = 0; m < kNNNodes; m++) s[m] = 0.0f;
#pragma unroll
        for (int d4 = 0; d4 < DIMP / 4; d4++) {
            const float4 v = sx4[q * (DIMP / 4) + d4];
            const float qv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int d = 4 * d4 + r;
                if (d < DIM) {
#pragma unroll
                    for (int m = 0; m < kNNNodes; m++) {
                        const float u = x[m][d] - qv[r];
                        s[m] = __fmaf_rn(u, u, s[m]);
                    }
                }
            }
        }
        unsigned long long key = ~0ull;
#pragma unroll
        for (int m = 0; m < kNNNodes; m++) {
            const bool ok = have[m] && (L.mode == 0 ? c[m] < sb[q] : sqrtf(s[m]) < sb[q]) && s[m] < FLT_MAX;
            const unsigned long long k = ((unsigned long long)__float_as_uint(s[m]) << 32) |
                                         (unsigned long long)(unsigned)(i0 + (long long)m * blockDim.x);
            if (ok && k < key) key = k;
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
            key = other < key ? other : key;
        }
        if (lane == 0) red[warp][q] = key;
    }
    __syncthreads();
    unsigned long long *best = L.best + L.q0[job];
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        unsigned long long k = red[0][q];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) k = red[w][q] < k ? red[w][q] : k;
        if (k != ~0ull) atomicMin(&best[q], k);
    }
}

cudaError_t launch_tree_nn(int dim, const NNLaunch &L, int njobs, long long max_n, cudaStream_t s) {
    const long long per_block = 256LL * kNNNodes;
    const dim3 grid((unsigned)std::max<long long>(1, (max_n + per_block - 1) / per_block), (unsigned)njobs);
    switch (dim) {
        case 7: tree_nn_kernel<7><<<grid, 256, 0, s>>>(L); break;
        case 14: tree_nn_kernel<14><<<grid, 256, 0, s>>>(L); break;
        case 21: tree_nn_kernel<21><<<grid, 256, 0, s>>>(L); break;
        case 28: tree_nn_kernel<28><<<grid, 256, 0, s>>>(L); break;
        case 35: tree_nn_kernel<35><<<grid, 256, 0, s>>>(L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Roadmap neighbour pairs: for every new node j in [n_old, n) and every node
// i < j, the pair (i, j) when the reference's distance (utils.cuh:123-133;
// node i minus node j, squares fused) is below `range`.  Pairs go to `out` in
// no particular order (the host sorts them); `count` receives how many there
// are, also beyond `cap`, so the caller can grow the buffer and search again.
__global__ void __launch_bounds__(256) roadmap_pairs_kernel(const float *__restrict__ q, int n_old, int n,
                                                            float range, int2 *__restrict__ out,
                                                            unsigned int *__restrict__ count, unsigned int cap) {
    const int j = n_old + (int)blockIdx.y;
    if (j >= n) return;
    float x[7];
#pragma unroll
    for (int d = 0; d < 7; d++) x[d] = q[(size_t)j * 7 + d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < j; i += gridDim.x * blockDim.x) {
        float s = 0.0f;
#pragma unroll
        for (int d = 0; d < 7; d++) {
            const float t = q[(size_t)i * 7 + d] - x[d];
            s = __fmaf_rn(t, t, s);
        }
        if (sqrtf(s) < range) {
            const unsigned int k = atomicAdd(count, 1u);
            if (k < cap) out[k] = make_int2(i, j);
        }
    }
}

cudaError_t launch_roadmap_pairs(const float *q, int n_old, int n, float range, int2 *out, unsigned int *count,
                                 unsigned int cap, cudaStream_t s) {
    const int n_new = n - n_old;
    if (n_new <= 0) return cudaSuccess;
    const unsigned gx = (unsigned)std::min<int64_t>(64, ((int64_t)n + 255) / 256);
    for (int y0 = 0; y0 < n_new; y0 += 65535) {  // gridDim.y limit
        const int ny = std::min(65535, n_new - y0);
        roadmap_pairs_kernel<<<dim3(gx, (unsigned)ny), 256, 0, s>>>(q, n_old + y0, n_old + y0 + ny, range, out,
                                                                    count, cap);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Validation on this library's kernels: page-locked staging buffers that the
// kernels read and write in place (mrpop_validate_edges_host).
// ---------------------------------------------------------------------------
struct GpuChecker {
    const mrpop_scene *scene = nullptr;
    const mrpop_robotset *robots = nullptr;
    mrpop_workspace *ws = nullptr;
    float *q0 = nullptr, *q1 = nullptr;
    uint8_t *valid = nullptr;
    int32_t *first = nullptr;
    size_t cap_f = 0, cap_e = 0;
    std::vector<cudaStream_t> group_streams;  // one per check of a group (call_many)

    ~GpuChecker() {
        for (cudaStream_t st : group_streams) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        if (q0) cudaFreeHost(q0);
        if (q1) cudaFreeHost(q1);
        if (valid) cudaFreeHost(valid);
        if (first) cudaFreeHost(first);
        if (ws) mrpop_workspace_destroy(ws);
    }
    static int call(void *ctx, const float *a, const float *b, int64_t n, int g, int rule, float range,
                    uint32_t flags, int arm, uint8_t *valid_out, int32_t *first_out) {
        GpuChecker &c = *static_cast<GpuChecker *>(ctx);
        const int dof = 7 * (arm >= 0 ? 1 : mrpop::robotset_arms(c.robots));
        const size_t nf = (size_t)n * dof;
        const int rc = c.reserve(nf, (size_t)n);
        if (rc) return rc;
        std::memcpy(c.q0, a, nf * sizeof(float));
        std::memcpy(c.q1, b, nf * sizeof(float));
        const mrpop_status st = mrpop_validate_edges_host(c.ws, c.scene, c.robots, c.q0, c.q1, n, g, flags, arm, rule,
                                                          range, c.valid, c.first);
        if (st != MRPOP_OK) return st;
        std::memcpy(valid_out, c.valid, (size_t)n);
        std::memcpy(first_out, c.first, (size_t)n * sizeof(int32_t));
        return 0;
    }

    // Page-locked staging of at least nf floats per endpoint array and ne edges.
    int reserve(size_t nf, size_t ne) {
        if (nf > cap_f) {
            cudaFreeHost(q0);
            cudaFreeHost(q1);
            q0 = q1 = nullptr;
            cap_f = 0;
            const size_t cap = std::max(nf, (size_t)1 << 16) * 2;
            if (cudaHostAlloc(&q0, cap * sizeof(float), cudaHostAllocDefault) != cudaSuccess ||
                cudaHostAlloc(&q1, cap * sizeof(float), cudaHostAllocDefault) != cudaSuccess)
                return mrpop::fail_status(MRPOP_ERR_OUT_OF_MEMORY, "drrt: page-locked staging buffers");
            cap_f = cap;
        }
        if (ne > cap_e) {
            cudaFreeHost(valid);
            cudaFreeHost(first);
            valid = nullptr;
            first = nullptr;
            cap_e = 0;
            const size_t cap = std::max(ne, (size_t)1 << 12) * 2;
            if (cudaHostAlloc(&valid, cap, cudaHostAllocDefault) != cudaSuccess ||
                cudaHostAlloc(&first, cap * sizeof(int32_t), cudaHostAllocDefault) != cudaSuccess)
                return mrpop::fail_status(MRPOP_ERR_OUT_OF_MEMORY, "drrt: page-locked staging buffers");
            cap_e = cap;
        }
        return 0;
    }

    // A group of checks (a roadmap round's checks of every arm): each is
    // enqueued on a stream of its own before one wait for all, so that they
    // run side by side on the device instead of one call after another.  The
    // kernels read the staged endpoints and write the verdicts in place.
    static int call_many(void *ctx, const mrpop_check_call *calls, int n) {
        GpuChecker &c = *static_cast<GpuChecker *>(ctx);
        const int arms = mrpop::robotset_arms(c.robots);
        size_t nf = 0, ne = 0;
        for (int i = 0; i < n; i++) {
            nf += (size_t)calls[i].n_edges * 7 * (calls[i].arm >= 0 ? 1 : arms);
            ne += (size_t)calls[i].n_edges;
        }
        int rc = c.reserve(nf, ne);
        if (rc) return rc;
        const int ns = std::min(n, MRPOP_MAX_ARMS);
        while ((int)c.group_streams.size() < ns) {
            cudaStream_t st = nullptr;
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
                return mrpop::fail_status(MRPOP_ERR_CUDA, "drrt: check streams");
            c.group_streams.push_back(st);
        }
        float *d0 = nullptr, *d1 = nullptr;
        uint8_t *dv = nullptr;
        int32_t *df = nullptr;
        if (cudaHostGetDevicePointer((void **)&d0, c.q0, 0) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&d1, c.q1, 0) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&dv, c.valid, 0) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&df, c.first, 0) != cudaSuccess)
            return mrpop::fail_status(MRPOP_ERR_CUDA, "drrt: staging device pointers");
        size_t fo = 0, eo = 0;
        mrpop_status st = MRPOP_OK;
        for (int i = 0; i < n && st == MRPOP_OK; i++) {
            const mrpop_check_call &k = calls[i];
            const size_t f = (size_t)k.n_edges * 7 * (k.arm >= 0 ? 1 : arms);
            std::memcpy(c.q0 + fo, k.q0, f * sizeof(float));
            std::memcpy(c.q1 + fo, k.q1, f * sizeof(float));
            st = mrpop::run_validator(c.scene, c.robots, d0 + fo, d1 + fo, k.n_edges, k.granularity, k.rule, k.range,
                                      k.flags, k.arm, dv + eo, df + eo, nullptr, nullptr, c.group_streams[i % ns],
                                      nullptr);
            fo += f;
            eo += (size_t)k.n_edges;
        }
        cudaError_t e = cudaSuccess;
        for (int i = 0; i < ns; i++) {
            const cudaError_t ei = cudaStreamSynchronize(c.group_streams[i]);
            if (e == cudaSuccess) e = ei;
        }
        if (st != MRPOP_OK) return st;
        if (e != cudaSuccess) return mrpop::fail_status(MRPOP_ERR_CUDA, "drrt: grouped checks");
        eo = 0;
        for (int i = 0; i < n; i++) {
            std::memcpy(calls[i].valid, c.valid + eo, (size_t)calls[i].n_edges);
            std::memcpy(calls[i].first_hit, c.first + eo, (size_t)calls[i].n_edges * sizeof(int32_t));
            eo += (size_t)calls[i].n_edges;
        }
        return 0;
    }
};

// ---------------------------------------------------------------------------
// Device resources of one solve (its stream, the trees' device rows, the
// nearest-neighbour staging block, the roadmap mirrors and pair buffers).
// Solves take them from a per-process pool and give them back, so a stream of
// solves allocates and frees nothing once warm: cudaFree waits for the whole
// device, and page-locked allocations take milliseconds.
// ---------------------------------------------------------------------------
struct DeviceWork {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t done_ev = nullptr;
    float *rows[2] = {nullptr, nullptr};
    size_t rows_bytes[2] = {0, 0};
    void *d_stage = nullptr, *h_stage = nullptr;
    size_t stage_cap = 0;
    std::vector<float *> d_rm;  // per arm, [cap][7]
    std::vector<int64_t> d_rm_cap;
    int2 *d_pairs = nullptr;
    size_t d_pairs_cap = 0;
    unsigned int *d_npairs = nullptr, *h_npairs = nullptr;

    void free_all() {
        if (stream) cudaStreamSynchronize(stream);
        for (float *&p : rows)
            if (p) cudaFree(p);
        if (d_stage) cudaFree(d_stage);
        if (h_stage) cudaFreeHost(h_stage);
        for (float *p : d_rm)
            if (p) cudaFree(p);
        if (d_pairs) cudaFree(d_pairs);
        if (d_npairs) cudaFree(d_npairs);
        if (h_npairs) cudaFreeHost(h_npairs);
        if (done_ev) cudaEventDestroy(done_ev);
        if (stream) cudaStreamDestroy(stream);
        *this = DeviceWork{};
    }
};

constexpr size_t kPoolKeep = 64;  // idle sets kept; more are freed on return
std::mutex g_pool_mu;
std::vector<DeviceWork> g_pool;

DeviceWork take_work(int device) {
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        for (size_t i = g_pool.size(); i-- > 0;)
            if (g_pool[i].device == device) {
                DeviceWork w = std::move(g_pool[i]);
                g_pool.erase(g_pool.begin() + (ptrdiff_t)i);
                return w;
            }
    }
    DeviceWork w;
    w.device = device;
    return w;
}

void give_work(DeviceWork &&w) {
    if (w.stream && cudaStreamSynchronize(w.stream) != cudaSuccess) {
        w.free_all();  // a failed stream is not reused
        return;
    }
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        if (g_pool.size() < kPoolKeep) {
            g_pool.push_back(std::move(w));
            return;
        }
    }
    w.free_all();
}

// ---------------------------------------------------------------------------
// The planner.
// ---------------------------------------------------------------------------
struct Solver {
    mrpop_drrt_settings S;
    int arms = 0, dim = 0, g = 0, num_goals = 0;
    int nthreads = 1;  // OpenMP threads of the host work
    mrpop_check_fn validate = nullptr;
    mrpop::check_many_fn validate_many = nullptr;  // optional: a group of checks in one call
    void *vctx = nullptr;
    bool device_nn = false;
    bool pooled = false;  // device resources taken from the pool (returned by the destructor)
    cudaStream_t stream = nullptr;
    void *d_stage = nullptr, *h_stage = nullptr;  // nearest-neighbour staging block (device, page-locked)
    cudaEvent_t done_ev = nullptr;  // blocking-sync event (settings.blocking_wait)

    // Waits for the solve's stream: by spinning (the CUDA default), or, with
    // blocking_wait, asleep on a blocking-sync event, so that many concurrent
    // solves leave the host's cores to each other.
    cudaError_t wait_stream() {
        if (!S.blocking_wait) return cudaStreamSynchronize(stream);
        if (!done_ev) {
            const cudaError_t e = cudaEventCreateWithFlags(&done_ev, cudaEventBlockingSync | cudaEventDisableTiming);
            if (e != cudaSuccess) return e;
        }
        const cudaError_t e = cudaEventRecord(done_ev, stream);
        return e == cudaSuccess ? cudaEventSynchronize(done_ev) : e;
    }
    mrpop_drrt_result *R = nullptr;
    mrpop_drrt_solution_fn on_solution = nullptr;
    void *sctx = nullptr;

    std::vector<float> start, goals;
    std::vector<Roadmap> rm;
    std::vector<Rng> rm_rng;  // [arm][block]
    std::vector<Rng> blk_rng;  // per rrtc block
    Tree T[2];
    int roadmap_launches = 0;
    float best_cost = FLT_MAX;
    // the reference's result state (pop_planner.cu:34-50, path_simplification.cu:14-15)
    std::vector<float> path_out, raw_path;
    int path_total = 0;
    float cost_sym = 0.0f;
    int solved_iters = 0;
    int64_t sol_tree[2] = {0, 0};
    bool init_sol = false;
    float res_cost = 0.0f;
    std::vector<float> res_path;
    // scratch
    std::vector<float> a0, a1;
    std::vector<uint8_t> ok;
    std::vector<int32_t> fh;

    // Takes a pooled set of device resources (device_nn solves).
    cudaError_t adopt_device() {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        DeviceWork w = take_work(dev);
        if (!w.stream) {
            e = cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return e;
        }
        stream = w.stream;
        done_ev = w.done_ev;
        for (int t = 0; t < 2; t++) {
            T[t].d_rows = w.rows[t];
            T[t].d_bytes = w.rows_bytes[t];
            T[t].dirty_from = 0;
        }
        d_stage = w.d_stage;
        h_stage = w.h_stage;
        d_cap_q = w.stage_cap;
        d_rm = std::move(w.d_rm);
        d_rm_cap = std::move(w.d_rm_cap);
        d_rm_up.assign(d_rm.size(), 0);
        d_pairs = w.d_pairs;
        d_pairs_cap = w.d_pairs_cap;
        d_npairs = w.d_npairs;
        h_npairs = w.h_npairs;
        pooled = true;
        return cudaSuccess;
    }

    ~Solver() {
        if (!pooled) return;
        DeviceWork w;
        cudaGetDevice(&w.device);
        w.stream = stream;
        w.done_ev = done_ev;
        for (int t = 0; t < 2; t++) {
            w.rows[t] = T[t].d_rows;
            w.rows_bytes[t] = T[t].d_bytes;
        }
        w.d_stage = d_stage;
        w.h_stage = h_stage;
        w.stage_cap = d_cap_q;
        w.d_rm = std::move(d_rm);
        w.d_rm_cap = std::move(d_rm_cap);
        w.d_pairs = d_pairs;
        w.d_pairs_cap = d_pairs_cap;
        w.d_npairs = d_npairs;
        w.h_npairs = h_npairs;
        give_work(std::move(w));
    }

    // Kind of a check for the statistics: roadmap (single-arm), extend
    // (composite plain), connect, B-spline, shortcut.
    static int check_kind(int rule, int arm) { return arm >= 0 ? 0 : rule == MRPOP_RULE_PLAIN ? 1 : 1 + rule; }

    int check(int64_t n, int rule, float range, uint32_t flags, int arm, int gran) {
        if (n == 0) return 0;
        ok.resize((size_t)n);
        fh.resize((size_t)n);
        const auto t0 = Clock::now();
        const int rc = validate(vctx, a0.data(), a1.data(), n, gran, rule, range, flags, arm, ok.data(), fh.data());
        const int64_t dt = ns_since(t0);
        R->validate_ns += dt;
        R->check_ns[check_kind(rule, arm)] += dt;
        R->check_calls[check_kind(rule, arm)]++;
        R->validate_calls++;
        R->edges_validated += n;
        return rc;
    }

    // A group of checks (calls with no edges are dropped): one call of
    // validate_many when the validator has it, else one validate call each.
    int check_many(std::vector<mrpop_check_call> &calls) {
        calls.erase(std::remove_if(calls.begin(), calls.end(), [](const mrpop_check_call &c) { return c.n_edges == 0; }),
                    calls.end());
        if (calls.empty()) return 0;
        const auto t0 = Clock::now();
        int rc = 0;
        if (validate_many) {
            rc = validate_many(vctx, calls.data(), (int)calls.size());
        } else {
            for (const auto &c : calls) {
                rc = validate(vctx, c.q0, c.q1, c.n_edges, c.granularity, c.rule, c.range, c.flags, c.arm, c.valid,
                              c.first_hit);
                if (rc) break;
            }
        }
        const int64_t dt = ns_since(t0);
        R->validate_ns += dt;
        R->check_ns[check_kind(calls[0].rule, calls[0].arm)] += dt;  // a group is of one kind
        for (const auto &c : calls) {
            R->check_calls[check_kind(c.rule, c.arm)]++;
            R->validate_calls++;
            R->edges_validated += c.n_edges;
        }
        return rc;
    }
    static mrpop_check_call plain_call(const float *q0, const float *q1, int64_t n, int g, int arm, uint8_t *valid,
                                       int32_t *first_hit) {
        mrpop_check_call c{};
        c.q0 = q0;
        c.q1 = q1;
        c.n_edges = n;
        c.granularity = g;
        c.rule = MRPOP_RULE_PLAIN;
        c.range = 0.0f;
        c.flags = MRPOP_CHECK_ENV | MRPOP_CHECK_SELF;
        c.arm = arm;
        c.valid = valid;
        c.first_hit = first_hit;
        return c;
    }

    // ---- nearest neighbours ------------------------------------------------
    // For both trees at once: idx[t][q] = the node of tree t nearest to
    // x[t][q] that passes the filter (lowest squared distance, then lowest
    // index), or -1; sqd[t][q] = its squared distance.  One upload, one launch
    // for every job of kNNChunk queries of both trees, one read-back.
    struct NNJob {
        std::vector<float> x, bound;
        std::vector<int> who, idx;
        std::vector<float> sqd;
        void clear() {
            x.clear();
            bound.clear();
            who.clear();
        }
    };
    size_t d_cap_q = 0;

    int nearest(NNJob *jobs, int mode) {
        const auto t0 = Clock::now();
        int nq_total = 0;
        for (int t = 0; t < 2; t++) {
            const int nq = (int)jobs[t].bound.size();
            jobs[t].idx.assign(nq, -1);
            jobs[t].sqd.assign(nq, FLT_MAX);
            nq_total += nq;
        }
        if (nq_total == 0) return 0;
        if (!device_nn) {
            for (int t = 0; t < 2; t++) {
                const Tree &tr = T[t];
                NNJob &J = jobs[t];
                const int nq = (int)J.bound.size();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
                for (int q = 0; q < nq; q++) {
                    const float *xq = &J.x[(size_t)q * dim];
                    uint64_t bestk = ~0ull;
                    for (int64_t i = 0; i < tr.size(); i++) {
                        const float sv = sq_l2(tr.node(i), xq, dim);
                        const bool pass = (mode == 0 ? tr.cost[i] < J.bound[q] : sqrtf(sv) < J.bound[q]) && sv < FLT_MAX;
                        if (!pass) continue;
                        uint32_t sb;
                        std::memcpy(&sb, &sv, 4);
                        const uint64_t k = ((uint64_t)sb << 32) | (uint64_t)(uint32_t)i;
                        bestk = std::min(bestk, k);
                    }
                    if (bestk != ~0ull) {
                        J.idx[q] = (int)(uint32_t)bestk;
                        const uint32_t sb = (uint32_t)(bestk >> 32);
                        std::memcpy(&J.sqd[q], &sb, 4);
                    }
                }
            }
            R->nn_ns += ns_since(t0);
            return 0;
        }
        // one staging block per search, uploaded with one copy: the result
        // words preset to "none", then tree 0's queries and tree 1's, then
        // their bounds
        cudaError_t e = cudaSuccess;
        const size_t stage_bytes = (size_t)nq_total * (sizeof(unsigned long long) + (dim + 1) * sizeof(float));
        if (stage_bytes > d_cap_q) {
            const size_t cap = std::max(stage_bytes, (size_t)512 * (sizeof(unsigned long long) + 36 * sizeof(float)));
            if (d_stage) cudaFree(d_stage);
            if (h_stage) cudaFreeHost(h_stage);
            d_stage = h_stage = nullptr;
            e = cudaMalloc(&d_stage, cap);
            if (e == cudaSuccess) e = cudaHostAlloc(&h_stage, cap, cudaHostAllocDefault);
            if (e != cudaSuccess) return mrpop::fail_status(MRPOP_ERR_CUDA, "drrt: nearest-neighbour buffers");
            d_cap_q = cap;
        }
        auto *h_best = reinterpret_cast<unsigned long long *>(h_stage);
        float *hx = reinterpret_cast<float *>(h_best + nq_total), *hb = hx + (size_t)nq_total * dim;
        auto *d_best = reinterpret_cast<unsigned long long *>(d_stage);
        float *d_qx = reinterpret_cast<float *>(d_best + nq_total), *d_qb = d_qx + (size_t)nq_total * dim;
        std::memset(h_best, 0xFF, (size_t)nq_total * sizeof(unsigned long long));
        int off = 0;
        for (int t = 0; t < 2; t++) {
            const int nq = (int)jobs[t].bound.size();
            std::memcpy(hx + (size_t)off * dim, jobs[t].x.data(), (size_t)nq * dim * sizeof(float));
            std::memcpy(hb + off, jobs[t].bound.data(), (size_t)nq * sizeof(float));
            off += nq;
        }
        for (int t = 0; t < 2 && e == cudaSuccess; t++)
            if (!jobs[t].bound.empty()) e = T[t].sync_device(stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_stage, h_stage, stage_bytes, cudaMemcpyHostToDevice, stream);
        NNLaunch L{};
        L.qx = d_qx;
        L.qb = d_qb;
        L.best = d_best;
        L.mode = mode;
        for (int t = 0; t < 2; t++) {
            L.rows[t] = T[t].d_rows;
            L.n[t] = T[t].size();
        }
        int njobs = 0;
        long long max_n = 0;
        off = 0;
        for (int t = 0; t < 2 && e == cudaSuccess; t++) {
            const int nq = (int)jobs[t].bound.size();
            for (int c0 = 0; c0 < nq && e == cudaSuccess; c0 += kNNChunk) {
                L.tree[njobs] = t;
                L.q0[njobs] = off + c0;
                L.nq[njobs] = std::min(kNNChunk, nq - c0);
                max_n = std::max<long long>(max_n, L.n[t]);
                if (++njobs == kNNMaxJobs) {
                    e = launch_tree_nn(dim, L, njobs, max_n, stream);
                    njobs = 0;
                    max_n = 0;
                }
            }
            off += nq;
        }
        if (e == cudaSuccess && njobs) e = launch_tree_nn(dim, L, njobs, max_n, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_best, d_best, (size_t)nq_total * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                stream);
        if (e == cudaSuccess) e = wait_stream();
        off = 0;
        for (int t = 0; t < 2 && e == cudaSuccess; t++) {
            const int nq = (int)jobs[t].bound.size();
            for (int q = 0; q < nq; q++) {
                const unsigned long long k = h_best[off + q];
                if (k == ~0ull) continue;
                jobs[t].idx[q] = (int)(uint32_t)k;
                const uint32_t sb = (uint32_t)(k >> 32);
                std::memcpy(&jobs[t].sqd[q], &sb, 4);
            }
            off += nq;
        }
        R->nn_ns += ns_since(t0);
        if (e != cudaSuccess) return mrpop::fail_status(MRPOP_ERR_CUDA, "drrt: nearest-neighbour search");
        return 0;
    }

    // ---- roadmaps (roadmap_interior.cuh:36-341) ------------------------------
    void init_roadmaps() {
        rm.assign(arms, Roadmap{});
        for (int a = 0; a < arms; a++) {
            rm[a].add(&start[7 * a]);
            for (int k = 0; k < num_goals; k++) rm[a].add(&goals[(size_t)k * dim + 7 * a]);
        }
    }
    bool connected(int a) {
        const int r0 = rm[a].find(0);
        for (int k = 0; k < num_goals; k++)
            if (rm[a].find(1 + k) == r0) return true;
        return false;
    }

    // Roadmap neighbour pairs on the device: each arm's nodes [0, n) mirrored
    // in device memory, every (i, j) with n_old <= j, i < j and the reference's
    // distance below `range` found by roadmap_pairs_kernel -- one launch per
    // arm, one read-back of the counts for all arms -- then sorted by (j, i),
    // the host loop's order, so both paths give the same edges.
    std::vector<float *> d_rm;
    std::vector<int64_t> d_rm_cap, d_rm_up;
    int2 *d_pairs = nullptr;     // MRPOP_MAX_ARMS regions of d_pairs_cap pairs
    unsigned int *d_npairs = nullptr, *h_npairs = nullptr;  // MRPOP_MAX_ARMS counters
    size_t d_pairs_cap = 0;

    int roadmap_pairs_device(const std::vector<int> &n_old, std::vector<std::vector<int>> &ea,
                             std::vector<std::vector<int>> &eb) {
        cudaError_t e = cudaSuccess;
        if (d_rm.size() < (size_t)arms) {
            d_rm.resize(arms, nullptr);
            d_rm_cap.resize(arms, 0);
            d_rm_up.resize(arms, 0);
        }
        for (int a = 0; a < arms && e == cudaSuccess; a++) {
            const Roadmap &M = rm[a];
            const int n = M.size();
            if (n > d_rm_cap[a]) {
                int64_t cap = std::max<int64_t>(2 * d_rm_cap[a], 16384);
                while (cap < n) cap *= 2;
                float *p = nullptr;
                e = cudaMalloc(&p, (size_t)cap * 7 * sizeof(float));
                if (e != cudaSuccess) break;
                if (d_rm[a]) cudaFree(d_rm[a]);
                d_rm[a] = p;
                d_rm_cap[a] = cap;
                d_rm_up[a] = 0;
            }
            if (n > d_rm_up[a])
                e = cudaMemcpyAsync(d_rm[a] + d_rm_up[a] * 7, M.node((int)d_rm_up[a]),
                                    (size_t)(n - d_rm_up[a]) * 7 * sizeof(float), cudaMemcpyHostToDevice, stream);
            d_rm_up[a] = n;
        }
        if (e == cudaSuccess && !d_npairs) {
            e = cudaMalloc(&d_npairs, MRPOP_MAX_ARMS * sizeof(unsigned int));
            if (e == cudaSuccess) e = cudaHostAlloc(&h_npairs, MRPOP_MAX_ARMS * sizeof(unsigned int), cudaHostAllocDefault);
        }
        for (int attempt = 0; attempt < 2 && e == cudaSuccess; attempt++) {
            if (!d_pairs) {
                d_pairs_cap = std::max<size_t>(d_pairs_cap, (size_t)1 << 18);
                e = cudaMalloc(&d_pairs, (size_t)MRPOP_MAX_ARMS * d_pairs_cap * sizeof(int2));
                if (e != cudaSuccess) break;
            }
            e = cudaMemsetAsync(d_npairs, 0, MRPOP_MAX_ARMS * sizeof(unsigned int), stream);
            for (int a = 0; a < arms && e == cudaSuccess; a++)
                if (rm[a].size() > n_old[a])
                    e = launch_roadmap_pairs(d_rm[a], n_old[a], rm[a].size(), S.range, d_pairs + (size_t)a * d_pairs_cap,
                                             d_npairs + a, (unsigned int)d_pairs_cap, stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(h_npairs, d_npairs, MRPOP_MAX_ARMS * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                    stream);
            if (e == cudaSuccess) e = wait_stream();
            if (e != cudaSuccess) break;
            size_t most = 0;
            for (int a = 0; a < arms; a++) most = std::max<size_t>(most, h_npairs[a]);
            if (most > d_pairs_cap) {  // grow and search again
                cudaFree(d_pairs);
                d_pairs = nullptr;
                d_pairs_cap = most + (most >> 2);
                continue;
            }
            for (int a = 0; a < arms && e == cudaSuccess; a++) {
                const size_t np = h_npairs[a];
                std::vector<int2> pairs(np);
                if (np)
                    e = cudaMemcpy(pairs.data(), d_pairs + (size_t)a * d_pairs_cap, np * sizeof(int2),
                                   cudaMemcpyDeviceToHost);
                std::sort(pairs.begin(), pairs.end(),
                          [](const int2 &p, const int2 &q) { return p.y != q.y ? p.y < q.y : p.x < q.x; });
                ea[a].resize(np);
                eb[a].resize(np);
                for (size_t k = 0; k < np; k++) {
                    ea[a][k] = pairs[k].x;
                    eb[a][k] = pairs[k].y;
                }
            }
            break;
        }
        if (e != cudaSuccess) return fail_cuda(e, "roadmap neighbour search");
        return 0;
    }
    static int fail_cuda(cudaError_t e, const char *what) {
        return mrpop::fail_status(MRPOP_ERR_CUDA, (std::string("drrt: ") + what + ": " + cudaGetErrorString(e)).c_str());
    }

    // One round: `blocks[a]` blocks of 230 samples grow arm a's roadmap.  The
    // reference grows every arm's roadmap in one launch (roadmap_interior.cuh:
    // 88-339); here the round's node checks of all arms go to the validator as
    // one group, then every arm's neighbour pairs are found, then the edge
    // checks of all arms go as one group.  Each arm draws from its own random
    // streams, so the grouping changes no sample.
    int roadmap_round(const std::vector<int> &blocks) {
        std::vector<std::vector<float>> smp(arms), e0(arms), e1(arms);
        std::vector<std::vector<uint8_t>> okv(arms);
        std::vector<std::vector<int32_t>> fhv(arms);
        std::vector<mrpop_check_call> calls;
        for (int a = 0; a < arms; a++) {
            const int nb = blocks[a];
            if (nb <= 0) continue;
            // samples in time order: iteration-major, block-minor
            const int64_t K = (int64_t)nb * kRoadmapIters;
            smp[a].resize((size_t)K * 7);
            for (int xx = 0; xx < kRoadmapIters; xx++)
                for (int b = 0; b < nb; b++) {
                    Rng &r = rm_rng[(size_t)a * S.block_per_robot + (b % S.block_per_robot)];
                    float *x = &smp[a][((size_t)xx * nb + b) * 7];
                    for (int j = 0; j < 7; j++) x[j] = fmaf(r.uniform(), kSm[j], kSa[j]);
                }
            okv[a].resize((size_t)K);
            fhv[a].resize((size_t)K);
            calls.push_back(plain_call(smp[a].data(), smp[a].data(), K, 1, a, okv[a].data(), fhv[a].data()));
        }
        int rc = check_many(calls);
        if (rc) return rc;
        // the valid samples become nodes; edges: every existing node within
        // `range` of each new node, the new node being the edge's end
        // (roadmap_interior.cuh:183-240), ordered by new node, then old node
        const auto t_nb = Clock::now();
        std::vector<int> n_old(arms, 0);
        for (int a = 0; a < arms; a++) {
            Roadmap &M = rm[a];
            n_old[a] = M.size();
            if (blocks[a] <= 0) continue;
            const int64_t K = (int64_t)okv[a].size();
            int added = 0;
            for (int64_t k = 0; k < K && n_old[a] + added < kMaxRoadmap; k++)
                if (okv[a][k]) {
                    M.add(&smp[a][(size_t)k * 7]);
                    added++;
                }
        }
        std::vector<std::vector<int>> ea(arms), eb(arms);
        if (device_nn) {
            rc = roadmap_pairs_device(n_old, ea, eb);
            if (rc) return rc;
        } else {
            for (int a = 0; a < arms; a++) {
                const Roadmap &M = rm[a];
                const int n_new = M.size() - n_old[a];
                if (n_new <= 0) continue;
                std::vector<std::vector<int>> nbr(n_new);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
                for (int j = 0; j < n_new; j++) {
                    const float *x = M.node(n_old[a] + j);
                    for (int i = 0; i < n_old[a] + j; i++)
                        if (l2(M.node(i), x, 7) < S.range) nbr[j].push_back(i);
                }
                for (int j = 0; j < n_new; j++)
                    for (int i : nbr[j]) {
                        ea[a].push_back(i);
                        eb[a].push_back(n_old[a] + j);
                    }
            }
        }
        R->roadmap_ns += ns_since(t_nb);
        calls.clear();
        for (int a = 0; a < arms; a++) {
            const Roadmap &M = rm[a];
            const int64_t ne = (int64_t)ea[a].size();
            if (!ne) continue;
            e0[a].resize((size_t)ne * 7);
            e1[a].resize((size_t)ne * 7);
            for (int64_t e = 0; e < ne; e++) {
                std::memcpy(&e0[a][(size_t)e * 7], M.node(ea[a][e]), 7 * sizeof(float));
                std::memcpy(&e1[a][(size_t)e * 7], M.node(eb[a][e]), 7 * sizeof(float));
            }
            okv[a].resize((size_t)ne);
            fhv[a].resize((size_t)ne);
            calls.push_back(plain_call(e0[a].data(), e1[a].data(), ne, g, a, okv[a].data(), fhv[a].data()));
        }
        rc = check_many(calls);
        if (rc) return rc;
        for (int a = 0; a < arms; a++) {
            std::vector<std::pair<int, int>> good;
            for (size_t e = 0; e < ea[a].size(); e++)
                if (okv[a][e]) good.emplace_back(ea[a][e], eb[a][e]);
            std::sort(good.begin(), good.end(),
                      [](auto &x, auto &y) { return x.second != y.second ? x.second < y.second : x.first < y.first; });
            for (auto &p : good) rm[a].link(p.first, p.second);
        }
        return 0;
    }

    // One build_roadmap launch: the first one loops rounds until every arm's
    // start and goal are connected (or a roadmap is full); later ones run one
    // round on every arm (roadmap_interior.cuh:88-339).  The first launch's
    // rounds are bounded by max_launches (the reference loops until its
    // roadmaps overflow).
    int build_roadmaps() {
        const bool first = roadmap_launches == 0;
        roadmap_launches++;
        if (!first) return roadmap_round(std::vector<int>(arms, S.block_per_robot));
        for (int round = 0; round < S.max_launches; round++) {
            std::vector<int> blocks(arms, 0);
            int first_open = -1, closed = 0;
            for (int a = 0; a < arms; a++) {
                if (connected(a)) {
                    closed++;
                } else {
                    blocks[a] = S.block_per_robot;
                    if (first_open < 0) first_open = a;
                }
            }
            if (first_open < 0) return 0;
            if (S.roadmap_reassign) blocks[first_open] += closed * S.block_per_robot;
            for (int a = 0; a < arms; a++)
                if (rm[a].size() >= kMaxRoadmap) return 0;
            const int rc = roadmap_round(blocks);
            if (rc) return rc;
        }
        return 0;
    }

    // ---- informed sampling set-up (pop_planner.cu:290-341) ----------------
    std::vector<float> tf, center;
    void phs_setup() {
        tf.assign((size_t)dim * dim, 0.0f);
        center.assign(dim, 0.0f);
        const float *f1 = T[0].node(0), *f2 = T[1].node(0);
        const float dmin = l2(f1, f2, dim);
        const float dtr = best_cost;
        std::vector<float> rot((size_t)dim * dim, 0.0f), axis(dim);
        for (int t = 0; t < dim; t++) center[t] = (f1[t] + f2[t]) / 2.0f;
        if (dmin < 1e-6f) {
            for (int t = 0; t < dim; t++) rot[(size_t)t * dim + t] = 1.0f;
        } else {
            for (int d = 0; d < dim; d++) axis[d] = (f2[d] - f1[d]) / dmin;
            const float v0 = 1.0f - axis[0];
            float vtv = v0 * v0;
            for (int i = 1; i < dim; i++) vtv = fmaf(-axis[i], -axis[i], vtv);
            const float beta = 2.0f / vtv;
            for (int c = 0; c < dim; c++) {
                const float vc = c == 0 ? 1.0f - axis[0] : -axis[c];
                for (int r = 0; r < dim; r++) {
                    const float vr = r == 0 ? 1.0f - axis[0] : -axis[r];
                    float val = -beta * vr * vc;
                    if (r == c) val += 1.0f;
                    rot[(size_t)r * dim + c] = val;
                }
            }
        }
        const float conj = sqrtf(fmaf(dtr, dtr, -(dmin * dmin)));
        std::vector<float> diag(dim, conj / 2);
        diag[0] = dtr / 2;
        for (int r = 0; r < dim; r++)
            for (int c = 0; c < dim; c++) tf[(size_t)r * dim + c] = rot[(size_t)r * dim + c] * diag[c];
    }
    // One informed sample (pop_planner.cu:398-445), then clamped to the limits.
    void phs_sample(Rng &r, float *x) {
        const float k = sqrtf((float)(M_PI / 8.0f));
        for (int d = 0; d < dim; d++) {
            const float u = r.uniform();
            x[d] = logf(u * (1.0f / (1.0f - u))) * k;
        }
        float n = 0.0f;
        for (int d = 0; d < dim; d++) n = fmaf(x[d], x[d], n);
        n = sqrtf(n);
        for (int d = 0; d < dim; d++) x[d] = x[d] / n;
        const float rad = powf(r.uniform(), 1.0f / (float)dim);
        for (int d = 0; d < dim; d++) x[d] = x[d] * rad;
        std::vector<float> y(dim);
        for (int t = 0; t < dim; t++) {
            float v = 0.0f;
            for (int c = 0; c < dim; c++) v = fmaf(tf[(size_t)t * dim + c], x[c], v);
            y[t] = v + center[t];
        }
        for (int t = 0; t < dim; t++) {
            const int j = t % 7;
            float u = (y[t] - kSa[j]) / kSm[j];
            u = fmaxf(fminf(1.0f, u), 0.0f);
            x[t] = fmaf(u, kSm[j], kSa[j]);
        }
    }

    // ---- direction oracle (nn_angle_mr, utils.cuh:688-759) ------------------
    bool nn_angle(int tree, const float *sample, int near, float bound, bool optimize, float *out, int *ids) const {
        const Tree &t = T[tree];
        const float *vn = t.node(near);
        for (int a = 0; a < arms; a++) {
            const int r0 = t.rid[(size_t)near * arms + a];
            if (r0 < 0) return false;
            const Roadmap &M = rm[a];
            int best = -1;
            float best_angle = 1e3f;
            for (int v : M.adj[r0]) {
                if (v == r0) continue;
                const float ed = l2(vn + 7 * a, M.node(v), 7);
                if ((optimize && ed > bound) || ed > S.range) continue;
                const float ang = angle_at(vn + 7 * a, sample + 7 * a, M.node(v), 7);
                if (ang < best_angle) {
                    best_angle = ang;
                    best = v;
                }
            }
            ids[a] = best;
            if (best < 0) return false;
            std::memcpy(out + 7 * a, M.node(best), 7 * sizeof(float));
            bound -= l2(M.node(best), vn + 7 * a, 7);
        }
        return true;
    }

    // ---- a solution (record_connected_path, path_processing.cu:11-70) -------
    void record_path(int t, int ti, int oi, int iter) {
        const int o = 1 - t;
        float c = 0.0f;
        std::vector<int> pt, po;
        for (int cur = ti; T[t].parent[cur] != cur; cur = T[t].parent[cur]) {
            c += l2(T[t].node(cur), T[t].node(T[t].parent[cur]), dim);
            pt.push_back(cur);
        }
        pt.push_back(0);
        for (int cur = oi; T[o].parent[cur] != cur; cur = T[o].parent[cur]) {
            c += l2(T[o].node(cur), T[o].node(T[o].parent[cur]), dim);
            po.push_back(cur);
        }
        po.push_back(0);
        const std::vector<int> &p1 = t == 1 ? pt : po, &p0 = t == 0 ? pt : po;
        path_out.clear();
        for (auto it = p1.rbegin(); it != p1.rend(); ++it) path_out.insert(path_out.end(), T[1].node(*it), T[1].node(*it) + dim);
        for (int i : p0) path_out.insert(path_out.end(), T[0].node(i), T[0].node(i) + dim);
        path_total = (int)(path_out.size() / dim);
        raw_path = path_out;
        cost_sym = c;
        solved_iters = iter;
        best_cost = std::min(best_cost, c);
        sol_tree[0] = T[0].size();
        sol_tree[1] = T[1].size();
    }

    // ---- one rrtc launch (pop_planner.cu:220-737) -------------------------
    // Returns the status; *solved = 1 when a connection was made.  Per
    // iteration: every attempt's sample (in parallel: per-attempt random
    // streams), one nearest-neighbour search per tree, the direction oracle
    // and prunes (in parallel), one extend check, tree growth in attempt
    // order, one connect search per tree, one connect check.
    int rrtc(bool optimize, int *solved) {
        *solved = 0;
        const int N = S.num_new_configs;
        if (optimize && S.phs) phs_setup();
        std::vector<int> tsel(N, 0), near(N), ext_ok(N), ext_exist(N);
        std::vector<float> x((size_t)N * dim), crand(N, FLT_MAX), nd(N), ext_cost(N), ext_cfg((size_t)N * dim);
        std::vector<int> ext_ids((size_t)N * arms);
        std::vector<char> live(N);
        NNJob job[2];
        for (int iter = 1;; iter++) {
            if (iter > S.max_iters || (optimize && iter > S.optimize_iters)) return 0;
            if (T[0].size() >= S.max_samples || T[1].size() >= S.max_samples) return 0;
            R->iterations++;
            const int64_t sz[2] = {T[0].size(), T[1].size()};
            const float bc = best_cost;
            // tree choice, sample, cost bound
#pragma omp parallel for schedule(static) num_threads(nthreads)
            for (int b = 0; b < N; b++) {
                Rng &r = blk_rng[b];
                if (iter == 1) {
                    tsel[b] = b < N / 2 ? 0 : 1;
                } else if (S.balance == 2) {
                    const int t = tsel[b];
                    const float ratio = (float)std::llabs(sz[t] - sz[1 - t]) / (float)sz[t];
                    if (ratio < S.tree_ratio) tsel[b] = 1 - t;
                }
                float *xb = &x[(size_t)b * dim];
                if (!S.phs || !optimize) {
                    for (int d = 0; d < dim; d++) xb[d] = fmaf(r.uniform(), kSm[d % 7], kSa[d % 7]);
                } else {
                    phs_sample(r, xb);
                }
                live[b] = !(l2(T[0].node(0), xb, dim) + l2(T[1].node(0), xb, dim) >= bc);
                if (live[b] && optimize) {
                    const int t = tsel[b];
                    const float gh = l2(T[t].node(0), xb, dim);
                    const float hh = l2(T[1 - t].node(0), xb, dim);
                    const float range = std::max(bc - (gh + hh), 0.0f);
                    crand[b] = fmaf(r.uniform(), range, gh);
                }
            }
            // nearest node of each live attempt in its tree
            for (int t = 0; t < 2; t++) job[t].clear();
            for (int b = 0; b < N; b++)
                if (live[b]) {
                    NNJob &J = job[tsel[b]];
                    J.x.insert(J.x.end(), &x[(size_t)b * dim], &x[(size_t)b * dim] + dim);
                    J.bound.push_back(optimize ? crand[b] : FLT_MAX);
                    J.who.push_back(b);
                }
            int rc = nearest(job, 0);
            if (rc) return rc;
            for (int t = 0; t < 2; t++)
                for (size_t k = 0; k < job[t].who.size(); k++) {
                    const int b = job[t].who[k];
                    near[b] = job[t].idx[k] < 0 ? 0 : job[t].idx[k];
                    nd[b] = sqrtf(job[t].idx[k] < 0 ? FLT_MAX : job[t].sqd[k]);
                }
            // direction oracle, existing-node test, cost prunes
            const auto t_or = Clock::now();
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads)
            for (int b = 0; b < N; b++) {
                ext_ok[b] = 0;
                if (!live[b]) continue;
                const int t = tsel[b];
                const int nr = near[b];
                const float bound = optimize ? crand[b] - T[t].cost[nr] : FLT_MAX;
                float *cfg = &ext_cfg[(size_t)b * dim];
                int *ids = &ext_ids[(size_t)b * arms];
                if (!nn_angle(t, &x[(size_t)b * dim], nr, bound, optimize, cfg, ids)) continue;
                const int ex = T[t].existing(cfg, ids);
                const float nc = T[t].cost[nr] + nd[b];
                if (ex >= 0 && (!optimize || nc >= T[t].cost[ex])) continue;
                if (optimize && nc >= bc) continue;
                ext_ok[b] = 1;
                ext_exist[b] = ex;
                ext_cost[b] = nc;
            }
            R->oracle_ns += ns_since(t_or);
            std::vector<int> ext;
            for (int b = 0; b < N; b++)
                if (ext_ok[b]) ext.push_back(b);
            const int64_t ne = (int64_t)ext.size();
            a0.resize((size_t)ne * dim);
            a1.resize((size_t)ne * dim);
            for (int64_t k = 0; k < ne; k++) {
                const int b = ext[k];
                std::memcpy(&a0[(size_t)k * dim], T[tsel[b]].node(near[b]), dim * sizeof(float));
                std::memcpy(&a1[(size_t)k * dim], &ext_cfg[(size_t)b * dim], dim * sizeof(float));
            }
            rc = check(ne, MRPOP_RULE_PLAIN, 0.0f, MRPOP_CHECK_SELF, -1, g);
            if (rc) return rc;
            // grow the trees in attempt order; remember the new nodes to connect
            struct Con {
                int b, t, node;
            };
            std::vector<Con> con;
            for (int64_t k = 0; k < ne; k++) {
                if (!ok[k]) continue;
                const int b = ext[k];
                Tree &tt = T[tsel[b]];
                if (ext_exist[b] >= 0) {  // rewire (pop_planner.cu:571-577)
                    tt.parent[ext_exist[b]] = near[b];
                    tt.set_cost(ext_exist[b], ext_cost[b]);
                    continue;
                }
                const int ni = tt.add(&ext_cfg[(size_t)b * dim], near[b], ext_cost[b], &ext_ids[(size_t)b * arms]);
                con.push_back(Con{b, tsel[b], ni});
            }
            // connect: nearest node of the other tree
            for (int t = 0; t < 2; t++) job[t].clear();
            for (size_t k = 0; k < con.size(); k++) {
                NNJob &J = job[1 - con[k].t];
                const Tree &tt = T[con[k].t];
                J.x.insert(J.x.end(), tt.node(con[k].node), tt.node(con[k].node) + dim);
                J.bound.push_back(optimize ? best_cost - tt.cost[con[k].node] : FLT_MAX);
                J.who.push_back((int)k);
            }
            rc = nearest(job, 1);
            if (rc) return rc;
            std::vector<int> onear(con.size(), -1);
            std::vector<float> od(con.size(), 0.0f);
            for (int o = 0; o < 2; o++)
                for (size_t k = 0; k < job[o].who.size(); k++)
                    if (job[o].idx[k] >= 0) {
                        onear[job[o].who[k]] = job[o].idx[k];
                        od[job[o].who[k]] = sqrtf(job[o].sqd[k]);
                    }
            std::vector<int> ck;
            for (size_t k = 0; k < con.size(); k++)
                if (onear[k] >= 0) ck.push_back((int)k);
            const int64_t nc = (int64_t)ck.size();
            a0.resize((size_t)nc * dim);
            a1.resize((size_t)nc * dim);
            for (int64_t j = 0; j < nc; j++) {
                const Con &c = con[ck[j]];
                std::memcpy(&a0[(size_t)j * dim], T[c.t].node(c.node), dim * sizeof(float));
                std::memcpy(&a1[(size_t)j * dim], T[1 - c.t].node(onear[ck[j]]), dim * sizeof(float));
            }
            rc = check(nc, MRPOP_RULE_CONNECT, S.range, MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, -1, g);
            if (rc) return rc;
            for (int64_t j = 0; j < nc; j++) {
                if (!ok[j]) continue;
                const Con &c = con[ck[j]];
                Tree &tt = T[c.t];
                const float d = od[ck[j]];
                const int next = (int)(d / S.range) + 1;
                // the accumulated end of the connect loop (pop_planner.cu:684-716)
                std::vector<float> cur(tt.node(c.node), tt.node(c.node) + dim), vec(dim);
                const float *target = T[1 - c.t].node(onear[ck[j]]);
                for (int dd = 0; dd < dim; dd++) vec[dd] = (target[dd] - cur[dd]) / (float)next;
                for (int s2 = 0; s2 < next; s2++)
                    for (int dd = 0; dd < dim; dd++) cur[dd] += vec[dd];
                const float ncost = tt.cost[c.node] + d / (float)next;
                const int ni = tt.add(cur.data(), c.node, ncost, nullptr);
                if (!*solved) {
                    *solved = 1;
                    record_path(c.t, ni, onear[ck[j]], iter);
                }
            }
            if (*solved) return 0;
        }
    }

    // ---- simplification (multiBlock_simplify, path_simplification.cu:17-242)
    int simplify() {
        const int n = path_total;
        if (n < 1) return 0;
        std::vector<float> &P = path_out;
        for (int round = 0; round < S.simplify_round; round++) {
            std::vector<float> pc(n, FLT_MAX);
            std::vector<int> par(n, -1);
            pc[0] = 0.0f;
            // B-spline midpoint smoothing of the odd waypoints, bspline_step steps
            const int R = (int)ceilf((float)(n - 3) / (2.0f * kShortcutSpan));
            for (int step = 0; step < S.bspline_step && R > 0; step++) {
                std::vector<int> cand;
                std::vector<float> mids;
                // the odd waypoints the 16 blocks reach in R strides (the last one
                // can be left out, as in the reference)
                for (int i = 1; i < n - 1 && i <= 2 * kShortcutSpan * R - 1; i += 2) {
                    const float *c1 = &P[(size_t)(i - 1) * dim], *c2 = &P[(size_t)i * dim],
                                *c3 = &P[(size_t)(i + 1) * dim];
                    std::vector<float> mid(dim);
                    for (int d = 0; d < dim; d++) {
                        const float b1 = (c1[d] + c2[d]) / 2.0f, b2 = (c2[d] + c3[d]) / 2.0f;
                        mid[d] = (b1 + b2) / 2.0f;
                    }
                    if (l2(c2, mid.data(), dim) < S.bspline_min_change) continue;
                    cand.push_back(i);
                    mids.insert(mids.end(), mid.begin(), mid.end());
                }
                const int64_t m = (int64_t)cand.size();
                a0.resize((size_t)2 * m * dim);
                a1.resize((size_t)2 * m * dim);
                for (int64_t k = 0; k < m; k++) {
                    const int i = cand[k];
                    std::memcpy(&a0[(size_t)(2 * k) * dim], &P[(size_t)(i - 1) * dim], dim * sizeof(float));
                    std::memcpy(&a0[(size_t)(2 * k + 1) * dim], &P[(size_t)(i + 1) * dim], dim * sizeof(float));
                    std::memcpy(&a1[(size_t)(2 * k) * dim], &mids[(size_t)k * dim], dim * sizeof(float));
                    std::memcpy(&a1[(size_t)(2 * k + 1) * dim], &mids[(size_t)k * dim], dim * sizeof(float));
                }
                const int rc = check(2 * m, MRPOP_RULE_BSPLINE, S.range, MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, -1, g);
                if (rc) return rc;
                for (int64_t k = 0; k < m; k++)
                    if (ok[2 * k] && ok[2 * k + 1])
                        std::memcpy(&P[(size_t)cand[k] * dim], &mids[(size_t)k * dim], dim * sizeof(float));
            }
            // shortcut dynamic programme: edge i -> i+b+1 for b in 1..15 checked,
            // i -> i+1 taken as valid (path_simplification.cu:143-217)
            std::vector<int> ei, ej;
            for (int i = 0; i < n - 1; i++)
                for (int b = 1; b < kShortcutSpan; b++)
                    if (i + b + 1 < n) {
                        ei.push_back(i);
                        ej.push_back(i + b + 1);
                    }
            const int64_t m = (int64_t)ei.size();
            a0.resize((size_t)m * dim);
            a1.resize((size_t)m * dim);
            for (int64_t k = 0; k < m; k++) {
                std::memcpy(&a0[(size_t)k * dim], &P[(size_t)ei[k] * dim], dim * sizeof(float));
                std::memcpy(&a1[(size_t)k * dim], &P[(size_t)ej[k] * dim], dim * sizeof(float));
            }
            const int rc = check(m, MRPOP_RULE_SHORTCUT, S.range, MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, -1, g);
            if (rc) return rc;
            std::vector<uint8_t> good(ok.begin(), ok.begin() + m);
            int64_t k = 0;
            for (int i = 0; i < n - 1; i++) {
                for (int b = 0; b < kShortcutSpan; b++) {
                    const int j = i + b + 1;
                    if (j >= n) continue;
                    bool eg = true;
                    if (b > 0) eg = good[k++];
                    if (!eg) continue;
                    const float d = l2(&P[(size_t)i * dim], &P[(size_t)j * dim], dim);
                    if (pc[j] > d + pc[i]) {
                        pc[j] = d + pc[i];
                        par[j] = i;
                    }
                }
            }
            // reconstruct: waypoints skipped by a shortcut become copies of its start
            if (pc[n - 1] < best_cost) {
                int child = n - 1, p = par[child];
                while (p < n && p != -1) {
                    for (int b = 0; b < kShortcutSpan; b++) {
                        const int w = b + p + 1;
                        if (w < child) std::memcpy(&P[(size_t)w * dim], &P[(size_t)p * dim], dim * sizeof(float));
                    }
                    child = p;
                    p = par[child];
                }
            }
            cost_sym = pc[n - 1];
            best_cost = std::min(best_cost, cost_sym);
        }
        return 0;
    }

    void report(int pass, int solved_flag) {
        // copy_path_to_result (path_processing.cu:73-122), called when the pass
        // solved and its cost improves on the reported one (pop_planner.cu:1007)
        if (!(solved_flag > 0 && (!init_sol || res_cost > cost_sym))) return;
        init_sol = true;
        res_cost = cost_sym;
        res_path.assign(path_out.begin(), path_out.begin() + (size_t)path_total * dim);
        R->solved = 1;
        R->cost = cost_sym;
        R->iters = solved_iters;
        R->path_length = path_total;
        R->start_tree_size = sol_tree[0];
        R->goal_tree_size = sol_tree[1];
        R->solutions++;
        if (on_solution)
            on_solution(sctx, pass, cost_sym, res_path.data(), path_total, raw_path.data(),
                        (int64_t)(raw_path.size() / dim));
    }

    void reset_trees() {
        for (int t = 0; t < 2; t++) {
            T[t].clear();
            T[t].dim = dim;
            T[t].arms = arms;
        }
        std::vector<int> ids(arms, 0);
        T[0].add(start.data(), -1, 0.0f, ids.data());
        for (int k = 0; k < num_goals; k++) {
            std::fill(ids.begin(), ids.end(), 1 + k);
            T[1].add(&goals[(size_t)k * dim], -1, 0.0f, ids.data());
        }
    }

    int run() {
        const auto t_start = Clock::now();
        init_roadmaps();
        rm_rng.clear();
        for (int a = 0; a < arms; a++)
            for (int b = 0; b < S.block_per_robot; b++) rm_rng.push_back(rng_stream(S.seed, 1, (uint64_t)a * 4096 + b));
        blk_rng.clear();
        for (int b = 0; b < S.num_new_configs; b++) blk_rng.push_back(rng_stream(S.seed, 2, b));
        const auto t_kernel = Clock::now();
        for (int pass = 0; pass < S.rrtc_iter; pass++) {
            R->passes++;
            reset_trees();
            const bool optimize = pass != 0;
            int solved = 0;
            do {
                int rc = build_roadmaps();
                if (rc) return rc;
                rc = rrtc(optimize, &solved);
                if (rc) return rc;
                if (!optimize) R->launches++;
            } while (!solved && !optimize && R->launches < S.max_launches);
            if (S.path_simplify && path_total > 0) {
                const int rc = simplify();
                if (rc) return rc;
            }
            report(pass, solved);
        }
        for (int a = 0; a < arms && a < MRPOP_MAX_ARMS; a++) {
            R->roadmap_nodes[a] = rm[a].size();
            R->roadmap_edges[a] = rm[a].edges;
        }
        R->kernel_ns = ns_since(t_kernel);
        R->wall_ns = ns_since(t_start);
        return 0;
    }
};

mrpop_status check_settings(const mrpop_drrt_settings &S) {
    if (S.granularity < 1 || S.granularity > MRPOP_MAX_GRANULARITY || !(S.range > 0.0f) || S.num_new_configs < 1 ||
        S.max_iters < 0 || S.max_samples < 2 || S.block_per_robot < 1 || S.rrtc_iter < 0 || S.max_launches < 1 ||
        S.simplify_round < 0 || S.bspline_step < 0)
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "drrt: bad settings");
    return MRPOP_OK;
}

mrpop_status solve(Solver &sv, int arms, const float *start, const float *goals, int num_goals,
                   const mrpop_drrt_settings *settings, float *path_out, int64_t max_waypoints,
                   mrpop_drrt_solution_fn on_solution, void *sctx, mrpop_drrt_result *out) {
    sv.S = *settings;
    sv.nthreads = settings->host_threads > 0 ? settings->host_threads : omp_get_num_procs();
    sv.arms = arms;
    sv.dim = 7 * arms;
    sv.g = settings->granularity;
    sv.num_goals = num_goals;
    sv.start.assign(start, start + sv.dim);
    sv.goals.assign(goals, goals + (size_t)num_goals * sv.dim);
    sv.R = out;
    sv.on_solution = on_solution;
    sv.sctx = sctx;
    const int rc = sv.run();
    if (rc) return (mrpop_status)rc;
    if (path_out && max_waypoints > 0 && !sv.res_path.empty())
        std::memcpy(path_out, sv.res_path.data(),
                    (size_t)std::min<int64_t>(out->path_length, max_waypoints) * sv.dim * sizeof(float));
    return MRPOP_OK;
}

}  // namespace

extern "C" mrpop_status mrpop_drrt_settings_default(mrpop_drrt_settings *o) {
    if (!o) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "drrt_settings_default: null");
    *o = mrpop_drrt_settings{};
    // pop_settings.hh:3-32
    o->max_samples = 1000000;
    o->max_iters = 1000;
    o->optimize_iters = 400000;
    o->num_new_configs = 256;
    o->granularity = 16;
    o->range = 0.5f;
    o->balance = 2;
    o->tree_ratio = 1.0f;
    o->dynamic_domain = 0;
    o->dd_alpha = 0.0001f;
    o->dd_radius = 4.0f;
    o->dd_min_radius = 1.0f;
    o->roadmap_reassign = 0;
    o->rrtc_iter = 1;
    o->resample_iter = 5;
    o->cost_bound_resample = 0;
    o->path_simplify = 1;
    o->phs = 1;
    o->simplify_round = 1;
    o->bspline_step = 3;
    o->bspline_min_change = 0.01f;
    o->perturb_step = 3;
    o->perturb_empty_step = 2;
    // this library's additions
    o->block_per_robot = 8;
    o->max_launches = 20;
    o->seed = 1234;
    o->host_threads = 0;
    o->blocking_wait = 0;
    return MRPOP_OK;
}

namespace mrpop {

// The planner with any validator; device_nn: nearest-neighbour searches as a
// kernel on the current device (else on the host).
mrpop_status drrt_run(int arms, mrpop_check_fn validate, check_many_fn validate_many, void *ctx, bool device_nn,
                      const float *start, const float *goals, int num_goals, const mrpop_drrt_settings *settings,
                      float *path_out, int64_t max_waypoints, mrpop_drrt_solution_fn on_solution, void *solution_ctx,
                      mrpop_drrt_result *out) {
    if (arms < 1 || arms > MRPOP_MAX_ARMS || !validate || !start || !goals || num_goals < 1 || !settings || !out)
        return fail_status(MRPOP_ERR_INVALID_ARGUMENT, "drrt: bad argument");
    const mrpop_status st = check_settings(*settings);
    if (st != MRPOP_OK) return st;
    *out = mrpop_drrt_result{};
    Solver sv;
    sv.validate = validate;
    sv.validate_many = validate_many;
    sv.vctx = ctx;
    sv.device_nn = device_nn;
    if (device_nn && sv.adopt_device() != cudaSuccess) return fail_status(MRPOP_ERR_CUDA, "drrt: device resources");
    return solve(sv, arms, start, goals, num_goals, settings, path_out, max_waypoints, on_solution, solution_ctx, out);
}

}  // namespace mrpop

extern "C" int64_t mrpop_drrt_release_pool(void) {
    std::vector<DeviceWork> idle;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        idle.swap(g_pool);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    for (auto &w : idle) {
        cudaSetDevice(w.device);
        w.free_all();
    }
    cudaSetDevice(dev);
    return (int64_t)idle.size();
}

extern "C" mrpop_status mrpop_drrt_solve_with(int arms, mrpop_check_fn validate, void *ctx, const float *start,
                                              const float *goals, int num_goals, const mrpop_drrt_settings *settings,
                                              float *path_out, int64_t max_waypoints,
                                              mrpop_drrt_solution_fn on_solution, void *solution_ctx,
                                              mrpop_drrt_result *out) {
    return mrpop::drrt_run(arms, validate, nullptr, ctx, false, start, goals, num_goals, settings, path_out, max_waypoints,
                           on_solution, solution_ctx, out);
}

extern "C" mrpop_status mrpop_drrt_solve(const mrpop_scene *scene, const mrpop_robotset *robots, const float *start,
                                         const float *goals, int num_goals, const mrpop_drrt_settings *settings,
                                         float *path_out, int64_t max_waypoints, mrpop_drrt_solution_fn on_solution,
                                         void *solution_ctx, mrpop_drrt_result *out) {
    const int arms = mrpop::robotset_arms(robots);
    if (!scene || arms < 1) return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "drrt_solve: bad argument");
    GpuChecker chk;
    chk.scene = scene;
    chk.robots = robots;
    if (mrpop_workspace_create(&chk.ws) != MRPOP_OK) return MRPOP_ERR_CUDA;
    return mrpop::drrt_run(arms, &GpuChecker::call, &GpuChecker::call_many, &chk, true, start, goals, num_goals, settings, path_out,
                           max_waypoints, on_solution, solution_ctx, out);
}
