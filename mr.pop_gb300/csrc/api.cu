// api.cu -- C ABI of the GB300 edge validator (declared in include/mrpop.h).
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/mrpop.h"
#include "launch.h"

namespace {

thread_local std::string g_last_error;

mrpop_status fail(mrpop_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}

mrpop_status cuda_fail(cudaError_t err, const char *what) {
    return fail(MRPOP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

#define MRPOP_CUDA(call, what)                                                                             \
    do {                                                                                                   \
        cudaError_t _e = (call);                                                                           \
        if (_e != cudaSuccess) return cuda_fail(_e, what);                                                 \
    } while (0)

// Reference base layouts (row-major 4x4): panda.cuh:16-73.
const float kQuadBase[4][16] = {
    {-0.65122966f, -0.75888071f, 0.f, 0.40000000f, 0.75888071f, -0.65122966f, 0.f, -0.40000000f, 0.f, 0.f,
     1.f, 0.15000000f, 0.f, 0.f, 0.f, 1.f},
    {0.78999223f, -0.61311685f, 0.f, -0.40000000f, 0.61311685f, 0.78999223f, 0.f, -0.40000000f, 0.f, 0.f,
     1.f, 0.15000000f, 0.f, 0.f, 0.f, 1.f},
    {0.78999223f, 0.61311685f, 0.f, -0.40000000f, -0.61311685f, 0.78999223f, 0.f, 0.40000000f, 0.f, 0.f,
     1.f, 0.15000000f, 0.f, 0.f, 0.f, 1.f},
    {-0.65122966f, 0.75888071f, 0.f, 0.40000000f, -0.75888071f, -0.65122966f, 0.f, 0.40000000f, 0.f, 0.f,
     1.f, 0.15000000f, 0.f, 0.f, 0.f, 1.f}};
const float kFiveBase[5][16] = {
    {0.00079633f, -0.99999968f, 0.f, 0.60000000f, 0.99999968f, 0.00079633f, 0.f, -0.70000000f, 0.f, 0.f, 1.f,
     0.10000000f, 0.f, 0.f, 0.f, 1.f},
    {0.00079633f, -0.99999968f, 0.f, 0.00000000f, 0.99999968f, 0.00079633f, 0.f, -0.70000000f, 0.f, 0.f, 1.f,
     0.10000000f, 0.f, 0.f, 0.f, 1.f},
    {0.00079633f, 0.99999968f, 0.f, 0.60000000f, -0.99999968f, 0.00079633f, 0.f, 0.70000000f, 0.f, 0.f, 1.f,
     0.10000000f, 0.f, 0.f, 0.f, 1.f},
    {0.00079633f, 0.99999968f, 0.f, 0.00000000f, -0.99999968f, 0.00079633f, 0.f, 0.70000000f, 0.f, 0.f, 1.f,
     0.10000000f, 0.f, 0.f, 0.f, 1.f},
    {1.00000000f, 0.00000000f, 0.f, -0.60000000f, 0.00000000f, 1.00000000f, 0.f, -0.20000000f, 0.f, 0.f, 1.f,
     0.10000000f, 0.f, 0.f, 0.f, 1.f}};

unsigned long long *g_phase_counters = nullptr;  // development phase timers (see edge_kernel.cuh)

// Per-device pool for the split pipeline's stream-ordered scratch; keeps
// freed memory cached (release threshold = max) so steady-state calls do not
// map new memory.  Created on first use, never destroyed.
std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};

cudaError_t scratch_pool(cudaMemPool_t *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) return e;
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return cudaSuccess;
}

size_t block_scratch_bytes() { return sizeof(mrpop::WarpScratch) * mrpop::kWarpsPerBlock; }

// Optional per-kernel timing (mrpop_kernel_timing): a pair of CUDA events is
// recorded on the caller's stream around every validator launch while it is
// on; mrpop_kernel_times sums and releases them.
static_assert(mrpop::kFused == MRPOP_KERNEL_FUSED && mrpop::kBroad == MRPOP_KERNEL_BROAD &&
                  mrpop::kNarrow == MRPOP_KERNEL_NARROW,
              "kernel kinds of launch.h and mrpop.h differ");
struct TimedLaunch {
    cudaEvent_t start, stop;
    int kind;
};
std::mutex g_timing_mu;
bool g_timing_on = false;
std::vector<TimedLaunch> g_timed;

cudaError_t timed_launch(int arms, mrpop::KernelKind kind, const mrpop::EdgeParams &p, size_t smem,
                         cudaStream_t stream) {
    bool on;
    {
        std::lock_guard<std::mutex> lk(g_timing_mu);
        on = g_timing_on;
    }
    if (!on) return mrpop::launch_validate(arms, kind, p, smem, stream);
    TimedLaunch t{nullptr, nullptr,
                  (int)(kind == mrpop::kFusedPair || kind == mrpop::kArmwise ? mrpop::kFused : kind)};
    cudaError_t e = cudaEventCreate(&t.start);
    if (e == cudaSuccess) e = cudaEventCreate(&t.stop);
    if (e == cudaSuccess) e = cudaEventRecord(t.start, stream);
    if (e == cudaSuccess) e = mrpop::launch_validate(arms, kind, p, smem, stream);
    if (e == cudaSuccess) e = cudaEventRecord(t.stop, stream);
    if (e != cudaSuccess) {
        if (t.start) cudaEventDestroy(t.start);
        if (t.stop) cudaEventDestroy(t.stop);
        return e;
    }
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timed.push_back(t);
    return cudaSuccess;
}

// Algorithmic flops of the broad phase for one sample (FMA = 2): FK of every
// arm (7 joint composes of 81 and 11 sphere placements of 18), the 10
// env-tested spheres of every arm against every obstacle, the 21 intra-arm
// pairs and the 121 pairs of every arm pair, each test at 11 flops.
double broad_flops_per_sample(int A, double env_test_flops, uint32_t flags) {
    double f = A * (7.0 * 81.0 + 11.0 * 18.0);
    if (flags & MRPOP_CHECK_ENV) f += A * 10.0 * env_test_flops;
    if (flags & MRPOP_CHECK_SELF) f += A * 21.0 * 11.0 + (A * (A - 1) / 2) * 121.0 * 11.0;
    return f;
}

// Forearm-hand rows table (panda_model.cuh): built once per process on the
// host, copied once per device into g_row5 when the device's first scene is
// created.
__device__ uint32_t g_row5[mrpop::kRow5Words];

const std::vector<uint32_t> &row5_host_table() {
    static std::vector<uint32_t> tab;
    static std::once_flag once;
    std::call_once(once, [] {
        using namespace mrpop;
        tab.assign(kRow5Words, 0u);
        const double h6 = ((double)kRow5Hi6 - kRow5Lo6) / kRow5N6, h7 = ((double)kRow5Hi7 - kRow5Lo7) / kRow5N7;
        constexpr int s0 = 17, s1 = 28, t0 = 32, t1 = 58;
        double R[s1 - s0 + 1], slack[t1 - t0 + 1];
        for (int s = s0; s <= s1; s++)
            R[s - s0] = s + 4 <= s1 ? std::fmax(kDet[s].r, kDet[s + 4].r) : (double)kDet[s].r;
        for (int t = t0; t <= t1; t++) {
            const SphereDef &x = kDet[t];
            const double n = std::sqrt((double)x.x * x.x + (double)x.y * x.y + (double)x.z * x.z);
            const double rxy = std::sqrt((double)x.x * x.x + (double)x.y * x.y);
            // a hand sphere moves at most (distance from the joint axis) x (angle) per joint:
            // <= |F7 translation| + |x| from axis 6, exactly |x_xy| from axis 7
            slack[t - t0] = (0.088 + n) * (0.5 * h6 + 1e-4) + rxy * (0.5 * h7 + 1e-4);
        }
        for (int i6 = 0; i6 < kRow5N6; i6++) {
            const double q6 = kRow5Lo6 + (i6 + 0.5) * h6, c6 = std::cos(q6), sn6 = std::sin(q6);
            for (int i7 = 0; i7 < kRow5N7; i7++) {
                const double q7 = kRow5Lo7 + (i7 + 0.5) * h7, c7 = std::cos(q7), sn7 = std::sin(q7);
                double gap = 1e30;
                for (int t = t0; t <= t1 && gap > kRow5Margin; t++) {
                    // hand sphere in the joint-5 frame: F6 Rz(q6) F7 Rz(q7) x
                    const SphereDef &x = kDet[t];
                    const double y0 = c7 * x.x - sn7 * x.y + 0.088, y1 = -(double)x.z, y2 = sn7 * x.x + c7 * x.y;
                    const double p0 = c6 * y0 - sn6 * y1, p1 = -y2, p2 = sn6 * y0 + c6 * y1;
                    for (int s = s0; s <= s1; s++) {
                        const double d0 = kDet[s].x - p0, d1 = kDet[s].y - p1, d2 = kDet[s].z - p2;
                        gap = std::fmin(gap, std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) - R[s - s0] - x.r -
                                                 slack[t - t0]);
                    }
                }
                if (gap > kRow5Margin) {
                    const int cell = i6 * kRow5N7 + i7;
                    tab[cell >> 5] |= 1u << (cell & 31);
                }
            }
        }
    });
    return tab;
}

std::mutex g_row5_mu;
const uint32_t *g_row5_dev[64] = {};

// Device copy of the table on the current device (uploaded on first use).
cudaError_t row5_device_table(const uint32_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const std::vector<uint32_t> &tab = row5_host_table();
    std::lock_guard<std::mutex> lk(g_row5_mu);
    if (!g_row5_dev[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_row5);
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_row5, tab.data(), tab.size() * sizeof(uint32_t));
        if (e != cudaSuccess) return e;
        g_row5_dev[dev] = (const uint32_t *)p;
    }
    *out = g_row5_dev[dev];
    return cudaSuccess;
}

// Largest staged scene: the block's dynamic shared memory stays below this.
constexpr size_t kMaxDynSmem = 200 * 1024;

}  // namespace

struct mrpop_scene {
    float4 *d_buf = nullptr;          // packed obstacles (float4 units)
    const uint32_t *row5 = nullptr;   // forearm-hand rows table on the scene's device
    unsigned int *d_status = nullptr; // bounded-wait error word
    mrpop::SceneCounts counts{};
    int total_f4 = 0;
    double env_test_flops = 0.0;
    int device = 0;
};

struct mrpop_robotset {
    int n_arms = 0;
    float base[mrpop::kMaxArms][12] = {};
};

struct mrpop_workspace {
    cudaStream_t stream = nullptr;
    int device = 0;
    float *d_q0 = nullptr, *d_q1 = nullptr;
    uint8_t *d_valid = nullptr;
    int32_t *d_first = nullptr;
    size_t cap_cfg = 0, cap_edges = 0;
};

extern "C" {

const char *mrpop_last_error(void) { return g_last_error.c_str(); }
const char *mrpop_version(void) { return "mrpop-gb300 0.1.0 (sm_103a)"; }

mrpop_status mrpop_scene_create(const mrpop_scene_desc *desc, mrpop_scene **out) {
    if (!desc || !out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "scene_create: null argument");
    *out = nullptr;
    auto need = [](const float *p, uint32_t n) { return n == 0 || p != nullptr; };
    if (!need(desc->spheres, desc->num_spheres) || !need(desc->capsules, desc->num_capsules) ||
        !need(desc->z_capsules, desc->num_z_capsules) || !need(desc->cuboids, desc->num_cuboids) ||
        !need(desc->z_cuboids, desc->num_z_cuboids) || !need(desc->cylinders, desc->num_cylinders))
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "scene_create: null array with nonzero count");
    mrpop::SceneCounts c{(int)desc->num_spheres, (int)desc->num_capsules, (int)desc->num_z_capsules,
                         (int)desc->num_cuboids, (int)desc->num_z_cuboids};
    const mrpop::SceneLayout L = mrpop::scene_layout(c);
    if ((size_t)L.total * sizeof(float4) + block_scratch_bytes() > kMaxDynSmem)
        return fail(MRPOP_ERR_UNSUPPORTED, "scene_create: scene too large to stage in shared memory (" +
                                               std::to_string(L.total * 16) + " bytes)");
    std::vector<float4> h((size_t)L.total);
    for (int i = 0; i < c.n_sph; i++) {
        const float *s = desc->spheres + 4 * i;
        h[L.sph + i] = make_float4(s[0], s[1], s[2], s[3]);
    }
    auto put_caps = [&](int off, const float *src, int n) {
        for (int i = 0; i < n; i++) {
            const float *s = src + 8 * i;
            h[off + 2 * i] = make_float4(s[0], s[1], s[2], s[6]);     // x1 y1 z1 r
            h[off + 2 * i + 1] = make_float4(s[3], s[4], s[5], s[7]); // xv yv zv rdv
        }
    };
    put_caps(L.cap, desc->capsules, c.n_cap);
    put_caps(L.zcap, desc->z_capsules, c.n_zcap);
    auto put_cubs = [&](int off, const float *src, int n) {
        for (int i = 0; i < n; i++) {
            const float *s = src + 15 * i;
            h[off + 4 * i] = make_float4(s[0], s[1], s[2], s[12]);    // centre, h1
            h[off + 4 * i + 1] = make_float4(s[3], s[4], s[5], s[13]); // axis 1, h2
            h[off + 4 * i + 2] = make_float4(s[6], s[7], s[8], s[14]); // axis 2, h3
            h[off + 4 * i + 3] = make_float4(s[9], s[10], s[11], 0.f); // axis 3
        }
    };
    put_cubs(L.cub, desc->cuboids, c.n_cub);
    put_cubs(L.zcub, desc->z_cuboids, c.n_zcub);
    // bounding spheres (culling only; exact tests decide every verdict)
    const double margin = mrpop::kCullMargin;
    auto bound = [&](double x, double y, double z, double r) {
        return make_float4((float)x, (float)y, (float)z, (float)(r * 1.002 + margin));
    };
    auto unit = [](double x, double y, double z) { return std::fabs(std::sqrt(x * x + y * y + z * z) - 1.0) < 1e-3; };
    for (int k = 0; k < 2; k++) {
        const float *src = k ? desc->z_cuboids : desc->cuboids;
        const int n = k ? c.n_zcub : c.n_cub, off = k ? L.b_zcub : L.b_cub;
        for (int i = 0; i < n; i++) {
            const float *b = src + 15 * i;
            bool ortho;
            if (k == 0)
                ortho = unit(b[3], b[4], b[5]) && unit(b[6], b[7], b[8]) && unit(b[9], b[10], b[11]) &&
                        std::fabs((double)b[3] * b[6] + (double)b[4] * b[7] + (double)b[5] * b[8]) < 1e-3 &&
                        std::fabs((double)b[3] * b[9] + (double)b[4] * b[10] + (double)b[5] * b[11]) < 1e-3 &&
                        std::fabs((double)b[6] * b[9] + (double)b[7] * b[10] + (double)b[8] * b[11]) < 1e-3;
            else
                ortho = unit(b[3], b[4], 0.0) && unit(b[6], b[7], 0.0) &&
                        std::fabs((double)b[3] * b[6] + (double)b[4] * b[7]) < 1e-3;
            const double hr = std::sqrt((double)b[12] * b[12] + (double)b[13] * b[13] + (double)b[14] * b[14]);
            h[off + i] = bound(b[0], b[1], b[2], ortho ? hr : 1e18);
        }
    }
    for (int k = 0; k < 2; k++) {
        const float *src = k ? desc->z_capsules : desc->capsules;
        const int n = k ? c.n_zcap : c.n_cap, off = k ? L.b_zcap : L.b_cap;
        for (int i = 0; i < n; i++) {
            const float *b = src + 8 * i;
            const double vx = k ? 0.0 : b[3], vy = k ? 0.0 : b[4], vz = b[5];
            const double len = std::sqrt(vx * vx + vy * vy + vz * vz);
            h[off + i] = bound(b[0] + 0.5 * vx, b[1] + 0.5 * vy, b[2] + 0.5 * vz, 0.5 * len + b[6]);
        }
    }
    for (int i = 0; i < c.n_sph; i++) {
        const float *b = desc->spheres + 4 * i;
        h[L.b_sph + i] = bound(b[0], b[1], b[2], b[3]);
    }

    mrpop_scene *sc = new (std::nothrow) mrpop_scene();
    if (!sc) return fail(MRPOP_ERR_OUT_OF_MEMORY, "scene_create: host allocation");
    sc->counts = c;
    sc->total_f4 = L.total;
    sc->env_test_flops = 27.0 * (c.n_cub + c.n_zcub) + 26.0 * (c.n_cap + c.n_zcap) + 11.0 * c.n_sph;
    cudaGetDevice(&sc->device);
    cudaError_t e = row5_device_table(&sc->row5);
    if (e == cudaSuccess) e = cudaMalloc(&sc->d_status, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(sc->d_status, 0, sizeof(unsigned int));
    if (e == cudaSuccess && L.total > 0) e = cudaMalloc(&sc->d_buf, (size_t)L.total * sizeof(float4));
    if (e == cudaSuccess && L.total > 0)
        e = cudaMemcpy(sc->d_buf, h.data(), (size_t)L.total * sizeof(float4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(sc->d_buf);
        cudaFree(sc->d_status);
        delete sc;
        return cuda_fail(e, "scene_create");
    }
    *out = sc;
    return MRPOP_OK;
}

mrpop_status mrpop_scene_destroy(mrpop_scene *scene) {
    if (!scene) return MRPOP_OK;
    cudaFree(scene->d_buf);
    cudaFree(scene->d_status);
    delete scene;
    return MRPOP_OK;
}

mrpop_status mrpop_scene_status(const mrpop_scene *scene, uint32_t *status_out) {
    if (!scene || !status_out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "scene_status: null argument");
    unsigned int v = 0;
    MRPOP_CUDA(cudaMemcpy(&v, scene->d_status, sizeof(v), cudaMemcpyDeviceToHost), "scene_status");
    *status_out = v;
    return MRPOP_OK;
}

mrpop_status mrpop_robotset_create(int n_arms, const float *base_T, mrpop_robotset **out) {
    if (!out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "robotset_create: null out");
    *out = nullptr;
    if (n_arms < 1 || n_arms > MRPOP_MAX_ARMS)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "robotset_create: n_arms must be 1..5");
    const float *src = base_T;
    static const float kIdent[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    if (!src) {
        if (n_arms == 1) src = kIdent;
        else if (n_arms == 4) src = &kQuadBase[0][0];
        else if (n_arms == 5) src = &kFiveBase[0][0];
        else
            return fail(MRPOP_ERR_INVALID_ARGUMENT,
                        "robotset_create: the reference has no built-in layout for this arm count");
    }
    mrpop_robotset *r = new (std::nothrow) mrpop_robotset();
    if (!r) return fail(MRPOP_ERR_OUT_OF_MEMORY, "robotset_create: host allocation");
    r->n_arms = n_arms;
    for (int a = 0; a < n_arms; a++)
        for (int i = 0; i < 12; i++) r->base[a][i] = src[16 * a + i];
    *out = r;
    return MRPOP_OK;
}

mrpop_status mrpop_robotset_destroy(mrpop_robotset *robots) {
    delete robots;
    return MRPOP_OK;
}

}  // extern "C"

namespace {

}  // namespace

namespace mrpop {

mrpop_status make_params(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0, const float *q1,
                         int64_t n_edges, int g, int rule, float range, uint32_t flags, int arm, uint8_t *valid,
                         int32_t *first_hit, int32_t *n_seg_out, double *flops, EdgeParams &p, int &A,
                         size_t &smem) {
    if (!scene || !robots) return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: null scene or robots");
    if (n_edges < 0) return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: n_edges < 0");
    if (n_edges > 0 && (!q0 || !q1 || ((!valid || !first_hit) && !flops)))
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: null device pointer");
    if (g < 1 || g > MRPOP_MAX_GRANULARITY)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: granularity must be 1..64");
    if (rule < MRPOP_RULE_PLAIN || rule > MRPOP_RULE_SHORTCUT)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: unknown segmentation rule");
    if (rule != MRPOP_RULE_PLAIN && !(range > 0.0f))
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: range must be > 0");
    if (flags & ~(MRPOP_CHECK_ENV | MRPOP_CHECK_SELF | MRPOP_MODE_EXACT))
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: unknown flag bits");
    if (arm >= robots->n_arms) return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: arm out of range");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != scene->device) return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate: scene lives on another device");

    p = EdgeParams{};
    p.q0 = q0;
    p.q1 = q1;
    p.n_edges = n_edges;
    p.g = g;
    p.flags = (int)flags;
    p.single = arm >= 0 ? 1 : 0;
    p.rule = rule;
    p.range = range;
    p.valid = valid;
    p.first_hit = first_hit;
    p.n_seg_out = n_seg_out;
    p.flops = flops;
    p.scene = scene->d_buf;
    p.sc = scene->counts;
    p.status = scene->d_status;
    p.phase = g_phase_counters;
    p.env_test_flops = scene->env_test_flops;
    p.row5 = scene->row5;
    static const int kGroupFirst[12] = {0, 1, 5, 9, 13, 17, 19, 21, 29, 32, 37, 59};
    for (int gi = 0; gi < 11; gi++) {
        double lo[3] = {1e9, 1e9, 1e9}, hi[3] = {-1e9, -1e9, -1e9};
        for (int i = kGroupFirst[gi]; i < kGroupFirst[gi + 1]; i++) {
            const double v[3] = {kDet[i].x, kDet[i].y, kDet[i].z};
            for (int c = 0; c < 3; c++) {
                lo[c] = std::fmin(lo[c], v[c]);
                hi[c] = std::fmax(hi[c], v[c]);
            }
        }
        const double cx = 0.5 * (lo[0] + hi[0]), cy = 0.5 * (lo[1] + hi[1]), cz = 0.5 * (lo[2] + hi[2]);
        double r = 0.0;
        for (int i = kGroupFirst[gi]; i < kGroupFirst[gi + 1]; i++) {
            const SphereDef &d = kDet[i];
            r = std::fmax(r, std::sqrt((d.x - cx) * (d.x - cx) + (d.y - cy) * (d.y - cy) + (d.z - cz) * (d.z - cz)) + d.r);
        }
        p.grp[gi] = make_float4((float)cx, (float)cy, (float)cz, (float)(r * 1.001 + kCullMargin));
        const SphereDef &ref = kApprox[grp_ref(gi)];
        const double ox = cx - ref.x, oy = cy - ref.y, oz = cz - ref.z;
        p.gofs[gi] = (float)(std::sqrt(ox * ox + oy * oy + oz * oz) * 1.001 + r * 1.001 + kCullMargin);
    }
    // the hand group's three parts (bits of hand_part over spheres kHandFirst..)
    for (int s = 0; s < kHandParts; s++) {
        double lo[3] = {1e9, 1e9, 1e9}, hi[3] = {-1e9, -1e9, -1e9};
        for (uint32_t m = hand_part(s); m; m &= m - 1) {
            const SphereDef &d = kDet[kHandFirst + __builtin_ctz(m)];
            const double v[3] = {d.x, d.y, d.z};
            for (int c = 0; c < 3; c++) {
                lo[c] = std::fmin(lo[c], v[c]);
                hi[c] = std::fmax(hi[c], v[c]);
            }
        }
        const double cx = 0.5 * (lo[0] + hi[0]), cy = 0.5 * (lo[1] + hi[1]), cz = 0.5 * (lo[2] + hi[2]);
        double r = 0.0;
        for (uint32_t m = hand_part(s); m; m &= m - 1) {
            const SphereDef &d = kDet[kHandFirst + __builtin_ctz(m)];
            r = std::fmax(r, std::sqrt((d.x - cx) * (d.x - cx) + (d.y - cy) * (d.y - cy) + (d.z - cz) * (d.z - cz)) + d.r);
        }
        p.hsub[s] = make_float4((float)cx, (float)cy, (float)cz, (float)(r * 1.001 + kCullMargin));
    }
    A = arm >= 0 ? 1 : robots->n_arms;
    for (int a = 0; a < A; a++)
        for (int i = 0; i < 12; i++) p.base[a][i] = robots->base[arm >= 0 ? arm : a][i];
    p.fbp = broad_flops_per_sample(A, scene->env_test_flops, flags);
    smem = (size_t)scene->total_f4 * sizeof(float4) + block_scratch_bytes();
    return MRPOP_OK;
}

// A 128-byte head with the two work counters, then per edge: flag words,
// candidate masks, reference-sphere bounds and segment state.  The kernels
// stage the flag words as 32-bit pairs for up to 4 arms, in the first half
// of their slice (which keeps its 64-bit size).
int robotset_arms(const mrpop_robotset *robots) { return robots ? robots->n_arms : 0; }

void set_split_scratch(EdgeParams &p, void *scratch, int64_t n_edges, int g, int A) {
    const int spl = g > 32 ? 2 : 1;
    const size_t flag_bytes = (size_t)n_edges * 32 * spl * 2 * sizeof(uint64_t);
    const size_t mask_bytes = (size_t)n_edges * 2 * sizeof(uint64_t);
    const size_t bound_bytes = (size_t)n_edges * A * kRefSpheres * sizeof(float4);
    p.work = (unsigned long long *)scratch;
    char *b = (char *)scratch + kSplitScratchHead;
    p.sflags = (uint64_t *)b;
    p.smasks = (uint64_t *)(b + flag_bytes);
    p.sbounds = (float4 *)(b + flag_bytes + mask_bytes);
    p.snseg = (int32_t *)(b + flag_bytes + mask_bytes + bound_bytes);
    p.sdone = p.snseg + n_edges;
}

// ext_scratch: caller-provided device scratch for the single-segment pipeline
// (at least split_scratch_bytes(n_edges, g, arms) bytes); nullptr = the
// library's stream-ordered pool.
// Calls of at most this many edges run as one fused launch (mrpop_set_fused_edges).
constexpr int64_t kFusedEdgesDefault = 2048;
std::atomic<int64_t> g_fused_edges{kFusedEdgesDefault};

mrpop_status run_validator(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0,
                           const float *q1, int64_t n_edges, int g, int rule, float range, uint32_t flags,
                           int arm, uint8_t *valid, int32_t *first_hit, int32_t *n_seg_out, double *flops,
                           cudaStream_t stream, void *ext_scratch) {
    EdgeParams p;
    int A = 0;
    size_t smem = 0;
    const mrpop_status st = make_params(scene, robots, q0, q1, n_edges, g, rule, range, flags, arm, valid, first_hit,
                                        n_seg_out, flops, p, A, smem);
    if (st != MRPOP_OK || n_edges == 0) return st;

    // scratch outputs when only the tally is wanted
    uint8_t *tmp_valid = nullptr;
    int32_t *tmp_first = nullptr;
    if (!valid || !first_hit) {
        MRPOP_CUDA(cudaMallocAsync(&tmp_valid, (size_t)n_edges, stream), "validate: tally scratch");
        MRPOP_CUDA(cudaMallocAsync(&tmp_first, (size_t)n_edges * 4, stream), "validate: tally scratch");
        p.valid = tmp_valid;
        p.first_hit = tmp_first;
    }
    // a small call: one fused launch from segment 0, no staging; with 3 or
    // more arms one warp per arm, else above 32 samples per segment two warps
    // per edge (one per 32-sample slot), unless the flop tally is wanted
    cudaError_t err;
    if (n_edges <= g_fused_edges.load(std::memory_order_relaxed)) {
        p.seg0 = 0;
        err = timed_launch(A, flops ? kFused : A >= 3 ? kArmwise : g > 32 ? kFusedPair : kFused, p, smem, stream);
        if (tmp_valid) cudaFreeAsync(tmp_valid, stream);
        if (tmp_first) cudaFreeAsync(tmp_first, stream);
        if (err != cudaSuccess) return cuda_fail(err, "validate: launch");
        return MRPOP_OK;
    }
    // split pipeline: staged flags, masks, bounds and segment state in
    // stream-ordered scratch.  Single-segment edges: one broad and one narrow
    // launch.  Segmented rules: segment r of every undecided edge per round
    // (broad + narrow), kSegRounds rounds, then the fused kernel for the edges
    // that still have segments left, from segment kSegRounds on.
    void *scratch = ext_scratch;
    if (!scratch) {
        cudaMemPool_t pool;
        err = scratch_pool(&pool);
        if (err == cudaSuccess) err = cudaMallocFromPoolAsync(&scratch, split_scratch_bytes(n_edges, g, A), pool, stream);
    } else {
        err = cudaSuccess;
    }
    if (err == cudaSuccess) {
        set_split_scratch(p, scratch, n_edges, g, A);
        const int rounds = rule == MRPOP_RULE_PLAIN ? 1 : kSegRounds;
        for (int r = 0; r < rounds && err == cudaSuccess; r++) {
            p.seg0 = r;
            err = cudaMemsetAsync(p.work, 0, 2 * sizeof(unsigned long long), stream);
            if (err == cudaSuccess) err = timed_launch(A, kBroad, p, smem, stream);
            if (err == cudaSuccess) err = timed_launch(A, kNarrow, p, smem, stream);
        }
        if (err == cudaSuccess && rule != MRPOP_RULE_PLAIN) {
            p.seg0 = kSegRounds;
            err = timed_launch(A, kFused, p, smem, stream);
        }
        if (!ext_scratch) cudaFreeAsync(scratch, stream);
    }
    if (tmp_valid) cudaFreeAsync(tmp_valid, stream);
    if (tmp_first) cudaFreeAsync(tmp_first, stream);
    if (err != cudaSuccess) return cuda_fail(err, "validate: launch");
    return MRPOP_OK;
}

mrpop_status fail_status(mrpop_status st, const char *msg) { return fail(st, msg); }

int64_t set_fused_edges(int64_t max_edges) {
    return g_fused_edges.exchange(max_edges == 0 ? kFusedEdgesDefault : max_edges < 0 ? -1 : max_edges);
}

}  // namespace mrpop

namespace {

struct Base12 {
    float m[12];
};

__global__ void fk_spheres_kernel(const float *q, long long n, int detailed, const Base12 base, float *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float b[12];
    for (int i = 0; i < 12; i++) b[i] = base.m[i];
    float qq[7];
    for (int d = 0; d < 7; d++) qq[d] = q[t * 7 + d];
    if (!detailed) {
        mrpop::ArmSpheres s;
        mrpop::fk_approx_arm(b, qq, s);
        for (int i = 0; i < mrpop::kNumApprox; i++) {
            out[(t * mrpop::kNumApprox + i) * 3 + 0] = s.x[i];
            out[(t * mrpop::kNumApprox + i) * 3 + 1] = s.y[i];
            out[(t * mrpop::kNumApprox + i) * 3 + 2] = s.z[i];
        }
        return;
    }
    // detailed: the narrow phase's run-time path (joint chain + placement)
    float Tj[mrpop::kNumJoints][12];
    mrpop::Xf T;
    mrpop::load_base(T, b);
    for (int i = 0; i < 12; i++) Tj[0][i] = T.m[i];
    for (int j = 1; j < mrpop::kNumJoints; j++) {
        mrpop::joint_step_rt(T, qq[j - 1], j);
        for (int i = 0; i < 12; i++) Tj[j][i] = T.m[i];
    }
    for (int i = 0; i < mrpop::kNumDet; i++) {
        const float3 p = mrpop::place_rt(Tj[mrpop::det_joint(i)], mrpop::c_det[i]);
        out[(t * mrpop::kNumDet + i) * 3 + 0] = p.x;
        out[(t * mrpop::kNumDet + i) * 3 + 1] = p.y;
        out[(t * mrpop::kNumDet + i) * 3 + 2] = p.z;
    }
}

// One CTA waits, with the kernels' bounded copy wait, on an mbarrier whose
// expected bytes no copy will deliver: the wait runs out after limit_ns,
// sets the status bit and returns.
__global__ void wait_timeout_kernel(unsigned long long limit_ns, unsigned int *status, unsigned long long *elapsed) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mrpop::smem_u32(&bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mrpop::smem_u32(&bar)), "r"(16u)
                     : "memory");
    const unsigned long long t0 = mrpop::global_ns();
    const bool ok = mrpop::copy_wait(&bar, 0, status, limit_ns);
    if (threadIdx.x == 0) *elapsed = ok ? 0ull : mrpop::global_ns() - t0;
}

__global__ void trig_kernel(const float *x, long long n, float *c, float *s) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float v = x[t];
    c[t] = __cosf(v);
    s[t] = __sinf(v);
}

}  // namespace

namespace mrpop {
size_t warp_scratch_bytes() { return sizeof(WarpScratch); }

cudaError_t batch_occupancy(int arms, int mode, bool seg, int spl, size_t smem_bytes, int warps, int *blocks_per_sm) {
    switch (arms) {
    case 1: return batch_occupancy_arms<1>(mode, seg, spl, smem_bytes, warps, blocks_per_sm);
    case 2: return batch_occupancy_arms<2>(mode, seg, spl, smem_bytes, warps, blocks_per_sm);
    case 3: return batch_occupancy_arms<3>(mode, seg, spl, smem_bytes, warps, blocks_per_sm);
    case 4: return batch_occupancy_arms<4>(mode, seg, spl, smem_bytes, warps, blocks_per_sm);
    case 5: return batch_occupancy_arms<5>(mode, seg, spl, smem_bytes, warps, blocks_per_sm);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch(int arms, int mode, bool seg, int spl, const BatchParams &b, size_t smem_bytes, int grid,
                         int warps, cudaStream_t stream) {
    switch (arms) {
    case 1: return launch_batch_arms<1>(mode, seg, spl, b, smem_bytes, grid, warps, stream);
    case 2: return launch_batch_arms<2>(mode, seg, spl, b, smem_bytes, grid, warps, stream);
    case 3: return launch_batch_arms<3>(mode, seg, spl, b, smem_bytes, grid, warps, stream);
    case 4: return launch_batch_arms<4>(mode, seg, spl, b, smem_bytes, grid, warps, stream);
    case 5: return launch_batch_arms<5>(mode, seg, spl, b, smem_bytes, grid, warps, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_validate(int arms, KernelKind kind, const EdgeParams &p, size_t smem_bytes, cudaStream_t stream) {
    switch (arms) {
    case 1: return launch_validate_arms<1>(kind, p, smem_bytes, stream);
    case 2: return launch_validate_arms<2>(kind, p, smem_bytes, stream);
    case 3: return launch_validate_arms<3>(kind, p, smem_bytes, stream);
    case 4: return launch_validate_arms<4>(kind, p, smem_bytes, stream);
    case 5: return launch_validate_arms<5>(kind, p, smem_bytes, stream);
    default: return cudaErrorInvalidValue;
    }
}
}  // namespace mrpop

extern "C" {

// Development hook: device array of >= 16 counters for builds with
// MRPOP_PHASE_TIMERS (ignored otherwise).  Not part of the public header.
void mrpop_dev_phase_counters(unsigned long long *dev_counters) { g_phase_counters = dev_counters; }

mrpop_status mrpop_validate_edges(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0,
                                  const float *q1, int64_t n_edges, int granularity, uint32_t flags, int arm,
                                  uint8_t *valid, int32_t *first_hit, void *stream) {
    return mrpop::run_validator(scene, robots, q0, q1, n_edges, granularity, MRPOP_RULE_PLAIN, 0.0f, flags, arm,
                                valid, first_hit, nullptr, nullptr, (cudaStream_t)stream, nullptr);
}

mrpop_status mrpop_validate_segments(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0,
                                     const float *q1, int64_t n_edges, int granularity, int rule, float range,
                                     uint32_t flags, int arm, uint8_t *valid, int32_t *first_hit,
                                     int32_t *n_seg_out, void *stream) {
    return mrpop::run_validator(scene, robots, q0, q1, n_edges, granularity, rule, range, flags, arm, valid,
                                first_hit, n_seg_out, nullptr, (cudaStream_t)stream, nullptr);
}

mrpop_status mrpop_count_flops(const mrpop_scene *scene, const mrpop_robotset *robots, const float *q0,
                               const float *q1, int64_t n_edges, int granularity, int rule, float range,
                               uint32_t flags, int arm, double *flops, void *stream) {
    if (!flops) return fail(MRPOP_ERR_INVALID_ARGUMENT, "count_flops: null output");
    return mrpop::run_validator(scene, robots, q0, q1, n_edges, granularity, rule, range, flags, arm, nullptr,
                                nullptr, nullptr, flops, (cudaStream_t)stream, nullptr);
}

mrpop_status mrpop_broad_flops_per_sample(const mrpop_scene *scene, const mrpop_robotset *robots, uint32_t flags,
                                          int arm, double *out) {
    if (!scene || !robots || !out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "broad_flops_per_sample: null argument");
    if (arm >= robots->n_arms) return fail(MRPOP_ERR_INVALID_ARGUMENT, "broad_flops_per_sample: arm out of range");
    *out = broad_flops_per_sample(arm >= 0 ? 1 : robots->n_arms, scene->env_test_flops, flags);
    return MRPOP_OK;
}

mrpop_status mrpop_debug_row5_table(uint32_t *out, int64_t words, int *n6, int *n7) {
    if (!out || !n6 || !n7) return fail(MRPOP_ERR_INVALID_ARGUMENT, "debug_row5_table: null argument");
    if (words < mrpop::kRow5Words) return fail(MRPOP_ERR_INVALID_ARGUMENT, "debug_row5_table: buffer too small");
    const std::vector<uint32_t> &tab = row5_host_table();
    std::memcpy(out, tab.data(), tab.size() * sizeof(uint32_t));
    *n6 = mrpop::kRow5N6;
    *n7 = mrpop::kRow5N7;
    return MRPOP_OK;
}

int64_t mrpop_set_fused_edges(int64_t max_edges) { return mrpop::set_fused_edges(max_edges); }

mrpop_status mrpop_kernel_timing(int enable) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timing_on = enable != 0;
    return MRPOP_OK;
}

mrpop_status mrpop_kernel_times(int64_t *launches, double *ms) {
    if (!launches || !ms) return fail(MRPOP_ERR_INVALID_ARGUMENT, "kernel_times: null argument");
    std::vector<TimedLaunch> taken;
    {
        std::lock_guard<std::mutex> lk(g_timing_mu);
        taken.swap(g_timed);
    }
    for (int k = 0; k < MRPOP_KERNEL_KINDS; k++) {
        launches[k] = 0;
        ms[k] = 0.0;
    }
    cudaError_t first_err = cudaSuccess;
    for (const TimedLaunch &t : taken) {
        float dt = 0.0f;
        cudaError_t e = cudaEventSynchronize(t.stop);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&dt, t.start, t.stop);
        if (e == cudaSuccess) {
            launches[t.kind] += 1;
            ms[t.kind] += dt;
        } else if (first_err == cudaSuccess) {
            first_err = e;
        }
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    if (first_err != cudaSuccess) return cuda_fail(first_err, "kernel_times");
    return MRPOP_OK;
}

mrpop_status mrpop_fk_spheres(const mrpop_robotset *robots, int arm, const float *q, int64_t n, int detailed,
                              float *out, void *stream) {
    if (!robots || !q || !out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "fk_spheres: null argument");
    if (arm < 0 || arm >= robots->n_arms) return fail(MRPOP_ERR_INVALID_ARGUMENT, "fk_spheres: arm out of range");
    if (n <= 0) return MRPOP_OK;
    Base12 b;
    for (int i = 0; i < 12; i++) b.m[i] = robots->base[arm][i];
    const int tpb = 128;
    fk_spheres_kernel<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, (cudaStream_t)stream>>>(q, n, detailed, b, out);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return cuda_fail(err, "fk_spheres: launch");
    return MRPOP_OK;
}

mrpop_status mrpop_debug_wait_timeout(int64_t limit_ns, uint32_t *status_out, int64_t *elapsed_ns_out) {
    if (!status_out || !elapsed_ns_out || limit_ns <= 0 || limit_ns > 2000000000ll)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "debug_wait_timeout: limit 1 ns .. 2 s, non-null outputs");
    unsigned int *d_status = nullptr;
    unsigned long long *d_elapsed = nullptr;
    MRPOP_CUDA(cudaMalloc(&d_status, sizeof(unsigned int)), "debug_wait_timeout: status");
    cudaError_t e = cudaMalloc(&d_elapsed, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d_status, 0, sizeof(unsigned int));
    if (e == cudaSuccess) {
        wait_timeout_kernel<<<1, 32>>>((unsigned long long)limit_ns, d_status, d_elapsed);
        e = cudaGetLastError();
    }
    unsigned int st = 0;
    unsigned long long el = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, d_status, sizeof(st), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&el, d_elapsed, sizeof(el), cudaMemcpyDeviceToHost);
    cudaFree(d_status);
    cudaFree(d_elapsed);
    MRPOP_CUDA(e, "debug_wait_timeout: run");
    *status_out = st;
    *elapsed_ns_out = (int64_t)el;
    return MRPOP_OK;
}

mrpop_status mrpop_debug_trig(const float *x, int64_t n, float *cos_out, float *sin_out, void *stream) {
    if (!x || !cos_out || !sin_out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "debug_trig: null argument");
    if (n <= 0) return MRPOP_OK;
    const int tpb = 256;
    trig_kernel<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, (cudaStream_t)stream>>>(x, n, cos_out, sin_out);
    MRPOP_CUDA(cudaGetLastError(), "debug_trig: launch");
    return MRPOP_OK;
}

mrpop_status mrpop_workspace_create(mrpop_workspace **out) {
    if (!out) return fail(MRPOP_ERR_INVALID_ARGUMENT, "workspace_create: null out");
    mrpop_workspace *w = new (std::nothrow) mrpop_workspace();
    if (!w) return fail(MRPOP_ERR_OUT_OF_MEMORY, "workspace_create: host allocation");
    cudaGetDevice(&w->device);
    cudaError_t e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete w;
        return cuda_fail(e, "workspace_create");
    }
    *out = w;
    return MRPOP_OK;
}

mrpop_status mrpop_workspace_destroy(mrpop_workspace *ws) {
    if (!ws) return MRPOP_OK;
    cudaStreamSynchronize(ws->stream);
    cudaFree(ws->d_q0);
    cudaFree(ws->d_q1);
    cudaFree(ws->d_valid);
    cudaFree(ws->d_first);
    cudaStreamDestroy(ws->stream);
    delete ws;
    return MRPOP_OK;
}

// Device address of a page-locked host buffer (mapped into the GPU's address
// space), or nullptr for any other memory.
static void *mapped_host(const void *h) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

mrpop_status mrpop_validate_edges_host(mrpop_workspace *ws, const mrpop_scene *scene, const mrpop_robotset *robots,
                                       const float *q0, const float *q1, int64_t n_edges, int granularity,
                                       uint32_t flags, int arm, int rule, float range, uint8_t *valid,
                                       int32_t *first_hit) {
    if (!ws || !robots) return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate_edges_host: null argument");
    if (n_edges <= 0) return n_edges == 0 ? MRPOP_OK : fail(MRPOP_ERR_INVALID_ARGUMENT, "n_edges < 0");
    if (!q0 || !q1 || !valid || !first_hit)
        return fail(MRPOP_ERR_INVALID_ARGUMENT, "validate_edges_host: null host pointer");
    const int dof = 7 * (arm >= 0 ? 1 : robots->n_arms);
    const size_t ncfg = (size_t)n_edges * dof;
    // Page-locked host buffers are used in place: the kernels read the
    // endpoints from host memory and write the verdicts there (over NVLink-C2C
    // on a Grace host), so no staging copy precedes or follows them.  Other
    // buffers go through the workspace's device arrays.
    const float *m_q0 = static_cast<const float *>(mapped_host(q0));
    const float *m_q1 = static_cast<const float *>(mapped_host(q1));
    uint8_t *m_valid = static_cast<uint8_t *>(mapped_host(valid));
    int32_t *m_first = static_cast<int32_t *>(mapped_host(first_hit));
    if (m_q0 && m_q1 && m_valid && m_first) {
        mrpop_status s = mrpop::run_validator(scene, robots, m_q0, m_q1, n_edges, granularity, rule, range, flags,
                                              arm, m_valid, m_first, nullptr, nullptr, ws->stream, nullptr);
        if (s != MRPOP_OK) return s;
        MRPOP_CUDA(cudaStreamSynchronize(ws->stream), "validate_edges_host: sync");
        return MRPOP_OK;
    }
    if (ncfg > ws->cap_cfg) {
        cudaFree(ws->d_q0);
        cudaFree(ws->d_q1);
        ws->d_q0 = ws->d_q1 = nullptr;
        ws->cap_cfg = 0;
        MRPOP_CUDA(cudaMalloc(&ws->d_q0, ncfg * sizeof(float)), "validate_edges_host: alloc");
        MRPOP_CUDA(cudaMalloc(&ws->d_q1, ncfg * sizeof(float)), "validate_edges_host: alloc");
        ws->cap_cfg = ncfg;
    }
    if ((size_t)n_edges > ws->cap_edges) {
        cudaFree(ws->d_valid);
        cudaFree(ws->d_first);
        ws->d_valid = nullptr;
        ws->d_first = nullptr;
        ws->cap_edges = 0;
        MRPOP_CUDA(cudaMalloc(&ws->d_valid, (size_t)n_edges), "validate_edges_host: alloc");
        MRPOP_CUDA(cudaMalloc(&ws->d_first, (size_t)n_edges * 4), "validate_edges_host: alloc");
        ws->cap_edges = (size_t)n_edges;
    }
    cudaStream_t st = ws->stream;
    MRPOP_CUDA(cudaMemcpyAsync(ws->d_q0, q0, ncfg * sizeof(float), cudaMemcpyHostToDevice, st), "H2D q0");
    MRPOP_CUDA(cudaMemcpyAsync(ws->d_q1, q1, ncfg * sizeof(float), cudaMemcpyHostToDevice, st), "H2D q1");
    mrpop_status s = mrpop::run_validator(scene, robots, ws->d_q0, ws->d_q1, n_edges, granularity, rule, range,
                                          flags, arm, ws->d_valid, ws->d_first, nullptr, nullptr, st, nullptr);
    if (s != MRPOP_OK) return s;
    MRPOP_CUDA(cudaMemcpyAsync(valid, ws->d_valid, (size_t)n_edges, cudaMemcpyDeviceToHost, st), "D2H valid");
    MRPOP_CUDA(cudaMemcpyAsync(first_hit, ws->d_first, (size_t)n_edges * 4, cudaMemcpyDeviceToHost, st),
               "D2H first_hit");
    MRPOP_CUDA(cudaStreamSynchronize(st), "validate_edges_host: sync");
    return MRPOP_OK;
}

}  // extern "C"
