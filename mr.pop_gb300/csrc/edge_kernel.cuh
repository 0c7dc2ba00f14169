// edge_kernel.cuh -- the batched edge validator (sm_103a).
//
// One warp owns one edge at a time; warps take edges from a per-launch work
// counter (persistent grid).  Lane L evaluates samples k = L+1 (+32) of the
// edge.  Single-segment edges run as two kernels (broad, then narrow, the
// narrow kernel a programmatic dependent of the broad one); segmented rules
// run those two per segment round and a fused kernel for the tail.
//   broad phase  per lane: FK of every arm (FP32 FMA, __sinf/__cosf as the
//                reference), the 11 broad-phase spheres per arm against the
//                scene staged in shared memory (one bulk-async copy per CTA,
//                bounded mbarrier wait), the intra-arm pairs and the arm-vs-arm
//                pairs, each screened one pair per lane against swept bounds of
//                the warp's samples first; the result is a per-(arm, joint)
//                flag word and per-sample sphere counts, staged in HBM with the
//                swept bounds for the narrow kernel.
//   decision     per warp: shuffle reductions give the edge totals; the
//                reference's proportional 4g-thread split (utils.cuh:476-517)
//                is evaluated exactly to pick the samples that get a detailed
//                check (or every flagged sample in EXACT mode); ballots form
//                the candidate masks.
//   narrow phase lane per candidate sample: all lanes walk the arms' joint
//                chains in step (lanes without a candidate keep the others
//                company), test the detailed spheres of flagged joints against
//                obstacles that survive a warp-wide screen per sphere group,
//                the flagged intra-arm rows (the forearm-hand rows skipped
//                where a (q6, q7) table certifies them apart) and the
//                arm-vs-arm group pairs that survive a warp-wide screen; the
//                first hit is the lowest set bit of a warp ballot.
// Culling: every obstacle carries a bounding sphere (1 mm margin) and every
// arm / joint group a bounding sphere computed from its own sphere set; an
// exact test is skipped only where the bounds prove it cannot fire, so the
// set of tests that can fire -- and therefore every verdict -- is unchanged.
#pragma once
#include "panda_model.cuh"

namespace mrpop {

#ifndef MRPOP_MIN_BLOCKS
#define MRPOP_MIN_BLOCKS 3
#endif
// Optional per-phase warp timers (development builds with
// -DMRPOP_PHASE_TIMERS; compiled out otherwise): clock64() deltas of lane 0
// accumulated into P.phase[i].
#ifdef MRPOP_PHASE_TIMERS
#define MRPOP_PHASE_START() long long _phase_t = clock64();
#define MRPOP_PHASE(P, i)                                                                          \
    do {                                                                                           \
        __syncwarp();                                                                              \
        const long long _n = clock64();                                                            \
        if ((P).phase && (threadIdx.x & 31) == 0)                                                  \
            atomicAdd((P).phase + (i), (unsigned long long)(_n - _phase_t));                       \
        _phase_t = _n;                                                                             \
    } while (0)
#define MRPOP_COUNT(P, i, v)                                                                       \
    do {                                                                                           \
        if ((P).phase && (threadIdx.x & 31) == 0) atomicAdd((P).phase + (i), (unsigned long long)(v)); \
    } while (0)
// counter update from code without the parameter block (warp-uniform v)
// (per translation unit; set from the parameter block by the kernel prologue)
static __device__ unsigned long long *g_dev_phase;
#define MRPOP_PHASE_BIND(P) do { if (threadIdx.x == 0) g_dev_phase = (P).phase; __syncthreads(); } while (0)
// count of lanes with pred set; the vote runs on every lane of the warp,
// only the add is lane 0's
#define MRPOP_COUNT_LANES(i, pred)                                                                 \
    do {                                                                                           \
        const uint32_t _votes = __ballot_sync(kFull, (pred));                                      \
        MRPOP_COUNT_W(i, __popc(_votes));                                                          \
    } while (0)
#define MRPOP_COUNT_W(i, v)                                                                        \
    do {                                                                                           \
        if (g_dev_phase && (threadIdx.x & 31) == 0) atomicAdd(g_dev_phase + (i), (unsigned long long)(v)); \
    } while (0)
#else
#define MRPOP_COUNT_W(i, v) do { } while (0)
#define MRPOP_PHASE_BIND(P) do { } while (0)
#define MRPOP_COUNT_LANES(i, pred) do { } while (0)
#define MRPOP_PHASE_START()
#define MRPOP_PHASE(P, i) do { } while (0)
#define MRPOP_COUNT(P, i, v) do { } while (0)
#endif

constexpr int kWarpsPerBlock = 6;
constexpr int kMaxArms = 5;
constexpr int kMaxDof = 7 * kMaxArms;
constexpr int kCrossStash = 16;        // per-lane arm-vs-arm candidate spheres
constexpr float kCullMargin = 1e-3f;   // metres added to every bounding radius
constexpr float kApproxMaxR = 0.176f;  // largest broad-phase sphere radius

struct SceneCounts {
    int n_sph, n_cap, n_zcap, n_cub, n_zcub;
};

// Float4 offsets inside the packed scene buffer: obstacle records by class,
// then one bounding sphere {cx, cy, cz, radius + margin} per obstacle in the
// order cuboids, z-cuboids, capsules, z-capsules, spheres.
struct SceneLayout {
    int sph, cap, zcap, cub, zcub;
    int b_cub, b_zcub, b_cap, b_zcap, b_sph;
    int total;
};

__host__ __device__ inline SceneLayout scene_layout(const SceneCounts &c) {
    SceneLayout l;
    l.sph = 0;
    l.cap = l.sph + c.n_sph;
    l.zcap = l.cap + 2 * c.n_cap;
    l.cub = l.zcap + 2 * c.n_zcap;
    l.zcub = l.cub + 4 * c.n_cub;
    l.b_cub = l.zcub + 4 * c.n_zcub;
    l.b_zcub = l.b_cub + c.n_cub;
    l.b_cap = l.b_zcub + c.n_zcub;
    l.b_zcap = l.b_cap + c.n_cap;
    l.b_sph = l.b_zcap + c.n_zcap;
    l.total = l.b_sph + c.n_sph;
    return l;
}

// Approx spheres whose swept bounds the narrow phase reuses: 0..8 (the
// reference sphere of every detailed sub-group, see grp_ref).
constexpr int kRefSpheres = 9;
// Segmented rules: segments checked by rounds of the split kernels before the
// fused kernel takes the remaining ones.
constexpr int kSegRounds = 4;

struct EdgeParams {
    const float *q0;
    const float *q1;
    long long n_edges;
    int g;           // samples per segment
    int flags;       // MRPOP_CHECK_* | MRPOP_MODE_EXACT
    int single;      // 1: single-arm (fkcc_single_buffer_mr) semantics
    int rule;        // MRPOP_RULE_*
    int seg0;        // segmented rules: the segment this launch checks (split kernels) or starts at (fused)
    float range;
    uint8_t *valid;
    int32_t *first_hit;
    int32_t *n_seg_out;
    double *flops;   // optional per-edge algorithmic flop tally
    double fbp;      // broad-phase flops per sample (for the tally)
    double env_test_flops;
    const float4 *scene;
    SceneCounts sc;
    unsigned int *status;
    unsigned long long *phase;  // phase timers (MRPOP_PHASE_TIMERS builds only)
    uint64_t *sflags;           // split pipeline: per-sample {env, self} flag words (32-bit for <= 4 arms)
    uint64_t *smasks;           // split pipeline: per-edge {env, self} candidate masks
    float4 *sbounds;            // split pipeline: per-edge swept reference-sphere bounds [A][kRefSpheres]
    int32_t *snseg;             // segmented rules: per-edge segment count (-1: too many), from segment 0
    int32_t *sdone;             // segmented rules: per-edge verdict written
    unsigned long long *work;   // split kernels: next-edge counters {broad, narrow}, zero before each launch
    float gofs[11];             // sub-group g: |group centre - reference sphere centre| + group radius
    float4 grp[11];             // detailed sub-group bounds in their joint frame (+margin)
    float4 hsub[3];             // bounds of the hand group's three parts in the joint-7 frame (+margin)
    const uint32_t *row5;       // forearm-hand rows table (kRow5N6 x kRow5N7 bits), or nullptr
    float base[kMaxArms][12];   // row-major 3x4 per arm of this check
};

// Per-warp shared scratch.  The broad-phase and narrow-phase parts are never
// live at the same time and share storage.
struct WarpScratch {
    float base[kMaxDof];   // segment start (accumulated for CONNECT)
    float stepg[kMaxDof];  // per-sample step (delta/g or vec/g)
    float delta[kMaxDof];  // per-segment step (B-spline / shortcut accumulation)
    // bound of the centres of approx spheres 0..kRefSpheres-1 of each arm over
    // every sample of the segment ({centre, radius}, sphere radius excluded);
    // written by the broad phase, read by the narrow phase's arm-vs-arm screen
    float4 rsw[kMaxArms][kRefSpheres];
    // sub-group bounds over the segment's samples derived from rsw (the
    // narrow phase's arm-vs-arm screen)
    float4 gbd[kMaxArms][11];
    union {
        struct {
            float4 swept[kMaxArms][kNumApprox]; // per-arm swept bound of each approx sphere
            float cur[kNumApprox][3][32];   // per-lane approx spheres of the current arm
            float low[kNumApprox][3][32];   // per-lane approx spheres of a lower arm
        } broad;
        struct {
            union {
                float stash[kDetRows][3][32];        // first sphere of each detailed self row
                float cstash[kCrossStash][4][32];    // arm-vs-arm candidates {x, y, z, r}
            };
        } lanes;
    };
};

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEnvBit = 1, kSelfBit = 2, kExactBit = 16;
constexpr int kRulePlain = 0, kRuleConnect = 1, kRuleBspline = 2, kRuleShortcut = 3;
constexpr int kMaxSegments = 1 << 16;

// ---------------------------------------------------------------------------
// shared-memory staging of the scene: one bulk asynchronous copy (TMA engine)
// completed on an mbarrier, with a bounded wait.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// The global nanosecond timer.
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Every wait on an mbarrier is bounded in time: a copy that has not completed
// after kWaitLimitNs is reported (scene status bit) instead of waited for.
constexpr uint64_t kWaitLimitNs = 1000000000ull;

// Wait for phase `parity` of mbarrier `bar`: true once it has completed,
// false after limit_ns of global time without it.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns) {
    const uint64_t t0 = global_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// The wait of a bulk copy into shared memory.  If it runs out, the status bit
// is set and the copy, which may still be writing this CTA's shared memory,
// gets a second bounded wait before the caller reports its edges and leaves.
__device__ __forceinline__ bool copy_wait(uint64_t *bar, uint32_t parity, unsigned int *status, uint64_t limit_ns) {
    if (bar_wait(bar, parity, limit_ns)) return true;
    atomicOr(status, 1u);
    bar_wait(bar, parity, limit_ns);
    return false;
}

__device__ __forceinline__ bool stage_scene(float4 *dst, const float4 *src, uint32_t bytes, uint64_t *bar,
                                            unsigned int *status) {
    if (bytes == 0) return true;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(dst)),
            "l"(src), "r"(bytes), "r"(smem_u32(bar))
            : "memory");
    }
    return __syncthreads_and(copy_wait(bar, 0, status, kWaitLimitNs));
}

__device__ __forceinline__ bool near3(float x, float y, float z, float4 b, float r) {
    const float dx = x - b.x, dy = y - b.y, dz = z - b.z;
    const float rr = r + b.w;
    return dx * dx + dy * dy + dz * dz < rr * rr;
}

// ---------------------------------------------------------------------------
// FK of one arm for one sample: approx sphere centres
// ---------------------------------------------------------------------------
struct ArmSpheres {
    float x[kNumApprox], y[kNumApprox], z[kNumApprox];
};

template <int I>
__device__ __forceinline__ void place_approx(const Xf &T, ArmSpheres &s) {
    s.x[I] = place_coord<I, false>(T, 0);
    s.y[I] = place_coord<I, false>(T, 1);
    s.z[I] = place_coord<I, false>(T, 2);
}

__device__ __forceinline__ void fk_approx_arm(const float *base12, const float (&q)[7], ArmSpheres &s) {
    Xf T;
    load_base(T, base12);
    place_approx<0>(T, s);
    joint_step<1>(T, q[0]);
    place_approx<1>(T, s);
    joint_step<2>(T, q[1]);
    place_approx<2>(T, s);
    joint_step<3>(T, q[2]);
    place_approx<3>(T, s);
    joint_step<4>(T, q[3]);
    place_approx<4>(T, s);
    joint_step<5>(T, q[4]);
    place_approx<5>(T, s);
    joint_step<6>(T, q[5]);
    place_approx<6>(T, s);
    joint_step<7>(T, q[6]);
    place_approx<7>(T, s);
    place_approx<8>(T, s);
    place_approx<9>(T, s);
    place_approx<10>(T, s);
}

// Joint values of arm `a` for sample k of segment `seg` (call-site formulas,
// see the rule constants).
__device__ __forceinline__ void sample_q(const WarpScratch &W, int rule, int seg, int a, int k, float (&q)[7]) {
    const float fk = (float)k;
#pragma unroll
    for (int d = 0; d < 7; d++) {
        const int i = 7 * a + d;
        float v = __fmaf_rn(fk, W.stepg[i], W.base[i]);
        if (rule == kRuleBspline || rule == kRuleShortcut)
            for (int s = 0; s < seg; s++) v = __fadd_rn(v, W.delta[i]);
        q[d] = v;
    }
}

// One joint value (dof index i) of sample k of segment `seg`.
__device__ __forceinline__ float sample_q1(const WarpScratch &W, int rule, int seg, int i, int k) {
    float v = __fmaf_rn((float)k, W.stepg[i], W.base[i]);
    if (rule == kRuleBspline || rule == kRuleShortcut)
        for (int s = 0; s < seg; s++) v = __fadd_rn(v, W.delta[i]);
    return v;
}

// Warp-wide float min / max (redux.sync on f32, sm_100a family).  NaN inputs
// are ignored; a lane with a NaN position can never pass an exact test, so the
// bounds built from these stay conservative.
__device__ __forceinline__ float warp_min(float v) {
    float r;
    asm volatile("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float warp_max(float v) {
    float r;
    asm volatile("redux.sync.max.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}

// FK of one arm for this lane's sample; the 11 approx centres go to column
// `lane` of dst.  With swept != nullptr it also writes, for every approx
// sphere, a bound of that sphere over the warp's 32 samples: the centre of
// the box around its 32 centres, radius = half the box diagonal (+0.4 %) +
// sphere radius + cull margin.  If the sphere touches something at any of the
// samples, its swept bound touches it too (the margin covers FP rounding).
__device__ __forceinline__ void fk_approx_lane(const float *base12, const WarpScratch &W, int rule, int seg,
                                                   int qarm, int k, float (*dst)[3][32], int lane, float4 *swept,
                                                   float4 *rsw, bool merge) {
    float q[7];
    sample_q(W, rule, seg, qarm, k, q);
    ArmSpheres s;
    fk_approx_arm(base12, q, s);
#pragma unroll
    for (int i = 0; i < kNumApprox; i++) {
        dst[i][0][lane] = s.x[i];
        dst[i][1][lane] = s.y[i];
        dst[i][2][lane] = s.z[i];
    }
    if (!swept) return;
    __syncwarp();
    {
        // spheres 1..10: lane t < 30 takes coordinate t % 3 of sphere 1 + t / 3
        // over the 32 columns (start skewed by lane: conflict-free banks);
        // sphere 0 (the base frame's) by warp reductions
        float lo = 0.0f, hi = 0.0f;
        if (lane < 30) {
            const float *col = &dst[1 + lane / 3][lane % 3][0];
            lo = hi = col[lane];
#pragma unroll 8
            for (int l = 1; l < 32; l++) {
                const float v = col[(l + lane) & 31];
                lo = fminf(lo, v);
                hi = fmaxf(hi, v);
            }
        }
        const float ly = __shfl_down_sync(kFull, lo, 1), hy = __shfl_down_sync(kFull, hi, 1);
        const float lz = __shfl_down_sync(kFull, lo, 2), hz = __shfl_down_sync(kFull, hi, 2);
        const float l0x = warp_min(s.x[0]), h0x = warp_max(s.x[0]);
        const float l0y = warp_min(s.y[0]), h0y = warp_max(s.y[0]);
        const float l0z = warp_min(s.z[0]), h0z = warp_max(s.z[0]);
        const bool own = lane < 30 && lane % 3 == 0;
        const int i = own ? 1 + lane / 3 : 0;
        if (own || lane == 30) {
            const float ax = own ? lo : l0x, bx = own ? hi : h0x;
            const float ay = own ? ly : l0y, by = own ? hy : h0y;
            const float az = own ? lz : l0z, bz = own ? hz : h0z;
            const float dx = bx - ax, dy = by - ay, dz = bz - az;
            swept[i] = make_float4(0.5f * (ax + bx), 0.5f * (ay + by), 0.5f * (az + bz),
                                   0.5f * sqrtf(dx * dx + dy * dy + dz * dz) * 1.004f + c_approx[i].w + kCullMargin);
        }
    }
    __syncwarp();
    // bounds of the reference spheres' centres for the narrow phase (sphere
    // radius and margin taken off again, +1e-6 m for the rounding), grown
    // over the segment's earlier samples when merging
    if (lane < kRefSpheres) {
        const float4 sv = swept[lane];
        const float hd = sv.w - c_approx[lane].w - kCullMargin + 1e-6f;
        if (!merge) {
            rsw[lane] = make_float4(sv.x, sv.y, sv.z, hd);
        } else {
            const float4 o = rsw[lane];
            const float ex = sv.x - o.x, ey = sv.y - o.y, ez = sv.z - o.z;
            const float d = sqrtf(ex * ex + ey * ey + ez * ez) * 1.0001f;
            rsw[lane] = make_float4(o.x, o.y, o.z, fmaxf(o.w, d + hd) + 1e-6f);
        }
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// broad phase: approx spheres 1..10 of one arm (lane column `lane` of sp)
// against the scene.  Returns a bitmask over sphere index (bit i = sphere i
// of this lane's sample touches some obstacle).  The obstacles of each class
// are screened one per lane against the 10 spheres' swept bounds (sw, shared
// by the warp): the obstacle's bounding sphere, then for cuboids with
// orthonormal axes the exact sphere-cuboid test (both conservative; for
// spheres the record is its own bound).  Exact per-sample tests then run, for
// the whole warp, only for the (sphere, obstacle) pairs that survive.
// ---------------------------------------------------------------------------
template <typename BoundFn, typename RefineFn, typename ExactFn>
__device__ __forceinline__ void env_class(int n, int lane, const float4 *sw, const float (*sp)[3][32], uint32_t &m,
                                          BoundFn bound, RefineFn refine, ExactFn exact) {
#pragma unroll 1
    for (int o0 = 0; o0 < n; o0 += 32) {
        // one obstacle per lane: which swept sphere bounds reach it
        const int o = o0 + lane;
        uint32_t cand = 0;
        if (o < n) {
            const float4 bs = bound(o);
#pragma unroll
            for (int i = 1; i < kNumApprox; i++) {
                const float4 u = sw[i];
                if (near3(u.x, u.y, u.z, bs, u.w)) cand |= 1u << i;
            }
            for (uint32_t c = cand; c; c &= c - 1) {
                const int i = __ffs(c) - 1;
                if (!refine(o, bs, sw[i])) cand &= ~(1u << i);
            }
        }
        // exact per-sample tests of the surviving (sphere, obstacle) pairs
        uint32_t obal = __ballot_sync(kFull, cand != 0);
        while (obal) {
            const int src = __ffs(obal) - 1;
            obal &= obal - 1;
            uint32_t cm = __shfl_sync(kFull, cand, src);
            while (cm) {
                const int i = __ffs(cm) - 1;
                cm &= cm - 1;
                if (exact(o0 + src, sp[i][0][lane], sp[i][1][lane], sp[i][2][lane], c_approx[i].w)) m |= 1u << i;
            }
        }
    }
}

__device__ __forceinline__ uint32_t env_mask_approx(const float4 *S, const SceneLayout &L, const SceneCounts &C,
                                                    const float (*sp)[3][32], int lane, const float4 *sw) {
    uint32_t m = 0;
    env_class(
        C.n_cub, lane, sw, sp, m, [&](int o) { return S[L.b_cub + o]; },
        [&](int o, float4 bs, float4 u) {
            const float4 *r = S + L.cub + 4 * o;
            return bs.w > 1e17f || hit_cuboid(r[0], r[1], r[2], r[3], u.x, u.y, u.z, u.w * u.w);
        },
        [&](int o, float x, float y, float z, float rad) {
            const float4 *r = S + L.cub + 4 * o;
            return hit_cuboid(r[0], r[1], r[2], r[3], x, y, z, __fmul_rn(rad, rad));
        });
    env_class(
        C.n_zcub, lane, sw, sp, m, [&](int o) { return S[L.b_zcub + o]; },
        [&](int o, float4 bs, float4 u) {
            const float4 *r = S + L.zcub + 4 * o;
            return bs.w > 1e17f || hit_zcuboid(r[0], r[1], r[2], u.x, u.y, u.z, u.w * u.w);
        },
        [&](int o, float x, float y, float z, float rad) {
            const float4 *r = S + L.zcub + 4 * o;
            return hit_zcuboid(r[0], r[1], r[2], x, y, z, __fmul_rn(rad, rad));
        });
    env_class(
        C.n_cap, lane, sw, sp, m, [&](int o) { return S[L.b_cap + o]; }, [&](int, float4, float4) { return true; },
        [&](int o, float x, float y, float z, float rad) {
            return hit_capsule(S[L.cap + 2 * o], S[L.cap + 2 * o + 1], x, y, z, rad);
        });
    env_class(
        C.n_zcap, lane, sw, sp, m, [&](int o) { return S[L.b_zcap + o]; }, [&](int, float4, float4) { return true; },
        [&](int o, float x, float y, float z, float rad) {
            return hit_zcapsule(S[L.zcap + 2 * o], S[L.zcap + 2 * o + 1], x, y, z, rad);
        });
    env_class(
        C.n_sph, lane, sw, sp, m, [&](int o) { return S[L.sph + o]; }, [&](int, float4, float4) { return true; },
        [&](int o, float x, float y, float z, float rad) {
            const float4 c0 = S[L.sph + o];
            return hit_sphere_sphere(c0.x, c0.y, c0.z, c0.w, x, y, z, rad);
        });
    return m;
}

// Broad-phase intra-arm rows (panda_multi_geometry.cuh:133-139) as 21 pairs.
static __constant__ uint8_t c_intra_pairs[21][2] = {
    {0, 5}, {0, 6}, {0, 7}, {0, 8}, {0, 9}, {0, 10}, {1, 5}, {1, 6}, {1, 7}, {1, 8}, {1, 9},
    {1, 10}, {2, 5}, {2, 7}, {2, 8}, {2, 9}, {2, 10}, {5, 7}, {5, 8}, {5, 9}, {5, 10}};

// Broad phase of one sample (every lane of the warp calls it; lanes past the
// segment's last sample evaluate sample g and discard the result).
// Intra-arm pairs of one arm (panda_four.cuh:140-176): the 21 approx sphere
// pairs, one per lane, screened by the swept bounds sw of the warp's samples;
// exact per-sample tests for the survivors.  Returns the lane's flag bits (by
// joint of the pair's first sphere).
__device__ __forceinline__ uint32_t intra_flags(const float (*sp)[3][32], const float4 *sw, int lane) {
    // pair `lane` of c_intra_pairs, computed rather than read per lane
    const int p1 = lane < 6 ? 0 : lane < 12 ? 1 : lane < 17 ? 2 : 5;
    const int p2 = lane < 12 ? 5 + lane % 6 : lane == 12 ? 5 : lane < 17 ? lane - 6 : lane - 10;
    const float4 u1 = sw[p1];
    const bool c = lane < 21 && near3(u1.x, u1.y, u1.z, sw[p2], u1.w);
    uint32_t bal = __ballot_sync(kFull, c);
    uint32_t jm = 0;
    while (bal) {
        const int t = __ffs(bal) - 1;
        bal &= bal - 1;
        const int s1 = c_intra_pairs[t][0], s2 = c_intra_pairs[t][1];
        if (hit_sphere_sphere(sp[s1][0][lane], sp[s1][1][lane], sp[s1][2][lane], c_approx[s1].w, sp[s2][0][lane],
                              sp[s2][1][lane], sp[s2][2][lane], c_approx[s2].w))
            jm |= 1u << approx_joint(s1);
    }
    return jm;
}

template <int A>
__device__ __forceinline__ void broad_sample(const EdgeParams &P, WarpScratch &W, const float4 *S,
                                             const SceneLayout &L, int seg, int k, bool merge, uint64_t &envw,
                                             uint64_t &selfw) {
    const int lane = threadIdx.x & 31;
    envw = 0;
    selfw = 0;
    const bool do_env = P.flags & kEnvBit, do_self = P.flags & kSelfBit;
    auto &cur = W.broad.cur;
    auto &low = W.broad.low;
#pragma unroll 1
    for (int b = 0; b < A; b++) {
        MRPOP_PHASE_START();
        float4 *sw = W.broad.swept[b];
        fk_approx_lane(P.base[b], W, P.rule, seg, P.single ? 0 : b, k, cur, lane, sw, W.rsw[b], merge);
        MRPOP_PHASE(P, 0);
        if (do_env) {
            const uint32_t m = env_mask_approx(S, L, P.sc, cur, lane, sw);
            uint32_t jm = 0;
#pragma unroll
            for (int i = 1; i < kNumApprox; i++)
                if (m >> i & 1u) jm |= 1u << approx_joint(i);
            envw |= (uint64_t)jm << (8 * b);
        }
        MRPOP_PHASE(P, 1);
        if (!do_self) continue;
        // intra-arm pairs: one pair per lane screened by swept bounds, exact
        // per-sample tests for the survivors
        const uint32_t jm = intra_flags(cur, sw, lane);
        selfw |= (uint64_t)jm << (8 * b);
        MRPOP_PHASE(P, 2);
        if (A == 1) continue;
        // arm-vs-arm against every lower arm a < b; flags go to arm a
        // (panda_four.cuh:178-214).  The 121 sphere pairs are screened by
        // swept bounds, four rounds of one pair per lane; arm a's spheres are
        // rebuilt only when some pair survives.
#pragma unroll 1
        for (int a = 0; a < b; a++) {
            const float4 *swa = W.broad.swept[a];
            uint32_t bal[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int t = 32 * r + lane;
                const int i = t / kNumApprox, j = t - kNumApprox * i;
                bal[r] = __ballot_sync(kFull, t < kNumApprox * kNumApprox &&
                                                  near3(swa[i].x, swa[i].y, swa[i].z, sw[j], swa[i].w));
            }
            if (!(bal[0] | bal[1] | bal[2] | bal[3])) continue;
            fk_approx_lane(P.base[a], W, P.rule, seg, a, k, low, lane, nullptr, nullptr, false);
            uint32_t am = 0;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                uint32_t q = bal[r];
                while (q) {
                    const int t = 32 * r + __ffs(q) - 1;
                    q &= q - 1;
                    const int i = t / kNumApprox, j = t - kNumApprox * i;
                    if (hit_sphere_sphere(low[i][0][lane], low[i][1][lane], low[i][2][lane], c_approx[i].w,
                                          cur[j][0][lane], cur[j][1][lane], cur[j][2][lane], c_approx[j].w))
                        am |= 1u << approx_joint(i);
                }
            }
            selfw |= (uint64_t)am << (8 * a);
        }
        MRPOP_PHASE(P, 3);
    }
}

__device__ __forceinline__ int flag_count(uint64_t w) {
    int n = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const uint64_t col = (w >> j) & 0x0101010101ull; // joint j of arms 0..4
        n += det_count(j) * __popcll(col);
    }
    return n;
}

// reference thread split (utils.cuh:478-497): share of 4g threads, truncated
__device__ __forceinline__ int ref_share(int cnt, int total, int g) {
    if (total == 0) return 0; // 0/0 is NaN on the device; its int conversion is 0
    return __float2int_rz(__fmul_rn(__fdiv_rn((float)cnt, (float)total), (float)(4 * g)));
}

// dense narrow-phase tally for one sample (per the flop convention)
static __device__ __noinline__ double narrow_flops(const EdgeParams &P, int A, uint64_t envw, uint64_t selfw, bool de,
                                               bool ds) {
    double f = 0.0;
    const bool quirk = !P.single && !(P.flags & kExactBit);
    for (int a = 0; a < A; a++) {
        const uint32_t em = de ? (uint32_t)(envw >> (8 * a)) & 0xffu : 0u;
        const uint32_t sm = ds ? (uint32_t)(selfw >> (8 * a)) & 0xffu : 0u;
        for (int j = 0; j < 8; j++) {
            if ((em | sm) >> j & 1u) f += 18.0 * det_count(j);
            if (em >> j & 1u) f += P.env_test_flops * (j == 0 ? 0 : det_count(j));
        }
        if (sm) {
            for (int r = 0; r < kDetRows; r++) {
                const int idx = quirk ? r : det_row_first(r);
                if (sm >> det_joint(idx) & 1u) f += 11.0 * (det_row_hi(r) - det_row_lo(r) + 1);
            }
            for (int j = 0; j < 8; j++)
                if (sm >> j & 1u) f += 11.0 * kNumDet * (A - 1 - a) * det_count(j);
        }
    }
    return f;
}

// ---------------------------------------------------------------------------
// narrow phase
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t joint_sphere_mask(uint32_t jm) {
    uint64_t m = 0;
#pragma unroll
    for (int j = 0; j < kNumJoints; j++)
        if (jm >> j & 1u) m |= ((1ull << det_count(j)) - 1ull) << det_first(j);
    return m;
}

// position of the n-th (0-based) set bit of m
__device__ __forceinline__ int nth_bit(uint64_t m, int n) {
    const uint32_t lo = (uint32_t)m;
    const int pl = __popc(lo);
    if (n < pl) return (int)__fns(lo, 0, n + 1);
    return 32 + (int)__fns((uint32_t)(m >> 32), 0, n - pl + 1);
}

// bit r set: detailed self row r is checked for an arm with self flags sm
// Rows whose first-read sphere is on joint j (quirk: sphere r, else first(r)).
__host__ __device__ constexpr uint32_t joint_rows(int j, bool quirk) {
    uint32_t m = 0;
    for (int r = 0; r < kDetRows; r++)
        if (det_joint(quirk ? r : det_row_first(r)) == j) m |= 1u << r;
    return m;
}

__device__ __forceinline__ uint32_t row_mask(uint32_t sm, bool quirk) {
    uint32_t m = 0;
#pragma unroll
    for (int j = 0; j < kNumJoints; j++)
        if (sm >> j & 1u) m |= quirk ? joint_rows(j, true) : joint_rows(j, false);
    return m;
}

// Row bookkeeping of the detailed self check, per sphere index i:
//   first[q][i]  rows whose first-read sphere is i (q = 1: the composite
//                robots' reading, sphere r; q = 0: sphere first(r))
//   cover[i]     rows whose target range lo..hi contains i
// and the same ORed over the spheres of each joint.
struct RowTab {
    uint32_t first[2][kNumDet];
    uint32_t cover[kNumDet];
    uint32_t jfirst[2][kNumJoints];
    uint32_t jcover[kNumJoints];
};

__host__ __device__ constexpr RowTab make_row_tab() {
    RowTab t{};
    for (int r = 0; r < kDetRows; r++) {
        t.first[0][det_row_first(r)] |= 1u << r;
        t.first[1][r] |= 1u << r;
        for (int i = det_row_lo(r); i <= det_row_hi(r); i++) t.cover[i] |= 1u << r;
    }
    for (int i = 0; i < kNumDet; i++) {
        const int j = det_joint(i);
        t.jfirst[0][j] |= t.first[0][i];
        t.jfirst[1][j] |= t.first[1][i];
        t.jcover[j] |= t.cover[i];
    }
    return t;
}

static __constant__ RowTab c_rows = make_row_tab();

// Detailed sphere centre, transform in registers (the reference's full
// expression, panda_four.cuh:363-366).
__device__ __forceinline__ float3 place_reg(const Xf &T, float4 s) {
    float3 p;
    p.x = __fadd_rn(__fmaf_rn(T.m[2], s.z, pair_fma(T.m[0], s.x, T.m[1], s.y)), T.m[3]);
    p.y = __fadd_rn(__fmaf_rn(T.m[6], s.z, pair_fma(T.m[4], s.x, T.m[5], s.y)), T.m[7]);
    p.z = __fadd_rn(__fmaf_rn(T.m[10], s.z, pair_fma(T.m[8], s.x, T.m[9], s.y)), T.m[11]);
    return p;
}

// Sub-groups of the detailed spheres (contiguous index ranges within one
// joint): [0] [1-4] [5-8] [9-12] [13-16] [17-18] [19-20] [21-28] [29-31]
// [32-36] [37-58].  EdgeParams::grp holds each group's bounding sphere in its
// joint frame; a group's world bound is that centre through the joint frame.
constexpr int kNumGroups = 11;
__host__ __device__ __forceinline__ constexpr int grp_first(int g) {
    return g == 0 ? 0 : g == 1 ? 1 : g == 2 ? 5 : g == 3 ? 9 : g == 4 ? 13 : g == 5 ? 17 : g == 6 ? 19 : g == 7 ? 21
         : g == 8 ? 29 : g == 9 ? 32 : g == 10 ? 37 : 59;
}
// groups of joint j: [jgrp_first(j), jgrp_first(j + 1))
__host__ __device__ __forceinline__ constexpr int jgrp_first(int j) {
    return j < 5 ? j : j == 5 ? 5 : j == 6 ? 8 : j == 7 ? 9 : 11;
}
// The hand group (spheres 37..58: a 6 x 3 grid along the gripper's diagonal
// plus four finger-tip spheres) is screened in three parts along the diagonal:
// the two columns and finger tips on each side, and the two middle columns.
// Bits are sphere index - kHandFirst; EdgeParams::hsub holds each part's bound.
constexpr int kHandGroup = 10;
constexpr int kHandFirst = 37;
constexpr int kHandParts = 3;
__host__ __device__ __forceinline__ constexpr uint32_t hand_part(int s) {
    return s == 0 ? 0x3030C3u : s == 1 ? 0x00C30Cu : 0x0F0C30u;
}

// Exact env test of one sphere against obstacle o (index over all classes in
// the bound order cuboids, z-cuboids, capsules, z-capsules, spheres).
__device__ __forceinline__ bool env_exact(const float4 *S, const SceneLayout &L, const SceneCounts &C, int o, float x,
                                          float y, float z, float r) {
    if (o < C.n_cub) {
        const float4 *c = S + L.cub + 4 * o;
        return hit_cuboid(c[0], c[1], c[2], c[3], x, y, z, __fmul_rn(r, r));
    }
    o -= C.n_cub;
    if (o < C.n_zcub) {
        const float4 *c = S + L.zcub + 4 * o;
        return hit_zcuboid(c[0], c[1], c[2], x, y, z, __fmul_rn(r, r));
    }
    o -= C.n_zcub;
    if (o < C.n_cap) return hit_capsule(S[L.cap + 2 * o], S[L.cap + 2 * o + 1], x, y, z, r);
    o -= C.n_cap;
    if (o < C.n_zcap) return hit_zcapsule(S[L.zcap + 2 * o], S[L.zcap + 2 * o + 1], x, y, z, r);
    o -= C.n_zcap;
    const float4 c0 = S[L.sph + o];
    return hit_sphere_sphere(c0.x, c0.y, c0.z, c0.w, x, y, z, r);
}

// Conservative screen of obstacle o (index over all classes, in the order of
// env_exact) against ball U: the obstacle's bounding sphere, then for cuboids
// with orthonormal axes the exact sphere-cuboid test with U's radius.
__device__ __forceinline__ bool screen_obstacle(const float4 *S, const SceneLayout &L, const SceneCounts &C, int o,
                                                float4 U) {
    const float4 bs = S[L.b_cub + o];
    if (!near3(U.x, U.y, U.z, bs, U.w)) return false;
    if (bs.w > 1e17f) return true;
    if (o < C.n_cub) {
        const float4 *c = S + L.cub + 4 * o;
        return hit_cuboid(c[0], c[1], c[2], c[3], U.x, U.y, U.z, U.w * U.w);
    }
    o -= C.n_cub;
    if (o < C.n_zcub) {
        const float4 *c = S + L.zcub + 4 * o;
        return hit_zcuboid(c[0], c[1], c[2], U.x, U.y, U.z, U.w * U.w);
    }
    return true;
}

// Env test of the spheres of sub-group g (sphere 0 is never env-tested) for
// the lanes with act set; every lane of the warp calls it.  The active lanes'
// group bounds are merged into one ball U (box of their centres, half
// diagonal + group radius); obstacles are screened against U one per lane, 32
// at a time, and each active lane tests its spheres against the survivors.
__device__ __forceinline__ bool env_group_warp(const float4 *S, const SceneLayout &L, const SceneCounts &C,
                                                   const Xf &T, int g, float4 gl, bool act) {
    const int lane = threadIdx.x & 31;
    const float3 gc = place_reg(T, gl);
    constexpr float kBig = 3.0e38f;
    const float lx = warp_min(act ? gc.x : kBig), hx = warp_max(act ? gc.x : -kBig);
    const float ly = warp_min(act ? gc.y : kBig), hy = warp_max(act ? gc.y : -kBig);
    const float lz = warp_min(act ? gc.z : kBig), hz = warp_max(act ? gc.z : -kBig);
    const float dx = hx - lx, dy = hy - ly, dz = hz - lz;
    const float4 U = make_float4(0.5f * (lx + hx), 0.5f * (ly + hy), 0.5f * (lz + hz),
                                 0.5f * sqrtf(dx * dx + dy * dy + dz * dz) * 1.004f + gl.w);
    const int n_obst = C.n_cub + C.n_zcub + C.n_cap + C.n_zcap + C.n_sph;
    const int i0 = grp_first(g) == 0 ? 1 : grp_first(g), i1 = grp_first(g + 1);
    bool hit = false;
#pragma unroll 1
    for (int base = 0; base < n_obst; base += 32) {
        if (__all_sync(kFull, !act || hit)) break;
        const int o = base + lane;
        const uint32_t m = __ballot_sync(kFull, o < n_obst && screen_obstacle(S, L, C, o, U));
        MRPOP_COUNT_W(11, 1);
        MRPOP_COUNT_W(12, __popc(m));
        MRPOP_COUNT_LANES(13, act && !hit);
        if (!m || !act || hit) continue;
        for (int i = i0; i < i1 && !hit; i++) {
            const float4 sd = c_det[i];
            const float3 p = place_reg(T, sd);
            uint32_t mm = m;
            while (mm) {
                const int t = __ffs(mm) - 1;
                mm &= mm - 1;
                if (near3(p.x, p.y, p.z, S[L.b_cub + base + t], sd.w) &&
                    env_exact(S, L, C, base + t, p.x, p.y, p.z, sd.w)) {
                    hit = true;
                    break;
                }
            }
        }
    }
    return hit;
}

// True when the forearm-hand rows cannot fire at joint values (q6, q7): the
// cell's bit of the table is set.  NaN or out-of-range values give false.
__device__ __forceinline__ bool row5_apart(const uint32_t *tab, float q6, float q7) {
    const float f6 = (q6 - kRow5Lo6) * ((float)kRow5N6 / (kRow5Hi6 - kRow5Lo6));
    const float f7 = (q7 - kRow5Lo7) * ((float)kRow5N7 / (kRow5Hi7 - kRow5Lo7));
    if (!(f6 >= 0.0f && f6 < (float)kRow5N6 && f7 >= 0.0f && f7 < (float)kRow5N7)) return false;
    const int cell = (int)f6 * kRow5N7 + (int)f7;
    return (__ldg(tab + (cell >> 5)) >> (cell & 31)) & 1u;
}

// Per-lane state of the lane-parallel detailed check of one arm.
struct LaneCtx {
    uint32_t em;  // env-flagged joints
    uint32_t rm;  // flagged detailed self rows
    int quirk;
    bool hit;
};

// Joint j of one arm, frame T: env tests of an env-flagged joint, stash of the
// first spheres of flagged rows, and the row tests whose targets are here
// (screened by the target group's bound).
__device__ __forceinline__ void lane_env(int j, const EdgeParams &P, const Xf &T, LaneCtx &c, const float4 *S,
                                         const SceneLayout &L) {
    // every lane takes part in the env screening (warp-wide votes inside)
    if (__any_sync(kFull, !c.hit && (c.em >> j & 1u))) {
#pragma unroll 1
        for (int g = jgrp_first(j); g < jgrp_first(j + 1); g++)
            if (env_group_warp(S, L, P.sc, T, g, P.grp[g], !c.hit && (c.em >> j & 1u))) c.hit = true;
    }
}

template <int A>
__device__ __forceinline__ void lane_rows(int j, const EdgeParams &P, const Xf &T, LaneCtx &c, WarpScratch &W,
                                          const float4 *det_tab, int lane) {
    if (c.hit || !c.rm) return;
    uint32_t m1 = c.rm & c_rows.jfirst[c.quirk][j];
    while (m1) {
        const int r = __ffs(m1) - 1;
        m1 &= m1 - 1;
        const float3 p = place_reg(T, det_tab[c.quirk ? r : det_row_first(r)]);
        W.lanes.stash[r][0][lane] = p.x;
        W.lanes.stash[r][1][lane] = p.y;
        W.lanes.stash[r][2][lane] = p.z;
    }
#pragma unroll 1
    for (int g = jgrp_first(j); g < jgrp_first(j + 1); g++) {
        uint32_t rows = c.rm & c_rows.cover[grp_first(g)];
        if (!rows) continue;
        const float4 gl = P.grp[g];
        const float3 gc = place_reg(T, gl);
        uint32_t nr = 0;
        while (rows) {
            const int r = __ffs(rows) - 1;
            rows &= rows - 1;
            if (near3(W.lanes.stash[r][0][lane], W.lanes.stash[r][1][lane], W.lanes.stash[r][2][lane],
                      make_float4(gc.x, gc.y, gc.z, gl.w), det_tab[det_row_first(r)].w))
                nr |= 1u << r;
        }
        if (!nr) continue;
        bool h = false;
        if (A == 1 && g == kHandGroup) {
            // single-arm form: the hand's parts screened per row first, then
            // their spheres (in the composite forms the extra screens cost
            // more than they save)
#pragma unroll 1
            for (int s = 0; s < kHandParts; s++) {
                const float4 sl = P.hsub[s];
                const float3 sc = place_reg(T, sl);
                uint32_t ns = 0;
                for (uint32_t m = nr; m; m &= m - 1) {
                    const int r = __ffs(m) - 1;
                    if (near3(W.lanes.stash[r][0][lane], W.lanes.stash[r][1][lane], W.lanes.stash[r][2][lane],
                              make_float4(sc.x, sc.y, sc.z, sl.w), det_tab[det_row_first(r)].w))
                        ns |= 1u << r;
                }
                if (!ns) continue;
                for (uint32_t pm = hand_part(s); pm; pm &= pm - 1) {
                    const float4 sd = c_det[kHandFirst + __ffs(pm) - 1];
                    const float3 p = place_reg(T, sd);
                    for (uint32_t m = ns; m; m &= m - 1) {
                        const int r = __ffs(m) - 1;
                        h |= hit_sphere_sphere(W.lanes.stash[r][0][lane], W.lanes.stash[r][1][lane],
                                               W.lanes.stash[r][2][lane], det_tab[det_row_first(r)].w, p.x, p.y,
                                               p.z, sd.w);
                    }
                }
            }
        } else {
            for (int i = grp_first(g); i < grp_first(g + 1); i++) {
                const float4 sd = c_det[i];
                const float3 p = place_reg(T, sd);
                uint32_t m = nr;
                while (m) {
                    const int r = __ffs(m) - 1;
                    m &= m - 1;
                    h |= hit_sphere_sphere(W.lanes.stash[r][0][lane], W.lanes.stash[r][1][lane],
                                           W.lanes.stash[r][2][lane], det_tab[det_row_first(r)].w, p.x, p.y, p.z,
                                           sd.w);
                }
            }
        }
        if (h) {
            c.hit = true;
            return;
        }
    }
}

// Lane-parallel detailed check of this lane's sample, called by every lane of
// the warp (de = ds = false for a lane without a candidate sample): every
// arm's chain is rebuilt in registers; env tests of env-flagged joints
// (screened warp-wide per sub-group) and the intra-arm rows of self-flagged
// joints run as the frames stream by (the first sphere of each row is stashed
// until its targets come).  Returns true if a test fired.
// ONE: only arm one_arm's chain (the arm-per-warp kernel).
template <int A, bool ONE = false>
__device__ __forceinline__ bool narrow_lane(const EdgeParams &P, WarpScratch &W, const float4 *S,
                                                const SceneLayout &L, const float4 *det_tab, int seg, int k,
                                                uint64_t envw, uint64_t selfw, bool de, bool ds, int one_arm = 0) {
    const int lane = threadIdx.x & 31;
    LaneCtx c;
    c.quirk = (!P.single && !(P.flags & kExactBit)) ? 1 : 0;
    c.hit = false;
    MRPOP_PHASE_START();
#pragma unroll 1
    for (int a = ONE ? one_arm : 0; a < (ONE ? one_arm + 1 : A); a++) {
        if (__all_sync(kFull, c.hit || !(de || ds))) break;
        c.em = de ? (uint32_t)(envw >> (8 * a)) & 0xffu : 0u;
        const uint32_t sm = ds ? (uint32_t)(selfw >> (8 * a)) & 0xffu : 0u;
        c.rm = sm ? row_mask(sm, c.quirk != 0) : 0u;
        const int qa = 7 * (P.single ? 0 : a);
        if (P.row5 && (c.rm & row5_rows(c.quirk)) &&
            row5_apart(P.row5, sample_q1(W, P.rule, seg, qa + 5, k), sample_q1(W, P.rule, seg, qa + 6, k)))
            c.rm &= ~row5_rows(c.quirk);
        // the arm's chain is walked only if some lane has env or row tests on it
        if (!__any_sync(kFull, !c.hit && (c.em | c.rm))) continue;
        Xf T;
        load_base(T, P.base[a]);
#pragma unroll 1
        for (int j = 0; j < kNumJoints; j++) {
            if (j > 0) joint_step_rt(T, sample_q1(W, P.rule, seg, qa + j - 1, k), j);
            MRPOP_PHASE(P, 8);
            lane_env(j, P, T, c, S, L);
            MRPOP_PHASE(P, 9);
            lane_rows<A>(j, P, T, c, W, det_tab, lane);
            MRPOP_PHASE(P, 10);
        }
    }
    return c.hit;
}

// Arm a, joint j: stash the flagged spheres (index >= from) that can reach
// bound bb, until the stash is full; `next` receives the first sphere left out.
__device__ __forceinline__ void stash_joint(int j, const Xf &T, uint32_t sma, uint32_t qa, int from, int &n,
                                            int &next, WarpScratch &W, int lane) {
    if (next >= 0 || !(sma >> j & 1u) || det_first(j + 1) <= from) return;
#pragma unroll 1
    for (int g = jgrp_first(j); g < jgrp_first(j + 1); g++) {
        if (!(qa >> g & 1u) || grp_first(g + 1) <= from) continue;
#pragma unroll 1
        for (int i = max(grp_first(g), from); i < grp_first(g + 1); i++) {
            const float4 sd = c_det[i];
            const float3 p = place_reg(T, sd);
            if (n == kCrossStash) {
                next = i;
                return;
            }
            W.lanes.cstash[n][0][lane] = p.x;
            W.lanes.cstash[n][1][lane] = p.y;
            W.lanes.cstash[n][2][lane] = p.z;
            W.lanes.cstash[n][3][lane] = sd.w;
            n++;
        }
    }
}

// Arm b, joint j: its spheres against the stashed spheres, by sub-group.
__device__ __forceinline__ void probe_joint(int j, const EdgeParams &P, const Xf &T, uint32_t qb, int n, bool &hit,
                                            WarpScratch &W, int lane) {
    if (hit) return;
#pragma unroll 1
    for (int g = jgrp_first(j); g < jgrp_first(j + 1); g++) {
        if (!(qb >> g & 1u)) continue;
        const float4 gl = P.grp[g];
        const float3 gc = place_reg(T, gl);
        const float4 gb = make_float4(gc.x, gc.y, gc.z, gl.w);
        uint32_t near = 0;
        for (int e = 0; e < n; e++)
            if (near3(W.lanes.cstash[e][0][lane], W.lanes.cstash[e][1][lane], W.lanes.cstash[e][2][lane], gb,
                      W.lanes.cstash[e][3][lane]))
                near |= 1u << e;
        if (!near) continue;
        bool h = false;
        for (int i = grp_first(g); i < grp_first(g + 1); i++) {
            const float4 sd = c_det[i];
            const float3 p = place_reg(T, sd);
            uint32_t m = near;
            while (m) {
                const int e = __ffs(m) - 1;
                m &= m - 1;
                // sphere_1 = the lower arm's sphere (panda_four.cuh:441-443)
                h |= hit_sphere_sphere(W.lanes.cstash[e][0][lane], W.lanes.cstash[e][1][lane],
                                       W.lanes.cstash[e][2][lane], W.lanes.cstash[e][3][lane], p.x, p.y, p.z, sd.w);
            }
        }
        if (h) {
            hit = true;
            return;
        }
    }
}

// Joint of detailed sub-group g.
__device__ __forceinline__ constexpr int grp_joint(int g) { return g < 5 ? g : g < 8 ? 5 : g < 9 ? 6 : 7; }
// Reference approx sphere of sub-group g: an approx sphere on the same joint
// (the nearest one for the hand), so that the group's centre is at a fixed
// distance from it (EdgeParams::gofs adds that distance and the group radius).
__host__ __device__ __forceinline__ constexpr int grp_ref(int g) {
    return g < 5 ? g : g < 8 ? 5 : g < 9 ? 6 : g < 10 ? 7 : 8;
}

// Arm pairs (a < b) in order: pair index of (a, b), and the count.
__host__ __device__ __forceinline__ constexpr int pair_index(int a, int b, int A) {
    return a * (2 * A - a - 1) / 2 + (b - a - 1);
}
__host__ __device__ __forceinline__ constexpr int num_pairs(int A) { return A * (A - 1) / 2; }

// Arm-vs-arm detailed test (panda_four.cuh:415-453) of this lane's sample;
// every lane of the warp calls it, lanes with act set take part.  For each arm
// pair (a, b) the 121 sub-group pairs are screened warp-wide, one per lane,
// with bounds over the segment's samples (the swept bound of the group's
// reference approx sphere, W.rsw, grown by EdgeParams::gofs; groups of a
// restricted to joints some active lane has self-flagged).  Pairs with no
// surviving group pair are skipped by the whole warp.  Otherwise each active
// lane stashes arm a's flagged spheres of the surviving groups that can reach
// arm b's bound (chunks of kCrossStash) and streams arm b's surviving groups
// against them.  Returns true if a test fired.
// SEL: only the arm pairs whose bit (pair_index) is set in `pairs`.
template <int A, bool SEL = false>
__device__ __forceinline__ bool cross_swept(const EdgeParams &P, WarpScratch &W, int seg, int k, uint64_t selfw,
                                            bool act, uint32_t pairs = 0) {
    const int lane = threadIdx.x & 31;
    bool hit = false;
#pragma unroll 1
    for (int a = 0; a < A - 1; a++) {
        const uint32_t sma = act ? (uint32_t)(selfw >> (8 * a)) & 0xffu : 0u;
        const uint32_t uj = __reduce_or_sync(kFull, sma);
        if (!uj) continue;
#pragma unroll 1
        for (int b = a + 1; b < A; b++) {
            if (SEL && !(pairs >> pair_index(a, b, A) & 1u)) continue;
            uint32_t qa = 0, qb = 0;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int t = 32 * r + lane;
                const int ga = t / kNumGroups, gb = t - kNumGroups * ga;
                bool pass = false;
                if (t < kNumGroups * kNumGroups && (uj >> grp_joint(ga) & 1u)) {
                    const float4 u = W.gbd[a][ga];
                    pass = near3(u.x, u.y, u.z, W.gbd[b][gb], u.w);
                }
                uint32_t bal = __ballot_sync(kFull, pass);
                while (bal) {
                    const int tt = 32 * r + __ffs(bal) - 1;
                    bal &= bal - 1;
                    qa |= 1u << (tt / kNumGroups);
                    qb |= 1u << (tt % kNumGroups);
                }
            }
            if (!qa || !act || hit) continue;
            int from = 0;
            while (from >= 0 && !hit) {
                int n = 0, next = -1;
                {
                    Xf T;
                    load_base(T, P.base[a]);
#pragma unroll 1
                    for (int j = 0; j < kNumJoints; j++) {
                        if (j > 0) joint_step_rt(T, sample_q1(W, P.rule, seg, 7 * a + j - 1, k), j);
                        stash_joint(j, T, sma, qa, from, n, next, W, lane);
                    }
                }
                from = next;
                if (n == 0) break;
                Xf T;
                load_base(T, P.base[b]);
#pragma unroll 1
                for (int j = 0; j < kNumJoints; j++) {
                    if (j > 0) joint_step_rt(T, sample_q1(W, P.rule, seg, 7 * b + j - 1, k), j);
                    probe_joint(j, P, T, qb, n, hit, W, lane);
                }
            }
        }
    }
    return hit;
}

// ---------------------------------------------------------------------------
// per-edge building blocks shared by the kernels
// ---------------------------------------------------------------------------
// Edge set-up: segment start and per-sample / per-segment steps of every dof
// into warp scratch (call-site formulas, see the rule constants).  Returns
// the segment count; too_many marks counts beyond kMaxSegments.
__device__ __forceinline__ int edge_setup(const EdgeParams &P, WarpScratch &W, long long e, int dof, int g, int lane,
                                          bool &too_many) {
    const float *qa = P.q0 + e * dof, *qb = P.q1 + e * dof;
    float diff0 = 0.f, diff1 = 0.f;
    if (lane < dof) diff0 = __fsub_rn(qb[lane], qa[lane]);
    if (lane + 32 < dof) diff1 = __fsub_rn(qb[lane + 32], qa[lane + 32]);
    int nseg = 1;
    too_many = false;
    if (P.rule != kRulePlain) {
        // |q1 - q0| with the reference's sequential FMA chain (utils.cuh:123-133)
        float acc = 0.0f;
        for (int d = 0; d < dof; d++) {
            const float v = __shfl_sync(kFull, d < 32 ? diff0 : diff1, d & 31);
            acc = __fmaf_rn(v, v, acc);
        }
        const float dist = __fsqrt_rn(acc);
        float n;
        if (P.rule == kRuleConnect) n = truncf(__fdiv_rn(dist, P.range)) + 1.0f;
        else if (P.rule == kRuleBspline) n = ceilf(__fdiv_rn(dist, P.range));
        else n = ceilf(__fdiv_rn(__fsub_rn(dist, 0.001f), P.range));
        if (n > (float)kMaxSegments) too_many = true;
        else nseg = (int)n; // may be <= 0: no segment is checked (the reference's loop runs 0 times)
    }
    for (int d = lane; d < dof; d += 32) {
        const float df = d < 32 ? diff0 : diff1;
        W.base[d] = qa[d];
        if (P.rule == kRulePlain) {
            W.stepg[d] = __fdiv_rn(df, (float)g);
            W.delta[d] = 0.0f;
        } else {
            const float step = __fdiv_rn(df, (float)nseg);
            W.delta[d] = step;
            W.stepg[d] = __fdiv_rn(step, (float)g);
        }
    }
    __syncwarp();
    return nseg;
}

// CONNECT: the segment start of segment `seg` (the caller's loop adds the
// per-segment step once per finished segment, pop_planner.cu:697).
__device__ __forceinline__ void connect_advance(WarpScratch &W, int dof, int seg, int lane) {
    for (int d = lane; d < dof; d += 32) {
        float b = W.base[d];
        for (int s = 0; s < seg; s++) b = __fadd_rn(b, W.delta[d]);
        W.base[d] = b;
    }
    __syncwarp();
}

// Broad phase of one segment for this lane's samples plus the decision: which
// samples get the detailed check (the reference's thread split, or every
// flagged sample in EXACT mode).  Returns false when no sample is flagged.
// The candidate masks of a segment from its samples' flag counts (totals over
// the segment given): every flagged sample in EXACT mode, else the samples the
// reference's proportional 4g-thread split gives at least one thread
// (utils.cuh:476-517), the remainder going to the last sample.
template <int SPL>
__device__ __forceinline__ void thread_split(bool exact, int g, int lane, const int (&envc)[SPL],
                                             const int (&selfc)[SPL], int tot_env, int tot_self, uint64_t &cand_env,
                                             uint64_t &cand_self) {
    if (exact) {
#pragma unroll
        for (int s = 0; s < SPL; s++) {
            const uint64_t be = __ballot_sync(kFull, envc[s] > 0);
            const uint64_t bs = __ballot_sync(kFull, selfc[s] > 0);
            cand_env |= be << (32 * s);
            cand_self |= bs << (32 * s);
        }
        return;
    }
    int de[SPL], ds[SPL], sum_e = 0, sum_s = 0;
#pragma unroll
    for (int s = 0; s < SPL; s++) {
        const int k = lane + 1 + 32 * s;
        de[s] = k <= g ? ref_share(envc[s], tot_env, g) : 0;
        ds[s] = k <= g ? ref_share(selfc[s], tot_self, g) : 0;
        sum_e += de[s];
        sum_s += ds[s];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum_e += __shfl_xor_sync(kFull, sum_e, o);
        sum_s += __shfl_xor_sync(kFull, sum_s, o);
    }
#pragma unroll
    for (int s = 0; s < SPL; s++) {
        const int k = lane + 1 + 32 * s;
        if (k == g) { // the remainder goes to the last sample
            de[s] += 4 * g - sum_e;
            ds[s] += 4 * g - sum_s;
        }
        const uint64_t be = __ballot_sync(kFull, tot_env > 0 && de[s] > 0);
        const uint64_t bs = __ballot_sync(kFull, tot_self > 0 && ds[s] > 0);
        cand_env |= be << (32 * s);
        cand_self |= bs << (32 * s);
    }
}

template <int A, int SPL>
__device__ __forceinline__ bool broad_decide(const EdgeParams &P, WarpScratch &W, const float4 *S,
                                             const SceneLayout &L, int seg, int g, int lane, uint64_t (&envw)[SPL],
                                             uint64_t (&selfw)[SPL], uint64_t &cand_env, uint64_t &cand_self,
                                             double &tally) {
    MRPOP_PHASE_START();
    int envc[SPL], selfc[SPL];
    int tot_env = 0, tot_self = 0;
    // one copy of the per-sample code for both slots (not unrolled); slot
    // arrays are written by constant index so they stay in registers
#pragma unroll 1
    for (int s = 0; s < SPL; s++) {
        const int k = lane + 1 + 32 * s;
        uint64_t ew, sw;
        broad_sample<A>(P, W, S, L, seg, k <= g ? k : g, s > 0, ew, sw);
        if (k > g) ew = sw = 0;
        const int ec = flag_count(ew), sc = flag_count(sw);
        if (s == 0) {
            envw[0] = ew;
            selfw[0] = sw;
            envc[0] = ec;
            selfc[0] = sc;
        } else {
            envw[SPL - 1] = ew;
            selfw[SPL - 1] = sw;
            envc[SPL - 1] = ec;
            selfc[SPL - 1] = sc;
        }
        tot_env += ec;
        tot_self += sc;
    }
    __syncwarp();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tot_env += __shfl_xor_sync(kFull, tot_env, o);
        tot_self += __shfl_xor_sync(kFull, tot_self, o);
    }
    if (P.flops) tally += P.fbp * g;
    cand_env = cand_self = 0;
    if (tot_env == 0 && tot_self == 0) return false;
    MRPOP_PHASE(P, 7);
    thread_split<SPL>((P.flags & kExactBit) != 0, g, lane, envc, selfc, tot_env, tot_self, cand_env, cand_self);
    if (P.flops) {
        double f = 0.0;
#pragma unroll
        for (int s = 0; s < SPL; s++) {
            const int bit = lane + 32 * s;
            const bool dE = cand_env >> bit & 1ull, dS = cand_self >> bit & 1ull;
            if (dE || dS) f += narrow_flops(P, P.single ? 1 : A, envw[s], selfw[s], dE, dS);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(kFull, f, o);
        tally += f;
    }
    MRPOP_PHASE(P, 4);
    return true;
}

// Detailed phase of one segment: every candidate sample in parallel, one lane
// each (samples k0 + 1 ..; k0 = 32 for the second warp of a pair).  Returns
// the 0-based index (from k0) of the first colliding sample, or 64.
template <int A, int SPL>
__device__ __forceinline__ int narrow_segment(const EdgeParams &P, WarpScratch &W, const float4 *S,
                                              const SceneLayout &L, const float4 *det_tab, int seg, int lane,
                                              const uint64_t (&envw)[SPL], const uint64_t (&selfw)[SPL],
                                              uint64_t cand_env, uint64_t cand_self, int k0 = 0) {
    MRPOP_PHASE_START();
    // sub-group bounds over the segment's samples, from the reference-sphere bounds
    for (int t = lane; t < A * kNumGroups; t += 32) {
        const int a = t / kNumGroups, g = t - kNumGroups * a;
        const float4 u = W.rsw[a][grp_ref(g)];
        W.gbd[a][g] = make_float4(u.x, u.y, u.z, u.w + P.gofs[g]);
    }
    __syncwarp();
    uint64_t hits = 0;
    // one copy of the per-sample code for both slots (not unrolled)
#pragma unroll 1
    for (int s = 0; s < SPL; s++) {
        const int bit = lane + 32 * s;
        const bool dE = cand_env >> bit & 1ull, dS = cand_self >> bit & 1ull;
        const uint64_t ew = s == 0 ? envw[0] : envw[SPL - 1], sw = s == 0 ? selfw[0] : selfw[SPL - 1];
        // every lane walks the arms (warp-wide screening inside); lanes
        // without a candidate sample keep the others company on sample
        // min(k, g), so that the warp's merged bounds stay on real samples
        const int k = k0 + bit + 1 <= P.g ? k0 + bit + 1 : P.g;
        bool h = narrow_lane<A>(P, W, S, L, det_tab, seg, k, ew, sw, dE, dS);
        MRPOP_PHASE(P, 5);
        MRPOP_COUNT_LANES(14, dE || dS);
        if (A > 1 && __any_sync(kFull, dS && !h)) {
            MRPOP_COUNT_W(15, 1);
            h |= cross_swept<A>(P, W, seg, k, sw, dS && !h);
        }
        MRPOP_PHASE(P, 6);
        hits |= (uint64_t)__ballot_sync(kFull, h) << (32 * s);
        if (hits) break; // later slots hold only later samples
    }
    return hits ? __ffsll((long long)hits) - 1 : 64;
}

// Common kernel prologue: scene staged in shared memory, warp scratch.
#define MRPOP_KERNEL_PROLOGUE()                                                                        \
    extern __shared__ __align__(128) unsigned char smem_raw[];                                         \
    __shared__ __align__(8) uint64_t bar;                                                              \
    __shared__ float4 det_tab[kNumDet];                                                                \
    const SceneLayout L = scene_layout(P.sc);                                                          \
    float4 *S = reinterpret_cast<float4 *>(smem_raw);                                                  \
    WarpScratch *Wall = reinterpret_cast<WarpScratch *>(smem_raw + (size_t)L.total * sizeof(float4));  \
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;                                        \
    WarpScratch &W = Wall[warp];                                                                       \
    for (int i = threadIdx.x; i < kNumDet; i += blockDim.x) det_tab[i] = c_det[i];                     \
    const bool staged = stage_scene(S, P.scene, (uint32_t)(L.total * sizeof(float4)), &bar, P.status); \
    MRPOP_PHASE_BIND(P);                                                                               \
    const int g = P.g;                                                                                 \
    const int dof = 7 * (P.single ? 1 : A);                                                            \
    const long long nwarps = (long long)gridDim.x * kWarpsPerBlock;                                    \
    (void)det_tab;

// ---------------------------------------------------------------------------
// fused kernel: every rule, segments in order with early exit
// ---------------------------------------------------------------------------
// One edge through the fused kernel: segments from P.seg0 in order, both
// phases per segment, early exit at the first colliding one.  Edges decided by
// earlier split rounds (P.seg0 > 0) are skipped.
template <int A, int SPL>
__device__ __forceinline__ void fused_edge(const EdgeParams &P, WarpScratch &W, const float4 *S, const SceneLayout &L,
                                           const float4 *det_tab, long long e, int dof, int g, int lane,
                                           bool staged) {
    if (!staged) {
        if (lane == 0) {
            P.valid[e] = 0;
            P.first_hit[e] = -2;
        }
        return;
    }
    if (P.seg0 > 0 && (P.sdone[e] || P.snseg[e] <= P.seg0)) return; // decided by the split rounds
    bool too_many;
    const int nseg = edge_setup(P, W, e, dof, g, lane, too_many);
    int first = 0;
    double tally = 0.0;
    const int nseg_run = too_many ? 0 : nseg;
    if (P.rule == kRuleConnect && P.seg0 > 0) connect_advance(W, dof, P.seg0, lane);
    for (int seg = P.seg0; seg < nseg_run && first == 0; seg++) {
        uint64_t envw[SPL], selfw[SPL], cand_env, cand_self;
        if (broad_decide<A, SPL>(P, W, S, L, seg, g, lane, envw, selfw, cand_env, cand_self, tally)) {
            const int fb = narrow_segment<A, SPL>(P, W, S, L, det_tab, seg, lane, envw, selfw, cand_env, cand_self);
            if (fb < 64) first = seg * g + fb + 1;
        }
        if (P.rule == kRuleConnect) {
            __syncwarp();
            for (int d = lane; d < dof; d += 32) W.base[d] = __fadd_rn(W.base[d], W.delta[d]);
            __syncwarp();
        }
    }
    if (lane == 0) {
        P.valid[e] = (first == 0 && !too_many) ? 1 : 0;
        P.first_hit[e] = too_many ? -2 : (first ? first : -1);
        if (P.n_seg_out) P.n_seg_out[e] = nseg;
        if (P.flops) P.flops[e] = P.seg0 > 0 ? P.flops[e] + tally : tally;
    }
    __syncwarp();
}

template <int A, int SPL>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MRPOP_MIN_BLOCKS)
    validate_kernel(const __grid_constant__ EdgeParams P) {
    MRPOP_KERNEL_PROLOGUE()
    for (long long e = (long long)blockIdx.x * kWarpsPerBlock + warp; e < P.n_edges; e += nwarps)
        fused_edge<A, SPL>(P, W, S, L, det_tab, e, dof, g, lane, staged);
}

// ---------------------------------------------------------------------------
// fused kernel, two warps per edge (granularity above 32, small calls): warp
// `half` of a pair takes samples 32 * half + 1 .. 32 * half + 32 of every
// segment, so an edge takes the time of one 32-sample slot instead of two.
// The thread split's totals and shares are summed over the pair (integers,
// so in any order), the segment's swept bounds merged with the single-warp
// kernel's formula, and both warps leave a segment together at its first
// hit: the verdicts are those of the one-warp kernels.
// ---------------------------------------------------------------------------
struct PairShare {
    int tot[2][2];  // [half] env, self flag totals of the slot
    int sum[2][2];  // [half] env, self thread shares of the slot
    int fb[2];      // [half] first colliding sample of the slot (from its k0), or 64
};

__device__ __forceinline__ void pair_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }

template <int A>
__device__ __forceinline__ void fused_edge_pair(const EdgeParams &P, WarpScratch &W, const WarpScratch &Wo,
                                                const float4 *S, const SceneLayout &L, const float4 *det_tab,
                                                long long e, int dof, int g, int lane, int half, PairShare &X,
                                                int bar_id, bool staged) {
    if (!staged) {
        if (half == 0 && lane == 0) {
            P.valid[e] = 0;
            P.first_hit[e] = -2;
        }
        return;
    }
    bool too_many;
    const int nseg = edge_setup(P, W, e, dof, g, lane, too_many);
    const int nseg_run = too_many ? 0 : nseg;
    const int k = lane + 1 + 32 * half;
    int first = 0;
    for (int seg = 0; seg < nseg_run && first == 0; seg++) {
        uint64_t ew, sw;
        broad_sample<A>(P, W, S, L, seg, k <= g ? k : g, false, ew, sw);
        if (k > g) ew = sw = 0;
        const int ec = flag_count(ew), sc = flag_count(sw);
        int te = ec, ts = sc;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            te += __shfl_xor_sync(kFull, te, o);
            ts += __shfl_xor_sync(kFull, ts, o);
        }
        if (lane == 0) {
            X.tot[half][0] = te;
            X.tot[half][1] = ts;
        }
        pair_sync(bar_id);  // A: both slots' totals and swept bounds written
        const int tot_env = X.tot[0][0] + X.tot[1][0], tot_self = X.tot[0][1] + X.tot[1][1];
        if (tot_env > 0 || tot_self > 0) {
            // the segment's bounds: slot 0's grown by slot 1's (fk_approx_lane's merge)
            const WarpScratch &W0 = half == 0 ? W : Wo, &W1 = half == 0 ? Wo : W;
            float4 mg[2];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int t = lane + 32 * r;
                if (t < A * kRefSpheres) {
                    const float4 o = (&W0.rsw[0][0])[t], sv = (&W1.rsw[0][0])[t];
                    const float ex = sv.x - o.x, ey = sv.y - o.y, ez = sv.z - o.z;
                    const float d = sqrtf(ex * ex + ey * ey + ez * ez) * 1.0001f;
                    mg[r] = make_float4(o.x, o.y, o.z, fmaxf(o.w, d + sv.w) + 1e-6f);
                }
            }
            bool cE, cS;
            if (P.flags & kExactBit) {
                cE = ec > 0;
                cS = sc > 0;
                pair_sync(bar_id);  // B (both warps read the bounds)
            } else {
                int de = k <= g ? ref_share(ec, tot_env, g) : 0, ds = k <= g ? ref_share(sc, tot_self, g) : 0;
                int se = de, ss = ds;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    se += __shfl_xor_sync(kFull, se, o);
                    ss += __shfl_xor_sync(kFull, ss, o);
                }
                if (lane == 0) {
                    X.sum[half][0] = se;
                    X.sum[half][1] = ss;
                }
                pair_sync(bar_id);  // B: shares written, bounds read
                if (k == g) {  // the remainder goes to the last sample
                    de += 4 * g - (X.sum[0][0] + X.sum[1][0]);
                    ds += 4 * g - (X.sum[0][1] + X.sum[1][1]);
                }
                cE = tot_env > 0 && de > 0;
                cS = tot_self > 0 && ds > 0;
            }
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int t = lane + 32 * r;
                if (t < A * kRefSpheres) (&W.rsw[0][0])[t] = mg[r];
            }
            const uint64_t cand_env = __ballot_sync(kFull, cE), cand_self = __ballot_sync(kFull, cS);
            __syncwarp();
            const uint64_t envw[1] = {ew}, selfw[1] = {sw};
            const int fb = (cand_env | cand_self)
                               ? narrow_segment<A, 1>(P, W, S, L, det_tab, seg, lane, envw, selfw, cand_env, cand_self,
                                                      32 * half)
                               : 64;
            if (lane == 0) X.fb[half] = fb;
            pair_sync(bar_id);  // C: both slots' first hits written
            const int f0 = X.fb[0], f1 = X.fb[1];
            if (f0 < 64) first = seg * g + f0 + 1;
            else if (f1 < 64) first = seg * g + 32 + f1 + 1;
        }
        if (P.rule == kRuleConnect) {
            __syncwarp();
            for (int d = lane; d < dof; d += 32) W.base[d] = __fadd_rn(W.base[d], W.delta[d]);
            __syncwarp();
        }
        pair_sync(bar_id);  // D: the pair's shared words are read before the next segment writes them
    }
    if (half == 0 && lane == 0) {
        P.valid[e] = (first == 0 && !too_many) ? 1 : 0;
        P.first_hit[e] = too_many ? -2 : (first ? first : -1);
        if (P.n_seg_out) P.n_seg_out[e] = nseg;
    }
    __syncwarp();
}

template <int A>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MRPOP_MIN_BLOCKS)
    pair_kernel(const __grid_constant__ EdgeParams P) {
    MRPOP_KERNEL_PROLOGUE()
    static_assert(kWarpsPerBlock % 2 == 0, "warps come in pairs");
    __shared__ PairShare X[kWarpsPerBlock / 2];
    const WarpScratch &Wo = Wall[warp ^ 1];
    const int pair = warp >> 1, half = warp & 1;
    (void)nwarps;
    for (long long e = (long long)blockIdx.x * (kWarpsPerBlock / 2) + pair; e < P.n_edges;
         e += (long long)gridDim.x * (kWarpsPerBlock / 2))
        fused_edge_pair<A>(P, W, Wo, S, L, det_tab, e, dof, g, lane, half, X[pair], 1 + pair, staged);
}

// ---------------------------------------------------------------------------
// fused kernel, one warp per arm (small calls of 2 to 5 arms): a CTA of A
// warps takes one edge at a time and warp a does arm a's share of it -- its
// forward kinematics, env and intra-arm screens and exact tests, its detailed
// chain walk -- and every A-th arm pair of the arm-vs-arm screens and tests,
// each over every slot of the segment.  Flag words are ORed together in
// shared memory, the thread split is evaluated from them by every warp (the
// same integers), and a sample collides when any warp's tests fire: the
// verdicts are those of the one-warp kernels.  The lower arm's spheres of a
// pair are read from the warp that placed them instead of being placed again.
// ---------------------------------------------------------------------------
struct ArmShare {
    unsigned long long env[2][32], self[2][32];  // [slot][lane] flag words of the segment
    unsigned int hits[2];                        // [slot] lanes whose sample collided
    unsigned int next[3];                        // arm pairs handed out: broad, narrow slot 0, slot 1
};

// The next arm pair for this warp from counter *c (lane 0 takes it).
__device__ __forceinline__ int take_pair(unsigned int *c, int lane) {
    unsigned int p = 0;
    if (lane == 0) p = atomicAdd(c, 1u);
    return (int)__shfl_sync(kFull, p, 0);
}

// Arm pair p (pair_index order): its lower and upper arm.
template <int A>
__host__ __device__ __forceinline__ constexpr void pair_arms(int p, int &a, int &b) {
    a = 0;
    while (p >= A - 1 - a) {
        p -= A - 1 - a;
        a++;
    }
    b = a + 1 + p;
}

// pair_arms inverts pair_index for every pair of up to 5 arms
template <int A>
constexpr bool pair_order_round_trips() {
    for (int p = 0; p < num_pairs(A); p++) {
        int a = 0, b = 0;
        pair_arms<A>(p, a, b);
        if (!(0 <= a && a < b && b < A) || pair_index(a, b, A) != p) return false;
    }
    return true;
}
static_assert(pair_order_round_trips<2>() && pair_order_round_trips<3>() && pair_order_round_trips<4>() &&
                  pair_order_round_trips<5>(),
              "arm pair order");

template <int A, int SPL>
__device__ __forceinline__ void armwise_edge(const EdgeParams &P, unsigned char *wbase, const float4 *S,
                                             const SceneLayout &L, const float4 *det_tab, long long e, int dof,
                                             int g, int lane, int arm, ArmShare &X, bool staged) {
    WarpScratch &W = reinterpret_cast<WarpScratch *>(wbase)[arm];
    if (!staged) {
        if (arm == 0 && lane == 0) {
            P.valid[e] = 0;
            P.first_hit[e] = -2;
        }
        return;
    }
    bool too_many;
    const int nseg = edge_setup(P, W, e, dof, g, lane, too_many);
    const int nseg_run = too_many ? 0 : nseg;
    const bool do_env = P.flags & kEnvBit, do_self = P.flags & kSelfBit;
    int first = 0;
    for (int seg = 0; seg < nseg_run && first == 0; seg++) {
        if (arm == 0) {
#pragma unroll
            for (int t = 0; t < 2; t++) X.env[t][lane] = X.self[t][lane] = 0;
            if (lane < 2) X.hits[lane] = 0;
            if (lane < 3) X.next[lane] = 0;
        }
        __syncthreads();
        // this arm: placement, swept bounds, env and intra-arm screens (the
        // slots' spheres stay in broad.cur / broad.low for the pair tests)
#pragma unroll 1
        for (int s = 0; s < SPL; s++) {
            const int k = lane + 1 + 32 * s;
            float(*sp)[3][32] = s == 0 ? W.broad.cur : W.broad.low;
            float4 *sw = W.broad.swept[s];
            fk_approx_lane(P.base[arm], W, P.rule, seg, P.single ? 0 : arm, k <= g ? k : g, sp, lane, sw, W.rsw[arm],
                           s > 0);
            uint32_t em = 0, im = 0;
            if (do_env) {
                const uint32_t m = env_mask_approx(S, L, P.sc, sp, lane, sw);
#pragma unroll
                for (int i = 1; i < kNumApprox; i++)
                    if (m >> i & 1u) em |= 1u << approx_joint(i);
            }
            if (do_self) im = intra_flags(sp, sw, lane);
            if (k <= g) {
                if (em) atomicOr(&X.env[s][lane], (unsigned long long)em << (8 * arm));
                if (im) atomicOr(&X.self[s][lane], (unsigned long long)im << (8 * arm));
            }
        }
        __syncthreads();
        // arm pairs (a, b), a < b, handed out one at a time to the warps as
        // they finish (their costs differ): flags go to arm a
        // (panda_four.cuh:178-214); screened by the slot's swept bounds
        if (A > 1 && do_self) {
            const WarpScratch *Wa = reinterpret_cast<const WarpScratch *>(wbase);
#pragma unroll 1
            for (int p = take_pair(&X.next[0], lane); p < num_pairs(A); p = take_pair(&X.next[0], lane)) {
                int a, b;
                pair_arms<A>(p, a, b);
#pragma unroll 1
                for (int s = 0; s < SPL; s++) {
                    const int k = lane + 1 + 32 * s;
                    const float4 *swa = Wa[a].broad.swept[s], *swb = Wa[b].broad.swept[s];
                    uint32_t bal[4];
#pragma unroll
                    for (int r = 0; r < 4; r++) {
                        const int t = 32 * r + lane;
                        const int i = t / kNumApprox, j = t - kNumApprox * i;
                        bal[r] = __ballot_sync(kFull, t < kNumApprox * kNumApprox &&
                                                          near3(swa[i].x, swa[i].y, swa[i].z, swb[j], swa[i].w));
                    }
                    if (!(bal[0] | bal[1] | bal[2] | bal[3])) continue;
                    const float(*low)[3][32] = s == 0 ? Wa[a].broad.cur : Wa[a].broad.low;
                    const float(*cur)[3][32] = s == 0 ? Wa[b].broad.cur : Wa[b].broad.low;
                    uint32_t am = 0;
#pragma unroll
                    for (int r = 0; r < 4; r++) {
                        uint32_t q = bal[r];
                        while (q) {
                            const int t = 32 * r + __ffs(q) - 1;
                            q &= q - 1;
                            const int i = t / kNumApprox, j = t - kNumApprox * i;
                            if (hit_sphere_sphere(low[i][0][lane], low[i][1][lane], low[i][2][lane],
                                                  c_approx[i].w, cur[j][0][lane], cur[j][1][lane],
                                                  cur[j][2][lane], c_approx[j].w))
                                am |= 1u << approx_joint(i);
                        }
                    }
                    if (am && k <= g) atomicOr(&X.self[s][lane], (unsigned long long)am << (8 * a));
                }
                }
        }
        __syncthreads();
        // the thread split, from the ORed words (every warp alike)
        uint64_t envw[SPL], selfw[SPL];
        int envc[SPL], selfc[SPL], tot_env = 0, tot_self = 0;
#pragma unroll
        for (int s = 0; s < SPL; s++) {
            envw[s] = X.env[s][lane];
            selfw[s] = X.self[s][lane];
            envc[s] = flag_count(envw[s]);
            selfc[s] = flag_count(selfw[s]);
            tot_env += envc[s];
            tot_self += selfc[s];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tot_env += __shfl_xor_sync(kFull, tot_env, o);
            tot_self += __shfl_xor_sync(kFull, tot_self, o);
        }
        if (tot_env > 0 || tot_self > 0) {
            uint64_t cand_env = 0, cand_self = 0;
            thread_split<SPL>((P.flags & kExactBit) != 0, g, lane, envc, selfc, tot_env, tot_self, cand_env,
                              cand_self);
            // the segment's sub-group bounds for the arm-vs-arm screens, from
            // every arm's reference-sphere bounds (each warp's own row)
            const WarpScratch *Wa = reinterpret_cast<const WarpScratch *>(wbase);
            for (int t = lane; t < A * kNumGroups; t += 32) {
                const int a = t / kNumGroups, gg = t - kNumGroups * a;
                const float4 u = Wa[a].rsw[a][grp_ref(gg)];
                W.gbd[a][gg] = make_float4(u.x, u.y, u.z, u.w + P.gofs[gg]);
            }
            __syncwarp();
#pragma unroll 1
            for (int s = 0; s < SPL; s++) {
                const int bit = lane + 32 * s;
                const bool dE = cand_env >> bit & 1ull, dS = cand_self >> bit & 1ull;
                const int k = bit + 1 <= g ? bit + 1 : g;
                bool h = narrow_lane<A, true>(P, W, S, L, det_tab, seg, k, envw[s], selfw[s], dE, dS, arm);
                // the slot's arm pairs, one at a time to whichever warp is free
                if (A > 1 && __any_sync(kFull, dS)) {
                    unsigned int *next = &X.next[1 + s];
                    for (int p = take_pair(next, lane); p < num_pairs(A); p = take_pair(next, lane))
                        if (__any_sync(kFull, dS && !h))
                            h |= cross_swept<A, true>(P, W, seg, k, selfw[s], dS && !h, 1u << p);
                }
                const unsigned int hb = __ballot_sync(kFull, h);
                if (lane == 0 && hb) atomicOr(&X.hits[s], hb);
            }
            __syncthreads();
            const uint64_t hits = (uint64_t)X.hits[0] | (SPL > 1 ? (uint64_t)X.hits[1] << 32 : 0ull);
            if (hits) first = seg * g + __ffsll((long long)hits);
        }
        if (P.rule == kRuleConnect) {
            __syncwarp();
            for (int d = lane; d < dof; d += 32) W.base[d] = __fadd_rn(W.base[d], W.delta[d]);
            __syncwarp();
        }
        __syncthreads();  // the shared words are read before the next segment clears them
    }
    if (arm == 0 && lane == 0) {
        P.valid[e] = (first == 0 && !too_many) ? 1 : 0;
        P.first_hit[e] = too_many ? -2 : (first ? first : -1);
        if (P.n_seg_out) P.n_seg_out[e] = nseg;
    }
}

template <int A, int SPL>
__global__ void __launch_bounds__(32 * A) armwise_kernel(const __grid_constant__ EdgeParams P) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ float4 det_tab[kNumDet];
    __shared__ ArmShare X;
    const SceneLayout L = scene_layout(P.sc);
    const float4 *S = reinterpret_cast<const float4 *>(smem_raw);
    const int arm = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kNumDet; i += blockDim.x) det_tab[i] = c_det[i];
    const bool staged = stage_scene(reinterpret_cast<float4 *>(smem_raw), P.scene,
                                    (uint32_t)(L.total * sizeof(float4)), &bar, P.status);
    unsigned char *wbase = smem_raw + (size_t)L.total * sizeof(float4);
    const int dof = 7 * (P.single ? 1 : A);
    for (long long e = blockIdx.x; e < P.n_edges; e += gridDim.x)
        armwise_edge<A, SPL>(P, wbase, S, L, det_tab, e, dof, P.g, lane, arm, X, staged);
}

// ---------------------------------------------------------------------------
// split pipeline for single-segment edges: the broad kernel writes every
// sample's flag words, each edge's candidate masks and reference-sphere
// bounds to HBM (P.sflags, P.smasks, P.sbounds); the narrow kernel runs the
// detailed phase of edges with candidates.  Each kernel's code fits the
// instruction cache on its own.  broad_edge / narrow_edge are one warp's work
// on edge e, shared by the plain kernels and the batch kernels.
// ---------------------------------------------------------------------------
// Staged flag words of sample slot o (= edge * 32 * SPL + sample - 1): 8 flag
// bits per arm, so 32-bit words hold up to 4 arms.
template <int A>
__device__ __forceinline__ void store_flags(const EdgeParams &P, long long o, uint64_t env, uint64_t self) {
    if (A <= 4) reinterpret_cast<uint2 *>(P.sflags)[o] = make_uint2((uint32_t)env, (uint32_t)self);
    else reinterpret_cast<ulonglong2 *>(P.sflags)[o] = make_ulonglong2(env, self);
}
template <int A>
__device__ __forceinline__ void load_flags(const EdgeParams &P, long long o, uint64_t &env, uint64_t &self) {
    if (A <= 4) {
        const uint2 v = reinterpret_cast<const uint2 *>(P.sflags)[o];
        env = v.x;
        self = v.y;
    } else {
        const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(P.sflags)[o];
        env = v.x;
        self = v.y;
    }
}

template <int A, int SPL, bool SEG>
__device__ __forceinline__ void broad_edge(const EdgeParams &P, WarpScratch &W, const float4 *S, const SceneLayout &L,
                                           long long e, int dof, int g, int lane, bool staged) {
    if (!staged) {
        if (lane == 0) {
            P.valid[e] = 0;
            P.first_hit[e] = -2;
            P.smasks[2 * e] = P.smasks[2 * e + 1] = 0;
        }
        return;
    }
    // SEG: a segment round of a segmented rule (r = P.seg0); otherwise a
    // single-segment edge (r = 0, compiled as a constant)
    const int r = SEG ? P.seg0 : 0;
    constexpr bool segmented = SEG;
    if (segmented && r > 0 && (P.sdone[e] || P.snseg[e] <= r)) {
        if (lane == 0) P.smasks[2 * e] = P.smasks[2 * e + 1] = 0;
        return;
    }
    bool too_many;
    const int nseg = edge_setup(P, W, e, dof, g, lane, too_many);
    if (segmented) {
        if (r == 0) {
            const bool none = too_many || nseg <= 0; // decided without a check
            if (lane == 0) {
                P.snseg[e] = too_many ? -1 : nseg;
                if (P.n_seg_out) P.n_seg_out[e] = nseg;
                P.sdone[e] = none ? 1 : 0;
                if (none) {
                    P.valid[e] = too_many ? 0 : 1;
                    P.first_hit[e] = too_many ? -2 : -1;
                    P.smasks[2 * e] = P.smasks[2 * e + 1] = 0;
                    if (P.flops) P.flops[e] = 0.0;
                }
            }
            if (none) {
                __syncwarp();
                return;
            }
        } else if (P.rule == kRuleConnect) {
            connect_advance(W, dof, r, lane);
        }
    } else {
        (void)nseg;
    }
    uint64_t envw[SPL], selfw[SPL], cand_env, cand_self;
    double tally = 0.0;
    const bool any = broad_decide<A, SPL>(P, W, S, L, r, g, lane, envw, selfw, cand_env, cand_self, tally);
    if (any) {
#pragma unroll
        for (int s = 0; s < SPL; s++) store_flags<A>(P, e * (32 * SPL) + lane + 32 * s, envw[s], selfw[s]);
        for (int t = lane; t < A * kRefSpheres; t += 32) P.sbounds[e * (A * kRefSpheres) + t] = (&W.rsw[0][0])[t];
    }
    if (lane == 0) {
        P.smasks[2 * e] = cand_env;
        P.smasks[2 * e + 1] = cand_self;
        if (!any && (!segmented || r == nseg - 1)) { // the last segment passed the broad phase
            P.valid[e] = 1;
            P.first_hit[e] = -1;
            if (segmented) P.sdone[e] = 1;
        }
        if (!segmented && P.n_seg_out) P.n_seg_out[e] = 1;
        if (P.flops) P.flops[e] = (segmented && r > 0) ? P.flops[e] + tally : tally;
    }
    __syncwarp();
}

template <int A, int SPL, bool SEG>
__device__ __forceinline__ void narrow_edge(const EdgeParams &P, WarpScratch &W, const float4 *S, const SceneLayout &L,
                                            const float4 *det_tab, long long e, int dof, int g, int lane,
                                            bool staged) {
    const uint64_t cand_env = P.smasks[2 * e], cand_self = P.smasks[2 * e + 1];
    if (!(cand_env | cand_self)) return; // verdict written by the broad kernel
    if (!staged) {
        if (lane == 0) {
            P.valid[e] = 0;
            P.first_hit[e] = -2;
        }
        return;
    }
    const int r = SEG ? P.seg0 : 0;
    constexpr bool segmented = SEG;
    bool too_many;
    const int nseg = edge_setup(P, W, e, dof, g, lane, too_many);
    if (SEG && P.rule == kRuleConnect && r > 0) connect_advance(W, dof, r, lane);
    uint64_t envw[SPL], selfw[SPL];
#pragma unroll
    for (int s = 0; s < SPL; s++) load_flags<A>(P, e * (32 * SPL) + lane + 32 * s, envw[s], selfw[s]);
    for (int t = lane; t < A * kRefSpheres; t += 32) (&W.rsw[0][0])[t] = P.sbounds[e * (A * kRefSpheres) + t];
    __syncwarp();
    const int fb = narrow_segment<A, SPL>(P, W, S, L, det_tab, r, lane, envw, selfw, cand_env, cand_self);
    if (lane == 0) {
        if (fb < 64) {
            P.valid[e] = 0;
            P.first_hit[e] = r * g + fb + 1;
            if (segmented) P.sdone[e] = 1;
        } else if (!segmented || r == nseg - 1) {
            P.valid[e] = 1;
            P.first_hit[e] = -1;
            if (segmented) P.sdone[e] = 1;
        }
    }
    __syncwarp();
}

// Next edge for this warp: a shared counter handed out one edge at a time, so
// that warps whose edges finish early take more (edge costs vary by orders of
// magnitude: an edge without candidates skips the narrow phase entirely).
__device__ __forceinline__ long long next_edge(unsigned long long *counter, int lane) {
    unsigned long long e = 0;
    if (lane == 0) e = atomicAdd(counter, 1ull);
    return (long long)__shfl_sync(kFull, e, 0);
}

template <int A, int SPL, bool SEG>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MRPOP_MIN_BLOCKS)
    broad_kernel(const __grid_constant__ EdgeParams P) {
    MRPOP_KERNEL_PROLOGUE()
    (void)nwarps;
    for (long long e = next_edge(P.work, lane); e < P.n_edges; e = next_edge(P.work, lane))
        broad_edge<A, SPL, SEG>(P, W, S, L, e, dof, g, lane, staged);
    // no edges left for this warp: the narrow kernel (launched as a
    // programmatic dependent) may start its CTAs once every CTA got here
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <int A, int SPL, bool SEG>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MRPOP_MIN_BLOCKS)
    narrow_kernel(const __grid_constant__ EdgeParams P) {
    MRPOP_KERNEL_PROLOGUE()
    (void)nwarps;
    // the scene is staged; wait for the broad kernel (complete, its writes
    // visible) before reading its output
    asm volatile("griddepcontrol.wait;" ::: "memory");
    for (long long e = next_edge(P.work + 1, lane); e < P.n_edges; e = next_edge(P.work + 1, lane))
        narrow_edge<A, SPL, SEG>(P, W, S, L, det_tab, e, dof, g, lane, staged);
}

// ---------------------------------------------------------------------------
// batch kernels: many independent instances (each with its own scene, arm
// layout, edges, granularity and outputs; one EdgeParams each, all of arm
// count A and samples-per-lane SPL) in one persistent launch.  An instance's
// edges form chunks; CTAs take chunks from a counter, in instance order, and
// copy the instance's parameters to shared memory and restage its scene with
// the bulk-copy engine when the instance changes; the CTA's warps then take
// the chunk's edges one at a time.  MODE picks the broad, narrow or fused
// per-edge body; SEG marks groups of segmented instances (connect, B-spline,
// shortcut), which run the split kernels in rounds (BatchParams::seg0) and
// the fused kernel for the edges left after them.
// ---------------------------------------------------------------------------
struct BatchParams {
    const EdgeParams *items;      // device array, one per instance
    const int4 *chunks;           // {instance, first edge, edge count, -}, instances in order
    int n_chunks;
    int seg0;                     // segmented groups: the round (split kernels) or first segment (fused)
    unsigned long long *work;     // next-chunk counter, zero before each launch
};

// Batch kernel modes: the split pipeline's two kernels, and the fused kernel
// that finishes segmented edges after the split rounds.
constexpr int kBatchBroad = 0, kBatchNarrow = 1, kBatchFused = 2;
// Batch mode of the arm-per-warp kernel (whole edges from segment 0, a CTA of
// A warps per edge): batch_armwise_kernel.
constexpr int kBatchArmwise = 3;

// One bulk copy of `bytes` from global to shared memory, completed on `bar`
// in phase `parity`; bounded wait.  Every thread of the CTA calls it after a
// barrier that follows its last read of `dst`; the proxy fence orders those
// reads before the copy's writes.  Returns false (for the whole CTA) if the
// copy did not complete in time.
__device__ __forceinline__ bool stage_bulk(float4 *dst, const float4 *src, uint32_t bytes, uint64_t *bar,
                                           uint32_t parity, unsigned int *status) {
    if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(dst)),
            "l"(src), "r"(bytes), "r"(smem_u32(bar))
            : "memory");
    }
    return __syncthreads_and(copy_wait(bar, parity, status, kWaitLimitNs));
}

template <int A, int SPL, int MODE, bool SEG>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MRPOP_MIN_BLOCKS)
    batch_kernel(const __grid_constant__ BatchParams B) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ float4 det_tab[kNumDet];
    __shared__ __align__(16) EdgeParams Ps;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kNumDet; i += blockDim.x) det_tab[i] = c_det[i];
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    __shared__ int s_chunk;
    __shared__ unsigned int s_next;
    int item = -1;
    uint32_t parity = 0;
    bool staged = false;
    for (;;) {
        // the CTA takes the next chunk of one instance's edges ...
        if (threadIdx.x == 0) {
            s_chunk = (int)atomicAdd(B.work, 1ull);
            s_next = 0;
        }
        __syncthreads();
        const int c = s_chunk;
        if (c >= B.n_chunks) break;
        const int4 ch = B.chunks[c];
        if (ch.x != item) {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(B.items + ch.x);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&Ps);
            for (int i = threadIdx.x; i < (int)(sizeof(EdgeParams) / 4); i += blockDim.x) dst[i] = src[i];
            __syncthreads();
            if (SEG) { // the round of this launch
                if (threadIdx.x == 0) Ps.seg0 = B.seg0;
                __syncthreads();
            }
            const uint32_t bytes = (uint32_t)(scene_layout(Ps.sc).total * sizeof(float4));
            staged = true;
            if (bytes) {
                staged = stage_bulk(reinterpret_cast<float4 *>(smem_raw), Ps.scene, bytes, &bar, parity, Ps.status);
                parity ^= 1u;
            }
            item = ch.x;
        }
        const EdgeParams &P = Ps;
        const SceneLayout L = scene_layout(P.sc);
        const float4 *S = reinterpret_cast<const float4 *>(smem_raw);
        WarpScratch &W = reinterpret_cast<WarpScratch *>(smem_raw + (size_t)L.total * sizeof(float4))[warp];
        const int dof = 7 * (P.single ? 1 : A);
        // ... and its warps take the chunk's edges one at a time
        for (;;) {
            unsigned int k = 0;
            if (lane == 0) k = atomicAdd(&s_next, 1u);
            k = __shfl_sync(kFull, k, 0);
            if ((int)k >= ch.z) break;
            const long long e = (long long)ch.y + k;
            if (MODE == kBatchBroad) broad_edge<A, SPL, SEG>(P, W, S, L, e, dof, P.g, lane, staged);
            else if (MODE == kBatchNarrow) narrow_edge<A, SPL, SEG>(P, W, S, L, det_tab, e, dof, P.g, lane, staged);
            else fused_edge<A, SPL>(P, W, S, L, det_tab, e, dof, P.g, lane, staged);
        }
        __syncthreads(); // every warp is done with this chunk (and instance)
    }
}

// Batch form of armwise_kernel: the CTA takes chunks (of single edges) from the
// launch's counter, stages each instance's parameters and scene as
// batch_kernel does, and runs the arm-per-warp body on every edge of the chunk.
template <int A, int SPL>
__global__ void __launch_bounds__(32 * A) batch_armwise_kernel(const __grid_constant__ BatchParams B) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ float4 det_tab[kNumDet];
    __shared__ __align__(16) EdgeParams Ps;
    __shared__ ArmShare X;
    __shared__ int s_chunk;
    const int arm = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kNumDet; i += blockDim.x) det_tab[i] = c_det[i];
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int item = -1;
    uint32_t parity = 0;
    bool staged = false;
    for (;;) {
        if (threadIdx.x == 0) s_chunk = (int)atomicAdd(B.work, 1ull);
        __syncthreads();
        const int c = s_chunk;
        if (c >= B.n_chunks) break;
        const int4 ch = B.chunks[c];
        if (ch.x != item) {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(B.items + ch.x);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&Ps);
            for (int i = threadIdx.x; i < (int)(sizeof(EdgeParams) / 4); i += blockDim.x) dst[i] = src[i];
            __syncthreads();
            const uint32_t bytes = (uint32_t)(scene_layout(Ps.sc).total * sizeof(float4));
            staged = true;
            if (bytes) {
                staged = stage_bulk(reinterpret_cast<float4 *>(smem_raw), Ps.scene, bytes, &bar, parity, Ps.status);
                parity ^= 1u;
            }
            item = ch.x;
        }
        const SceneLayout L = scene_layout(Ps.sc);
        const float4 *S = reinterpret_cast<const float4 *>(smem_raw);
        unsigned char *wbase = smem_raw + (size_t)L.total * sizeof(float4);
        const int dof = 7 * (Ps.single ? 1 : A);
        for (int k = 0; k < ch.z; k++)
            armwise_edge<A, SPL>(Ps, wbase, S, L, det_tab, (long long)ch.y + k, dof, Ps.g, lane, arm, X, staged);
        __syncthreads();  // every warp is done with this chunk (and instance)
    }
}

}  // namespace mrpop
