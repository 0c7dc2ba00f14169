// ref_harness.cu -- runs the reference's own edge check on a GPU.
//
// TEST INFRASTRUCTURE ONLY (the checker, and the timed reference arm of
// bench.py).  This translation unit includes the reference's unmodified
// headers from the reference source tree (-I <reference root>, see
// oracle/build.py) and wraps its block-collective routines
//   ppln::device_utils::fkcc_single_buffer<Robot>       utils.cuh:447-534
//   ppln::device_utils::fkcc_single_buffer_drrt<Robot>  utils.cuh:626-686
//   ppln::device_utils::fkcc_single_buffer_mr<Panda>    utils.cuh:536-624
// in batch kernels: one block of 4*g threads per edge (the planner's launch
// shape, pop_planner.cu:973), edges strided over a persistent grid.  The edge
// interpolation and segmentation are written exactly as at the reference's
// call sites (pop_planner.cu:551-564 extend, :666-703 connect,
// roadmap_interior.cuh:219-240 roadmap, path_simplification.cu:85-129
// B-spline and :155-200 shortcut).  The include order is that of
// pop_planner.cu:1-14 (the robot headers have no include guards).
#include "Planners.hh"
#include "Robots.hh"
#include "utils.cuh"
#include "pop_settings.hh"
#include "src/collision/environment.hh"
#include "src/collision/panda_collision.cuh"
#include "src/robots/panda.cuh"
#include "src/robots/panda_multi_geometry.cuh"
#include "src/robots/panda_four.cuh"
#include "src/robots/panda_five.cuh"

using ppln::collision::Capsule;
using ppln::collision::Cuboid;
using ppln::collision::Environment;
using ppln::collision::Sphere;

namespace {
constexpr int kMaxThreads = 256;        // 4 * MAX_GRANULARITY (pop_planner_state.cuh:13-14)
constexpr int kSpherePosStride = 57344; // >= 5 arms * 59 spheres * 64 samples * 3
constexpr int kLinkCCStride = 8000;     // all_block_linkCC row (pop_planner.cu:38)

// Segmentation rules (same numbering as include/mrpop.h)
constexpr int kPlain = 0, kConnect = 1, kBspline = 2, kShortcut = 3;
// Variants
constexpr int kComposite = 0, kExtend = 1, kSingle = 2;
}  // namespace

extern "C" __global__ void ref_sizes(int *out) {
    out[0] = (int)sizeof(Environment<float>);
    out[1] = (int)sizeof(Sphere<float>);
    out[2] = (int)sizeof(Capsule<float>);
    out[3] = (int)sizeof(Cuboid<float>);
}

// Fill reference-layout obstacle arrays from packed records (include/mrpop.h
// field order) and point an Environment<float> at them.  Only the numeric
// fields are written; the device code never reads Shape::name.
extern "C" __global__ void ref_env_build(Environment<float> *env, const float *sph, int n_sph, const float *cap,
                                         int n_cap, const float *zcap, int n_zcap, const float *cub, int n_cub,
                                         const float *zcub, int n_zcub, Sphere<float> *o_sph,
                                         Capsule<float> *o_cap, Capsule<float> *o_zcap, Cuboid<float> *o_cub,
                                         Cuboid<float> *o_zcub) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int i = 0; i < n_sph; i++) {
        const float *s = sph + 4 * i;
        o_sph[i].x = s[0]; o_sph[i].y = s[1]; o_sph[i].z = s[2]; o_sph[i].r = s[3];
    }
    auto fill_caps = [](Capsule<float> *o, const float *c, int n) {
        for (int i = 0; i < n; i++) {
            const float *s = c + 8 * i;
            o[i].x1 = s[0]; o[i].y1 = s[1]; o[i].z1 = s[2];
            o[i].xv = s[3]; o[i].yv = s[4]; o[i].zv = s[5];
            o[i].r = s[6]; o[i].rdv = s[7];
        }
    };
    fill_caps(o_cap, cap, n_cap);
    fill_caps(o_zcap, zcap, n_zcap);
    auto fill_cubs = [](Cuboid<float> *o, const float *c, int n) {
        for (int i = 0; i < n; i++) {
            const float *s = c + 15 * i;
            o[i].x = s[0]; o[i].y = s[1]; o[i].z = s[2];
            o[i].axis_1_x = s[3]; o[i].axis_1_y = s[4]; o[i].axis_1_z = s[5];
            o[i].axis_2_x = s[6]; o[i].axis_2_y = s[7]; o[i].axis_2_z = s[8];
            o[i].axis_3_x = s[9]; o[i].axis_3_y = s[10]; o[i].axis_3_z = s[11];
            o[i].axis_1_r = s[12]; o[i].axis_2_r = s[13]; o[i].axis_3_r = s[14];
        }
    };
    fill_cubs(o_cub, cub, n_cub);
    fill_cubs(o_zcub, zcub, n_zcub);
    env->spheres = o_sph; env->num_spheres = (unsigned)n_sph;
    env->capsules = o_cap; env->num_capsules = (unsigned)n_cap;
    env->z_aligned_capsules = o_zcap; env->num_z_aligned_capsules = (unsigned)n_zcap;
    env->cylinders = nullptr; env->num_cylinders = 0;
    env->cuboids = o_cub; env->num_cuboids = (unsigned)n_cub;
    env->z_aligned_cuboids = o_zcub; env->num_z_aligned_cuboids = (unsigned)n_zcub;
}

template <typename Robot, int VARIANT>
__device__ void ref_edges(Environment<float> *env, const float *q0, const float *q1, int n_edges, int g, int rule,
                          float range, int num_robot, int robot_id, float *sphere_pos_all, int *linkcc_all,
                          int *valid, int *seg_fail) {
    constexpr int dim = Robot::dimension;
    const int tid = threadIdx.x;
    __shared__ volatile unsigned int local_cc_result[1];
    __shared__ volatile unsigned int any_approx_env_collision[1];
    __shared__ volatile unsigned int any_approx_self_collision[1];
    __shared__ volatile int env_sphere_to_check[kMaxThreads];
    __shared__ volatile int self_sphere_to_check[kMaxThreads];
    __shared__ volatile int env_thread_dist[kMaxThreads];
    __shared__ volatile int self_thread_dist[kMaxThreads];
    __align__(16) __shared__ float T[64 * 2 * 16];
    __shared__ float config[dim];
    __shared__ volatile float delta[dim];
    __shared__ volatile float vec[dim];
    __shared__ volatile unsigned int n_extensions;
    volatile float *sphere_pos = sphere_pos_all + (size_t)blockIdx.x * kSpherePosStride;
    volatile int *link_CC = linkcc_all + (size_t)blockIdx.x * kLinkCCStride;

    auto check = [&](float *interp_cfg) {
        if (VARIANT == kComposite)
            ppln::device_utils::fkcc_single_buffer<Robot>(
                interp_cfg, env, tid, sphere_pos, link_CC, T, local_cc_result, any_approx_env_collision,
                any_approx_self_collision, env_sphere_to_check, self_sphere_to_check, env_thread_dist,
                self_thread_dist, g);
        else if (VARIANT == kExtend)
            ppln::device_utils::fkcc_single_buffer_drrt<Robot>(
                interp_cfg, env, tid, sphere_pos, link_CC, T, local_cc_result, any_approx_env_collision,
                any_approx_self_collision, self_sphere_to_check, self_thread_dist, g);
        else
            ppln::device_utils::fkcc_single_buffer_mr<Robot>(
                interp_cfg, env, tid, sphere_pos, link_CC, T, local_cc_result, any_approx_env_collision,
                any_approx_self_collision, env_sphere_to_check, self_sphere_to_check, env_thread_dist,
                self_thread_dist, g, num_robot, robot_id);
    };

    for (int e = blockIdx.x; e < n_edges; e += gridDim.x) {
        const float *nearest_node = q0 + (size_t)e * dim; // edge start
        const float *other = q1 + (size_t)e * dim;        // edge end
        __syncthreads();
        if (tid == 0) {
            local_cc_result[0] = 0;
            any_approx_env_collision[0] = 0;
            any_approx_self_collision[0] = 0;
        }
        __syncthreads();
        int failed_seg = -1;
        if (rule == kPlain) {
            // extend (pop_planner.cu:551-561) / roadmap edge (roadmap_interior.cuh:219-234)
            if (tid < dim) delta[tid] = (other[tid] - nearest_node[tid]) / (float)g;
            __syncthreads();
            float interp_cfg[dim];
            for (int i = 0; i < dim; i++) interp_cfg[i] = nearest_node[i] + (int(tid / 4 + 1) * delta[i]);
            __syncthreads();
            check(interp_cfg);
            if (local_cc_result[0] != 0) failed_seg = 0;
            __syncthreads();
        } else if (rule == kConnect) {
            // connect (pop_planner.cu:657-703): config = new node, nearest = other tree's node
            if (tid == 0) {
                float d = sqrt(ppln::device_utils::sq_l2_dist((float *)other, (float *)nearest_node, dim));
                n_extensions = int(d / range) + 1;
            }
            if (tid < dim) config[tid] = nearest_node[tid];
            __syncthreads();
            if (tid < dim) vec[tid] = (other[tid] - config[tid]) / (float)n_extensions;
            __syncthreads();
            float interp_cfg[dim];
            for (int t = 0; t < (int)n_extensions; t++) {
                for (int i = 0; i < dim; i++) interp_cfg[i] = config[i] + (int(tid / 4 + 1) * (vec[i] / (float)g));
                check(interp_cfg);
                bool ext_edge_good = local_cc_result[0] == 0;
                __syncthreads();
                if (!ext_edge_good) {
                    failed_seg = t;
                    break;
                }
                if (tid < dim) config[tid] += vec[tid];
                __syncthreads();
            }
        } else {
            // B-spline (path_simplification.cu:85-129) and shortcut (:155-200)
            const float granularity_tolerance = 0.001;
            int cc_iter;
            if (rule == kBspline)
                cc_iter = ceil(ppln::device_utils::l2_dist((float *)nearest_node, (float *)other, dim) / (float)range);
            else
                cc_iter = ceil((ppln::device_utils::l2_dist((float *)nearest_node, (float *)other, dim) -
                                granularity_tolerance) /
                               (float)range);
            if (tid < dim) delta[tid] = (other[tid] - nearest_node[tid]) / cc_iter;
            float interp_cfg[dim];
            for (int d = 0; d < dim; d++) interp_cfg[d] = nearest_node[d];
            __syncthreads();
            for (int d = 0; d < dim; d++) interp_cfg[d] += (int(tid / 4 + 1) * (delta[d] / (float)g));
            for (int cc_round = 0; cc_round < cc_iter; cc_round++) {
                if (tid == 0) {
                    any_approx_env_collision[0] = 0;
                    any_approx_self_collision[0] = 0;
                    local_cc_result[0] = 0;
                }
                __syncthreads();
                check(interp_cfg);
                bool edge_good = (local_cc_result[0] == 0);
                __syncthreads();
                if (!edge_good) {
                    failed_seg = cc_round;
                    break;
                }
                for (int d = 0; d < dim; d++) interp_cfg[d] += delta[d];
                __syncthreads();
            }
        }
        if (tid == 0) {
            valid[e] = failed_seg < 0 ? 1 : 0;
            seg_fail[e] = failed_seg;
        }
    }
}

// robots: 4 -> Panda_four, 5 -> Panda_five (composite variants); the single-arm
// variant always uses Panda with (num_robot, robot_id) choosing its base.
extern "C" __global__ void __launch_bounds__(256)
    ref_validate(Environment<float> *env, const float *q0, const float *q1, int n_edges, int g, int variant,
                 int rule, float range, int num_robot, int robot_id, float *sphere_pos_all, int *linkcc_all,
                 int *valid, int *seg_fail) {
    if (variant == kSingle)
        ref_edges<ppln::robots::Panda, kSingle>(env, q0, q1, n_edges, g, rule, range, num_robot, robot_id,
                                                sphere_pos_all, linkcc_all, valid, seg_fail);
    else if (num_robot == 4) {
        if (variant == kComposite)
            ref_edges<ppln::robots::Panda_four, kComposite>(env, q0, q1, n_edges, g, rule, range, 4, 0,
                                                            sphere_pos_all, linkcc_all, valid, seg_fail);
        else
            ref_edges<ppln::robots::Panda_four, kExtend>(env, q0, q1, n_edges, g, rule, range, 4, 0,
                                                         sphere_pos_all, linkcc_all, valid, seg_fail);
    } else if (num_robot == 5) {
        if (variant == kComposite)
            ref_edges<ppln::robots::Panda_five, kComposite>(env, q0, q1, n_edges, g, rule, range, 5, 0,
                                                            sphere_pos_all, linkcc_all, valid, seg_fail);
        else
            ref_edges<ppln::robots::Panda_five, kExtend>(env, q0, q1, n_edges, g, rule, range, 5, 0,
                                                         sphere_pos_all, linkcc_all, valid, seg_fail);
    }
}

// Sphere centres from the reference FK: block of 256 threads = 64 configs.
// kind 0: fk_approx_mr/fk_mr<Panda>(num_robot, robot_id); 4/5: fk_approx/fk
// of the composite robot.  out: [config][arm][sphere][3].
template <typename Robot>
__device__ void ref_fk_composite(const float *q, int n, int detailed, float *sphere_pos, float *out) {
    constexpr int dim = Robot::dimension;
    constexpr int arms = dim / 7;
    __align__(16) __shared__ float T[64 * 2 * 16];
    const int tid = threadIdx.x, b = tid / 4;
    int c = blockIdx.x * 64 + b;
    const int src = c < n ? c : n - 1;
    float cfg[dim];
    for (int i = 0; i < dim; i++) cfg[i] = q[(size_t)src * dim + i];
    if (detailed) ppln::collision::fk<Robot>(cfg, sphere_pos, T, tid);
    else ppln::collision::fk_approx<Robot>(cfg, sphere_pos, T, tid);
    __syncthreads();
    const int ns = detailed ? 59 : 11;
    if (c < n && tid % 4 == 0)
        for (int a = 0; a < arms; a++)
            for (int s = 0; s < ns; s++)
                for (int k = 0; k < 3; k++)
                    out[(((size_t)c * arms + a) * ns + s) * 3 + k] = sphere_pos[a * ns * 3 * 64 + s * 64 * 3 + b * 3 + k];
}

extern "C" __global__ void __launch_bounds__(256)
    ref_fk(const float *q, int n, int kind, int num_robot, int robot_id, int detailed, float *sphere_pos_all,
           float *out) {
    float *sphere_pos = sphere_pos_all + (size_t)blockIdx.x * kSpherePosStride;
    if (kind == 4) {
        ref_fk_composite<ppln::robots::Panda_four>(q, n, detailed, sphere_pos, out);
        return;
    }
    if (kind == 5) {
        ref_fk_composite<ppln::robots::Panda_five>(q, n, detailed, sphere_pos, out);
        return;
    }
    __align__(16) __shared__ float T[64 * 2 * 16];
    const int tid = threadIdx.x, b = tid / 4;
    const int c = blockIdx.x * 64 + b;
    const int src = c < n ? c : n - 1;
    float cfg[7];
    for (int i = 0; i < 7; i++) cfg[i] = q[(size_t)src * 7 + i];
    if (detailed) ppln::collision::fk_mr<ppln::robots::Panda>(cfg, sphere_pos, T, tid, num_robot, robot_id);
    else ppln::collision::fk_approx_mr<ppln::robots::Panda>(cfg, sphere_pos, T, tid, num_robot, robot_id);
    __syncthreads();
    const int ns = detailed ? 59 : 11;
    if (c < n && tid % 4 == 0)
        for (int s = 0; s < ns; s++)
            for (int k = 0; k < 3; k++) out[((size_t)c * ns + s) * 3 + k] = sphere_pos[s * 64 * 3 + b * 3 + k];
}
