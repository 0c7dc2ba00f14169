// mrpop_compat.hpp -- header-only C++ layer between the reference planner's
// host types and the C ABI in mrpop.h.
//
// The reference describes a scene as ppln::collision::Environment<float>
// (src/collision/environment.hh:11-40) holding arrays of Sphere / Capsule /
// Cuboid structs (src/collision/shapes.hh:28-185), each with a std::string
// name and a min_distance ahead of the numeric fields.  Those structs are not
// POD, so this header reads them field by field into the packed records of
// mrpop_scene_desc.  It is a template over the environment type: any struct
// with the reference's member names works (the reference's own headers
// included first, or a look-alike), and nothing here depends on them.
//
//   #include "src/collision/environment.hh"   // the reference's type
//   #include "mrpop_compat.hpp"
//   mrpop::ScenePtr scene = mrpop::make_scene(env);
//   mrpop::RobotsPtr arms = mrpop::make_robots(4);        // reference layout
//   mrpop::check(mrpop_validate_edges(scene.get(), arms.get(), d_q0, d_q1, n, 32,
//                                     MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, -1,
//                                     d_valid, d_first, stream));
#pragma once

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mrpop.h"

namespace mrpop {

inline void check(mrpop_status s) {
    if (s != MRPOP_OK) throw std::runtime_error(std::string("mrpop: ") + mrpop_last_error());
}

struct SceneDeleter {
    void operator()(mrpop_scene *s) const { mrpop_scene_destroy(s); }
};
struct RobotsDeleter {
    void operator()(mrpop_robotset *r) const { mrpop_robotset_destroy(r); }
};
struct WorkspaceDeleter {
    void operator()(mrpop_workspace *w) const { mrpop_workspace_destroy(w); }
};
using ScenePtr = std::unique_ptr<mrpop_scene, SceneDeleter>;
using RobotsPtr = std::unique_ptr<mrpop_robotset, RobotsDeleter>;
using WorkspacePtr = std::unique_ptr<mrpop_workspace, WorkspaceDeleter>;

// Packed float records of an Environment-like scene (see mrpop.h for the
// record layouts).
struct SceneRecords {
    std::vector<float> spheres, capsules, z_capsules, cylinders, cuboids, z_cuboids;

    mrpop_scene_desc desc() const {
        mrpop_scene_desc d{};
        d.spheres = spheres.data();
        d.num_spheres = (uint32_t)(spheres.size() / 4);
        d.capsules = capsules.data();
        d.num_capsules = (uint32_t)(capsules.size() / 8);
        d.z_capsules = z_capsules.data();
        d.num_z_capsules = (uint32_t)(z_capsules.size() / 8);
        d.cylinders = cylinders.data();
        d.num_cylinders = (uint32_t)(cylinders.size() / 8);
        d.cuboids = cuboids.data();
        d.num_cuboids = (uint32_t)(cuboids.size() / 15);
        d.z_cuboids = z_cuboids.data();
        d.num_z_cuboids = (uint32_t)(z_cuboids.size() / 15);
        return d;
    }
};

template <class Cap>
inline void append_capsule(std::vector<float> &out, const Cap &c) {
    out.insert(out.end(), {c.x1, c.y1, c.z1, c.xv, c.yv, c.zv, c.r, c.rdv});
}

template <class Cub>
inline void append_cuboid(std::vector<float> &out, const Cub &c) {
    out.insert(out.end(), {c.x, c.y, c.z, c.axis_1_x, c.axis_1_y, c.axis_1_z, c.axis_2_x, c.axis_2_y, c.axis_2_z,
                           c.axis_3_x, c.axis_3_y, c.axis_3_z, c.axis_1_r, c.axis_2_r, c.axis_3_r});
}

// Reads an Environment<float>-shaped value (member names of environment.hh).
template <class Env>
inline SceneRecords records_from_environment(const Env &env) {
    SceneRecords r;
    for (unsigned i = 0; i < env.num_spheres; i++)
        r.spheres.insert(r.spheres.end(), {env.spheres[i].x, env.spheres[i].y, env.spheres[i].z, env.spheres[i].r});
    for (unsigned i = 0; i < env.num_capsules; i++) append_capsule(r.capsules, env.capsules[i]);
    for (unsigned i = 0; i < env.num_z_aligned_capsules; i++) append_capsule(r.z_capsules, env.z_aligned_capsules[i]);
    for (unsigned i = 0; i < env.num_cylinders; i++) append_capsule(r.cylinders, env.cylinders[i]);
    for (unsigned i = 0; i < env.num_cuboids; i++) append_cuboid(r.cuboids, env.cuboids[i]);
    for (unsigned i = 0; i < env.num_z_aligned_cuboids; i++) append_cuboid(r.z_cuboids, env.z_aligned_cuboids[i]);
    return r;
}

template <class Env>
inline ScenePtr make_scene(const Env &env) {
    const SceneRecords rec = records_from_environment(env);
    const mrpop_scene_desc d = rec.desc();
    mrpop_scene *s = nullptr;
    check(mrpop_scene_create(&d, &s));
    return ScenePtr(s);
}

// base_T: n_arms row-major 4x4, or nullptr for the reference's compiled-in
// layouts (1, 4 or 5 arms).
inline RobotsPtr make_robots(int n_arms, const float *base_T = nullptr) {
    mrpop_robotset *r = nullptr;
    check(mrpop_robotset_create(n_arms, base_T, &r));
    return RobotsPtr(r);
}

inline WorkspacePtr make_workspace() {
    mrpop_workspace *w = nullptr;
    check(mrpop_workspace_create(&w));
    return WorkspacePtr(w);
}

// The three forms the reference's planner kernels use, batched:
//   extend   (fkcc_single_buffer_drrt, pop_planner.cu:551-564)   self only
//   connect  (fkcc_single_buffer,      pop_planner.cu:666-703)   env + self, segmented
//   roadmap  (fkcc_single_buffer_mr,   roadmap_interior.cuh:219-240) one arm
inline void validate_extend(const mrpop_scene *s, const mrpop_robotset *r, const float *q0, const float *q1,
                            int64_t n, int g, uint8_t *valid, int32_t *first_hit, void *stream = nullptr) {
    check(mrpop_validate_edges(s, r, q0, q1, n, g, MRPOP_CHECK_SELF, -1, valid, first_hit, stream));
}

inline void validate_connect(const mrpop_scene *s, const mrpop_robotset *r, const float *q0, const float *q1,
                             int64_t n, int g, float range, uint8_t *valid, int32_t *first_hit,
                             int32_t *n_seg = nullptr, void *stream = nullptr) {
    check(mrpop_validate_segments(s, r, q0, q1, n, g, MRPOP_RULE_CONNECT, range, MRPOP_CHECK_ENV | MRPOP_CHECK_SELF,
                                  -1, valid, first_hit, n_seg, stream));
}

// Serving: RAII handles for the validation service and its sessions, and a
// served solve that fills a PlannerResult-shaped struct (the member names of
// the reference's PlannerResult<Robot>, Planners.hh:14-32) from the library's
// planner.  Config is the reference's Robot::Configuration (std::array<float, D>).
struct ServerDeleter {
    void operator()(mrpop_server *s) const { mrpop_server_destroy(s); }
};
struct SessionDeleter {
    void operator()(mrpop_session *s) const { mrpop_session_close(s); }
};
using ServerPtr = std::unique_ptr<mrpop_server, ServerDeleter>;
using SessionPtr = std::unique_ptr<mrpop_session, SessionDeleter>;

inline ServerPtr make_server(int64_t budget_bytes = 0, int streams = 0, int64_t host_bytes = 0) {
    mrpop_server_config c{};
    c.budget_bytes = budget_bytes;
    c.streams = streams;
    c.host_bytes = host_bytes;
    mrpop_server *s = nullptr;
    check(mrpop_server_create(&c, &s));
    return ServerPtr(s);
}

inline SessionPtr open_session(mrpop_server *server, int arms, int64_t max_edges, int max_granularity,
                               int64_t timeout_ms = -1) {
    mrpop_session *ss = nullptr;
    check(mrpop_session_open(server, arms, max_edges, max_granularity, timeout_ms, &ss));
    return SessionPtr(ss);
}

template <class Result, class Config>
inline Result solve_served(mrpop_session *ss, const mrpop_scene *s, const mrpop_robotset *r, const Config &start,
                           const Config &goal, const mrpop_plan_settings &ps,
                           uint32_t flags = MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, int64_t max_waypoints = 4096) {
    const size_t dof = start.size();
    std::vector<float> path((size_t)max_waypoints * dof);
    mrpop_plan_result pr{};
    const auto t0 = std::chrono::steady_clock::now();
    check(mrpop_session_plan(ss, s, r, flags, start.data(), goal.data(), &ps, path.data(), max_waypoints, &pr));
    Result out{};
    out.solved = pr.solved != 0;
    for (int64_t i = 0; i < std::min(pr.waypoints, max_waypoints); i++) {
        Config c{};
        std::copy(path.begin() + i * dof, path.begin() + (i + 1) * dof, c.begin());
        out.path.push_back(c);
    }
    out.start_tree_size = (int)pr.start_tree;
    out.goal_tree_size = (int)pr.goal_tree;
    out.path_length = (int)out.path.size();
    out.iters = pr.iterations;
    out.cost = (float)pr.cost;
    out.wall_ns = (std::size_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                      std::chrono::steady_clock::now() - t0).count();
    out.kernel_ns = (std::size_t)pr.validate_ns;  // time spent waiting on the service's validation
    out.copy_ns = 0;                              // session buffers are read and written in place
    return out;
}

inline void validate_roadmap(const mrpop_scene *s, const mrpop_robotset *r, int robot_id, const float *q0,
                             const float *q1, int64_t n, int g, uint8_t *valid, int32_t *first_hit,
                             void *stream = nullptr) {
    check(mrpop_validate_edges(s, r, q0, q1, n, g, MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, robot_id, valid, first_hit,
                               stream));
}

}  // namespace mrpop
