// mrpop_drrt.hpp -- the reference planner's host API on this library.
//
// The reference declares
//   template <typename Robot> PlannerResult<Robot>
//   dRRT::solve(Robot::Configuration &start, std::vector<Robot::Configuration> &goals,
//               ppln::collision::Environment<float> &env, pop_settings &settings,
//               const int num_robots, const int block_per_robot);
// in src/planning/Planners.hh:57-64, with PlannerResult at :14-32 and
// pop_settings in src/planning/pop_settings.hh:3-32, and defines it in
// pop_planner.cu:739-1030 (explicit instantiations for Panda_four and
// Panda_five at :1032-1039).  mrpop::drrt_solve below is that function on
// mrpop_drrt_solve (include/mrpop.h): it is a template over the robot,
// environment, settings and result types, so the reference's own types work
// (its headers included first) and so does any type with their member names.
// mr.pop_gb300/dropin/pop_planner_gb300.cu is the translation unit that
// replaces pop_planner.cu in the reference's build: it defines dRRT::solve
// with this function and instantiates it for the two robots.
//
// Behaviour as the reference's:
//   - the scene is read from the environment's spheres, capsules, z-aligned
//     capsules, cuboids and z-aligned cuboids (cylinders are never tested);
//   - the arms sit on the reference's compiled-in bases for num_robots
//     (quad_franka_base_transform / five_franka_base_transform), unless the
//     caller passes its own base_T;
//   - PlannerResult::path holds the reported solution from the goal to the
//     start, simplified when settings.path_simplify is set; seed_paths holds
//     every improving solution with its cost; iters, cost, path_length and the
//     tree sizes are the reported solution's; wall_ns, kernel_ns, copy_ns
//     are timed like the reference's (copy_ns is 0: nothing is staged);
//   - errors are printed and an unsolved result is returned (the reference
//     prints its CUDA errors and carries on, pop_planner.cu:967-994).
// In addition, simplified_path holds the reported path when it was
// simplified (the reference leaves it empty).
#pragma once

#include <array>
#include <chrono>
#include <cstdio>
#include <utility>
#include <vector>

#include "mrpop_compat.hpp"

namespace mrpop {

// pop_settings -> mrpop_drrt_settings, field by field (pop_settings.hh:3-32).
template <class Settings>
inline mrpop_drrt_settings drrt_settings_from(const Settings &s, int block_per_robot) {
    mrpop_drrt_settings o{};
    mrpop_drrt_settings_default(&o);
    o.max_samples = s.max_samples;
    o.max_iters = s.max_iters;
    o.optimize_iters = s.optimize_iters;
    o.num_new_configs = s.num_new_configs;
    o.granularity = s.granularity;
    o.range = s.range;
    o.balance = s.balance;
    o.tree_ratio = s.tree_ratio;
    o.dynamic_domain = s.dynamic_domain ? 1 : 0;
    o.dd_alpha = s.dd_alpha;
    o.dd_radius = s.dd_radius;
    o.dd_min_radius = s.dd_min_radius;
    o.roadmap_reassign = s.roadmap_reassign ? 1 : 0;
    o.rrtc_iter = s.rrtc_iter;
    o.resample_iter = s.resample_iter;
    o.cost_bound_resample = s.cost_bound_resample ? 1 : 0;
    o.path_simplify = s.path_simplify ? 1 : 0;
    o.phs = s.phs ? 1 : 0;
    o.simplify_round = s.simplify_round;
    o.bspline_step = s.bspline_step;
    o.bspline_min_change = s.bspline_min_change;
    o.perturb_step = s.perturb_step;
    o.perturb_empty_step = s.perturb_empty_step;
    o.block_per_robot = block_per_robot;
    return o;
}

template <class Robot, class Result>
struct DrrtCollect {
    Result *res;
    bool simplified;
    static void on_solution(void *ctx, int32_t, float cost, const float *path, int64_t n, const float *, int64_t) {
        auto *c = static_cast<DrrtCollect *>(ctx);
        constexpr int dim = Robot::dimension;
        std::vector<typename Robot::Configuration> p((size_t)n);
        for (int64_t i = 0; i < n; i++)
            for (int d = 0; d < dim; d++) p[(size_t)i][(size_t)d] = path[i * dim + d];
        c->res->path = p;
        if (c->simplified) c->res->simplified_path = p;
        c->res->seed_paths.emplace_back(cost, std::move(p));
    }
};

template <class Robot, class Env, class Settings, class Result>
inline Result drrt_solve(typename Robot::Configuration &start, std::vector<typename Robot::Configuration> &goals,
                         const Env &env, const Settings &settings, int num_robots, int block_per_robot,
                         const float *base_T = nullptr) {
    const auto t0 = std::chrono::steady_clock::now();
    Result res{};
    try {
        if ((int)Robot::dimension != 7 * num_robots) throw std::runtime_error("dRRT::solve: num_robots != dimension / 7");
        ScenePtr scene = make_scene(env);
        RobotsPtr robots = make_robots(num_robots, base_T);
        const mrpop_drrt_settings st = drrt_settings_from(settings, block_per_robot);
        std::vector<float> gl;
        for (const auto &c : goals) gl.insert(gl.end(), c.begin(), c.end());
        DrrtCollect<Robot, Result> col{&res, st.path_simplify != 0};
        mrpop_drrt_result out{};
        check(mrpop_drrt_solve(scene.get(), robots.get(), start.data(), gl.data(), (int)goals.size(), &st, nullptr,
                               0, &DrrtCollect<Robot, Result>::on_solution, &col, &out));
        res.solved = out.solved != 0;
        res.cost = out.cost;
        res.iters = out.iters;
        res.path_length = (int)res.path.size();
        res.start_tree_size = (int)out.start_tree_size;
        res.goal_tree_size = (int)out.goal_tree_size;
        res.kernel_ns = (std::size_t)out.kernel_ns;
        res.copy_ns = 0;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
    }
    res.wall_ns = (std::size_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() -
                                                                                     t0)
                      .count();
    return res;
}

}  // namespace mrpop
