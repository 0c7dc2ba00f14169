// A driver that calls the reference's host API exactly as its benchmark
// driver does (scripts/evaluate_mr.cu:111-136): an Environment<float> of
// boxes, the evaluate settings (:162-166) and dRRT::solve<Robot>(start,
// goals, env, settings, arms, 8).  It is compiled against the reference's own
// headers and linked with mr.pop_gb300/dropin/pop_planner_gb300.cu and the
// library.  Input (text): arms, n_boxes, boxes (15 floats each: centre, three
// axes, half extents), start, goal.  Output: one line with the result.
#include <cstdio>
#include <fstream>
#include <iostream>

#include "src/planning/Planners.hh"
#include "src/planning/Robots.hh"
#include "src/planning/pop_settings.hh"
#include "src/collision/environment.hh"

template <typename Robot>
int run(std::ifstream &in, int n_boxes) {
    using Configuration = typename Robot::Configuration;
    ppln::collision::Environment<float> env{};
    env.cuboids = new ppln::collision::Cuboid<float>[n_boxes];
    env.num_cuboids = n_boxes;
    for (int i = 0; i < n_boxes; i++) {
        auto &c = env.cuboids[i];
        in >> c.x >> c.y >> c.z >> c.axis_1_x >> c.axis_1_y >> c.axis_1_z >> c.axis_2_x >> c.axis_2_y >> c.axis_2_z >>
            c.axis_3_x >> c.axis_3_y >> c.axis_3_z >> c.axis_1_r >> c.axis_2_r >> c.axis_3_r;
    }
    Configuration start{};
    std::vector<Configuration> goals(1);
    for (auto &v : start) in >> v;
    for (auto &v : goals[0]) in >> v;
    pop_settings settings;
    settings.num_new_configs = 300;
    settings.granularity = 64;
    settings.range = 2.0;
    settings.rrtc_iter = 3;
    const int arms = Robot::dimension / 7;
    PlannerResult<Robot> r = dRRT::solve<Robot>(start, goals, env, settings, arms, 8);
    std::printf("result solved=%d cost=%.6f path_length=%d iters=%d seeds=%zu simplified=%zu start_tree=%d "
                "goal_tree=%d wall_ns=%zu\n",
                (int)r.solved, r.cost, r.path_length, r.iters, r.seed_paths.size(), r.simplified_path.size(),
                r.start_tree_size, r.goal_tree_size, r.wall_ns);
    for (const auto &cfg : r.path) {
        for (int i = 0; i < Robot::dimension; i++) std::printf("%.9g ", cfg[i]);
        std::printf("\n");
    }
    return 0;
}

int main(int argc, char **argv) {
    if (argc != 2) return 2;
    std::ifstream in(argv[1]);
    int arms = 0, n_boxes = 0;
    in >> arms >> n_boxes;
    if (arms == 4) return run<ppln::robots::Panda_four>(in, n_boxes);
    if (arms == 5) return run<ppln::robots::Panda_five>(in, n_boxes);
    return 2;
}
