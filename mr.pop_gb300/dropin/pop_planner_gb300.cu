// pop_planner_gb300.cu -- replaces src/planning/pop_planner.cu in the
// reference's build.  It defines the reference's host entry point,
// dRRT::solve<Robot> (declared in src/planning/Planners.hh:57-64), on this
// library's planner (mrpop::drrt_solve, include/mrpop_drrt.hpp), and
// instantiates it for the two composite robots as pop_planner.cu:1032-1039
// does, so that the reference's drivers (scripts/evaluate_mr.cu:133-136,
// scripts/export_seeds.cu:126-129) link against libmrpop_gb300 unchanged.
//
// Build it from the reference's source root with this repository's include
// directory on the path, and link the library:
//   nvcc -std=c++17 -I<reference> -I<reference>/src/planning -I<repo>/include \
//        -c pop_planner_gb300.cu
//   ... -L<repo>/mr.pop_gb300/_build/default -lmrpop_gb300
#include "src/planning/Planners.hh"
#include "src/planning/Robots.hh"
#include "src/collision/environment.hh"

#include "mrpop_drrt.hpp"

namespace dRRT {

template <typename Robot>
PlannerResult<Robot> solve(typename Robot::Configuration &start, std::vector<typename Robot::Configuration> &goals,
                           ppln::collision::Environment<float> &environment, pop_settings &settings,
                           const int num_robots, const int block_per_robot) {
    return mrpop::drrt_solve<Robot, ppln::collision::Environment<float>, pop_settings, PlannerResult<Robot>>(
        start, goals, environment, settings, num_robots, block_per_robot);
}

template PlannerResult<ppln::robots::Panda_four> solve<ppln::robots::Panda_four>(
    std::array<float, 28> &, std::vector<std::array<float, 28>> &, ppln::collision::Environment<float> &,
    pop_settings &, const int, const int);
template PlannerResult<ppln::robots::Panda_five> solve<ppln::robots::Panda_five>(
    std::array<float, 35> &, std::vector<std::array<float, 35>> &, ppln::collision::Environment<float> &,
    pop_settings &, const int, const int);

}  // namespace dRRT
