"""The header-only C++ layer (include/mrpop_compat.hpp) compiles against an
Environment<float>-shaped type with the reference's member names, packs its
obstacles into the C ABI's records, and links against the library."""
import subprocess
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = textwrap.dedent(r'''
    #include <array>
    #include <cstdio>
    #include <string>
    #include <vector>
    #include "mrpop_compat.hpp"
    // look-alike of the reference's shape structs (name/min_distance first)
    struct Shape { std::string name; float min_distance; };
    struct Sphere : Shape { float x, y, z, r; };
    struct Capsule : Shape { float x1, y1, z1, xv, yv, zv, r, rdv; };
    struct Cuboid : Shape { float x, y, z, axis_1_x, axis_1_y, axis_1_z, axis_2_x, axis_2_y, axis_2_z,
                            axis_3_x, axis_3_y, axis_3_z, axis_1_r, axis_2_r, axis_3_r; };
    struct Env {
        Sphere *spheres; unsigned num_spheres;
        Capsule *capsules; unsigned num_capsules;
        Capsule *z_aligned_capsules; unsigned num_z_aligned_capsules;
        Capsule *cylinders; unsigned num_cylinders;
        Cuboid *cuboids; unsigned num_cuboids;
        Cuboid *z_aligned_cuboids; unsigned num_z_aligned_cuboids;
    };
    // look-alike of the reference's PlannerResult<Robot> (Planners.hh:14-32)
    struct Result {
        bool solved = false;
        std::vector<std::array<float, 28>> path;
        int start_tree_size = 0, goal_tree_size = 0, path_length = 0, iters = 0;
        float cost = 0.0f;
        std::size_t wall_ns = 0, kernel_ns = 0, copy_ns = 0;
    };
    // compiled, not called: serving needs a GPU
    Result served(mrpop_session *ss, const mrpop_scene *s, const mrpop_robotset *r) {
        std::array<float, 28> a{}, b{};
        mrpop_plan_settings ps = {64, 60, 32, 5, 32, 1.0f, 1.0f, 42};
        return mrpop::solve_served<Result>(ss, s, r, a, b, ps);
    }
    int main(int argc, char **) {
        if (argc > 5) served(nullptr, nullptr, nullptr);
        try { mrpop::make_server(1 << 20, 17); return 6; } catch (const std::runtime_error &) {}
        Sphere s[1]; s[0].x = 1; s[0].y = 2; s[0].z = 3; s[0].r = 0.5f; s[0].name = "ball";
        Capsule c[1] = {}; c[0].x1 = 0.1f; c[0].zv = 0.4f; c[0].r = 0.05f; c[0].rdv = 6.25f;
        Cuboid b[2] = {}; b[1].x = 7; b[1].axis_1_x = 1; b[1].axis_2_y = 1; b[1].axis_3_z = 1; b[1].axis_3_r = 0.25f;
        Env env{s, 1, c, 1, nullptr, 0, nullptr, 0, b, 2, nullptr, 0};
        mrpop::SceneRecords r = mrpop::records_from_environment(env);
        mrpop_scene_desc d = r.desc();
        if (d.num_spheres != 1 || d.num_capsules != 1 || d.num_cuboids != 2) return 1;
        if (d.spheres[2] != 3.f || d.capsules[5] != 0.4f || d.capsules[7] != 6.25f) return 2;
        if (d.cuboids[15 + 0] != 7.f || d.cuboids[15 + 14] != 0.25f || d.cuboids[15 + 11] != 1.f) return 3;
        mrpop::RobotsPtr arms = mrpop::make_robots(4);
        if (!arms) return 4;
        try { mrpop::make_robots(3); return 5; } catch (const std::runtime_error &) {}
        std::printf("ok\n");
        return 0;
    }
''')


def test_compat_header_compiles_and_packs(tmp_path, lib_path):
    src = tmp_path / "compat.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "compat"
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(src), str(lib_path), "-o", str(exe),
                        f"-Wl,-rpath,{lib_path.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0 and run.stdout.strip() == "ok", (run.returncode, run.stdout, run.stderr)
