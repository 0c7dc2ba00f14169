"""mrpop_gb300 -- GB300-native batched edge validation for the MR.POP planner.

The compute path is the CUDA library built from csrc/ (C ABI in
include/mrpop.h); this package holds its build recipe, a ctypes host binding
and the seeded workload generators.
"""
from . import build, drrt, evaluate, mrpop, planner, problems, serving, workloads  # noqa: F401
from .mrpop import (CHECK_ENV, CHECK_SELF, MODE_EXACT, RULE_BSPLINE, RULE_CONNECT, RULE_PLAIN,  # noqa: F401
                    RULE_SHORTCUT, Batch, MrpopError, RobotSet, Scene, SceneArrays, Server, Session, Workspace, broad_flops_per_sample,
                    count_flops, debug_trig, fk_spheres, kernel_timing, kernel_times, library, validate)

__version__ = "0.1.0"
