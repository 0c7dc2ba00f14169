"""Planning-problem files of the reference benchmark as validator inputs.

The reference's driver reads `scripts/<robot>_problems.json` (a list of
problem dicts) and turns each into an Environment<float> with
problem_dict_to_env (scripts/evaluate_mr.cu:14-79).  load_problems does the
same for this library:

- "sphere" entries become spheres (position, radius);
- "cylinder" entries become capsules from centre, Euler XYZ angles, radius and
  length -- except in problems named "box", where each becomes a box with half
  extents (radius, radius, radius / 2), as the reference does;
- "box" entries become boxes from centre, Euler XYZ angles (R = Rz Ry Rx) and
  half extents, after any cylinder-boxes;
- problems whose "valid" is false are skipped, like the reference's loop
  (evaluate_mr.cu:125-127).
The values are cast to float32 first and the obstacles built in float32 the
way the reference's Eigen factories evaluate them (workloads.box_f32 /
capsule_f32); precision="f64" builds them in float64 and rounds once.

Each Problem also carries the start and goal configurations and, when the
file gives them, the arm bases (base_positions, base_orientation_wxyz) as
row-major 4x4 transforms for RobotSet.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .mrpop import SceneArrays
from .workloads import box, box_f32, capsule, capsule_f32


@dataclass
class Problem:
    name: str
    index: int
    scene: SceneArrays
    start: np.ndarray                 # (dof,)
    goals: np.ndarray                 # (n_goals, dof)
    bases: np.ndarray | None = None   # (arms, 4, 4) when the file gives them
    raw: dict = field(default_factory=dict, repr=False)


def quat_base(position, wxyz) -> np.ndarray:
    """Row-major 4x4 from a position and a unit quaternion (w, x, y, z)."""
    w, x, y, z = (float(v) for v in wxyz)
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    t = np.eye(4)
    t[:3, :3] = r
    t[:3, 3] = np.asarray(position, np.float64)
    return t.astype(np.float32)


def problem_scene(problem: dict, precision: str = "f32") -> SceneArrays:
    """The obstacles of one problem dict (evaluate_mr.cu:14-79)."""
    if precision == "f32":
        box_fn, capsule_fn = box_f32, capsule_f32
    elif precision == "f64":
        box_fn, capsule_fn = box, capsule
    else:
        raise ValueError(precision)
    name = problem.get("name", "")
    spheres = [np.array([*o["position"], o["radius"]], np.float32) for o in problem.get("sphere", [])]
    caps, cubs = [], []
    for o in problem.get("cylinder", []):
        r = float(o["radius"])
        if name == "box":
            cubs.append(box_fn(o["position"], o["orientation_euler_xyz"], (r, r, np.float32(r) / np.float32(2.0))))
        else:
            caps.append(capsule_fn(o["position"], o["orientation_euler_xyz"], r, float(o["length"])))
    for o in problem.get("box", []):
        cubs.append(box_fn(o["position"], o["orientation_euler_xyz"], o["half_extents"]))
    kw = {}
    if spheres:
        kw["spheres"] = np.stack(spheres)
    if caps:
        kw["capsules"] = np.stack(caps)
    if cubs:
        kw["cuboids"] = np.stack(cubs)
    return SceneArrays(**kw)


def load_problems(src, include_invalid: bool = False) -> list[Problem]:
    """Problems from a JSON file path, JSON text, or an already parsed list."""
    if isinstance(src, str) and src.lstrip()[:1] in ("[", "{"):
        data = json.loads(src)
    elif isinstance(src, (str, Path)):
        data = json.loads(Path(src).read_text())
    else:
        data = src
    out = []
    for i, p in enumerate(data):
        if not p.get("valid", True) and not include_invalid:
            continue
        bases = None
        if "base_positions" in p and "base_orientation_wxyz" in p:
            bases = np.stack([quat_base(a, q) for a, q in zip(p["base_positions"], p["base_orientation_wxyz"])])
        out.append(Problem(name=p.get("name", ""), index=int(p.get("source_index", i)), scene=problem_scene(p),
                           start=np.asarray(p["start"], np.float32),
                           goals=np.asarray(p.get("goals", []), np.float32).reshape(-1, len(p["start"])),
                           bases=bases, raw=p))
    return out
