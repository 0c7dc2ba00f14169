"""Seeded synthetic workloads for the edge validator (scenes, arm layouts, edges).

No public benchmark suite exists for this path; these generators stand in
for the planner's inputs with the shapes and value ranges of the benchmark
configurations:
  config 1  one Panda (identity base), 4096 edges x 32 samples, 16 yawed boxes +
            8 vertical capsules in a 1.2 m cube in front of the base;
  config 2  four Pandas at the corners of a 1.0 m square facing the centre,
            65536 edges x 32 samples, |dq| <= 1.5 rad, a bin-picking scene
            (table + 4 open bins of 0.01 m walls + 30 boxes, 51 boxes total);
  config 3  five Pandas on a 1.8 m line facing a 4x3 shelf (0.02 m boards,
            0.35 x 0.3 x 0.3 m cells) holding 20 capsules, 262144 edges x 64,
            plus a shortcut batch (1024 paths, 64 pairs each);
  config 4  512 planning instances with 1-5 arms, lognormal edge counts
            (median 2000, sigma 1) and granularity in {16, 32, 64}.
Obstacle construction follows the reference's factories: boxes from centre,
Euler XYZ (R = Rz*Ry*Rx, axes = columns of R) and half extents
(factory.hh:26-41); capsules from centre, Euler, radius and length with end
points at +-length/2 on the local z axis and rdv = 1/|v|^2 (factory.hh:100-114,
70-80).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .mrpop import SceneArrays

# Panda joint limits as q = u*s_m + s_a (Robots.hh:13-23)
PANDA_SM = np.array([5.9342, 3.6652, 5.9342, 3.2289, 5.9342, 3.9095999999999997, 5.9342], np.float32)
PANDA_SA = np.array([-2.9671, -1.8326, -2.9671, -3.1416, -2.9671, -0.0873, -2.9671], np.float32)
PANDA_LO = PANDA_SA
PANDA_HI = (PANDA_SA + PANDA_SM).astype(np.float32)


def rot_xyz(rho: float, theta: float, phi: float) -> np.ndarray:
    cx, sx = math.cos(rho), math.sin(rho)
    cy, sy = math.cos(theta), math.sin(theta)
    cz, sz = math.cos(phi), math.sin(phi)
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    return rz @ ry @ rx


def box(center, euler_xyz, half) -> np.ndarray:
    r = rot_xyz(*euler_xyz)
    rec = [*center, *r[:, 0], *r[:, 1], *r[:, 2], *half]
    return np.array(rec, np.float32)


def capsule(center, euler_xyz, radius, length) -> np.ndarray:
    r = rot_xyz(*euler_xyz)
    c = np.asarray(center, np.float64)
    p1 = (c + r @ np.array([0, 0, length / 2])).astype(np.float32)
    p2 = (c + r @ np.array([0, 0, -length / 2])).astype(np.float32)
    v = (p2 - p1).astype(np.float32)
    dot = np.float32(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return np.array([*p1, *v, radius, np.float32(1.0 / float(dot))], np.float32)


# ---------------------------------------------------------------------------
# The reference's factories in float32, as its host code evaluates them:
# Eigen::AngleAxisf(phi, Z) * AngleAxisf(theta, Y) * AngleAxisf(rho, X) is a
# product of unit quaternions (factory.hh:29-31, 103-105), applied to the unit
# axes (box) or turned into a rotation matrix of an affine transform (capsule).
# Restated from Eigen 3.4's scalar (non-vectorised) code paths -- AngleAxis to
# Quaternion (w = cos(a/2), v = sin(a/2) * axis), the generic quaternion product,
# QuaternionBase::_transformVector (uv = 2 * v x p; p + w * uv + v x uv) and
# toRotationMatrix -- every operation rounded to float32 without fused
# multiply-adds.  The reference's build enables SSE/AVX2/FMA (CMakeLists.txt:30),
# under which Eigen may take vectorised paths that round differently, so these
# are pinned against the float64 construction (box, capsule above) to 1e-6.
# ---------------------------------------------------------------------------
_F = np.float32


def _quat_axis(angle, axis: int):
    ha = _F(0.5) * _F(angle)
    s = _F(math.sin(ha))  # std::sin on float
    q = [_F(math.cos(ha)), _F(0), _F(0), _F(0)]
    q[1 + axis] = _F(s * _F(1))
    return q


def _quat_mul(a, b):
    aw, ax, ay, az = a
    bw, bx, by, bz = b
    return [_F(_F(_F(aw * bw) - _F(ax * bx)) - _F(ay * by)) - _F(az * bz),
            _F(_F(_F(aw * bx) + _F(ax * bw)) + _F(ay * bz)) - _F(az * by),
            _F(_F(_F(aw * by) + _F(ay * bw)) + _F(az * bx)) - _F(ax * bz),
            _F(_F(_F(aw * bz) + _F(az * bw)) + _F(ax * by)) - _F(ay * bx)]


def _cross(a, b):
    return [_F(_F(a[1] * b[2]) - _F(a[2] * b[1])), _F(_F(a[2] * b[0]) - _F(a[0] * b[2])),
            _F(_F(a[0] * b[1]) - _F(a[1] * b[0]))]


def _quat_rotate(q, p):
    v = q[1:]
    uv = _cross(v, p)
    uv = [_F(u + u) for u in uv]
    vuv = _cross(v, uv)
    return [_F(_F(p[i] + _F(q[0] * uv[i])) + vuv[i]) for i in range(3)]


def euler_quat_f32(euler_xyz):
    rho, theta, phi = (_F(e) for e in euler_xyz)
    return _quat_mul(_quat_mul(_quat_axis(phi, 2), _quat_axis(theta, 1)), _quat_axis(rho, 0))


def quat_matrix_f32(q):
    w, x, y, z = q
    tx, ty, tz = _F(2) * x, _F(2) * y, _F(2) * z
    twx, twy, twz = tx * w, ty * w, tz * w
    txx, txy, txz = tx * x, ty * x, tz * x
    tyy, tyz, tzz = ty * y, tz * y, tz * z
    return np.array([[_F(1) - (tyy + tzz), txy - twz, txz + twy],
                     [txy + twz, _F(1) - (txx + tzz), tyz - twx],
                     [txz - twy, tyz + twx, _F(1) - (txx + tyy)]], np.float32)


def box_f32(center, euler_xyz, half) -> np.ndarray:
    """factory::cuboid::flat (factory.hh:26-41) in float32."""
    q = euler_quat_f32(euler_xyz)
    axes = [_quat_rotate(q, [_F(1) if i == k else _F(0) for i in range(3)]) for k in range(3)]
    return np.array([*(_F(c) for c in center), *axes[0], *axes[1], *axes[2], *(_F(h) for h in half)], np.float32)


def capsule_f32(center, euler_xyz, radius, length) -> np.ndarray:
    """factory::cylinder::center::flat (factory.hh:100-114, endpoints at
    +-length/2 on the local z axis, rdv = 1/|v|^2 in double, :70-80) in float32."""
    r = quat_matrix_f32(euler_quat_f32(euler_xyz))
    c = np.asarray(center, np.float32)
    hl = _F(_F(length) / _F(2))
    p1 = np.array([_F(_F(r[i, 2] * hl) + c[i]) for i in range(3)], np.float32)
    p2 = np.array([_F(_F(r[i, 2] * -hl) + c[i]) for i in range(3)], np.float32)
    v = (p2 - p1).astype(np.float32)
    dot = np.float32(np.float32(np.float32(v[0] * v[0]) + np.float32(v[1] * v[1])) + np.float32(v[2] * v[2]))
    return np.array([*p1, *v, _F(radius), np.float32(1.0 / float(dot))], np.float32)


def yaw_base(x: float, y: float, z: float, yaw: float) -> np.ndarray:
    c, s = math.cos(yaw), math.sin(yaw)
    return np.array([[c, -s, 0, x], [s, c, 0, y], [0, 0, 1, z], [0, 0, 0, 1]], np.float32)


def bases_facing_centre(n: int, radius: float, z: float = 0.0, phase: float = math.pi / 4) -> np.ndarray:
    """n arms evenly on a circle, each yawed to face the centre (n=1: identity)."""
    if n == 1:
        return np.eye(4, dtype=np.float32)[None]
    out = []
    for a in range(n):
        ang = phase + 2 * math.pi * a / n
        x, y = radius * math.cos(ang), radius * math.sin(ang)
        out.append(yaw_base(x, y, z, math.atan2(-y, -x)))
    return np.stack(out)


# ---------------------------------------------------------------------------
# scenes
# ---------------------------------------------------------------------------
def scene_config1(seed: int = 0) -> SceneArrays:
    rng = np.random.default_rng(seed)
    lo, hi = np.array([0.2, -0.6, 0.0]), np.array([1.4, 0.6, 1.2])
    boxes = [box(rng.uniform(lo, hi), (0.0, 0.0, rng.uniform(-math.pi, math.pi)), rng.uniform(0.03, 0.2, 3))
             for _ in range(16)]
    caps = [capsule(rng.uniform(lo, hi), (0.0, 0.0, 0.0), rng.uniform(0.02, 0.08), rng.uniform(0.1, 0.5))
            for _ in range(8)]
    return SceneArrays(cuboids=np.stack(boxes), capsules=np.stack(caps))


def scene_config2(seed: int = 0) -> SceneArrays:
    rng = np.random.default_rng(seed)
    boxes = [box((0.0, 0.0, 0.15), (0, 0, 0), (0.35, 0.35, 0.15))]  # table, top at z=0.30
    t, h = 0.005, 0.06  # wall half thickness, wall half height
    bins = [(-0.17, -0.17), (0.17, -0.17), (-0.17, 0.17), (0.17, 0.17)]
    half_w = 0.14
    for bx, by in bins:
        boxes.append(box((bx, by, 0.30 + t), (0, 0, 0), (half_w, half_w, t)))  # floor
        for sx, sy, hx, hy in ((half_w - t, 0, t, half_w), (-(half_w - t), 0, t, half_w),
                               (0, half_w - t, half_w, t), (0, -(half_w - t), half_w, t)):
            boxes.append(box((bx + sx, by + sy, 0.30 + 2 * t + h), (0, 0, 0), (hx, hy, h)))
    for i in range(30):
        bx, by = bins[i % 4]
        half = rng.uniform(0.015, 0.06, 3)
        c = (bx + rng.uniform(-0.08, 0.08), by + rng.uniform(-0.08, 0.08), 0.30 + 2 * t + half[2])
        boxes.append(box(c, (0, 0, rng.uniform(-math.pi, math.pi)), half))
    return SceneArrays(cuboids=np.stack(boxes))


def scene_config3(seed: int = 0) -> SceneArrays:
    rng = np.random.default_rng(seed)
    cols, rows, cw, ch, cd, bt = 4, 3, 0.35, 0.30, 0.30, 0.01  # bt = board half thickness
    x0, y0, z0 = -cols * cw / 2, 0.45, 0.20  # shelf front face at y0, bottom at z0
    boxes = []
    width, height = cols * cw, rows * ch
    for r in range(rows + 1):  # horizontal boards
        boxes.append(box((0.0, y0 + cd / 2, z0 + r * ch), (0, 0, 0), (width / 2 + bt, cd / 2, bt)))
    for c in range(cols + 1):  # vertical boards
        boxes.append(box((x0 + c * cw, y0 + cd / 2, z0 + height / 2), (0, 0, 0), (bt, cd / 2, height / 2)))
    boxes.append(box((0.0, y0 + cd + bt, z0 + height / 2), (0, 0, 0), (width / 2 + bt, bt, height / 2)))  # back
    caps = []
    for i in range(20):
        c, r = i % cols, (i // cols) % rows
        rad, ln = rng.uniform(0.02, 0.05), rng.uniform(0.08, 0.2)
        cx = x0 + (c + 0.5) * cw + rng.uniform(-0.1, 0.1)
        cy = y0 + cd / 2 + rng.uniform(-0.08, 0.08)
        caps.append(capsule((cx, cy, z0 + r * ch + bt + rad + ln / 2), (0, 0, 0), rad, ln))
    return SceneArrays(cuboids=np.stack(boxes), capsules=np.stack(caps))


def bases_config2() -> np.ndarray:
    return np.stack([yaw_base(x, y, 0.0, math.atan2(-y, -x)) for x, y in
                     ((0.5, -0.5), (-0.5, -0.5), (-0.5, 0.5), (0.5, 0.5))])


def bases_config3() -> np.ndarray:
    return np.stack([yaw_base(x, -0.35, 0.0, math.pi / 2) for x in np.linspace(-0.9, 0.9, 5)])


# ---------------------------------------------------------------------------
# edges
# ---------------------------------------------------------------------------
def random_configs(rng: np.random.Generator, n: int, arms: int) -> np.ndarray:
    lo, hi = np.tile(PANDA_LO, arms), np.tile(PANDA_HI, arms)
    return rng.uniform(lo, hi, size=(n, 7 * arms)).astype(np.float32)


def random_edges(rng: np.random.Generator, n: int, arms: int, max_dist: float) -> tuple[np.ndarray, np.ndarray]:
    """q0 uniform in the limits; q1 = q0 + L*u (|u| = 1, L ~ U(0, max_dist)), clipped to the limits."""
    lo, hi = np.tile(PANDA_LO, arms), np.tile(PANDA_HI, arms)
    q0 = random_configs(rng, n, arms)
    u = rng.normal(size=q0.shape)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    ln = rng.uniform(0.0, max_dist, size=(n, 1))
    q1 = np.clip(q0 + ln * u, lo, hi).astype(np.float32)
    return q0, q1


@dataclass
class Workload:
    name: str
    scene: SceneArrays
    bases: np.ndarray        # (arms, 4, 4)
    q0: np.ndarray
    q1: np.ndarray
    granularity: int
    flags: int
    arm: int = -1
    rule: int = 0
    range_: float = 0.0


def config1(n_edges: int = 4096, seed: int = 0) -> Workload:
    from .mrpop import CHECK_ENV, CHECK_SELF
    rng = np.random.default_rng(1000 + seed)
    q0, q1 = random_edges(rng, n_edges, 1, 1.0)
    return Workload("config1_panda_4096x32", scene_config1(seed), np.eye(4, dtype=np.float32)[None], q0, q1, 32,
                    CHECK_ENV | CHECK_SELF, arm=0)


def config2(n_edges: int = 65536, seed: int = 0) -> Workload:
    from .mrpop import CHECK_ENV, CHECK_SELF
    rng = np.random.default_rng(2000 + seed)
    q0, q1 = random_edges(rng, n_edges, 4, 1.5)
    return Workload("config2_4panda_65536x32", scene_config2(seed), bases_config2(), q0, q1, 32,
                    CHECK_ENV | CHECK_SELF)


def config3(n_edges: int = 262144, seed: int = 0) -> Workload:
    from .mrpop import CHECK_ENV, CHECK_SELF
    rng = np.random.default_rng(3000 + seed)
    q0, q1 = random_edges(rng, n_edges, 5, 1.5)
    return Workload("config3_5panda_262144x64", scene_config3(seed), bases_config3(), q0, q1, 64,
                    CHECK_ENV | CHECK_SELF)


def config3_shortcuts(n_paths: int = 1024, pairs: int = 64, seed: int = 0) -> Workload:
    """Shortcut batch: random-walk paths of 20-200 waypoints, `pairs` (i<j) per path."""
    from .mrpop import CHECK_ENV, CHECK_SELF, RULE_SHORTCUT
    rng = np.random.default_rng(3500 + seed)
    lo, hi = np.tile(PANDA_LO, 5), np.tile(PANDA_HI, 5)
    a, b = [], []
    for _ in range(n_paths):
        m = int(rng.integers(20, 201))
        steps = rng.normal(size=(m, 35))
        steps *= (rng.uniform(0.1, 0.5, size=(m, 1)) / np.linalg.norm(steps, axis=1, keepdims=True))
        path = np.clip(random_configs(rng, 1, 5)[0] + np.cumsum(steps, axis=0), lo, hi).astype(np.float32)
        i = rng.integers(0, m - 1, size=pairs)
        j = np.minimum(m - 1, i + 1 + rng.integers(0, m, size=pairs) % (m - 1 - i))
        a.append(path[i])
        b.append(path[j])
    return Workload("config3_shortcut_1024x64", scene_config3(seed), bases_config3(), np.concatenate(a),
                    np.concatenate(b), 64, CHECK_ENV | CHECK_SELF, rule=RULE_SHORTCUT, range_=2.0)


def config4_instances(n_instances: int = 512, seed: int = 0, scale: float = 1.0) -> list[Workload]:
    """Uneven multi-instance batch: 1-5 arms, lognormal edge counts, g in {16,32,64}."""
    from .mrpop import CHECK_ENV, CHECK_SELF
    rng = np.random.default_rng(4000 + seed)
    out = []
    for i in range(n_instances):
        arms = int(rng.integers(1, 6))
        n = max(1, int(round(scale * rng.lognormal(math.log(2000.0), 1.0))))
        g = int(rng.choice([16, 32, 64]))
        sc = scene_config1(seed * 7919 + i) if rng.random() < 0.5 else scene_config2(seed * 7919 + i)
        bases = bases_facing_centre(arms, 0.71)
        q0, q1 = random_edges(rng, n, arms, 1.5)
        out.append(Workload(f"inst{i}", sc, bases, q0, q1, g, CHECK_ENV | CHECK_SELF))
    return out
