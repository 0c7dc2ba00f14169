// panda_model.cuh -- Franka Panda sphere model, FK and collision primitives
// for the GB300 edge validator.
//
// Geometry tables are the reference's data (panda_multi_geometry.cuh:17-516,
// identical to panda.cuh:97-595), regrouped per joint: the spheres of joint j
// are kApprox/kDet[first[j] .. first[j+1]).
//
// Arithmetic contract: every value that feeds a collision verdict is computed
// with the rounding sequence of the reference's compiled device code.  The
// reference builds each joint step column-wise with 0/1 select arithmetic
// (utils.cuh:400-427) and composes with a 4-term dot product per entry
// (utils.cuh:443-445, contracted to an FMA chain by nvcc).  For the Panda's
// fixed transforms (rotation blocks are signed permutations) most terms of
// those chains are exact products with 0 or 1, so the chains reduce exactly to
// the short forms below; the only places where two non-trivial products meet
// are written with pair_fma(), whose fused operand follows MRPOP_PAIR_ORDER
// (0: fma(a,b,c*d), the first product fused).  All operations use the _rn
// intrinsics so nvcc cannot re-contract them.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#ifndef MRPOP_PAIR_ORDER
#define MRPOP_PAIR_ORDER 0
#endif

namespace mrpop {

struct SphereDef {
    float x, y, z, r;
};

constexpr int kNumJoints = 8;
constexpr int kNumApprox = 11;
constexpr int kNumDet = 59;

// Broad-phase ("approx") spheres, panda_multi_geometry.cuh:17-29.
constexpr SphereDef kApprox[kNumApprox] = {
    {0.0f, 0.0f, 0.05f, 0.08f},        {-0.001f, -0.039f, -0.085f, 0.154f},
    {0.0f, -0.085f, 0.04f, 0.154f},    {0.039f, 0.028f, -0.052f, 0.128f},
    {-0.042f, 0.049f, 0.029f, 0.126f}, {-0.001f, 0.037f, -0.11f, 0.176f},
    {0.042f, 0.014f, 0.0f, 0.095f},    {0.015f, 0.015f, 0.075f, 0.072f},
    {0.0f, 0.0f, 0.129f, 0.104f},      {0.054447f, 0.054447f, 0.1984f, 0.024f},
    {-0.054447f, -0.054447f, 0.1984f, 0.024f}};
// joint j owns approx spheres [kApproxFirst[j], kApproxFirst[j+1]) (:83-106)
constexpr int kApproxFirst[kNumJoints + 1] = {0, 1, 2, 3, 4, 5, 6, 7, 11};

// Detailed spheres, panda_multi_geometry.cuh:186-246.
constexpr SphereDef kDet[kNumDet] = {
    {0.0f, 0.0f, 0.05f, 0.08f},        {0.0f, -0.08f, 0.0f, 0.06f},
    {0.0f, -0.03f, 0.0f, 0.06f},       {0.0f, 0.0f, -0.12f, 0.06f},
    {0.0f, 0.0f, -0.17f, 0.06f},       {0.0f, 0.0f, 0.03f, 0.06f},
    {0.0f, 0.0f, 0.08f, 0.06f},        {0.0f, -0.12f, 0.0f, 0.06f},
    {0.0f, -0.17f, 0.0f, 0.06f},       {0.0f, 0.0f, -0.1f, 0.06f},
    {0.0f, 0.0f, -0.06f, 0.05f},       {0.08f, 0.06f, 0.0f, 0.055f},
    {0.08f, 0.02f, 0.0f, 0.055f},      {-0.08f, 0.095f, 0.0f, 0.06f},
    {0.0f, 0.0f, 0.02f, 0.055f},       {0.0f, 0.0f, 0.06f, 0.055f},
    {-0.08f, 0.06f, 0.0f, 0.055f},     {0.0f, 0.055f, 0.0f, 0.06f},
    {0.0f, 0.075f, 0.0f, 0.06f},       {0.0f, 0.0f, -0.22f, 0.06f},
    {0.0f, 0.05f, -0.18f, 0.05f},      {0.01f, 0.08f, -0.14f, 0.025f},
    {0.01f, 0.085f, -0.11f, 0.025f},   {0.01f, 0.09f, -0.08f, 0.025f},
    {0.01f, 0.095f, -0.05f, 0.025f},   {-0.01f, 0.08f, -0.14f, 0.025f},
    {-0.01f, 0.085f, -0.11f, 0.025f},  {-0.01f, 0.09f, -0.08f, 0.025f},
    {-0.01f, 0.095f, -0.05f, 0.025f},  {0.0f, 0.0f, 0.0f, 0.05f},
    {0.08f, -0.01f, 0.0f, 0.05f},      {0.08f, 0.035f, 0.0f, 0.052f},
    {0.0f, 0.0f, 0.07f, 0.05f},        {0.02f, 0.04f, 0.08f, 0.025f},
    {0.04f, 0.02f, 0.08f, 0.025f},     {0.04f, 0.06f, 0.085f, 0.02f},
    {0.06f, 0.04f, 0.085f, 0.02f},     {-0.053033f, -0.053033f, 0.117f, 0.028f},
    {-0.03182f, -0.03182f, 0.117f, 0.028f}, {-0.010607f, -0.010607f, 0.117f, 0.028f},
    {0.010607f, 0.010607f, 0.117f, 0.028f}, {0.03182f, 0.03182f, 0.117f, 0.028f},
    {0.053033f, 0.053033f, 0.117f, 0.028f}, {-0.053033f, -0.053033f, 0.137f, 0.026f},
    {-0.03182f, -0.03182f, 0.137f, 0.026f}, {-0.010607f, -0.010607f, 0.137f, 0.026f},
    {0.010607f, 0.010607f, 0.137f, 0.026f}, {0.03182f, 0.03182f, 0.137f, 0.026f},
    {0.053033f, 0.053033f, 0.137f, 0.026f}, {-0.053033f, -0.053033f, 0.157f, 0.024f},
    {-0.03182f, -0.03182f, 0.157f, 0.024f}, {-0.010607f, -0.010607f, 0.157f, 0.024f},
    {0.010607f, 0.010607f, 0.157f, 0.024f}, {0.03182f, 0.03182f, 0.157f, 0.024f},
    {0.053033f, 0.053033f, 0.157f, 0.024f}, {0.056569f, 0.056569f, 0.1874f, 0.012f},
    {0.051619f, 0.051619f, 0.2094f, 0.012f}, {-0.056569f, -0.056569f, 0.1874f, 0.012f},
    {-0.051619f, -0.051619f, 0.2094f, 0.012f}};
// joint j owns detailed spheres [kDetFirst[j], kDetFirst[j+1]) (counts :362-371)
constexpr int kDetFirst[kNumJoints + 1] = {0, 1, 5, 9, 13, 17, 29, 32, 59};
constexpr int kDetCount[kNumJoints] = {1, 4, 4, 4, 4, 12, 3, 27};

// Device copies for run-time indexing ({x, y, z, r} per sphere).
static __constant__ float4 c_approx[kNumApprox] = {
#define MRPOP_ROW(i) {kApprox[i].x, kApprox[i].y, kApprox[i].z, kApprox[i].r}
    MRPOP_ROW(0), MRPOP_ROW(1), MRPOP_ROW(2), MRPOP_ROW(3), MRPOP_ROW(4), MRPOP_ROW(5),
    MRPOP_ROW(6), MRPOP_ROW(7), MRPOP_ROW(8), MRPOP_ROW(9), MRPOP_ROW(10)};
#undef MRPOP_ROW
static __constant__ float4 c_det[kNumDet] = {
#define MRPOP_ROW(i) {kDet[i].x, kDet[i].y, kDet[i].z, kDet[i].r}
    MRPOP_ROW(0),  MRPOP_ROW(1),  MRPOP_ROW(2),  MRPOP_ROW(3),  MRPOP_ROW(4),  MRPOP_ROW(5),
    MRPOP_ROW(6),  MRPOP_ROW(7),  MRPOP_ROW(8),  MRPOP_ROW(9),  MRPOP_ROW(10), MRPOP_ROW(11),
    MRPOP_ROW(12), MRPOP_ROW(13), MRPOP_ROW(14), MRPOP_ROW(15), MRPOP_ROW(16), MRPOP_ROW(17),
    MRPOP_ROW(18), MRPOP_ROW(19), MRPOP_ROW(20), MRPOP_ROW(21), MRPOP_ROW(22), MRPOP_ROW(23),
    MRPOP_ROW(24), MRPOP_ROW(25), MRPOP_ROW(26), MRPOP_ROW(27), MRPOP_ROW(28), MRPOP_ROW(29),
    MRPOP_ROW(30), MRPOP_ROW(31), MRPOP_ROW(32), MRPOP_ROW(33), MRPOP_ROW(34), MRPOP_ROW(35),
    MRPOP_ROW(36), MRPOP_ROW(37), MRPOP_ROW(38), MRPOP_ROW(39), MRPOP_ROW(40), MRPOP_ROW(41),
    MRPOP_ROW(42), MRPOP_ROW(43), MRPOP_ROW(44), MRPOP_ROW(45), MRPOP_ROW(46), MRPOP_ROW(47),
    MRPOP_ROW(48), MRPOP_ROW(49), MRPOP_ROW(50), MRPOP_ROW(51), MRPOP_ROW(52), MRPOP_ROW(53),
    MRPOP_ROW(54), MRPOP_ROW(55), MRPOP_ROW(56), MRPOP_ROW(57), MRPOP_ROW(58)};
#undef MRPOP_ROW

__host__ __device__ __forceinline__ constexpr int det_joint(int i) {
    return i < 1 ? 0 : i < 5 ? 1 : i < 9 ? 2 : i < 13 ? 3 : i < 17 ? 4 : i < 29 ? 5 : i < 32 ? 6 : 7;
}
__host__ __device__ __forceinline__ constexpr int approx_joint(int i) { return i < 7 ? i : 7; }
__host__ __device__ __forceinline__ constexpr int det_first(int j) {
    return j == 0 ? 0 : j == 1 ? 1 : j == 2 ? 5 : j == 3 ? 9 : j == 4 ? 13 : j == 5 ? 17 : j == 6 ? 29 : j == 7 ? 32 : 59;
}
__host__ __device__ __forceinline__ constexpr int det_count(int j) {
    return j == 0 ? 1 : j < 5 ? 4 : j == 5 ? 12 : j == 6 ? 3 : 27;
}

// Detailed self-check rows (panda_multi_geometry.cuh:446-472): row r tests
// sphere first(r) against spheres lo(r)..hi(r) of the same arm.
__host__ __device__ __forceinline__ constexpr int det_row_first(int r) {
    return r < 5 ? r : r < 13 ? 5 + ((r - 5) >> 1) : r + 4;
}
__host__ __device__ __forceinline__ constexpr int det_row_lo(int r) {
    return r < 5 ? 17 : (r < 13 && ((r - 5) & 1) == 0) ? 17 : 32;
}
__host__ __device__ __forceinline__ constexpr int det_row_hi(int r) {
    return r < 5 ? 58 : (r < 13 && ((r - 5) & 1) == 0) ? 28 : 58;
}
constexpr int kDetRows = 25;

// Forearm-hand rows.  The rows whose first-read sphere sits on joint 5
// (positions 17..28: rows 13..24 by sphere index, rows 17..24 in the
// composite robots' reading) test it against the hand spheres 32..58 of
// joint 7.  Their distances depend only on q6 and q7 (the frames between are
// F6 Rz(q6) F7 Rz(q7)), and the Panda's approx spheres 5 and 7/8 overlap in
// every configuration, so these rows are flagged in every sample.  A table
// over (q6, q7) cells, built on the host in double precision, marks the cells
// where every such pair is apart by more than kRow5Margin for every
// configuration in the cell (distance at the cell centre minus the largest
// displacement a hand sphere can make inside the cell, with the larger of the
// two radii a row can read).  For a sample in a marked cell those rows cannot
// fire (the FP32 evaluation errs by ~1e-5 m at most), so they are skipped;
// samples outside the table's range are tested as usual.
constexpr int kRow5N6 = 256, kRow5N7 = 384;
constexpr int kRow5Words = kRow5N6 * kRow5N7 / 32;
constexpr float kRow5Lo6 = -0.0873f, kRow5Hi6 = 3.8223f;  // joint 6 limits (Robots.hh:13-23)
constexpr float kRow5Lo7 = -2.9671f, kRow5Hi7 = 2.9671f;  // joint 7 limits
constexpr double kRow5Margin = 2e-4;
// rows covered, by reading: [0] sphere index (single arm, EXACT), [1] composite
__host__ __device__ __forceinline__ constexpr uint32_t row5_rows(int quirk) {
    return quirk ? 0x01FE0000u /* rows 17..24 */ : 0x01FFE000u /* rows 13..24 */;
}

// ---------------------------------------------------------------------------
// exact-order arithmetic helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pair_fma(float a, float b, float c, float d) {
#if MRPOP_PAIR_ORDER == 0
    return __fmaf_rn(a, b, __fmul_rn(c, d));
#else
    return __fmaf_rn(c, d, __fmul_rn(a, b));
#endif
}

// 3x4 rigid transform, row-major: m[r*4 + c].
struct Xf {
    float m[12];
};

__device__ __forceinline__ void load_base(Xf &T, const float *base12) {
#pragma unroll
    for (int i = 0; i < 12; i++) T.m[i] = base12[i];
}

// T <- T * (F_J * Rz(q)) for Panda joint J (1..7).  F_J rows are
// panda_multi_geometry.cuh:255-295.  See the header comment for why these
// short forms equal the reference's dense chains bit for bit.
template <int J>
__device__ __forceinline__ void joint_step(Xf &T, float q) {
    const float c = __cosf(q);
    const float s = __sinf(q);
    const float ns = -s;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const float t0 = T.m[r * 4 + 0], t1 = T.m[r * 4 + 1], t2 = T.m[r * 4 + 2],
                    t3 = T.m[r * 4 + 3];
        float n0, n1, n2, n3;
        if constexpr (J == 1) {  // F = I, translation z 0.333
            n0 = pair_fma(t0, c, t1, s);
            n1 = pair_fma(t0, ns, t1, c);
            n2 = t2;
            n3 = __fadd_rn(t3, __fmul_rn(t2, 0.333f));
        } else if constexpr (J == 2 || J == 5) {  // rows e0, e2, -e1
            n0 = __fmaf_rn(t2, ns, __fmul_rn(t0, c));
            n1 = __fmaf_rn(t2, -c, __fmul_rn(t0, ns));
            n2 = t1;
            if constexpr (J == 2) n3 = t3;
            else n3 = __fadd_rn(t3, pair_fma(t0, -0.0825f, t1, 0.384f));
        } else {  // J = 3, 4, 6, 7: rows e0, -e2, e1
            n0 = __fmaf_rn(t2, s, __fmul_rn(t0, c));
            n1 = __fmaf_rn(t2, c, __fmul_rn(t0, ns));
            n2 = -t1;
            if constexpr (J == 3) n3 = __fadd_rn(t3, __fmul_rn(t1, -0.316f));
            else if constexpr (J == 4) n3 = __fadd_rn(t3, __fmul_rn(t0, 0.0825f));
            else if constexpr (J == 6) n3 = t3;
            else n3 = __fadd_rn(t3, __fmul_rn(t0, 0.088f));
        }
        T.m[r * 4 + 0] = n0;
        T.m[r * 4 + 1] = n1;
        T.m[r * 4 + 2] = n2;
        T.m[r * 4 + 3] = n3;
    }
}

// Joints 2..7 share one form: rows of F_J are e0, A*e2, -A*e1 (A = +-1) with
// translation (tx, ty, 0).  The reference's chains then reduce to
//   n0 = fma(t2, A*s, t0*c), n1 = fma(t2, A*c, t0*(-s)), n2 = -A*t1,
//   n3 = t3 + (t0*tx + t1*ty)
// where a zero translation term contributes an exact signed zero, exactly as
// the reference's zero products do.  {A, tx, ty} per joint 2..7:
static __constant__ float c_joint_k[6][3] = {{-1.f, 0.f, 0.f},      {1.f, 0.f, -0.316f}, {1.f, 0.0825f, 0.f},
                                             {-1.f, -0.0825f, 0.384f}, {1.f, 0.f, 0.f},     {1.f, 0.088f, 0.f}};

__device__ __forceinline__ void joint_step_rt(Xf &T, float q, int j) {
    if (j == 1) {
        joint_step<1>(T, q);
        return;
    }
    const float A = c_joint_k[j - 2][0], tx = c_joint_k[j - 2][1], ty = c_joint_k[j - 2][2];
    const float c = __cosf(q);
    const float s = __sinf(q);
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const float t0 = T.m[r * 4 + 0], t1 = T.m[r * 4 + 1], t2 = T.m[r * 4 + 2], t3 = T.m[r * 4 + 3];
        T.m[r * 4 + 0] = __fmaf_rn(t2, A * s, __fmul_rn(t0, c));
        T.m[r * 4 + 1] = __fmaf_rn(t2, A * c, __fmul_rn(t0, -s));
        T.m[r * 4 + 2] = -A * t1;
        T.m[r * 4 + 3] = __fadd_rn(t3, pair_fma(t0, tx, t1, ty));
    }
}

// One coordinate of a sphere centre, T(c,0)x + T(c,1)y + T(c,2)z + T(c,3)
// (panda_four.cuh:117-125) with compile-time offsets: structural zero terms
// are dropped (they only add signed zeros in the reference's chain).
template <int I, bool DET>
__device__ __forceinline__ float place_coord(const Xf &T, int c) {
    constexpr SphereDef s = DET ? kDet[I] : kApprox[I];
    const float t0 = T.m[c * 4 + 0], t1 = T.m[c * 4 + 1], t2 = T.m[c * 4 + 2], t3 = T.m[c * 4 + 3];
    float acc = 0.0f;
    if constexpr (s.x != 0.0f && s.y != 0.0f) acc = pair_fma(t0, s.x, t1, s.y);
    else if constexpr (s.x != 0.0f) acc = __fmul_rn(t0, s.x);
    else if constexpr (s.y != 0.0f) acc = __fmul_rn(t1, s.y);
    if constexpr (s.z != 0.0f) {
        if constexpr (s.x != 0.0f || s.y != 0.0f) acc = __fmaf_rn(t2, s.z, acc);
        else acc = __fmul_rn(t2, s.z);
    }
    if constexpr (s.x == 0.0f && s.y == 0.0f && s.z == 0.0f) return t3;
    else return __fadd_rn(acc, t3);
}

// Same with run-time offsets: the reference's full expression (zeros included).
__device__ __forceinline__ float3 place_rt(const float *T12, float4 s) {
    float3 p;
    p.x = __fadd_rn(__fmaf_rn(T12[2], s.z, pair_fma(T12[0], s.x, T12[1], s.y)), T12[3]);
    p.y = __fadd_rn(__fmaf_rn(T12[6], s.z, pair_fma(T12[4], s.x, T12[5], s.y)), T12[7]);
    p.z = __fadd_rn(__fmaf_rn(T12[10], s.z, pair_fma(T12[8], s.x, T12[9], s.y)), T12[11]);
    return p;
}

// ---------------------------------------------------------------------------
// collision primitives (utils.cuh:100-228).  Each returns true when the
// reference's "< 0" test fires.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sql2(float xs, float ys, float zs) {
    return __fmaf_rn(zs, zs, pair_fma(xs, xs, ys, ys));
}

// sphere_sphere_sql2 (:100-107): |a-b|^2 - (ra+rb)^2 < 0
__device__ __forceinline__ bool hit_sphere_sphere(float ax, float ay, float az, float ar, float bx,
                                                  float by, float bz, float br) {
    const float s = sql2(__fsub_rn(ax, bx), __fsub_rn(ay, by), __fsub_rn(az, bz));
    const float rs = __fadd_rn(ar, br);
    return __fmaf_rn(-rs, rs, s) < 0.0f;
}

// sphere_capsule (:148-158).  c0 = {x1,y1,z1,r}, c1 = {xv,yv,zv,rdv}
__device__ __forceinline__ bool hit_capsule(float4 c0, float4 c1, float x, float y, float z,
                                            float r) {
    const float dot =
        __fmaf_rn(__fsub_rn(z, c0.z), c1.z, pair_fma(__fsub_rn(x, c0.x), c1.x, __fsub_rn(y, c0.y), c1.y));
    const float cdf = fmaxf(fminf(__fmul_rn(dot, c1.w), 1.0f), 0.0f);
    const float s = sql2(__fsub_rn(x, __fmaf_rn(c1.x, cdf, c0.x)), __fsub_rn(y, __fmaf_rn(c1.y, cdf, c0.y)),
                         __fsub_rn(z, __fmaf_rn(c1.z, cdf, c0.z)));
    const float rs = __fadd_rn(r, c0.w);
    return __fmaf_rn(-rs, rs, s) < 0.0f;
}

// sphere_z_aligned_capsule (:165-174)
__device__ __forceinline__ bool hit_zcapsule(float4 c0, float4 c1, float x, float y, float z,
                                             float r) {
    const float dot = __fmul_rn(__fsub_rn(z, c0.z), c1.z);
    const float cdf = fmaxf(fminf(__fmul_rn(dot, c1.w), 1.0f), 0.0f);
    const float s = sql2(__fsub_rn(x, c0.x), __fsub_rn(y, c0.y), __fsub_rn(z, __fmaf_rn(c1.z, cdf, c0.z)));
    const float rs = __fadd_rn(r, c0.w);
    return __fmaf_rn(-rs, rs, s) < 0.0f;
}

// sphere_cuboid (:185-201).  c0 = {cx,cy,cz,h1}, c1 = {a1,h2}, c2 = {a2,h3}, c3 = {a3,-}
__device__ __forceinline__ bool hit_cuboid(float4 c0, float4 c1, float4 c2, float4 c3, float x,
                                           float y, float z, float rsq) {
    const float xs = __fsub_rn(x, c0.x), ys = __fsub_rn(y, c0.y), zs = __fsub_rn(z, c0.z);
    const float d1 = __fmaf_rn(c1.z, zs, pair_fma(c1.x, xs, c1.y, ys));
    const float d2 = __fmaf_rn(c2.z, zs, pair_fma(c2.x, xs, c2.y, ys));
    const float d3 = __fmaf_rn(c3.z, zs, pair_fma(c3.x, xs, c3.y, ys));
    const float a1 = fmaxf(0.0f, __fsub_rn(fabsf(d1), c0.w));
    const float a2 = fmaxf(0.0f, __fsub_rn(fabsf(d2), c1.w));
    const float a3 = fmaxf(0.0f, __fsub_rn(fabsf(d3), c2.w));
    return __fsub_rn(sql2(a1, a2, a3), rsq) < 0.0f;
}

// sphere_z_aligned_cuboid (:208-221)
__device__ __forceinline__ bool hit_zcuboid(float4 c0, float4 c1, float4 c2, float x, float y,
                                            float z, float rsq) {
    const float xs = __fsub_rn(x, c0.x), ys = __fsub_rn(y, c0.y), zs = __fsub_rn(z, c0.z);
    const float a1 = fmaxf(0.0f, __fsub_rn(fabsf(pair_fma(c1.x, xs, c1.y, ys)), c0.w));
    const float a2 = fmaxf(0.0f, __fsub_rn(fabsf(pair_fma(c2.x, xs, c2.y, ys)), c1.w));
    const float a3 = fmaxf(0.0f, __fsub_rn(fabsf(zs), c2.w));
    return __fsub_rn(sql2(a1, a2, a3), rsq) < 0.0f;
}

}  // namespace mrpop
