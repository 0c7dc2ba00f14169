/*
 * edge_oracle.c -- CPU restatement of MR.POP's batched edge validation.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library under
 * mr.pop_gb300/) links, loads or calls this file; only tests/, the smoke check
 * and bench.py's CPU-baseline leg use it, and only as the checker.
 *
 * Parity pinning: the reference ships no tests and no golden vectors.  This
 * restatement is pinned against outputs of the reference's own device code
 * (its fkcc_single_buffer* routines compiled from the reference sources into a
 * cubin, see oracle/ref_harness.cu) run on a GB300; the captured outputs are
 * committed under tests/golden/ together with the script that made them.
 *
 * What it restates (file:line in the reference project):
 *   - edge interpolation at the call sites: pop_planner.cu:551-561 (extend),
 *     pop_planner.cu:666-703 (connect, n_extensions segments),
 *     roadmap_interior.cuh:219-234 (roadmap), path_simplification.cu:85-129
 *     (B-spline) and :155-200 (shortcut);
 *   - the block-collective edge checks fkcc_single_buffer (utils.cuh:447-534),
 *     fkcc_single_buffer_mr (utils.cuh:536-624) and fkcc_single_buffer_drrt
 *     (utils.cuh:626-686), including the proportional thread split
 *     (utils.cuh:476-517) that decides which samples get a detailed check;
 *   - the Panda FK (panda_four.cuh:44-131 / 289-373, panda.cuh:598-669 /
 *     761-829) with the joint-step builders of utils.cuh:400-445;
 *   - the approx and detailed env/self checks (panda_four.cuh:133-276 /
 *     375-489, panda.cuh:672-748 / 832-888) and the primitives of
 *     utils.cuh:100-260.
 *
 * Arithmetic: FP32, with every multiply-add that nvcc contracts into an FMA in
 * the reference written as an explicit fmaf() (build with -ffp-contract=off so
 * the C compiler adds no fusion of its own).  For a sum of two products
 * a*b + c*d the reference's compiled code fuses one of the two products; which
 * one is the `pair_order` argument (0: fmaf(a,b,c*d), 1: fmaf(c,d,a*b)).
 * sin/cos: the reference calls the __sinf/__cosf hardware approximations.  The
 * oracle either uses (float)sin((double)x) or a table of device-produced
 * values handed in by the caller (trig lookup), which makes the restatement
 * bit-exact against device code.
 *
 * FP64 "truth": sphere centres and true signed distances in double precision,
 * used to (1) check device sphere centres to 1e-5 m and (2) mark an edge
 * ambiguous when a minimum signed distance that decides one of its flags or
 * detailed verdicts lies within `band` metres of zero.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Panda geometry, restated from panda_multi_geometry.cuh:17-516 (identical  */
/* to panda.cuh:97-595).  Layout here: one row per sphere {x, y, z, r}.      */
/* ------------------------------------------------------------------------ */
static const float OR_APPROX_SPH[11][4] = {
    {0.0f, 0.0f, 0.05f, 0.08f},          {-0.001f, -0.039f, -0.085f, 0.154f},
    {0.0f, -0.085f, 0.04f, 0.154f},      {0.039f, 0.028f, -0.052f, 0.128f},
    {-0.042f, 0.049f, 0.029f, 0.126f},   {-0.001f, 0.037f, -0.11f, 0.176f},
    {0.042f, 0.014f, 0.0f, 0.095f},      {0.015f, 0.015f, 0.075f, 0.072f},
    {0.0f, 0.0f, 0.129f, 0.104f},        {0.054447f, 0.054447f, 0.1984f, 0.024f},
    {-0.054447f, -0.054447f, 0.1984f, 0.024f}};
static const int OR_APPROX_S2J[11] = {0, 1, 2, 3, 4, 5, 6, 7, 7, 7, 7};
static const int OR_APPROX_JCOUNT[8] = {1, 1, 1, 1, 1, 1, 1, 4};
static const int OR_APPROX_RANGES[5][3] = {{0, 5, 10}, {1, 5, 10}, {2, 5, 5}, {2, 7, 10}, {5, 7, 10}};

static const float OR_DET_SPH[59][4] = {
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
static const int OR_DET_JCOUNT[8] = {1, 4, 4, 4, 4, 12, 3, 27};
static const int OR_DET_RANGES[25][3] = {
    {0, 17, 58}, {1, 17, 58}, {2, 17, 58}, {3, 17, 58}, {4, 17, 58}, {5, 17, 28}, {5, 32, 58},
    {6, 17, 28}, {6, 32, 58}, {7, 17, 28}, {7, 32, 58}, {8, 17, 28}, {8, 32, 58}, {17, 32, 58},
    {18, 32, 58}, {19, 32, 58}, {20, 32, 58}, {21, 32, 58}, {22, 32, 58}, {23, 32, 58},
    {24, 32, 58}, {25, 32, 58}, {26, 32, 58}, {27, 32, 58}, {28, 32, 58}};

/* Fixed joint transforms, row-major 4x4 (joint 0 is the base placeholder).  */
static const float OR_FIXED[8][16] = {
    {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1},
    {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0.333f, 0, 0, 0, 1},
    {1, 0, 0, 0, 0, 0, 1, 0, 0, -1, 0, 0, 0, 0, 0, 1},
    {1, 0, 0, 0, 0, 0, -1, -0.316f, 0, 1, 0, 0, 0, 0, 0, 1},
    {1, 0, 0, 0.0825f, 0, 0, -1, 0, 0, 1, 0, 0, 0, 0, 0, 1},
    {1, 0, 0, -0.0825f, 0, 0, 1, 0.384f, 0, -1, 0, 0, 0, 0, 0, 1},
    {1, 0, 0, 0, 0, 0, -1, 0, 0, 1, 0, 0, 0, 0, 0, 1},
    {1, 0, 0, 0.088f, 0, 0, -1, 0, 0, 1, 0, 0, 0, 0, 0, 1}};

#define OR_MAX_ARMS 5
#define OR_NA 11
#define OR_ND 59
#define OR_MAX_G 64

#define OR_ENV 1
#define OR_SELF 2
#define OR_EXACT 16

static int OR_DET_S2J[59];
static void or_init_tables(void) {
    int s = 0;
    for (int j = 0; j < 8; j++)
        for (int c = 0; c < OR_DET_JCOUNT[j]; c++) OR_DET_S2J[s++] = j;
}

/* ------------------------------------------------------------------------ */
/* Inputs                                                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    const float *spheres;   int32_t n_spheres;   /* {x,y,z,r}                      */
    const float *capsules;  int32_t n_capsules;  /* {x1,y1,z1,xv,yv,zv,r,rdv}      */
    const float *zcapsules; int32_t n_zcapsules; /* same record, z-aligned         */
    const float *cuboids;   int32_t n_cuboids;   /* {x,y,z,a1(3),a2(3),a3(3),h1,h2,h3} */
    const float *zcuboids;  int32_t n_zcuboids;  /* same record, z-aligned         */
} orc_scene;

typedef struct {
    int32_t n_arms;
    float base[OR_MAX_ARMS][16]; /* row-major 4x4 per arm */
} orc_robots;

typedef struct {            /* optional device trig values keyed by input bits */
    const uint32_t *keys;   /* sorted ascending */
    const float *cosv;
    const float *sinv;
    int64_t n;
} orc_trig;

static const orc_trig *g_trig = NULL; /* set per call, read-only during it */
static int g_trig_miss = 0;

static void or_sincos(float x, float *c, float *s) {
    if (g_trig) {
        uint32_t key;
        memcpy(&key, &x, 4);
        int64_t lo = 0, hi = g_trig->n - 1;
        while (lo <= hi) {
            int64_t mid = (lo + hi) >> 1;
            uint32_t k = g_trig->keys[mid];
            if (k == key) {
                *c = g_trig->cosv[mid];
                *s = g_trig->sinv[mid];
                return;
            }
            if (k < key) lo = mid + 1; else hi = mid - 1;
        }
#pragma omp atomic write
        g_trig_miss = 1;
    }
    *c = (float)cos((double)x);
    *s = (float)sin((double)x);
}

/* a*b + c*d with one product fused, as the reference's compiled code does. */
static inline float or_pair(int order, float a, float b, float c, float d) {
    return order == 0 ? fmaf(a, b, c * d) : fmaf(c, d, a * b);
}

/* ------------------------------------------------------------------------ */
/* FP32 FK mirror (dense form of utils.cuh:400-445 + panda_four.cuh:74-128)  */
/* T is 4x4 stored like the reference: column-major, T[c*4 + r] = T(r,c).    */
/* ------------------------------------------------------------------------ */
static void or_zrot_step(const float *F, float angle, float S[16], int po) {
    /* utils.cuh:400-427: column c of F * Rz(angle), built branch-free. */
    float cs, sn;
    or_sincos(angle, &cs, &sn);
    float n_sin = -1.0f * sn;
    for (int col = 0; col < 4; col++) {
        int by2 = col / 2, per2 = col % 2;
        float f1 = or_pair(po, (float)(1 - per2), cs, (float)per2, n_sin);
        float f2 = or_pair(po, (float)(1 - per2), sn, (float)per2, cs);
        f1 = fmaf((float)by2, 1.0f, (float)(1 - by2) * f1); /* exact: 0/1 factors */
        f2 = (float)(1 - by2) * f2;
        int off = by2 * col;
        for (int r = 0; r < 3; r++) S[col * 4 + r] = or_pair(po, F[4 * r + off], f1, f2, F[4 * r + 1]);
        S[col * 4 + 3] = F[12 + off] * (float)by2;
    }
}

static inline float or_dot4_col(const float *Tp, int r, const float *s, int po) {
    /* dot4_col (utils.cuh:443-445): T(r,0)s0 + T(r,1)s1 + T(r,2)s2 + T(r,3)s3 */
    float acc = or_pair(po, Tp[0 * 4 + r], s[0], Tp[1 * 4 + r], s[1]);
    acc = fmaf(Tp[2 * 4 + r], s[2], acc);
    return fmaf(Tp[3 * 4 + r], s[3], acc);
}

static void or_compose(float T[16], const float S[16], int po) {
    float N[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) N[c * 4 + r] = or_dot4_col(T, r, &S[c * 4], po);
    memcpy(T, N, sizeof(N));
}

static inline void or_place(const float T[16], const float *sp, float out[3], int po) {
    for (int c = 0; c < 3; c++) {
        float acc = or_pair(po, T[0 * 4 + c], sp[0], T[1 * 4 + c], sp[1]);
        acc = fmaf(T[2 * 4 + c], sp[2], acc);
        out[c] = acc + T[3 * 4 + c];
    }
}

/* FK of one arm.  `base` row-major 4x4.  Writes approx (11) and/or detailed
 * (59) centres.  The base enters as I * base through the same dot4 chain the
 * composite robots use (panda_four.cuh:81-86), which is exact. */
static void or_fk_arm(const float *base, const float *q7, float apos[OR_NA][3],
                      float dpos[OR_ND][3], int po) {
    float T[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) T[c * 4 + r] = (r == c) ? 1.0f : 0.0f;
    float S[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) S[c * 4 + r] = base[4 * r + c];
    or_compose(T, S, po);
    int ai = 0, di = 0;
    for (int j = 0; j < 8; j++) {
        if (j > 0) {
            or_zrot_step(OR_FIXED[j], q7[j - 1], S, po);
            or_compose(T, S, po);
        }
        if (apos)
            for (int s = 0; s < OR_APPROX_JCOUNT[j]; s++, ai++) or_place(T, OR_APPROX_SPH[ai], apos[ai], po);
        if (dpos)
            for (int s = 0; s < OR_DET_JCOUNT[j]; s++, di++) or_place(T, OR_DET_SPH[di], dpos[di], po);
    }
}

/* FP64 FK (exact sin/cos, double arithmetic). */
static void or_fk_arm64(const float *base, const float *q7, double apos[OR_NA][3],
                        double dpos[OR_ND][3]) {
    double T[3][4];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) T[r][c] = base[4 * r + c];
    int ai = 0, di = 0;
    for (int j = 0; j < 8; j++) {
        if (j > 0) {
            const float *F = OR_FIXED[j];
            double th = (double)q7[j - 1], cs = cos(th), sn = sin(th);
            double S[3][4]; /* F * Rz */
            for (int r = 0; r < 3; r++) {
                S[r][0] = F[4 * r + 0] * cs + F[4 * r + 1] * sn;
                S[r][1] = -F[4 * r + 0] * sn + F[4 * r + 1] * cs;
                S[r][2] = F[4 * r + 2];
                S[r][3] = F[4 * r + 3];
            }
            double N[3][4];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 4; c++) {
                    double v = T[r][0] * S[0][c] + T[r][1] * S[1][c] + T[r][2] * S[2][c];
                    if (c == 3) v += T[r][3];
                    N[r][c] = v;
                }
            memcpy(T, N, sizeof(T));
        }
        for (int s = 0; s < OR_APPROX_JCOUNT[j]; s++, ai++)
            for (int c = 0; c < 3; c++)
                apos[ai][c] = T[c][0] * OR_APPROX_SPH[ai][0] + T[c][1] * OR_APPROX_SPH[ai][1] +
                              T[c][2] * OR_APPROX_SPH[ai][2] + T[c][3];
        for (int s = 0; s < OR_DET_JCOUNT[j]; s++, di++)
            for (int c = 0; c < 3; c++)
                dpos[di][c] = T[c][0] * OR_DET_SPH[di][0] + T[c][1] * OR_DET_SPH[di][1] +
                              T[c][2] * OR_DET_SPH[di][2] + T[c][3];
    }
}

/* ------------------------------------------------------------------------ */
/* FP32 primitives (utils.cuh:100-228) and the scene loop (utils.cuh:231-260) */
/* ------------------------------------------------------------------------ */
static inline float or_sql2(float xs, float ys, float zs, int po) {
    return fmaf(zs, zs, or_pair(po, xs, xs, ys, ys));
}

static inline int or_sphere_sphere(const float *a, float ar, const float *b, float br, int po) {
    float s = or_sql2(a[0] - b[0], a[1] - b[1], a[2] - b[2], po);
    float rs = ar + br;
    return fmaf(-rs, rs, s) < 0.0f;
}

static inline float or_clamp01(float v) { return fmaxf(fminf(v, 1.0f), 0.0f); }

static int or_env_hit(const orc_scene *sc, const float *p, float r, int po) {
    const float x = p[0], y = p[1], z = p[2];
    const float rsq = r * r;
    for (int i = 0; i < sc->n_spheres; i++) {
        const float *o = sc->spheres + 4 * i;
        float s = or_sql2(o[0] - x, o[1] - y, o[2] - z, po);
        float rs = o[3] + r;
        if (fmaf(-rs, rs, s) < 0.0f) return 1;
    }
    for (int i = 0; i < sc->n_capsules; i++) {
        const float *c = sc->capsules + 8 * i;
        float dot = fmaf(z - c[2], c[5], or_pair(po, x - c[0], c[3], y - c[1], c[4]));
        float cdf = or_clamp01(dot * c[7]);
        float s = or_sql2(x - fmaf(c[3], cdf, c[0]), y - fmaf(c[4], cdf, c[1]),
                          z - fmaf(c[5], cdf, c[2]), po);
        float rs = r + c[6];
        if (fmaf(-rs, rs, s) < 0.0f) return 1;
    }
    for (int i = 0; i < sc->n_zcapsules; i++) {
        const float *c = sc->zcapsules + 8 * i;
        float dot = (z - c[2]) * c[5];
        float cdf = or_clamp01(dot * c[7]);
        float s = or_sql2(x - c[0], y - c[1], z - fmaf(c[5], cdf, c[2]), po);
        float rs = r + c[6];
        if (fmaf(-rs, rs, s) < 0.0f) return 1;
    }
    for (int i = 0; i < sc->n_cuboids; i++) {
        const float *c = sc->cuboids + 15 * i;
        float xs = x - c[0], ys = y - c[1], zs = z - c[2];
        float d1 = fmaf(c[5], zs, or_pair(po, c[3], xs, c[4], ys));
        float d2 = fmaf(c[8], zs, or_pair(po, c[6], xs, c[7], ys));
        float d3 = fmaf(c[11], zs, or_pair(po, c[9], xs, c[10], ys));
        float a1 = fmaxf(0.0f, fabsf(d1) - c[12]);
        float a2 = fmaxf(0.0f, fabsf(d2) - c[13]);
        float a3 = fmaxf(0.0f, fabsf(d3) - c[14]);
        if (or_sql2(a1, a2, a3, po) - rsq < 0.0f) return 1;
    }
    for (int i = 0; i < sc->n_zcuboids; i++) {
        const float *c = sc->zcuboids + 15 * i;
        float xs = x - c[0], ys = y - c[1], zs = z - c[2];
        float a1 = fmaxf(0.0f, fabsf(or_pair(po, c[3], xs, c[4], ys)) - c[12]);
        float a2 = fmaxf(0.0f, fabsf(or_pair(po, c[6], xs, c[7], ys)) - c[13]);
        float a3 = fmaxf(0.0f, fabsf(zs) - c[14]);
        if (or_sql2(a1, a2, a3, po) - rsq < 0.0f) return 1;
    }
    return 0;
}

/* FP64 signed distance of a sphere to the scene's closest obstacle surface
 * (same geometry as the FP32 formulas; returns the minimum). */
static double or_env_sd64(const orc_scene *sc, const double *p, double r) {
    double best = 1e30;
    for (int i = 0; i < sc->n_spheres; i++) {
        const float *o = sc->spheres + 4 * i;
        double dx = p[0] - o[0], dy = p[1] - o[1], dz = p[2] - o[2];
        double d = sqrt(dx * dx + dy * dy + dz * dz) - (o[3] + r);
        if (d < best) best = d;
    }
    for (int k = 0; k < 2; k++) {
        int n = k ? sc->n_zcapsules : sc->n_capsules;
        const float *arr = k ? sc->zcapsules : sc->capsules;
        for (int i = 0; i < n; i++) {
            const float *c = arr + 8 * i;
            double vx = k ? 0.0 : c[3], vy = k ? 0.0 : c[4], vz = c[5];
            double dot = (p[0] - c[0]) * vx + (p[1] - c[1]) * vy + (p[2] - c[2]) * vz;
            double vv = vx * vx + vy * vy + vz * vz;
            double t = vv > 0 ? dot / vv : 0.0;
            t = t < 0 ? 0 : (t > 1 ? 1 : t);
            double dx = p[0] - (c[0] + vx * t), dy = p[1] - (c[1] + vy * t), dz = p[2] - (c[2] + vz * t);
            double d = sqrt(dx * dx + dy * dy + dz * dz) - (r + c[6]);
            if (d < best) best = d;
        }
    }
    for (int i = 0; i < sc->n_cuboids; i++) {
        const float *c = sc->cuboids + 15 * i;
        double xs = p[0] - c[0], ys = p[1] - c[1], zs = p[2] - c[2], s = 0;
        for (int a = 0; a < 3; a++) {
            double d = fabs(c[3 + 3 * a] * xs + c[4 + 3 * a] * ys + c[5 + 3 * a] * zs) - c[12 + a];
            if (d > 0) s += d * d;
        }
        double d = sqrt(s) - r;
        if (d < best) best = d;
    }
    for (int i = 0; i < sc->n_zcuboids; i++) {
        const float *c = sc->zcuboids + 15 * i;
        double xs = p[0] - c[0], ys = p[1] - c[1], zs = p[2] - c[2], s = 0, d;
        d = fabs(c[3] * xs + c[4] * ys) - c[12]; if (d > 0) s += d * d;
        d = fabs(c[6] * xs + c[7] * ys) - c[13]; if (d > 0) s += d * d;
        d = fabs(zs) - c[14]; if (d > 0) s += d * d;
        d = sqrt(s) - r;
        if (d < best) best = d;
    }
    return best;
}

static inline double or_ss_sd64(const double *a, double ar, const double *b, double br) {
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz) - (ar + br);
}

/* ------------------------------------------------------------------------ */
/* Per-sample broad phase and per-edge decision                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    float q[OR_MAX_ARMS * 7];
    float apos[OR_MAX_ARMS][OR_NA][3];
    uint8_t envf[OR_MAX_ARMS];  /* bit j: joint j needs a detailed env check  */
    uint8_t selff[OR_MAX_ARMS]; /* bit j: joint j needs a detailed self check */
    int env_cnt, self_cnt;
} or_sample;

typedef struct {
    const orc_scene *sc;
    const orc_robots *rb;
    int n_arms;  /* arms in this check */
    int arm;     /* -1: composite; >= 0 single arm (fkcc_single_buffer_mr) */
    int flags;
    int po;
    double band;
} or_ctx;

static inline const float *or_base(const or_ctx *cx, int a) {
    return cx->rb->base[cx->arm >= 0 ? cx->arm : a];
}

static void or_broad(const or_ctx *cx, or_sample *sm) {
    const int A = cx->n_arms;
    for (int a = 0; a < A; a++) {
        or_fk_arm(or_base(cx, a), sm->q + 7 * a, sm->apos[a], NULL, cx->po);
        sm->envf[a] = 0;
        sm->selff[a] = 0;
    }
    if (cx->flags & OR_ENV) /* env_collision_check_approx: spheres 1..10 */
        for (int a = 0; a < A; a++)
            for (int i = 1; i < OR_NA; i++)
                if (or_env_hit(cx->sc, sm->apos[a][i], OR_APPROX_SPH[i][3], cx->po))
                    sm->envf[a] |= (uint8_t)(1u << OR_APPROX_S2J[i]);
    if (cx->flags & OR_SELF) {
        for (int a = 0; a < A; a++) {
            for (int i = 0; i < 5; i++) { /* intra-arm approx ranges */
                int s1 = OR_APPROX_RANGES[i][0];
                for (int j = OR_APPROX_RANGES[i][1]; j <= OR_APPROX_RANGES[i][2]; j++)
                    if (or_sphere_sphere(sm->apos[a][s1], OR_APPROX_SPH[s1][3], sm->apos[a][j],
                                         OR_APPROX_SPH[j][3], cx->po))
                        sm->selff[a] |= (uint8_t)(1u << OR_APPROX_S2J[s1]);
            }
            for (int i = 0; i < OR_NA; i++) /* cross-arm: flags the lower arm */
                for (int b = a + 1; b < A; b++)
                    for (int j = 0; j < OR_NA; j++)
                        if (or_sphere_sphere(sm->apos[a][i], OR_APPROX_SPH[i][3], sm->apos[b][j],
                                             OR_APPROX_SPH[j][3], cx->po))
                            sm->selff[a] |= (uint8_t)(1u << OR_APPROX_S2J[i]);
        }
    }
    sm->env_cnt = sm->self_cnt = 0;
    for (int a = 0; a < A; a++)
        for (int j = 0; j < 8; j++) {
            if (sm->envf[a] >> j & 1) sm->env_cnt += OR_DET_JCOUNT[j];
            if (sm->selff[a] >> j & 1) sm->self_cnt += OR_DET_JCOUNT[j];
        }
}

/* utils.cuh:477-498: proportional split of 4g threads over the samples. */
static void or_thread_dist(const int *cnt, int g, int *dist) {
    const int total_threads = 4 * g;
    int total = 0;
    for (int i = 0; i < g; i++) total += cnt[i];
    int used = 0;
    for (int i = 0; i < g; i++) {
        if (total == 0) {
            dist[i] = 0; /* 0/0 is NaN on the device; its int conversion gives 0 */
        } else {
            float f = ((float)cnt[i] / (float)total) * (float)total_threads;
            dist[i] = (int)f;
        }
        used += dist[i];
    }
    dist[g - 1] += total_threads - used;
}

static int or_narrow_env(const or_ctx *cx, const or_sample *sm, float dpos[][OR_ND][3]) {
    for (int a = 0; a < cx->n_arms; a++) {
        if (!sm->envf[a]) continue;
        for (int i = 1; i < OR_ND; i++)
            if ((sm->envf[a] >> OR_DET_S2J[i] & 1) &&
                or_env_hit(cx->sc, dpos[a][i], OR_DET_SPH[i][3], cx->po))
                return 1;
    }
    return 0;
}

static int or_narrow_self(const or_ctx *cx, const or_sample *sm, float dpos[][OR_ND][3]) {
    const int A = cx->n_arms;
    /* quirk: the composite robots read position and joint flag of sphere `i`
     * (the range index) but the radius of sphere ranges[i][0]
     * (panda_four.cuh:388-413); the single-arm robot does not (panda.cuh:841-859). */
    const int quirk = (cx->arm < 0) && !(cx->flags & OR_EXACT);
    for (int a = 0; a < A; a++) {
        if (!sm->selff[a]) continue;
        for (int i = 0; i < 25; i++) {
            int s1 = OR_DET_RANGES[i][0];
            int idx = quirk ? i : s1;
            if (!(sm->selff[a] >> OR_DET_S2J[idx] & 1)) continue;
            for (int j = OR_DET_RANGES[i][1]; j <= OR_DET_RANGES[i][2]; j++)
                if (or_sphere_sphere(dpos[a][idx], OR_DET_SPH[s1][3], dpos[a][j], OR_DET_SPH[j][3], cx->po))
                    return 1;
        }
        for (int i = 0; i < OR_ND; i++) {
            if (!(sm->selff[a] >> OR_DET_S2J[i] & 1)) continue;
            for (int b = a + 1; b < A; b++)
                for (int j = 0; j < OR_ND; j++)
                    if (or_sphere_sphere(dpos[a][i], OR_DET_SPH[i][3], dpos[b][j], OR_DET_SPH[j][3], cx->po))
                        return 1;
        }
    }
    return 0;
}

/* Algorithmic flop tally (FMA = 2), per the convention:
 * sphere placement 18, revolute compose 81, sphere-sphere 11, sphere-OBB 27,
 * sphere-capsule 26. */
static double or_env_test_flops(const orc_scene *sc) {
    return 27.0 * (sc->n_cuboids + sc->n_zcuboids) + 26.0 * (sc->n_capsules + sc->n_zcapsules) +
           11.0 * sc->n_spheres;
}

static double or_broad_flops(const or_ctx *cx) {
    const int A = cx->n_arms;
    double f = A * (7.0 * 81.0 + 11.0 * 18.0);
    if (cx->flags & OR_ENV) f += A * 10.0 * or_env_test_flops(cx->sc);
    if (cx->flags & OR_SELF) f += A * 21.0 * 11.0 + (A * (A - 1) / 2) * 121.0 * 11.0;
    return f;
}

static double or_narrow_flops(const or_ctx *cx, const or_sample *sm, int do_env, int do_self) {
    const int A = cx->n_arms;
    const int quirk = (cx->arm < 0) && !(cx->flags & OR_EXACT);
    double f = 0.0;
    for (int a = 0; a < A; a++) {
        uint8_t fl = (uint8_t)((do_env ? sm->envf[a] : 0) | (do_self ? sm->selff[a] : 0));
        for (int j = 0; j < 8; j++)
            if (fl >> j & 1) f += 18.0 * OR_DET_JCOUNT[j];
        if (do_env)
            for (int i = 1; i < OR_ND; i++)
                if (sm->envf[a] >> OR_DET_S2J[i] & 1) f += or_env_test_flops(cx->sc);
        if (do_self) {
            for (int i = 0; i < 25; i++) {
                int idx = quirk ? i : OR_DET_RANGES[i][0];
                if (sm->selff[a] >> OR_DET_S2J[idx] & 1)
                    f += 11.0 * (OR_DET_RANGES[i][2] - OR_DET_RANGES[i][1] + 1);
            }
            for (int i = 0; i < OR_ND; i++)
                if (sm->selff[a] >> OR_DET_S2J[i] & 1) f += 11.0 * OR_ND * (A - 1 - a);
        }
    }
    return f;
}

/* FP64 ambiguity of one sample.  A verdict can only flip where a minimum
 * crosses zero: the minimum signed distance behind each broad-phase flag
 * (per arm and joint, env and self), and the sample's minimum over the
 * detailed tests its FP32 flags select (both readings of the composite
 * robots' detailed self rows).  Ambiguous = any of those within band. */
static int or_sample_ambiguous(const or_ctx *cx, const or_sample *sm) {
    const int A = cx->n_arms;
    const double band = cx->band;
    double ap[OR_MAX_ARMS][OR_NA][3], dp[OR_MAX_ARMS][OR_ND][3];
    double envj[OR_MAX_ARMS][8], selfj[OR_MAX_ARMS][8];
    double narrow = 1e30;
    for (int a = 0; a < A; a++) {
        or_fk_arm64(or_base(cx, a), sm->q + 7 * a, ap[a], dp[a]);
        for (int j = 0; j < 8; j++) envj[a][j] = selfj[a][j] = 1e30;
    }
#define OR_MIN(dst, v) do { double _v = (v); if (_v < (dst)) (dst) = _v; } while (0)
    for (int a = 0; a < A; a++) {
        if (cx->flags & OR_ENV) {
            for (int i = 1; i < OR_NA; i++)
                OR_MIN(envj[a][OR_APPROX_S2J[i]], or_env_sd64(cx->sc, ap[a][i], OR_APPROX_SPH[i][3]));
            for (int i = 1; i < OR_ND; i++)
                if (sm->envf[a] >> OR_DET_S2J[i] & 1)
                    OR_MIN(narrow, or_env_sd64(cx->sc, dp[a][i], OR_DET_SPH[i][3]));
        }
        if (cx->flags & OR_SELF) {
            for (int i = 0; i < 5; i++) {
                int s1 = OR_APPROX_RANGES[i][0];
                for (int j = OR_APPROX_RANGES[i][1]; j <= OR_APPROX_RANGES[i][2]; j++)
                    OR_MIN(selfj[a][OR_APPROX_S2J[s1]],
                           or_ss_sd64(ap[a][s1], OR_APPROX_SPH[s1][3], ap[a][j], OR_APPROX_SPH[j][3]));
            }
            for (int i = 0; i < OR_NA; i++)
                for (int b = a + 1; b < A; b++)
                    for (int j = 0; j < OR_NA; j++)
                        OR_MIN(selfj[a][OR_APPROX_S2J[i]],
                               or_ss_sd64(ap[a][i], OR_APPROX_SPH[i][3], ap[b][j], OR_APPROX_SPH[j][3]));
            if (!sm->selff[a]) continue;
            for (int i = 0; i < 25; i++) {
                int s1 = OR_DET_RANGES[i][0];
                for (int v = 0; v < 2; v++) {
                    int idx = v ? i : s1;
                    if (!(sm->selff[a] >> OR_DET_S2J[idx] & 1)) continue;
                    for (int j = OR_DET_RANGES[i][1]; j <= OR_DET_RANGES[i][2]; j++)
                        OR_MIN(narrow, or_ss_sd64(dp[a][idx], OR_DET_SPH[s1][3], dp[a][j], OR_DET_SPH[j][3]));
                }
            }
            for (int i = 0; i < OR_ND; i++) {
                if (!(sm->selff[a] >> OR_DET_S2J[i] & 1)) continue;
                for (int b = a + 1; b < A; b++)
                    for (int j = 0; j < OR_ND; j++)
                        OR_MIN(narrow, or_ss_sd64(dp[a][i], OR_DET_SPH[i][3], dp[b][j], OR_DET_SPH[j][3]));
            }
        }
    }
#undef OR_MIN
    if (fabs(narrow) < band) return 1;
    for (int a = 0; a < A; a++)
        for (int j = 0; j < 8; j++)
            if (fabs(envj[a][j]) < band || fabs(selfj[a][j]) < band) return 1;
    return 0;
}

/* One fkcc_single_buffer* call: g samples already interpolated in sm[0..g-1]
 * (sample k+1 in sm[k]).  Returns the 1-based sample that fired first, or 0.
 * `amb` counts the ambiguous samples (only computed when band > 0; with
 * count_all = 0 it stops at the first). */
static int or_check_segment(const or_ctx *cx, or_sample *sm, int g, double *flops, int *amb, int count_all) {
    int envc[OR_MAX_G], selfc[OR_MAX_G], envd[OR_MAX_G], selfd[OR_MAX_G];
    int any_env = 0, any_self = 0;
    for (int k = 0; k < g; k++) {
        or_broad(cx, &sm[k]);
        envc[k] = sm[k].env_cnt;
        selfc[k] = sm[k].self_cnt;
        any_env |= envc[k] > 0;
        any_self |= selfc[k] > 0;
    }
    *flops += g * or_broad_flops(cx);
    if (cx->band > 0.0)
        for (int k = 0; k < g && (count_all || !*amb); k++) *amb += or_sample_ambiguous(cx, &sm[k]);
    if (!any_env && !any_self) return 0;
    int exact = (cx->flags & OR_EXACT) != 0;
    if (!exact) {
        or_thread_dist(envc, g, envd);
        or_thread_dist(selfc, g, selfd);
    }
    int first = 0;
    for (int k = 0; k < g; k++) {
        int do_env = any_env && (exact ? envc[k] > 0 : envd[k] > 0);
        int do_self = any_self && (exact ? selfc[k] > 0 : selfd[k] > 0);
        if (!do_env && !do_self) continue;
        *flops += or_narrow_flops(cx, &sm[k], do_env, do_self);
        if (first) continue; /* keep tallying the dense narrow work */
        float dpos[OR_MAX_ARMS][OR_ND][3];
        for (int a = 0; a < cx->n_arms; a++) or_fk_arm(or_base(cx, a), sm[k].q + 7 * a, NULL, dpos[a], cx->po);
        int hit = (do_env && or_narrow_env(cx, &sm[k], dpos)) || (do_self && or_narrow_self(cx, &sm[k], dpos));
        if (hit) first = k + 1;
    }
    return first;
}

/* Segmentation rules (call sites named in the file header). */
#define OR_RULE_PLAIN 0    /* delta=(q1-q0)/g, q_k = q0 + k*delta            */
#define OR_RULE_CONNECT 1  /* n=int(|d|/range)+1, restart from accumulated q */
#define OR_RULE_BSPLINE 2  /* n=ceil(|d|/range), accumulate per sample       */
#define OR_RULE_SHORTCUT 3 /* n=ceil((|d|-0.001)/range), accumulate          */

static float or_l2(const float *a, const float *b, int dim) {
    float ans = 0.0f;
    for (int i = 0; i < dim; i++) {
        float d = a[i] - b[i];
        ans = fmaf(d, d, ans);
    }
    return sqrtf(ans);
}

int oracle_segment_count(const float *q0, const float *q1, int dim, int rule, float range) {
    if (rule == OR_RULE_PLAIN) return 1;
    if (rule == OR_RULE_CONNECT) return (int)(or_l2(q1, q0, dim) / range) + 1;
    if (rule == OR_RULE_BSPLINE) return (int)ceilf(or_l2(q0, q1, dim) / range);
    return (int)ceilf((or_l2(q0, q1, dim) - 0.001f) / range);
}

/* ------------------------------------------------------------------------ */
/* Public entry points (ctypes)                                              */
/* ------------------------------------------------------------------------ */
int oracle_validate(const orc_scene *sc, const orc_robots *rb, const float *q0, const float *q1,
                    int64_t n_edges, int g, int flags, int arm, int rule, float range,
                    int pair_order, double band, const orc_trig *trig, int n_threads,
                    uint8_t *valid, int32_t *first_hit, uint8_t *ambiguous, double *flops_out,
                    int32_t *n_seg_out, int32_t *amb_samples) {
    or_init_tables();
    if (g < 1 || g > OR_MAX_G || rb->n_arms < 1 || rb->n_arms > OR_MAX_ARMS) return 1;
    if (arm >= rb->n_arms) return 1;
    g_trig = (trig && trig->n > 0) ? trig : NULL;
    g_trig_miss = 0;
    or_ctx cx = {sc, rb, arm >= 0 ? 1 : rb->n_arms, arm, flags, pair_order, band};
    const int dim = 7 * cx.n_arms;
    double total_flops = 0.0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total_flops)
    for (int64_t e = 0; e < n_edges; e++) {
        const float *a = q0 + e * dim, *b = q1 + e * dim;
        or_sample sm[OR_MAX_G];
        double fl = 0.0;
        int amb = 0, first = 0;
        int nseg = oracle_segment_count(a, b, dim, rule, range);
        float base[OR_MAX_ARMS * 7], step[OR_MAX_ARMS * 7], acc[OR_MAX_G][OR_MAX_ARMS * 7];
        for (int d = 0; d < dim; d++) {
            base[d] = a[d];
            if (rule == OR_RULE_PLAIN) step[d] = (b[d] - a[d]) / (float)g;
            else step[d] = (b[d] - a[d]) / (float)nseg;
        }
        if (rule == OR_RULE_BSPLINE || rule == OR_RULE_SHORTCUT)
            for (int k = 0; k < g; k++)
                for (int d = 0; d < dim; d++) acc[k][d] = fmaf((float)(k + 1), step[d] / (float)g, a[d]);
        for (int s = 0; s < nseg && !first; s++) {
            for (int k = 0; k < g; k++)
                for (int d = 0; d < dim; d++) {
                    float v;
                    if (rule == OR_RULE_PLAIN) v = fmaf((float)(k + 1), step[d], base[d]);
                    else if (rule == OR_RULE_CONNECT) v = fmaf((float)(k + 1), step[d] / (float)g, base[d]);
                    else v = acc[k][d];
                    sm[k].q[d] = v;
                }
            int f = or_check_segment(&cx, sm, g, &fl, &amb, amb_samples != NULL);
            if (f) first = s * g + f;
            if (rule == OR_RULE_CONNECT)
                for (int d = 0; d < dim; d++) base[d] = base[d] + step[d];
            else if (rule != OR_RULE_PLAIN)
                for (int k = 0; k < g; k++)
                    for (int d = 0; d < dim; d++) acc[k][d] = acc[k][d] + step[d];
        }
        valid[e] = first == 0;
        first_hit[e] = first ? first : -1;
        if (ambiguous) ambiguous[e] = (uint8_t)(amb > 0);
        if (amb_samples) amb_samples[e] = amb;
        if (n_seg_out) n_seg_out[e] = nseg;
        total_flops += fl;
    }
    if (flops_out) *flops_out = total_flops;
    int miss = g_trig_miss;
    g_trig = NULL;
    return miss ? 2 : 0;
}

/* Sphere centres of n configurations of one arm (base row-major 4x4).
 * detailed: 0 approx (11 spheres), 1 detailed (59).  fp64: 0 FP32 mirror
 * (pair_order, trig table honoured), 1 double precision truth. */
int oracle_fk_spheres(const float *base, const float *q, int64_t n, int detailed, int fp64,
                      int pair_order, const orc_trig *trig, double *out) {
    or_init_tables();
    g_trig = (trig && trig->n > 0) ? trig : NULL;
    g_trig_miss = 0;
    const int ns = detailed ? OR_ND : OR_NA;
    for (int64_t e = 0; e < n; e++) {
        double *o = out + e * ns * 3;
        if (fp64) {
            double ap[OR_NA][3], dp[OR_ND][3];
            or_fk_arm64(base, q + 7 * e, ap, dp);
            memcpy(o, detailed ? (double *)dp : (double *)ap, sizeof(double) * ns * 3);
        } else {
            float ap[OR_NA][3], dp[OR_ND][3];
            or_fk_arm(base, q + 7 * e, detailed ? NULL : ap, detailed ? dp : NULL, pair_order);
            for (int i = 0; i < ns * 3; i++) o[i] = detailed ? ((float *)dp)[i] : ((float *)ap)[i];
        }
    }
    int miss = g_trig_miss;
    g_trig = NULL;
    return miss ? 2 : 0;
}

/* Interpolated sample configurations of one edge (for building trig tables):
 * writes n_seg*g*dim floats (capped by max_out) and returns the count. */
int64_t oracle_edge_samples(const float *q0, const float *q1, int dim, int g, int rule, float range,
                            float *out, int64_t max_out) {
    int nseg = oracle_segment_count(q0, q1, dim, rule, range);
    int64_t w = 0;
    float base[OR_MAX_ARMS * 7], step[OR_MAX_ARMS * 7], acc[OR_MAX_G][OR_MAX_ARMS * 7];
    for (int d = 0; d < dim; d++) {
        base[d] = q0[d];
        step[d] = (rule == OR_RULE_PLAIN) ? (q1[d] - q0[d]) / (float)g : (q1[d] - q0[d]) / (float)nseg;
    }
    for (int k = 0; k < g; k++)
        for (int d = 0; d < dim; d++) acc[k][d] = fmaf((float)(k + 1), step[d] / (float)g, q0[d]);
    for (int s = 0; s < nseg; s++) {
        for (int k = 0; k < g; k++)
            for (int d = 0; d < dim; d++) {
                float v;
                if (rule == OR_RULE_PLAIN) v = fmaf((float)(k + 1), step[d], base[d]);
                else if (rule == OR_RULE_CONNECT) v = fmaf((float)(k + 1), step[d] / (float)g, base[d]);
                else v = acc[k][d];
                if (w < max_out) out[w] = v;
                w++;
            }
        if (rule == OR_RULE_CONNECT)
            for (int d = 0; d < dim; d++) base[d] = base[d] + step[d];
        else if (rule != OR_RULE_PLAIN)
            for (int k = 0; k < g; k++)
                for (int d = 0; d < dim; d++) acc[k][d] = acc[k][d] + step[d];
    }
    return w;
}

/* The detailed sphere table {x, y, z, r} x 59 (local frames), for tests. */
int oracle_det_spheres(float *out) {
    for (int i = 0; i < OR_ND; i++)
        for (int c = 0; c < 4; c++) out[4 * i + c] = OR_DET_SPH[i][c];
    return 0;
}

/* Host threads available (processors, not the current OpenMP setting, which a
 * one-thread call leaves at 1). */
int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

/* Primitive-level access for unit tests: FP32 verdict of one sphere against
 * the scene (the reference's scene loop) and its FP64 signed distance. */
int oracle_env_hit(const orc_scene *sc, float x, float y, float z, float r, int pair_order) {
    const float p[3] = {x, y, z};
    return or_env_hit(sc, p, r, pair_order);
}

double oracle_env_sd(const orc_scene *sc, double x, double y, double z, double r) {
    const double p[3] = {x, y, z};
    return or_env_sd64(sc, p, r);
}
