// planner.cu -- a compact composite-space planner whose every edge check goes
// through a validate callback: the client of the validation service in served
// planning (mrpop_session_plan in server.cu), and testable on the CPU with any
// validator.
//
// The reference's planner (dRRT with per-arm roadmaps plus AO-x optimisation,
// dRRT::solve in Planners.hh:57-64, pop_planner.cu) is not rebuilt here.  This
// one has its step pattern, which is what the service is measured on:
//   - extend: `batch` tree nodes steered towards uniform targets by at most
//     `step` (composite Euclidean), each edge one plain edge of `granularity`
//     samples (the extend form, pop_planner.cu:551-561);
//   - connect: every new node towards its nearest node of the other tree,
//     checked with the connect segmentation (pop_planner.cu:666-703);
//   - shortcut: after the first solution, `shortcut_passes` passes of
//     `shortcut_pairs` random (i < j) waypoint pairs checked with the shortcut
//     segmentation (path_simplification.cu:155-200); the valid pair saving the
//     most length is spliced in.
// It is deterministic given the seed and the verdicts it receives.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "launch.h"

namespace {

// Panda joint limits, lower bound and span (Robots.hh:13-23).
constexpr float kLo[7] = {-2.9671f, -1.8326f, -2.9671f, -3.1416f, -2.9671f, -0.0873f, -2.9671f};
constexpr float kSpan[7] = {5.9342f, 3.6652f, 5.9342f, 3.2289f, 5.9342f, 3.9095999999999997f, 5.9342f};

// splitmix64 (Steele, Lea, Flood 2014): the planner's only random source.
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    int64_t below(int64_t n) { return (int64_t)(next() % (uint64_t)n); }
};

struct Tree {
    int dof = 0;
    std::vector<float> q;
    std::vector<double> norm2;  // |node|^2, for the nearest-node search
    std::vector<int> parent;
    int64_t size() const { return (int64_t)parent.size(); }
    const float *node(int64_t i) const { return &q[(size_t)i * dof]; }
    void add(const float *x, int p) {
        double n2 = 0.0;
        for (int d = 0; d < dof; d++) {
            q.push_back(x[d]);
            n2 += (double)x[d] * x[d];
        }
        norm2.push_back(n2);
        parent.push_back(p);
    }
};

// Nearest node to x (squared Euclidean as |n|^2 - 2 n.x, ties to the lowest index).
int64_t nearest(const Tree &t, const float *x) {
    double best = INFINITY;
    int64_t bi = 0;
    for (int64_t i = 0; i < t.size(); i++) {
        const float *n = t.node(i);
        double dot = 0.0;
        for (int d = 0; d < t.dof; d++) dot += (double)n[d] * x[d];
        const double v = t.norm2[i] - 2.0 * dot;
        if (v < best) {
            best = v;
            bi = i;
        }
    }
    return bi;
}

double dist(const float *a, const float *b, int dof) {
    double s = 0.0;
    for (int d = 0; d < dof; d++) {
        const double v = (double)a[d] - b[d];
        s += v * v;
    }
    return std::sqrt(s);
}

// FNV-1a over the verdicts received, in order.
void digest_add(uint64_t &h, const void *p, size_t n) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 0x100000001B3ull;
    }
}

}  // namespace

extern "C" mrpop_status mrpop_plan(int arms, const float *start, const float *goal, const mrpop_plan_settings *settings,
                                   mrpop_validate_fn validate, void *ctx, float *path_out, int64_t max_waypoints,
                                   mrpop_plan_result *out) {
    if (arms < 1 || arms > MRPOP_MAX_ARMS || !start || !goal || !settings || !validate || !out)
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "plan: bad argument");
    const mrpop_plan_settings &S = *settings;
    if (S.batch < 1 || S.max_iters < 0 || S.granularity < 1 || S.granularity > MRPOP_MAX_GRANULARITY ||
        !(S.step > 0.0f) || !(S.range > 0.0f) || S.shortcut_passes < 0 || S.shortcut_pairs < 1)
        return mrpop::fail_status(MRPOP_ERR_INVALID_ARGUMENT, "plan: bad settings");
    const int dof = 7 * arms;
    *out = mrpop_plan_result{};
    uint64_t digest = 0xCBF29CE484222325ull;
    Rng rng{S.seed};
    Tree T[2];
    T[0].dof = T[1].dof = dof;
    T[0].add(start, -1);
    T[1].add(goal, -1);
    const int B = S.batch;
    std::vector<float> tgt(dof), q0((size_t)B * dof), q1((size_t)B * dof);
    std::vector<uint8_t> valid(B);
    std::vector<int32_t> first(B);
    std::vector<int64_t> nn(B);

    auto check = [&](int64_t n, int rule, float range) -> int {
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = validate(ctx, q0.data(), q1.data(), n, S.granularity, rule, range, valid.data(), first.data());
        out->validate_ns +=
            std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
        out->steps++;
        out->edges += n;
        digest_add(digest, valid.data(), (size_t)n);
        digest_add(digest, first.data(), (size_t)n * sizeof(int32_t));
        return rc;
    };

    int ja = -1;
    int64_t ia = -1, ib = -1;
    for (int it = 0; it < S.max_iters && ja < 0; it++) {
        out->iterations = it + 1;
        const int a = it % 2;
        for (int k = 0; k < B; k++) {
            for (int d = 0; d < dof; d++) tgt[d] = (float)(kLo[d % 7] + rng.uniform() * kSpan[d % 7]);
            nn[k] = nearest(T[a], tgt.data());
            const float *nr = T[a].node(nn[k]);
            double len2 = 0.0;
            for (int d = 0; d < dof; d++) len2 += ((double)tgt[d] - nr[d]) * ((double)tgt[d] - nr[d]);
            const double scale = std::min(1.0, (double)S.step / std::max(std::sqrt(len2), 1e-12));
            for (int d = 0; d < dof; d++) {
                q0[(size_t)k * dof + d] = nr[d];
                q1[(size_t)k * dof + d] = (float)(nr[d] + ((double)tgt[d] - nr[d]) * scale);
            }
        }
        int rc = check(B, MRPOP_RULE_PLAIN, 0.0f);
        if (rc) return mrpop::fail_status((mrpop_status)rc, "plan: extend check failed");
        const int64_t first_new = T[a].size();
        for (int k = 0; k < B; k++)
            if (valid[k]) T[a].add(&q1[(size_t)k * dof], (int)nn[k]);
        const int64_t added = T[a].size() - first_new;
        if (!added) continue;
        const Tree &o = T[1 - a];
        std::vector<int64_t> nb(added);
        for (int64_t k = 0; k < added; k++) {
            nb[k] = nearest(o, T[a].node(first_new + k));
            std::memcpy(&q0[(size_t)k * dof], T[a].node(first_new + k), dof * sizeof(float));
            std::memcpy(&q1[(size_t)k * dof], o.node(nb[k]), dof * sizeof(float));
        }
        rc = check(added, MRPOP_RULE_CONNECT, S.range);
        if (rc) return mrpop::fail_status((mrpop_status)rc, "plan: connect check failed");
        for (int64_t k = 0; k < added; k++)
            if (valid[k]) {
                ja = a;
                ia = first_new + k;
                ib = nb[k];
                break;
            }
    }
    out->digest = digest;
    out->start_tree = T[0].size();
    out->goal_tree = T[1].size();
    if (ja < 0) return MRPOP_OK;

    // path: start .. goal
    std::vector<int64_t> ha, hb;
    for (int64_t i = ia; i >= 0; i = T[ja].parent[i]) ha.push_back(i);
    for (int64_t i = ib; i >= 0; i = T[1 - ja].parent[i]) hb.push_back(i);
    std::vector<float> path;
    auto push = [&](const Tree &t, int64_t i) { path.insert(path.end(), t.node(i), t.node(i) + dof); };
    if (ja == 0) {
        for (auto it = ha.rbegin(); it != ha.rend(); ++it) push(T[0], *it);
        for (int64_t i : hb) push(T[1], i);
    } else {
        for (auto it = hb.rbegin(); it != hb.rend(); ++it) push(T[0], *it);
        for (int64_t i : ha) push(T[1], i);
    }
    // shortcut passes
    const int P = S.shortcut_pairs;
    if ((int)valid.size() < P) {
        valid.resize(P);
        first.resize(P);
        q0.resize((size_t)P * dof);
        q1.resize((size_t)P * dof);
    }
    std::vector<int64_t> pi(P), pj(P);
    for (int pass = 0; pass < S.shortcut_passes; pass++) {
        const int64_t m = (int64_t)path.size() / dof;
        if (m < 3) break;
        for (int k = 0; k < P; k++) {
            pi[k] = rng.below(m - 2);
            pj[k] = std::min<int64_t>(m - 1, pi[k] + 2 + rng.below(m) % (m - 1 - pi[k]));
            std::memcpy(&q0[(size_t)k * dof], &path[(size_t)pi[k] * dof], dof * sizeof(float));
            std::memcpy(&q1[(size_t)k * dof], &path[(size_t)pj[k] * dof], dof * sizeof(float));
        }
        const int rc = check(P, MRPOP_RULE_SHORTCUT, S.range);
        if (rc) return mrpop::fail_status((mrpop_status)rc, "plan: shortcut check failed");
        std::vector<double> csum(m, 0.0);
        for (int64_t i = 1; i < m; i++) csum[i] = csum[i - 1] + dist(&path[(i - 1) * dof], &path[i * dof], dof);
        int best = -1;
        double gain = 0.0;
        for (int k = 0; k < P; k++) {
            if (!valid[k]) continue;
            const double g = (csum[pj[k]] - csum[pi[k]]) - dist(&path[pi[k] * dof], &path[pj[k] * dof], dof);
            if (g > gain + 1e-9) {
                best = k;
                gain = g;
            }
        }
        if (best >= 0)
            path.erase(path.begin() + (pi[best] + 1) * dof, path.begin() + pj[best] * dof);
    }
    const int64_t m = (int64_t)path.size() / dof;
    double cost = 0.0;
    for (int64_t i = 1; i < m; i++) cost += dist(&path[(i - 1) * dof], &path[i * dof], dof);
    out->solved = 1;
    out->waypoints = m;
    out->cost = cost;
    out->digest = digest;
    if (path_out && max_waypoints > 0)
        std::memcpy(path_out, path.data(), (size_t)std::min(m, max_waypoints) * dof * sizeof(float));
    return MRPOP_OK;
}
