/*
 * mrpop.h -- C ABI of the GB300-native batched edge validator for MR.POP.
 *
 * The reference planner has no library boundary for this path: edge checks are
 * block-collective __device__ routines inlined into its planner kernels
 *   fkcc_single_buffer<Robot>       src/planning/utils.cuh:447-534  (env + self)
 *   fkcc_single_buffer_mr<Robot>    src/planning/utils.cuh:536-624  (one arm)
 *   fkcc_single_buffer_drrt<Robot>  src/planning/utils.cuh:626-686  (self only)
 * whose callers interpolate the edge first (pop_planner.cu:551-561 extend,
 * :666-703 connect, roadmap_interior.cuh:219-234 roadmap edges,
 * path_simplification.cu:85-129 B-spline, :155-200 shortcut).  This header is
 * the batched, stream-ordered replacement: one call validates many edges.
 *
 * Conventions
 *   - Every function returns an mrpop_status; nothing calls exit() (the
 *     reference's cudaCheckError does, utils.cuh:265-274).
 *   - Device entry points are asynchronous on the given cudaStream_t (passed as
 *     void*; NULL = legacy default stream).  Pointers documented "device" must
 *     be device-accessible for the whole call.
 *   - Handles are immutable after creation and may be shared by threads; calls
 *     on one handle from several host threads are safe.  The library keeps no
 *     global device state except the per-device tables it sets up on first use.
 *   - Configurations are float32, row-major [n_edges][dof] with dof = 7 * arms
 *     (the layout of the reference's Robot::Configuration arrays,
 *     Robots.hh:46-140).  Sample k (1..g) of an edge is q0 + k*(q1-q0)/g as the
 *     reference computes it; sample 0 (the edge start) is never tested.
 */
#ifndef MRPOP_H
#define MRPOP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MRPOP_OK = 0,
    MRPOP_ERR_INVALID_ARGUMENT = 1,
    MRPOP_ERR_CUDA = 2,
    MRPOP_ERR_UNSUPPORTED = 3,
    MRPOP_ERR_OUT_OF_MEMORY = 4,
    MRPOP_ERR_DEVICE_TIMEOUT = 5, /* a bounded device wait gave up (see mrpop_scene_status) */
} mrpop_status;

/* Check selection and semantics (flags argument). */
#define MRPOP_CHECK_ENV 0x1u   /* robot spheres vs scene obstacles                    */
#define MRPOP_CHECK_SELF 0x2u  /* intra-arm pairs and, for composites, arm-vs-arm     */
#define MRPOP_MODE_EXACT 0x10u /* every flagged sample gets the detailed check        */
/* Without MRPOP_MODE_EXACT the verdicts are those of the reference's own check,
 * including its proportional thread split (utils.cuh:476-517: samples whose share
 * of 4*g threads rounds to zero get no detailed check) and, for composites, its
 * detailed intra-arm row indexing (panda_four.cuh:388-413).
 *   fkcc_single_buffer       == MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, arm = -1
 *   fkcc_single_buffer_drrt  == MRPOP_CHECK_SELF,                   arm = -1
 *   fkcc_single_buffer_mr    == MRPOP_CHECK_ENV | MRPOP_CHECK_SELF, arm = robot_id */

/* Edge segmentation rules (mrpop_validate_segments). */
#define MRPOP_RULE_PLAIN 0    /* one segment: q_k = q0 + k*((q1-q0)/g)                       */
#define MRPOP_RULE_CONNECT 1  /* n = int(|q1-q0|/range)+1, q_k = q + k*(vec/g), q += vec     */
                              /*   (pop_planner.cu:666-703)                                  */
#define MRPOP_RULE_BSPLINE 2  /* n = ceil(|q1-q0|/range), q_k += delta per segment           */
                              /*   (path_simplification.cu:85-129)                           */
#define MRPOP_RULE_SHORTCUT 3 /* n = ceil((|q1-q0|-0.001)/range), q_k += delta per segment   */
                              /*   (path_simplification.cu:155-200)                          */

#define MRPOP_MAX_ARMS 5
#define MRPOP_MAX_GRANULARITY 64 /* the reference's MAX_GRANULARITY, pop_planner_state.cuh:13 */

/*
 * Scene description (host memory; the library copies it).  Records are packed
 * float32 in the field order of the reference's shape structs
 * (src/collision/shapes.hh:28-185, environment.hh:11-40):
 *   sphere  {x, y, z, r}                                         4 floats
 *   capsule {x1, y1, z1, xv, yv, zv, r, rdv}  rdv = 1/|v|^2      8 floats
 *   cuboid  {x, y, z, a1x, a1y, a1z, a2x, a2y, a2z, a3x, a3y, a3z, h1, h2, h3}  15 floats
 * z_capsules / z_cuboids use the z-aligned tests (utils.cuh:165-181, 208-228).
 * cylinders are accepted and never tested, as in the reference (its scene loop
 * utils.cuh:231-260 does not read Environment::cylinders).
 */
typedef struct {
    const float *spheres;
    uint32_t num_spheres;
    const float *capsules;
    uint32_t num_capsules;
    const float *z_capsules;
    uint32_t num_z_capsules;
    const float *cylinders;
    uint32_t num_cylinders;
    const float *cuboids;
    uint32_t num_cuboids;
    const float *z_cuboids;
    uint32_t num_z_cuboids;
} mrpop_scene_desc;

typedef struct mrpop_scene mrpop_scene;
typedef struct mrpop_robotset mrpop_robotset;
typedef struct mrpop_workspace mrpop_workspace;

/* Replaces setup_environment_on_device (pop_planner.cu:69-161): copies the
 * scene to the current device.  Synchronous. */
mrpop_status mrpop_scene_create(const mrpop_scene_desc *desc, mrpop_scene **out);
mrpop_status mrpop_scene_destroy(mrpop_scene *scene);
/* Device-side status word of the scene (0 = fine; nonzero = a bounded wait in a
 * kernel gave up; the kernel then reported its edges as invalid). Synchronous. */
mrpop_status mrpop_scene_status(const mrpop_scene *scene, uint32_t *status_out);

/* Arm bases.  base_T: n_arms row-major 4x4 transforms (host memory), or NULL
 * for the reference's compiled-in layouts: identity for 1 arm
 * (panda.cuh:78-83), quad_franka_base_transform for 4 (panda.cuh:16-40 ==
 * panda_four.cuh:17-41), five_franka_base_transform for 5 (panda.cuh:42-73 ==
 * panda_five.cuh:17-46).  The arms are Franka Pandas with the reference's
 * sphere model (panda_multi_geometry.cuh). */
mrpop_status mrpop_robotset_create(int n_arms, const float *base_T, mrpop_robotset **out);
mrpop_status mrpop_robotset_destroy(mrpop_robotset *robots);

/*
 * Validate n_edges edges q0[e] -> q1[e] (device pointers, [n_edges][dof]).
 *   arm < 0 : composite check over all arms, dof = 7 * n_arms
 *   arm >= 0: single-arm check of arm `arm` (its base), dof = 7
 * granularity: samples per edge, 1..64.
 * Outputs (device): valid[e] = 1 if collision-free; first_hit[e] = the 1-based
 * sample index of the first sample whose detailed check fired (-1 if valid).
 * Replaces one fkcc_single_buffer* call per edge (see flags above).
 * Launch form: a call of more than the fused-edge limit runs the split
 * pipeline (a broad and a narrow kernel; for segmented rules, segment rounds
 * of both and a fused tail); a smaller call runs as one fused launch (both
 * phases per edge in one warp, from segment 0), which saves the launches and
 * the staging that dominate small calls.  Verdicts are the same either way.
 * mrpop_set_fused_edges sets the limit for the process (0: the default, 2048
 * edges; -1: every call split) and returns the previous one.
 */
int64_t mrpop_set_fused_edges(int64_t max_edges);
mrpop_status mrpop_validate_edges(const mrpop_scene *scene, const mrpop_robotset *robots,
                                  const float *q0, const float *q1, int64_t n_edges,
                                  int granularity, uint32_t flags, int arm, uint8_t *valid,
                                  int32_t *first_hit, void *stream);

/*
 * Segmented edges (connect, B-spline and shortcut forms).  Each edge is split
 * into n segments of `granularity` samples by `rule` with `range` (settings.range);
 * segments are checked in order and checking stops at the first invalid one.
 * first_hit = segment * granularity + sample (1-based), -1 if valid.
 * n_seg_out (device, optional) receives each edge's segment count.
 */
mrpop_status mrpop_validate_segments(const mrpop_scene *scene, const mrpop_robotset *robots,
                                     const float *q0, const float *q1, int64_t n_edges,
                                     int granularity, int rule, float range, uint32_t flags,
                                     int arm, uint8_t *valid, int32_t *first_hit,
                                     int32_t *n_seg_out, void *stream);

/*
 * Same verdicts as mrpop_validate_edges (single-segment edges), for callers that
 * must not allocate device memory while they run -- e.g. a serving process that
 * reserves its whole device-memory budget at start-up and admits work against
 * it, or a planner loop that may not enter the allocator.  No counterpart in the
 * reference (its planner keeps all scratch in fixed __device__ arrays).
 *   - Calls no allocation routine.  Its scratch is one fixed array in the
 *     library's device memory, about 27.6 MiB per device
 *     (MRPOP_NOALLOC_MAX_EDGES edges at granularity 64), held by every GPU that
 *     loads the library until the process exits.
 *   - n_edges above MRPOP_NOALLOC_MAX_EDGES is rejected (MRPOP_ERR_INVALID_ARGUMENT).
 *   - The first call on a device looks up the array's device address (a one-time
 *     set-up per device, done with that device current); make that first call
 *     before any stream capture.  With CUDA's default lazy module loading the
 *     driver places the array, and loads each kernel variant, on first use: the
 *     first call per device -- and the first per arm count and granularity class
 *     (g <= 32 or not) -- is a warm-up in which the driver may take device
 *     memory.  A caller with a fixed budget makes those calls at start-up (or
 *     sets CUDA_MODULE_LOADING=EAGER); later calls take none.
 *   - The cached address, like every handle of this library, does not survive
 *     cudaDeviceReset.
 *   - Every call shares the array: calls that overlap on the GPU (different
 *     streams, other host threads) race on it and must be ordered by the caller.
 *     The array keeps the last call's contents; no call depends on them.
 */
#define MRPOP_NOALLOC_MAX_EDGES 16384
mrpop_status mrpop_validate_edges_noalloc(const mrpop_scene *scene, const mrpop_robotset *robots,
                                          const float *q0, const float *q1, int64_t n_edges,
                                          int granularity, uint32_t flags, int arm, uint8_t *valid,
                                          int32_t *first_hit, void *stream);

/*
 * Host-buffer form for callers without device memory (the reference's host
 * API, dRRT::solve in Planners.hh:57-64, hands host arrays across): validates
 * q0/q1 in host memory, writes valid/first_hit there and waits.  When all four
 * buffers are page-locked (cudaHostAlloc, cudaHostRegister, a pinned tensor)
 * the kernels read and write them in place (over NVLink-C2C on a Grace host);
 * otherwise the call copies through the workspace's device buffers, which
 * grow on demand.  A workspace belongs to one host thread.
 */
mrpop_status mrpop_workspace_create(mrpop_workspace **out);
mrpop_status mrpop_workspace_destroy(mrpop_workspace *ws);
mrpop_status mrpop_validate_edges_host(mrpop_workspace *ws, const mrpop_scene *scene,
                                       const mrpop_robotset *robots, const float *q0,
                                       const float *q1, int64_t n_edges, int granularity,
                                       uint32_t flags, int arm, int rule, float range,
                                       uint8_t *valid, int32_t *first_hit);

/*
 * Sphere centres of n single-arm configurations (device q [n][7], device out
 * [n][spheres][3]); detailed = 0: the 11 broad-phase spheres, 1: the 59
 * detailed spheres.  The same FK the validator runs (panda.cuh:598-669,
 * 761-829 with the base of arm `arm`).
 */
mrpop_status mrpop_fk_spheres(const mrpop_robotset *robots, int arm, const float *q, int64_t n,
                              int detailed, float *out, void *stream);

/*
 * Batched validation of many independent planning instances (no counterpart
 * in the reference, whose planner validates one edge per 256-thread block).
 * Each item is one mrpop_validate_edges call (rule MRPOP_RULE_PLAIN) or one
 * mrpop_validate_segments call without segment counts (connect, B-spline or
 * shortcut rule with its range): its scene, robot set, endpoints
 * [n_edges][7 * arms], granularity, check flags, arm selection, rule and
 * outputs; the items may differ in all of them.  Endpoints and outputs may
 * live in device memory or in page-locked host memory, which the kernels read
 * and write in place.  Results equal the per-item calls bit for bit.
 *
 * mrpop_batch_create checks every item, allocates the device scratch and the
 * per-group parameter tables (groups = arm count x (g <= 32 or not) x
 * (segmented or not)), and keeps the item pointers: their buffers must outlive
 * the batch.
 * mrpop_batch_run launches, per group on `stream`, one persistent broad-phase
 * and one narrow-phase kernel; a segmented group runs them in rounds (one
 * segment of every undecided edge per round) and then one fused kernel for the
 * edges with segments left.  It allocates nothing and reads the inputs as they
 * are at execution time, so a batch can be rerun on refilled buffers.
 * mrpop_batch_tune picks each group's launch shape by timing (synchronous):
 * the chunk size (edges a CTA takes at a time: 24, 48, 96 or 192) and, for the
 * broad and the narrow kernel, the warps per CTA (2, 3, 4 or 6; one edge per
 * warp at a time) and the grid (multiples of the SM count up to the resident
 * maximum at that CTA size).  It times launches on the items' own buffers, so it writes
 * their outputs: afterwards single-segment items hold their verdicts, but
 * segmented items hold only the first segment round's partial state (their
 * later rounds are not run) -- run the batch or launch its graph before
 * reading them.
 * mrpop_batch_capture records one run as a CUDA graph (each group on its own
 * branch) and mrpop_batch_launch launches that graph on `stream`.
 * mrpop_batch_info reports, per group, {arms, samples per lane, segmented,
 * broad grid, narrow grid} into grids[5 * i ..] for up to max_groups groups.
 * A batch's staged scratch and work counters serve every run of it, so runs
 * and graph launches of one batch must be ordered (one stream, or events
 * between streams); different batches are independent.
 */
typedef struct mrpop_batch_item {
    const mrpop_scene *scene;
    const mrpop_robotset *robots;
    const float *q0;
    const float *q1;
    int64_t n_edges;
    int32_t granularity;
    uint32_t flags;
    int32_t arm;
    uint8_t *valid;
    int32_t *first_hit;
    int32_t rule;  /* MRPOP_RULE_*; zero-initialised items are single-segment */
    float range;   /* segment length for the segmented rules (> 0) */
} mrpop_batch_item;

typedef struct mrpop_batch mrpop_batch;

mrpop_status mrpop_batch_create(const mrpop_batch_item *items, int64_t n_items, mrpop_batch **out);
mrpop_status mrpop_batch_run(mrpop_batch *batch, void *stream);
mrpop_status mrpop_batch_tune(mrpop_batch *batch, void *stream);
mrpop_status mrpop_batch_capture(mrpop_batch *batch);
mrpop_status mrpop_batch_launch(mrpop_batch *batch, void *stream);
mrpop_status mrpop_batch_info(const mrpop_batch *batch, int64_t *n_groups, int32_t *grids, int64_t max_groups);
/* Per group, MRPOP_BATCH_SHAPE_INTS values into out[12 * i ..]: {arms, samples
 * per lane, segmented, chunk edges, chunks, broad warps per CTA, broad grid,
 * narrow warps, narrow grid, fused warps, fused grid, 0}.
 * mrpop_batch_set_shape sets one group's shape by hand (chunk_edges and
 * warps[k] > 0 replace the current values; grids[k] > 0 is capped at the
 * resident maximum, 0 selects it; k = broad, narrow, fused) and drops a
 * captured graph.  Results do not depend on the shape. */
#define MRPOP_BATCH_SHAPE_INTS 12
mrpop_status mrpop_batch_shapes(const mrpop_batch *batch, int64_t *n_groups, int32_t *out, int64_t max_groups);
mrpop_status mrpop_batch_set_shape(mrpop_batch *batch, int64_t group, int32_t chunk_edges, const int32_t *warps,
                                   const int32_t *grids);
mrpop_status mrpop_batch_destroy(mrpop_batch *batch);

/*
 * Serving: a continuous-batching validation service for many concurrent
 * planning queries on one GPU.  No counterpart in the reference, which runs
 * one query per process (dRRT::solve, Planners.hh:57-64, owning the device)
 * and validates one edge per block (pop_planner.cu:973).
 *
 * mrpop_server_create reserves, once, an arena of budget_bytes of device
 * memory on the current device, `streams` launch slots and one worker thread.
 * A query opens a session (mrpop_session_open), which is admitted when the
 * scratch of its largest step (arms, max_edges, max_granularity) fits in the
 * arena's free space; otherwise the call waits, up to timeout_ms (< 0: no
 * limit, 0: do not wait; MRPOP_ERR_OUT_OF_MEMORY when it gives up).  A session
 * then submits one step at a time (mrpop_session_submit: an mrpop_batch_item,
 * plain or segmented, whose buffers are device memory or page-locked host
 * memory and must stay valid until the step is done) and waits for it
 * (mrpop_session_wait; timeout_ms as above, MRPOP_ERR_DEVICE_TIMEOUT if the
 * step is still running).  The worker (a dispatcher thread) gathers the
 * steps pending from all sessions, in submission order, into a wave (up to
 * max_wave_steps steps, and up to max_wave_chunks chunks counted at 96 edges
 * each), cuts it into chunks of 6 to 96 edges so that even a small wave
 * spreads over the SMs, and launches it as one set of persistent batch kernels
 * on the next free slot's stream, so waves formed while others run overlap on
 * the device.  While waves are in flight the worker polls an event recorded
 * after each wave (one host core busy) and wakes each session whose steps are
 * done; with nothing in flight or pending it sleeps.  Each step's verdicts
 * equal the same mrpop_validate_edges / mrpop_validate_segments call made
 * alone.
 * mrpop_session_close waits for the session's step and returns its memory to
 * the arena.  Sessions may be used from different host threads; one session
 * is used by one thread at a time.  Close every session before
 * mrpop_server_destroy, which finishes the pending steps and frees the server.
 * A session also reserves page-locked host buffers for its steps in a host
 * arena of host_bytes (mrpop_session_host_buffers).  Zero in a config field
 * selects the default: 1 GiB, 4 streams, 1024 steps, 16384 chunks, 256 MiB,
 * 4096 fused edges.
 */
typedef struct {
    int64_t budget_bytes;    /* device arena for the sessions' step scratch            */
    int32_t streams;
    int32_t max_wave_steps;
    int64_t max_wave_chunks;
    int64_t host_bytes;      /* page-locked host arena for the sessions' buffers       */
    int64_t fused_edges;     /* groups of at most this many edges in a wave run as one
                                fused launch instead of the split kernels; -1: never   */
} mrpop_server_config;

typedef struct {
    int64_t budget_bytes;        /* arena size                                        */
    int64_t bytes_in_use;        /* reserved by open sessions now                     */
    int64_t peak_bytes_in_use;   /* largest reservation seen at an admission          */
    int64_t sessions;            /* sessions admitted                                 */
    int64_t admission_waits;     /* sessions that had to wait for room                */
    int64_t admission_timeouts;  /* sessions refused after waiting                    */
    int64_t waves;               /* waves launched                                    */
    int64_t steps;               /* steps launched                                    */
    int64_t max_wave_steps;      /* most steps in one wave                            */
    int64_t max_waves_in_flight; /* most waves on the device at once                  */
    int64_t kernel_launches;     /* validator kernels launched                        */
    int64_t queue_ns;            /* summed over steps: submit to its wave's launch    */
    int64_t flight_ns;           /* summed over steps: wave launch to wave done       */
    int64_t device_ns;           /* summed over waves: first to last command on the GPU */
} mrpop_server_stats;

typedef struct mrpop_server mrpop_server;
typedef struct mrpop_session mrpop_session;

mrpop_status mrpop_server_create(const mrpop_server_config *cfg, mrpop_server **out);
mrpop_status mrpop_server_destroy(mrpop_server *server);
mrpop_status mrpop_server_get_stats(mrpop_server *server, mrpop_server_stats *out);
mrpop_status mrpop_session_open(mrpop_server *server, int arms, int64_t max_edges, int max_granularity,
                                int64_t timeout_ms, mrpop_session **out);
mrpop_status mrpop_session_submit(mrpop_session *session, const mrpop_batch_item *step);
/* Several steps submitted together (at most MRPOP_SESSION_MAX_ITEMS, their
 * edge counts summing to at most the session's max_edges): they enter the
 * pending queue together, so they normally share one wave, and
 * mrpop_session_wait returns when all are done.  Each item keeps its own
 * arm count (at most the session's), granularity and rule. */
#define MRPOP_SESSION_MAX_ITEMS 16
mrpop_status mrpop_session_submit_many(mrpop_session *session, const mrpop_batch_item *steps, int n_steps);
mrpop_status mrpop_session_wait(mrpop_session *session, int64_t timeout_ms);
mrpop_status mrpop_session_close(mrpop_session *session);
/* The session's page-locked host buffers for its steps, carved from the host
 * arena the server reserved at start-up (host_bytes): q0 and q1 of
 * [max_edges][7 * arms] floats, valid [max_edges], first_hit [max_edges].  The
 * kernels read and write them in place, so a step may point at them. */
mrpop_status mrpop_session_host_buffers(mrpop_session *session, float **q0, float **q1, uint8_t **valid,
                                        int32_t **first_hit);

/*
 * A compact composite-space planner with the reference planner's step
 * pattern: batched extends (plain edges, pop_planner.cu:551-561), connect
 * checks of the new nodes towards the other tree (connect rule,
 * pop_planner.cu:666-703) and shortcut passes (shortcut rule,
 * path_simplification.cu:155-200).  It is the client that served planning
 * measures; the reference's dRRT/AO-x planner (Planners.hh:57-64) is not
 * rebuilt.  Deterministic given the seed and the verdicts.
 *
 * mrpop_plan runs it with any validator: validate(ctx, q0, q1, n, g, rule,
 * range, valid, first_hit) checks n host edges and returns 0 (or an
 * mrpop_status, which aborts the plan).  path_out (optional) receives up to
 * max_waypoints waypoints [7 * arms] from start to goal.
 * mrpop_session_plan runs it with its steps validated by the session (scene,
 * robots and flags as for mrpop_validate_edges, composite check), in the
 * session's host buffers; the session must allow max(batch, shortcut_pairs)
 * edges at the settings' granularity, and the robot set must have the
 * session's arm count.
 */
typedef int (*mrpop_validate_fn)(void *ctx, const float *q0, const float *q1, int64_t n_edges, int granularity,
                                 int rule, float range, uint8_t *valid, int32_t *first_hit);

typedef struct {
    int32_t batch;           /* extend targets per iteration (64)                      */
    int32_t max_iters;       /* extend iterations before giving up (60)                */
    int32_t granularity;     /* samples per edge and per segment (32)                  */
    int32_t shortcut_passes; /* passes after the first solution (5)                    */
    int32_t shortcut_pairs;  /* random (i<j) pairs per pass (32)                       */
    float step;              /* extend length, composite Euclidean in rad (1.0)        */
    float range;             /* segment length of connect and shortcut checks (1.0)    */
    uint64_t seed;
} mrpop_plan_settings;

typedef struct {
    int32_t solved;
    int32_t iterations;
    int32_t steps;           /* validate calls                                         */
    int64_t edges;           /* edges validated                                        */
    int64_t waypoints;
    double cost;             /* path length, composite Euclidean                       */
    uint64_t digest;         /* FNV-1a of every verdict received, in order             */
    int64_t start_tree;      /* nodes of the tree grown from the start                 */
    int64_t goal_tree;       /* nodes of the tree grown from the goal                  */
    int64_t validate_ns;     /* host wall time spent inside validate calls             */
} mrpop_plan_result;

mrpop_status mrpop_plan(int arms, const float *start, const float *goal, const mrpop_plan_settings *settings,
                        mrpop_validate_fn validate, void *ctx, float *path_out, int64_t max_waypoints,
                        mrpop_plan_result *out);
mrpop_status mrpop_session_plan(mrpop_session *session, const mrpop_scene *scene, const mrpop_robotset *robots,
                                uint32_t flags, const float *start, const float *goal,
                                const mrpop_plan_settings *settings, float *path_out, int64_t max_waypoints,
                                mrpop_plan_result *out);

/*
 * The reference's planner, dRRT with per-arm roadmaps under the AO-x
 * meta-algorithm (dRRT::solve, Planners.hh:57-64, pop_planner.cu:173-1030,
 * roadmap_interior.cuh:36-341, utils.cuh:688-759, path_simplification.cu:17-242),
 * rebuilt on this library's batched validator.  The reference runs it as
 * persistent kernels that check one edge per 256-thread block; here the host
 * steps all `num_new_configs` extension attempts of an iteration together and
 * validates their edges in one call per form:
 *   roadmap nodes and edges  single-arm form (fkcc_single_buffer_mr), one call
 *                            per arm and round (roadmap_interior.cuh:167-263)
 *   extend                   self only (fkcc_single_buffer_drrt, pop_planner.cu:551-564)
 *   connect                  env + self, connect segmentation (pop_planner.cu:624-703)
 *   B-spline smoothing       env + self, B-spline segmentation (path_simplification.cu:55-141)
 *   shortcut DP              env + self, shortcut segmentation (path_simplification.cu:143-233)
 * Tree nearest-neighbour searches (pop_planner.cu:472-507, 630-663) run as a
 * kernel over the trees, which live in page-locked host memory that the GPU
 * reads in place.  The algorithm follows the reference step for step
 * (sampling, balance strategy, direction oracle, cost bounds, PHS sampling in
 * the optimising passes, B-spline and shortcut passes); its races between
 * blocks are replaced by a fixed order (attempts in block order within an
 * iteration), and its random numbers come from seeded per-block streams of
 * this library, so a solve is deterministic given the seed and the verdicts.
 *
 * Settings: the fields of the reference's pop_settings (pop_settings.hh:3-32)
 * in order, bools as int32, then this library's additions.
 * mrpop_drrt_settings_default fills the reference's defaults (and
 * block_per_robot 8, max_launches 20, seed 1234, host_threads 0,
 * blocking_wait 0).  The result depends on neither host_threads nor
 * blocking_wait: they trade one solve's latency against the share of the
 * host that many concurrent solves leave each other.  dd_radius, dd_min_radius,
 * resample_iter, cost_bound_resample and the perturb fields are carried but
 * read nowhere, as in the reference; dynamic_domain is honoured as the
 * reference computes it (its radii never leave FLT_MAX, so it never prunes).
 *
 * mrpop_drrt_solve validates with this library's kernels on the current
 * device.  start: [7 * arms]; goals: [num_goals][7 * arms] (host).  The
 * robot set gives the arms and their bases (arm count 1-5).  path_out
 * (optional) receives up to max_waypoints waypoints of the best solution, in
 * the reference's order: from the goal to the start (record_connected_path,
 * path_processing.cu:11-70), simplified when path_simplify is set.
 * on_solution (optional) is called for every improving solution, as the
 * reference's copy_path_to_result (path_processing.cu:73-122) appends to
 * PlannerResult::seed_paths: the pass, its cost, the path as path_out has it,
 * and the unsimplified path of that pass.  The pointers are valid during the
 * call only.  The first pass repeats (one roadmap round, then up to max_iters
 * iterations) until it finds a solution, as the reference's does, but at most
 * max_launches times (the reference repeats without limit); trees are capped
 * at max_samples nodes.
 * mrpop_drrt_solve_with takes any validator (validate(ctx, q0, q1, n, g,
 * rule, range, flags, arm, valid, first_hit) checks n host edges, returns 0 or
 * an mrpop_status) and searches nearest neighbours on the host with the same
 * arithmetic, so the same settings, seed and verdicts give the same solve:
 * the CPU tests drive it with the oracle.
 */
typedef int (*mrpop_check_fn)(void *ctx, const float *q0, const float *q1, int64_t n_edges, int granularity,
                              int rule, float range, uint32_t flags, int arm, uint8_t *valid, int32_t *first_hit);
/* One check of a group handed to a validator at once (the planner's roadmap
 * rounds check every arm's nodes, then every arm's edges, as one group). */
typedef struct {
    const float *q0;
    const float *q1;
    int64_t n_edges;
    int32_t granularity;
    int32_t rule;
    float range;
    uint32_t flags;
    int32_t arm;
    uint8_t *valid;
    int32_t *first_hit;
} mrpop_check_call;
typedef void (*mrpop_drrt_solution_fn)(void *ctx, int32_t pass, float cost, const float *path, int64_t n_waypoints,
                                       const float *raw_path, int64_t n_raw);

typedef struct {
    int32_t max_samples;      /* tree capacity (1000000)                                  */
    int32_t max_iters;        /* iterations per launch (1000)                             */
    int32_t optimize_iters;   /* iteration cap of the optimising passes (400000)          */
    int32_t num_new_configs;  /* extension attempts per iteration (256)                   */
    int32_t granularity;      /* samples per edge and segment (16)                        */
    float range;              /* roadmap radius, connect and shortcut segment length (0.5) */
    int32_t balance;          /* 2: swap trees unless the other is twice as large (2)     */
    float tree_ratio;         /* (1.0)                                                    */
    int32_t dynamic_domain;   /* (0)                                                      */
    float dd_alpha;           /* (0.0001)                                                 */
    float dd_radius;          /* (4.0, unused)                                            */
    float dd_min_radius;      /* (1.0, unused)                                            */
    int32_t roadmap_reassign; /* connected arms' roadmap blocks help the others (0)       */
    int32_t rrtc_iter;        /* AO-x passes: the first finds a path, the rest optimise (1) */
    int32_t resample_iter;    /* (5, unused)                                              */
    int32_t cost_bound_resample; /* (0, unused)                                           */
    int32_t path_simplify;    /* B-spline and shortcut passes after every pass (1)        */
    int32_t phs;              /* informed (prolate hyperspheroid) sampling when optimising (1) */
    int32_t simplify_round;   /* (1)                                                      */
    int32_t bspline_step;     /* (3)                                                      */
    float bspline_min_change; /* (0.01)                                                   */
    int32_t perturb_step;     /* (3, unused)                                              */
    int32_t perturb_empty_step; /* (2, unused)                                            */
    /* this library's additions */
    int32_t block_per_robot;  /* roadmap blocks per arm, 230 samples each per round (8)   */
    int32_t max_launches;     /* bound on the first pass's roadmap + rrtc repeats (20)    */
    uint64_t seed;            /* random streams (1234, the reference's curand seed)       */
    int32_t host_threads;     /* host threads for the attempts' work; 0: all (0)          */
    int32_t blocking_wait;    /* 1: sleep while the call's device work runs; 0: spin (0)  */
} mrpop_drrt_settings;

typedef struct {
    int32_t solved;
    int32_t iters;            /* iteration of the attempt that found the reported solution */
    float cost;               /* the reported solution's cost after simplification        */
    int32_t passes;           /* passes run                                               */
    int32_t solutions;        /* improving solutions reported (on_solution calls)         */
    int32_t launches;         /* first-pass repeats                                       */
    int64_t start_tree_size;  /* tree sizes when the reported solution was found          */
    int64_t goal_tree_size;
    int64_t path_length;      /* waypoints of the reported path                           */
    int64_t roadmap_nodes[MRPOP_MAX_ARMS];
    int64_t roadmap_edges[MRPOP_MAX_ARMS];
    int64_t validate_calls;
    int64_t edges_validated;
    int64_t iterations;       /* rrtc iterations over all passes                          */
    int64_t wall_ns;          /* whole call                                               */
    int64_t kernel_ns;        /* from the first pass's start to the end (reference's kernel_ns) */
    int64_t validate_ns;      /* inside validate calls                                    */
    int64_t nn_ns;            /* inside nearest-neighbour searches                        */
    int64_t oracle_ns;        /* direction oracle and prunes of the attempts (host)       */
    int64_t roadmap_ns;       /* roadmap neighbour searches (host)                        */
    int64_t check_ns[5];      /* validate time by kind of check: roadmap (single-arm),    */
    int64_t check_calls[5];   /* extend (composite plain), connect, B-spline, shortcut    */
} mrpop_drrt_result;

mrpop_status mrpop_drrt_settings_default(mrpop_drrt_settings *out);
mrpop_status mrpop_drrt_solve(const mrpop_scene *scene, const mrpop_robotset *robots, const float *start,
                              const float *goals, int num_goals, const mrpop_drrt_settings *settings,
                              float *path_out, int64_t max_waypoints, mrpop_drrt_solution_fn on_solution,
                              void *solution_ctx, mrpop_drrt_result *out);
mrpop_status mrpop_drrt_solve_with(int arms, mrpop_check_fn validate, void *ctx, const float *start,
                                   const float *goals, int num_goals, const mrpop_drrt_settings *settings,
                                   float *path_out, int64_t max_waypoints, mrpop_drrt_solution_fn on_solution,
                                   void *solution_ctx, mrpop_drrt_result *out);
/* Device resources of the solves (a stream, the trees' device rows, staging
 * blocks, roadmap mirrors) are kept in a per-process pool between solves, so
 * that a stream of solves allocates and frees nothing once warm; at most 64
 * idle sets are kept.  mrpop_drrt_release_pool frees the idle sets (after
 * waiting for their streams) and returns how many it freed; sets in use by
 * running solves are untouched. */
int64_t mrpop_drrt_release_pool(void);
/* The same planner with its checks served by a session of the validation
 * service (below): every check becomes steps of at most the session's edge
 * count, co-batched with the steps of the other sessions, and each roadmap
 * round's checks of all arms go in as one mrpop_session_submit_many group;
 * the tree searches run on the device on a stream of the call's own.  The
 * session needs the robot set's arm count and a granularity of at least
 * settings->granularity. */
mrpop_status mrpop_session_drrt(mrpop_session *session, const mrpop_scene *scene, const mrpop_robotset *robots,
                                const float *start, const float *goals, int num_goals,
                                const mrpop_drrt_settings *settings, float *path_out, int64_t max_waypoints,
                                mrpop_drrt_solution_fn on_solution, void *solution_ctx, mrpop_drrt_result *out);

/* Algorithmic flop count per edge (FMA = 2; the convention of the project's
 * roofline) for the same arguments as mrpop_validate_segments; writes
 * flops[e] (device, double).  Runs the validator with counting enabled. */
mrpop_status mrpop_count_flops(const mrpop_scene *scene, const mrpop_robotset *robots,
                               const float *q0, const float *q1, int64_t n_edges,
                               int granularity, int rule, float range, uint32_t flags, int arm,
                               double *flops, void *stream);

/* Algorithmic flops of the broad phase per sample (FMA = 2) for a scene,
 * robot set, check flags and arm selection: FK of every arm, every env-tested
 * broad sphere against every obstacle, every intra-arm and arm-vs-arm broad
 * pair, with no culling.  Measurement utility, no counterpart in the
 * reference (the broad phase is utils.cuh:461-475 there). */
mrpop_status mrpop_broad_flops_per_sample(const mrpop_scene *scene, const mrpop_robotset *robots,
                                          uint32_t flags, int arm, double *out);

/* Per-kernel timing, a measurement utility with no counterpart in the
 * reference.  While enabled, every validate call records a pair of CUDA
 * events on its stream around each kernel it launches.  mrpop_kernel_times
 * waits for the recorded launches, writes per kernel kind (index
 * MRPOP_KERNEL_FUSED / _BROAD / _NARROW) the number of launches and their
 * summed device time in ms since the previous read, and releases the events.
 * Read on the device the launches ran on. */
#define MRPOP_KERNEL_KINDS 3
#define MRPOP_KERNEL_FUSED 0  /* segmented rules, segments after the split rounds: both phases in one kernel */
#define MRPOP_KERNEL_BROAD 1  /* broad phase (single-segment edges, or one segment round) */
#define MRPOP_KERNEL_NARROW 2 /* narrow phase (single-segment edges, or one segment round) */
mrpop_status mrpop_kernel_timing(int enable);
mrpop_status mrpop_kernel_times(int64_t *launches, double *ms);

/* Test utility, no counterpart in the reference: the host copy of the
 * forearm-hand rows table (bit i6 * n7 + i7 set when the detailed self rows
 * between the joint-5 spheres and the hand cannot fire for any (q6, q7) in
 * cell (i6, i7) of the joint-6 x joint-7 limit box, cells of equal size).
 * out needs n6 * n7 / 32 words; 3072 today. */
mrpop_status mrpop_debug_row5_table(uint32_t *out, int64_t words, int *n6, int *n7);

/* The kernels' bounded wait on a bulk copy, run out on purpose: one CTA waits
 * on an mbarrier whose bytes no copy will deliver, with limit_ns (at most 2 s)
 * in place of the kernels' 1 s.  The wait gives up, sets bit 0 of the status
 * word and returns: *status_out receives the word, *elapsed_ns_out the time
 * from the wait's start to its giving up (both waits).  Synchronous; the
 * context stays usable.  Tests the failure path that reports a scene status
 * (mrpop_scene_status) without a fault or a hang. */
mrpop_status mrpop_debug_wait_timeout(int64_t limit_ns, uint32_t *status_out, int64_t *elapsed_ns_out);

/* The __cosf/__sinf values the validator uses for inputs x (device arrays). */
mrpop_status mrpop_debug_trig(const float *x, int64_t n, float *cos_out, float *sin_out,
                              void *stream);

/* Measurement utility: launches `blocks` x 256 threads of an FP32 FMA loop
 * (scratch: >= blocks floats of device memory) and reports its flop count, so
 * a caller can time the FP32 issue peak that bounds the validator.  No
 * counterpart in the reference. */
mrpop_status mrpop_fp32_peak_probe(int blocks, int iters, float *scratch, double *flops_out, void *stream);

/* Last error message of the calling thread ("" if none). */
const char *mrpop_last_error(void);
/* Library version string. */
const char *mrpop_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MRPOP_H */
