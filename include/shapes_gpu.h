/*
 * shapes_gpu.h — C ABI of the GB300 world step for ublubu/shapes.
 *
 * This is the drop-in boundary for `Physics.Engine.Main`
 * (shapes/src/Physics/Engine/Main.hs:32-98): a Haskell caller keeps its
 * `EngineST` API and marshals world state through `foreign import ccall` into
 * device-resident structure-of-arrays buffers owned by this library.  Every
 * entry point is plain C: pointers, sizes, status codes.
 *
 * Conventions
 *   - Every function returns an int status: SHAPES_OK (0) or a negative
 *     SHAPES_E_* code.  Nothing aborts, exits or traps.
 *   - Host pointers passed in are only read during the call (copied).
 *     Out-buffers are caller-allocated; size them with the matching count
 *     query first.
 *   - A handle is single-threaded, like the reference's `ST` state thread.
 *     Different handles may be used from different threads; each owns a CUDA
 *     stream on the current device.
 *   - Body indices in keys and pairs are world-local slot indices, exactly the
 *     reference's World slot keys after `fromList` (World.hs:118-124).
 *   - Limits: at most 2^20 bodies per world, 3..64 vertices per convex hull
 *     (counter-clockwise, strictly convex); a circle is one local point
 *     (radius, 0).
 */
#ifndef SHAPES_GPU_H
#define SHAPES_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SHAPES_OK 0
#define SHAPES_E_INVALID_ARG (-1)
#define SHAPES_E_UNSUPPORTED (-2) /* more than 64 vertices, custom External */
#define SHAPES_E_NONCONVEX (-3)   /* hull not strictly convex and counter-clockwise */
#define SHAPES_E_CAPACITY (-4)    /* internal buffer could not grow */
#define SHAPES_E_CUDA (-5)        /* CUDA runtime error (no device, launch failure) */
#define SHAPES_E_TIMEOUT (-6)     /* a bounded device wait gave up */
#define SHAPES_E_NAN (-7)         /* non-finite body state passed in */
#define SHAPES_E_BUFFER (-8)      /* caller's out-buffer too small */

/* Shapes (Contact.hs:19-20 `data Shape`).  A hull is 3..64 counter-clockwise
 * local vertices (makeHull, Engine.hs:47-51).  A circle (makeCircle,
 * Engine.hs:53-54) is ONE local point (radius, 0) with 0 < radius < 2^500;
 * its centre is the body's position (circleWithRadius, Contact/Circle.hs:24-25). */
#define SHAPES_SHAPE_HULL 0
#define SHAPES_SHAPE_CIRCLE 1

/* External effects (World.hs:33 `type External`): the reference's closures
 * cannot cross the FFI; the two the reference's scenes use are supported. */
#define SHAPES_EXTERNAL_NONE 0           /* `const id` (Scenes/TwoFlyingBoxes.hs:30-31) */
#define SHAPES_EXTERNAL_CONSTANT_ACCEL 1 /* constantAccel (World/External.hs:23-28) */

#define SHAPES_WARM_START_OFF 0
#define SHAPES_WARM_START_CACHE 1 /* applyCachedSlns (Solvers/Contact.hs:74-121) */

/* Structure-of-arrays body state: PhysicalObj (Constraint.hs:52-57) plus
 * Material (World.hs:35-38).  inv_mass_* are the stored InvMass2 fields, i.e.
 * toInvMass2 (Constraint.hs:79-83) already applied: 0 means infinite mass. */
typedef struct shapes_bodies {
  double* vel_x;
  double* vel_y;
  double* rot_vel;
  double* pos_x;
  double* pos_y;
  double* rot;
  double* inv_mass_lin;
  double* inv_mass_rot;
  double* mu;
  double* bounce;
} shapes_bodies;

/* EngineConfig (Engine/Main.hs:34-37) + ContactBehavior (Contact/Types.hs:20-25)
 * + the External, plus the solver sweep count the reference hard-codes to 2
 * (Engine/Main.hs:81-82). */
typedef struct shapes_config {
  double dt;
  double baumgarte;
  double slop;
  double accel_x;
  double accel_y;
  int32_t iterations; /* improveWorld sweeps per step; 2 = reference */
  int32_t warm_start; /* SHAPES_WARM_START_* */
  int32_t external;   /* SHAPES_EXTERNAL_* */
  int32_t flags;      /* SHAPES_FLAG_* */
} shapes_config;

/* Compute the per-world solver residual after each step's last sweep
 * (readable with shapes_batch_get_world_metrics).  No counterpart in the
 * reference, which reports no solver metrics. */
#define SHAPES_FLAG_RESIDUAL 1
/* Worlds of SHAPES_LARGE_WORLD_BODIES bodies or more are solved by a
 * graph-coloured sweep (contacts coloured so that no two of a colour share a
 * dynamic body, colours swept one after another) instead of the default
 * order-preserving path; the coloured order differs from the reference's, so
 * its results differ too.  No counterpart in the reference. */
#define SHAPES_FLAG_COLOURED 2
#define SHAPES_LARGE_WORLD_BODIES 4096
/* Learned warm start: contacts without a cache entry (the `newCache` branch
 * of applyCachedSlns, Solvers/Contact.hs:91-98, where the reference starts
 * from zero) start from the Lagrangians the attached network predicts, in
 * worlds whose learned mask is set (shapes_batch_set_mlp).  The results then
 * differ from the reference's.  No counterpart in the reference. */
#define SHAPES_FLAG_LEARNED 4

/* Counters of the most recent step or collide call, summed over worlds.
 * pairs and contacts are those of the call's last step; cache_hits,
 * solver_items and solver_levels are summed over all steps of the call. */
typedef struct shapes_stats {
  int64_t pairs;
  int64_t contacts;
  int64_t cache_hits;
  int64_t solver_items;  /* warm-start applications + sweep updates */
  int64_t solver_levels; /* sum over steps and solver groups of dependency levels */
  int64_t retries;       /* buffer regrowths during the last call */
  int64_t predicted;     /* contacts started from the network, summed over the call */
  int64_t reverted;      /* worlds switched back to the plain start during the call */
} shapes_stats;

typedef struct shapes_batch shapes_batch;

/* Build `n_worlds` independent worlds in one handle.
 *   world_body_offsets[n_worlds+1]: bodies of world w are [off[w], off[w+1]).
 *   bodies: SoA arrays of length off[n_worlds].
 *   vert_offsets[n_bodies+1]: local points of body b are
 *     local_verts_xy[2*vert_offsets[b] .. 2*vert_offsets[b+1]).
 *   shape_kind: per body SHAPES_SHAPE_*, or NULL for all hulls.  A body whose
 *     kind does not match its points (a circle with other than one point
 *     (radius, 0), a hull with fewer than 3) is SHAPES_E_INVALID_ARG.
 * Shapes are posed from the bodies' positions on creation (makeWorldObj,
 * World.hs:142-149) and the contact cache starts empty (initEngine,
 * Engine/Main.hs:43-46).
 * Replaces: makeWorld/fromList (Engine.hs:41-42, World.hs:118-124), makeHull /
 * makeRectangleHull + listToHull (Engine.hs:47-51, ConvexHull.hs:151-167),
 * initEngine (Engine/Main.hs:43-46). */
int shapes_batch_create(int32_t n_worlds, const int32_t* world_body_offsets,
                        const shapes_bodies* bodies, const int32_t* vert_offsets,
                        const double* local_verts_xy, const uint8_t* shape_kind,
                        shapes_batch** out);

/* Advance every world by `nsteps` world steps.
 * Replaces: updateWorld (Engine/Main.hs:71-84) and stepWorld (Engine/Main.hs:88-89). */
int shapes_batch_step(shapes_batch* b, const shapes_config* cfg, int32_t nsteps);

/* Steps n handles (each on its own stream, see shapes_batch_set_stream) by
 * `nsteps` steps each, with all of them in flight at once: the solver of one
 * handle's worlds overlaps the other stages of another's.  Each handle ends
 * exactly as shapes_batch_step would leave it; the first failing status is
 * returned.  Two handles sharing a stream are SHAPES_E_INVALID_ARG.
 * No counterpart in the reference (a way to shard worlds on one GPU). */
int shapes_batches_step(shapes_batch* const* bs, int32_t n, const shapes_config* cfg, int32_t nsteps);

/* One step of n handles with the body state in and out of caller buffers,
 * everything asynchronous until one wait per handle: for each handle, in[k]
 * is uploaded and checked (as shapes_batch_set_bodies), the step runs and the
 * result is written to out[k] (as shapes_batch_get_bodies), with all handles'
 * copies and steps in flight at once.  A handle whose input holds a
 * non-finite value returns SHAPES_E_NAN with its state as before the call
 * (its out[k] is then unspecified).  Pinned host buffers are copied by a
 * kernel over the host link. */
int shapes_batches_step_io(shapes_batch* const* bs, int32_t n, const shapes_config* cfg, const shapes_bodies* in,
                           shapes_bodies* out);

/* Called on the host after step `step` of handle `handle_index` has written
 * its result into state[handle_index]; the caller may read and change that
 * state before the next upload: the values in its arrays, not the array
 * pointers, whose device addresses are resolved once per call.  Non-zero
 * stops that handle's loop.  Calls for different handles may come from
 * different threads at once. */
typedef int (*shapes_step_callback)(void* user, int32_t handle_index, int32_t step);

/* nsteps steps of n handles whose body state lives in caller host memory:
 * every step of handle k uploads and checks state[k] (as
 * shapes_batch_set_bodies), steps, writes the result back into state[k] (the
 * arrays a step changes: vel_x, vel_y, rot_vel, pos_x, pos_y, rot; the inverse
 * masses and material in state[k] are the values just uploaded) and waits for
 * it, then calls on_step (may be NULL).  Each handle runs its steps
 * in order on a host thread of its own, so one handle's copies and host turn
 * overlap the others' steps.  Pinned buffers are resolved once per call and
 * copied by a kernel over the host link.  Returns the first error; a handle
 * whose input holds a non-finite value stops with SHAPES_E_NAN, its device
 * state as before that step (state[k] is then unspecified); the others run
 * to the end.  No counterpart in the
 * reference (its state is a Haskell value that each updateWorld returns,
 * Engine/Main.hs:71-84). */
int shapes_batches_run_io(shapes_batch* const* bs, int32_t n, const shapes_config* cfg, int32_t nsteps,
                          shapes_bodies* state, shapes_step_callback on_step, void* user);

/* Broadphase + contact generation on the current poses only (no forces, no
 * solve); results readable with the pair/contact getters.
 * Replaces: G.culledKeys . G.toGrid (Engine/Main.hs:75) followed by
 * prepareFrame (Solvers/Contact.hs:40-52), as the demo's worldContacts query
 * does (shapes-demo/src/Physics/Demo/IOWorld.hs:74-81). */
int shapes_batch_collide(shapes_batch* b);

/* Body state read/write.  set validates on the device (SHAPES_E_NAN leaves the
 * state untouched), re-poses the shapes and keeps the cache.
 * Replaces: readPhysObj / updatePhysObj (World.hs:93-97). */
int shapes_batch_get_bodies(shapes_batch* b, shapes_bodies* out);
int shapes_batch_set_bodies(shapes_batch* b, const shapes_bodies* in);

/* Counts of the handle. */
int shapes_batch_num_worlds(shapes_batch* b, int32_t* out);
int shapes_batch_num_bodies(shapes_batch* b, int64_t* out);
int shapes_batch_num_vertices(shapes_batch* b, int64_t* out);

/* World-space hull vertices and unit edge normals of the current pose, in
 * vertex order (2 doubles each).  Replaces: reading _hullVertices /
 * _hullEdgeNormals of the posed Shape (ConvexHull.hs:61-68, World.hs:111-112). */
int shapes_batch_get_shapes(shapes_batch* b, double* world_xy, double* normal_xy);

/* Broadphase pairs of the last step/collide, descending (i, j), i > j,
 * world-local indices, worlds in order; world_counts[n_worlds] may be NULL.
 * Replaces: the Descending (Int, Int) keys of Aabb.culledKeys / Grid.culledKeys
 * (Aabb.hs:168-183, Grid.hs:257-261). */
int shapes_batch_num_pairs(shapes_batch* b, int64_t* out);
int shapes_batch_get_pairs(shapes_batch* b, int32_t* ij, int64_t capacity, int32_t* world_counts);

/* Contacts of the last step/collide in descending key order:
 * keys5 = (i, j, feature_i, feature_j, flip), vals5 = (normal x, normal y,
 * point x, point y, depth).
 * Replaces: the Descending (ObjectFeatureKey Int, Flipping Contact) of
 * prepareFrame (Solvers/Contact.hs:40-52, Constraints/Contact.hs:49-57). */
int shapes_batch_num_contacts(shapes_batch* b, int64_t* out);
int shapes_batch_get_contacts(shapes_batch* b, int32_t* keys5, double* vals5, int64_t capacity,
                              int32_t* world_counts);

/* Contact-solution cache: keys4 = (i, j, feature_i, feature_j), lam2 =
 * (normal, friction) Lagrangians, per world in descending key order.
 * set replaces the whole cache (checkpoint/resume); keys must be strictly
 * descending within each world.
 * Replaces: EngineCache (Engine/Main.hs:32) carried in EngineState. */
int shapes_batch_num_cache(shapes_batch* b, int64_t* out);
int shapes_batch_get_cache(shapes_batch* b, int32_t* keys4, double* lam2, int64_t capacity,
                           int32_t* world_counts);
int shapes_batch_set_cache(shapes_batch* b, const int32_t* world_counts, const int32_t* keys4,
                           const double* lam2);

int shapes_batch_get_stats(shapes_batch* b, shapes_stats* out);

/* Per-world metrics (arrays of n_worlds, either may be NULL).
 *   residual: RMS over the world's contacts of the normal and friction
 *     impulses one more sweep would apply after the last step's final sweep
 *     (needs SHAPES_FLAG_RESIDUAL on that step; NaN otherwise);
 *   max_depth: the largest contact depth on the current poses (the next
 *     step's contacts), found by running shapes_batch_collide.
 * No counterpart in the reference. */
int shapes_batch_get_world_metrics(shapes_batch* b, double* residual, double* max_depth);

/* Solver packing.  Worlds are sorted by size and packed into groups, one warp
 * per group; target_bodies_per_group > 0 closes a group once it holds that many
 * bodies (0 = automatic: about one warp of updates per dependency level);
 * threads = warps per CTA x 32, at most 256 (0 = 32).  Results do not depend
 * on the packing. */
int shapes_batch_set_launch(shapes_batch* b, int32_t target_bodies_per_group, int32_t threads);
/* Same, with a fixed number of worlds per warp group (1..32), as chosen by
 * shapes_batch_autotune. */
int shapes_batch_set_launch_groups(shapes_batch* b, int32_t worlds_per_group, int32_t threads);

/* Cooperative groups: 2, 4 or 8 warps share each group (one group per CTA;
 * the level's updates are spread over all of them, __syncthreads between
 * levels); 1 (default) = one warp per group, `threads` / 32 groups per CTA.
 * Results do not depend on it. */
int shapes_batch_set_group_warps(shapes_batch* b, int32_t warps);
/* Cooperative groups compute the dependency levels of the updates in
 * parallel (default 1): one walk over each world's contacts records every
 * update's predecessors, then the passes are levelled chunk by chunk to a
 * fixed point; 0 walks over every update in order, one thread per world.
 * Both give every update the same level. */
int shapes_batch_set_parallel_levels(shapes_batch* b, int32_t enabled);
int shapes_batch_get_parallel_levels(shapes_batch* b, int32_t* enabled);
/* Cooperative groups: launch the heaviest groups first, one per SM, then the
 * others lightest first (default 0: heaviest first throughout), so a heavy
 * group shares its SM with light ones.  Results do not depend on it. */
int shapes_batch_set_spread_heavy(shapes_batch* b, int32_t enabled);
int shapes_batch_get_spread_heavy(shapes_batch* b, int32_t* enabled);
/* The packing in use (any pointer may be NULL); worlds_per_group is 0 when
 * groups are packed by body count (shapes_batch_get_group_target). */
int shapes_batch_get_launch(shapes_batch* b, int32_t* worlds_per_group, int32_t* threads, int32_t* group_warps);
/* The body count at which groups close (shapes_batch_set_launch; the
 * autotuner tries such packings for batches of uneven world sizes), 0 when
 * they are packed by world count. */
int shapes_batch_get_group_target(shapes_batch* b, int32_t* target_bodies);
/* The order in which worlds are packed into groups: a permutation of
 * 0..n_worlds-1 (NULL = by body count, largest first, the default).  The
 * autotuner may choose an order by dependency levels; get_world_order reads
 * the one in use so that another handle of the same scene can reuse it. */
int shapes_batch_set_world_order(shapes_batch* b, const int32_t* order);
int shapes_batch_get_world_order(shapes_batch* b, int32_t* order);
/* Dependency levels of each world's last solve (0 for large worlds). */
int shapes_batch_get_world_levels(shapes_batch* b, int32_t* levels);

/* Autotuner for the solver packing: from the current state, times
 * `steps_per_trial` steps for each candidate (worlds per group x warps per
 * CTA, and worlds per group x warps per cooperative group x parallel or
 * walked dependency levels, each in size and in level order) after one untimed
 * step, restores the state exactly after every trial, and keeps the fastest (read it back with
 * shapes_batch_get_launch).  The world state and cache are left exactly as they were; results
 * never depend on the packing.  Tune on a state that has contacts (e.g. after
 * the scene settles).  chosen_* may be NULL.  Allocates temporary device
 * memory for the saved state. */
int shapes_batch_autotune(shapes_batch* b, const shapes_config* cfg, int32_t steps_per_trial,
                          int32_t* chosen_worlds_per_group, int32_t* chosen_threads);

/* Run this handle's device work on a caller-owned CUDA stream (a
 * cudaStream_t passed as void*), e.g. a framework's current stream; NULL
 * returns to the handle's own stream.  The stream must stay valid while set. */
int shapes_batch_set_stream(shapes_batch* b, void* cuda_stream);

/* CUDA-graph replay of the step (default on): each step is captured once per
 * configuration and buffer layout and replayed with one graph launch; steps
 * are launched kernel by kernel while profiling, or when the stream is a
 * legacy default stream or already capturing.  Results are identical either
 * way. */
int shapes_batch_set_graphs(shapes_batch* b, int32_t enabled);

/* Incremental grid pairs (on by default).  Worlds on the grid broadphase
 * keep, per body, a fat box (its AABB grown by 1/32 of the world's cell size)
 * and the list of bodies whose fat boxes overlap it; only bodies whose AABB
 * left their fat box are searched again, and each row's pairs are the listed
 * bodies whose current AABBs overlap.  The pair list is identical either way;
 * off = every grid body searches its 3x3 cells every frame.
 * Replaces: nothing in the reference (Broadphase/Grid.hs:67-141 rebuilds the
 * grid every frame); the pair contract of culledKeys (Aabb.hs:168-183) stays. */
int shapes_batch_set_incremental(shapes_batch* b, int32_t enabled);

/* Sweep and prune for large worlds (off by default: min_bodies = 0).  With
 * incremental pairs off, grid worlds of at least min_bodies bodies pair their
 * small bodies by sorting them on their boxes' lower x (a counting sort over
 * 65,536 buckets of the world's range) and sweeping forward from each body
 * while the candidates' lower x can still reach its upper x, instead of
 * searching 3x3 grid cells; bodies too large for the grid keep their own
 * rows.  The pair list is identical either way (exact overlap test, rows
 * sorted descending).  Replaces: nothing in the reference
 * (Broadphase/Aabb.hs:155-183 tests every pair; the pair contract of
 * culledKeys stays). */
int shapes_batch_set_sweep_prune(shapes_batch* b, int32_t min_bodies);

/* Lanes per pair in the narrowphase: 1 (default) runs one pair per thread;
 * 2, 4, 8, 16 or 32 split each pair's separating-axis search over that many
 * lanes of a warp (32: one warp per pair) and reduce it with shuffles, then
 * build the manifold on the pair's first lane.  The contacts are identical
 * either way.  Replaces: nothing (SAT.hs:121-138's minOverlap fold is kept
 * exactly, including which axis wins among equal or NaN depths). */
int shapes_batch_set_narrowphase_lanes(shapes_batch* b, int32_t lanes);

/* The order-preserving solve of large worlds waits for each update's
 * predecessors by polling completion counts; a lane that polls one dependency
 * more than `polls` times (default 2^22, restored by 0) makes the step return
 * SHAPES_E_TIMEOUT, with the state of the steps that ran partly solved.  The
 * next run starts with the flag clear.  No counterpart in the reference. */
int shapes_batch_set_wait_limit(shapes_batch* b, int64_t polls);

/* Per-stage device timing.  While enabled, CUDA events on the handle's stream
 * bracket each stage of every step; get_profile returns the accumulated
 * milliseconds and kernel launches per stage since profiling was enabled or
 * last read (reading resets).  Stages, in order: broadphase, narrowphase,
 * constraint build, solver schedule, solver, integrate+pose, scans/offsets,
 * learned warm start (features, network, judge, sample collection). */
#define SHAPES_STAGE_COUNT 8
int shapes_batch_set_profiling(shapes_batch* b, int32_t enabled);
int shapes_batch_get_profile(shapes_batch* b, double* ms, int64_t* launches);
/* While profiling: per solver group of the last step, 8 int64 each
 * (clock at start, after the dependency scan, after the level sort, at end;
 * dependency levels; updates; bodies; worlds).  *n_groups receives the group
 * count; `out` may be NULL to query it. */
int shapes_batch_get_group_clocks(shapes_batch* b, int64_t* out, int32_t* n_groups);

void shapes_batch_destroy(shapes_batch* b);

/* ---- Contact generation without allocation ----------------------------------
 * No counterpart in the reference.  An extra entry point for callers that
 * cannot allocate device memory themselves: plugins whose host application
 * owns every device buffer and hands out pre-planned memory, and loops with a
 * latency budget in which cudaMalloc/cudaFree (they synchronize the whole
 * device) are not allowed.  It runs the same broadphase and contact
 * generation as shapes_batch_collide on one world given entirely as device
 * pointers (inputs and outputs), and its scratch memory is a fixed array
 * inside the library, so it calls no cudaMalloc, cudaFree or allocating
 * library routine.
 *   Limits: n_bodies <= SHAPES_NOALLOC_MAX_BODIES, n_verts <=
 *   SHAPES_NOALLOC_MAX_VERTS, broadphase pairs <= SHAPES_NOALLOC_MAX_PAIRS;
 *   beyond them it returns SHAPES_E_CAPACITY.  The array (about 10 MB) is
 *   held by every GPU that loads the library until the process exits.
 *   The call cannot be captured into a CUDA graph: it synchronizes
 *   `cuda_stream` and reads counters on the host between kernels.  The first
 *   call on a device looks up the array's device address
 *   (cudaGetSymbolAddress) and keeps it for the life of the process: after
 *   cudaDeviceReset on that device the function must not be called again.
 *   All calls share the one array: calls that overlap on the GPU (different
 *   streams, threads or processes sharing the library) race.  The call
 *   synchronizes `cuda_stream` (NULL = legacy default stream) before it
 *   returns, so consecutive calls on one stream are safe.
 *   Inputs (device): pos_x, pos_y, rot, inv_mass_lin, inv_mass_rot [n];
 *   vert_offsets [n+1]; local_verts_xy [2*n_verts].  Only convex hulls are
 *   accepted (no circles): every body needs 3..64 vertices (vert_offsets[0]
 *   = 0, vert_offsets[n] = n_verts) forming a strictly convex,
 *   counter-clockwise polygon of finite points, and finite position, angle
 *   and inverse masses.  These are checked on the device before any other
 *   kernel runs: bad offsets or a zero-length edge give
 *   SHAPES_E_INVALID_ARG, a non-finite value SHAPES_E_NAN, a hull that is not
 *   strictly convex and counter-clockwise SHAPES_E_NONCONVEX (as
 *   shapes_batch_create), with the reason in shapes_last_error_detail.
 *   Outputs (device): pairs_ij [2*pair_capacity],
 *   contact_keys5 / contact_vals5 [5*contact_capacity] in the layouts of
 *   shapes_batch_get_pairs / shapes_batch_get_contacts; *n_pairs and
 *   *n_contacts (host) are set even when the capacities are too small
 *   (SHAPES_E_BUFFER). */
#define SHAPES_NOALLOC_MAX_BODIES 4096
#define SHAPES_NOALLOC_MAX_VERTS 32768
#define SHAPES_NOALLOC_MAX_PAIRS 32768
int shapes_collide_noalloc(int32_t n_bodies, const double* pos_x, const double* pos_y, const double* rot,
                           const double* inv_mass_lin, const double* inv_mass_rot, const int32_t* vert_offsets,
                           const double* local_verts_xy, int32_t n_verts, int32_t* pairs_ij,
                           int64_t pair_capacity, int32_t* contact_keys5, double* contact_vals5,
                           int64_t contact_capacity, void* cuda_stream, int64_t* n_pairs,
                           int64_t* n_contacts);

/* ------------------------------------------------------------------------ */
/* Learned warm start (no counterpart in the reference)                      */
/* ------------------------------------------------------------------------ */

/* A 16 -> 64 -> 64 -> 64 -> 2 ReLU network (BF16 tensor-core products, FP32
 * accumulation, FP32 master weights) mapping 16 contact features to the
 * starting normal and friction Lagrangians of a contact without a cache
 * entry.  Parameters: 9538 floats, W1[64][16] b1[64] W2[64][64] b2[64]
 * W3[64][64] b3[64] W4[2][64] b4[2] (row = output).  Normalisation: 36
 * floats, feature mean[16], feature 1/scale[16], target mean[2], target
 * scale[2]; the network sees (f - mean) / scale clipped to [-8, 8] and predicts
 * (target - mean) / scale.  Features, in order: J_n.v, J_f.v, b_n, J_n M^-1
 * J_n^T, J_f M^-1 J_f^T, the isolated normal and friction updates, pair
 * friction, depth, normal x, normal y, one step of acceleration as a normal
 * impulse, contacts of the pair, one-body-static flag, the two angular
 * entries of the normal row. */
#define SHAPES_MLP_PARAMS 9538
#define SHAPES_MLP_NORM 36
#define SHAPES_MLP_FEATURES 16
typedef struct shapes_mlp shapes_mlp;

typedef struct shapes_train_config {
  int32_t epochs;
  int32_t batch; /* samples per Adam step, a multiple of 128 */
  float lr;      /* Adam learning rate (beta1 0.9, beta2 0.999, eps 1e-8) */
  uint64_t seed; /* shuffling */
} shapes_train_config;

/* He-uniform initialisation from `seed`; identity normalisation. */
int shapes_mlp_create(uint64_t seed, shapes_mlp** out);
void shapes_mlp_destroy(shapes_mlp* m);
int shapes_mlp_get_params(shapes_mlp* m, float* params, float* norm);
/* Either pointer may be NULL; new parameters reset the Adam state. */
int shapes_mlp_set_params(shapes_mlp* m, const float* params, const float* norm);
/* Sets the normalisation to the mean and standard deviation of a dataset. */
int shapes_mlp_fit_normalization(shapes_mlp* m, const float* features, const float* targets, int64_t n);
/* Predictions (de-normalised, unclamped) for n feature rows. */
int shapes_mlp_forward(shapes_mlp* m, const float* features, int64_t n, float* out2);
/* Gradient of the mean over n samples (n <= 2^20) of the squared error of
 * the normalised outputs; *loss gets that mean.  No update. */
int shapes_mlp_gradient(shapes_mlp* m, const float* features, const float* targets, int64_t n,
                        float* grad, float* loss);
/* Adam on the GPU over shuffled mini-batches; epoch_loss[e] (optional) is
 * epoch e's mean loss. */
int shapes_mlp_train(shapes_mlp* m, const float* features, const float* targets, int64_t n,
                     const shapes_train_config* tc, float* epoch_loss);

/* Attaches a network to a handle (NULL detaches).  The handle reads the
 * network's device parameters at each step; keep it alive while attached.
 * Every world's learned mask is set. */
int shapes_batch_set_mlp(shapes_batch* b, const shapes_mlp* m);
/* Per-world learned mask (n_worlds bytes, 1 = predicted start).  The judge
 * clears a world's byte when, after a step with SHAPES_FLAG_LEARNED, the
 * world's residual exceeds max_residual[w] or its largest contact depth
 * exceeds max_depth[w] (shapes_batch_set_judge); the world then starts from
 * the plain cache until its byte is set again. */
int shapes_batch_get_learned_mask(shapes_batch* b, uint8_t* mask);
int shapes_batch_set_learned_mask(shapes_batch* b, const uint8_t* mask);
/* Per-world limits of the judge (n_worlds doubles each; NULL = no limit). */
int shapes_batch_set_judge(shapes_batch* b, const double* max_residual, const double* max_depth);
/* Training samples: while capacity > 0, every step appends, for each contact
 * without a cache entry, its 16 features (before the solve) and its final
 * normal and friction Lagrangians (after the last sweep), up to `capacity`
 * samples in all.  capacity 0 stops and frees the buffer. */
int shapes_batch_collect(shapes_batch* b, int64_t capacity);
int shapes_batch_get_samples(shapes_batch* b, float* features, float* targets, int64_t capacity,
                             int64_t* n);

/* ------------------------------------------------------------------------ */
/* World mutation                                                             */
/* ------------------------------------------------------------------------ */

/* World.delete (World.hs:90-91) = EmptiesVector.safeDelete
 * (Utils/EmptiesVector.hs:57-69): the slot (world-local index) must be filled
 * (else SHAPES_E_INVALID_ARG); it becomes empty and the top of the world's
 * empty-slot stack.  An empty slot keeps its last state, takes no part in the
 * step and keeps its index, so contact keys of the other bodies do not change. */
int shapes_batch_delete_body(shapes_batch* b, int32_t world, int32_t slot);
/* World.append (World.hs:83-89) = EmptiesVector.append
 * (Utils/EmptiesVector.hs:72-86): fills the top of the world's empty-slot
 * stack (the slot freed last); with no empty slot the world grows by one slot
 * at its end (the reference's fixed-capacity vector would be full).  body10
 * holds the ten shapes_bodies fields of the new body in order; n_verts 1 is a
 * circle (local point (radius, 0)), 3..64 a hull; the shape is posed at once
 * (makeWorldObj, World.hs:142-149).  *slot receives the slot. */
int shapes_batch_append_body(shapes_batch* b, int32_t world, const double* body10, int32_t n_verts,
                             const double* local_verts_xy, int32_t* slot);
/* Filled (1) or empty (0) per slot, over all worlds' slots (n_bodies bytes). */
int shapes_batch_get_active(shapes_batch* b, uint8_t* out);

/* ------------------------------------------------------------------------ */
/* Checkpoint file of the engine state                                        */
/* ------------------------------------------------------------------------ */

/* EngineState (Engine/Main.hs:32-33) = World + EngineCache, written as one
 * little-endian file: "SHAPESCK", uint32 version (1), uint32 0x01020304,
 * int32 n_worlds, int32 n_bodies, int64 n_vertices, int64 n_cache, then
 * int32 world_body_offsets[n_worlds+1], int32 vert_offsets[n_bodies+1],
 * double local_xy[2 n_vertices], double bodies[10][n_bodies] (the
 * shapes_bodies fields in order), int32 cache_world_counts[n_worlds],
 * int32 cache_keys[4 n_cache], double cache_lambdas[2 n_cache], uint8
 * filled[n_bodies] (World.delete / append), int32 empty_count[n_worlds], the
 * worlds' empty-slot stacks (int32, bottom to top, world by world), and a
 * uint64 FNV-1a hash of everything before it.  save writes path + ".tmp" then
 * renames it; load checks the hash and the sizes and builds a new handle that
 * continues bit for bit where the saved one stopped.  The External and the
 * step configuration are not part of it (they are passed to every step). */
int shapes_batch_save(shapes_batch* b, const char* path);
int shapes_batch_load(const char* path, shapes_batch** out);

/* Single-world convenience wrappers over a batch of one world. */
int shapes_world_create(int32_t n_bodies, const shapes_bodies* bodies, const int32_t* vert_offsets,
                        const double* local_verts_xy, const uint8_t* shape_kind,
                        shapes_batch** out);

/* Human-readable text for a status code (static storage). */
const char* shapes_strerror(int status);

/* Text of the last CUDA error seen by any handle on this thread (static
 * storage, empty if none). */
const char* shapes_last_error_detail(void);

#ifdef __cplusplus
}
#endif

#endif /* SHAPES_GPU_H */
