/*
 * ogx.h -- C ABI of the GB300 batched GJK distance / EPA penetration engine.
 *
 * Every function returns an ogx_status (0 = OGX_OK); on failure
 * ogx_last_error() gives a message for the calling thread.  There is no CPU
 * fallback: without a usable GPU the calls fail with OGX_ERR_NO_DEVICE.
 *
 * Two layers:
 *   1. Engine API (ogx_ctx / ogx_pool): a device-resident polytope pool in the
 *      engine's padded SoA layout, batched queries over pairs of pool indices on
 *      device buffers, asynchronous on the context's stream.
 *   2. Reference-compatible entry points (ogx_compute_*, ogx_allocate_*, ...):
 *      the functions of OpenGJK-GPU's host API with the same arguments, meaning
 *      and output conventions, each replacing the reference function cited beside
 *      it.  opengjk_gpu.hpp wraps them under the reference's C++ names
 *      (GJK::GPU::computeDistances, compute_minimum_distance, ...).
 *
 * Output conventions (as the reference, GJK/gpu/openGJK.h:52-64, GJK/cpu/EPA.c):
 *   distance >= 0 for separated pairs, 0 when GJK finds the origin enclosed, and
 *   -penetration depth after EPA; witnesses in simplex.witnesses[0] (body 1) and
 *   [1] (body 2); contact normal unit length from body 1 towards body 2, (1,0,0)
 *   when undefined.
 */
#ifndef OGX_H_
#define OGX_H_

#include <stddef.h>
#include <stdint.h>

#include "ogx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int ogx_status;
#define OGX_OK 0
#define OGX_ERR_INVALID (-1)   /* bad argument: null pointer, negative size, bad index */
#define OGX_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define OGX_ERR_NOMEM (-3)     /* device or pinned host allocation failed */
#define OGX_ERR_NO_DEVICE (-4) /* no usable GPU */
#define OGX_ERR_CAPACITY (-5)  /* a size exceeds a capacity of the call */
#define OGX_ERR_BUSY (-6)      /* a wait timed out (serving loop) */

/* Run-time tolerances.  ogx_config_default() fills the engine defaults (FP32 bulk,
 * FP64 escalation and polish, distances to ~1e-5 relative of the FP64 oracle);
 * ogx_config_reference() the reference's FP32 constants (GJK/cpu/openGJK.c:41-42,
 * 955; GJK/cpu/EPA.c:46, 592). */
typedef struct ogx_config {
  float gjk_eps_rel;  /* GJK stops when |v|^2 - v.w <= eps_rel |v|^2 */
  float gjk_eps_tot;  /* ... or when |v|^2 - v.w < eps_tot */
  float gjk_noise;    /* ... or when |v|^2 - v.w is below noise * FLT_EPSILON |v|(|v|+|w|) */
  int gjk_max_iter;   /* GJK iteration cap (reference: 25) */
  float epa_tol;      /* EPA stops when the support improves the closest face by < tol */
  float epa_rel;      /* ... or by < epa_rel * (scale of the polytope) */
  float epa_vis;      /* face visibility threshold relative to the polytope scale */
  int epa_max_iter;   /* EPA iteration cap (reference: 64) */
  int flags;          /* OGX_FLAG_* */
  float polish_rel;   /* >= 0; no longer read: with OGX_FLAG_FP64_POLISH every separated
                       * pair's final simplex is certified and re-solved, or continued, in
                       * FP64 (the field keeps the structure's layout) */
} ogx_config;

#define OGX_FLAG_FP64_ESCALATE 1 /* near-degenerate steps re-run in FP64 */
#define OGX_FLAG_FP64_POLISH 2   /* final simplex / EPA face re-solved in FP64 */
#define OGX_FLAG_REFERENCE_TOL 4 /* reference termination rules */
#define OGX_FLAG_EPA_FP64_PLANES 8 /* every EPA face plane solved in FP64 (the engine
                                    * turns this on itself for contacts whose FP32
                                    * expansion ran out of room or met an inconsistent
                                    * horizon: they are run again from the start) */

/* Per-pair status bits (optional output of the engine API). */
#define OGX_PAIR_GJK_CAP 1
#define OGX_PAIR_GJK_ESCALATED 2
#define OGX_PAIR_POLISHED 4
#define OGX_PAIR_EPA_RUN 8
#define OGX_PAIR_EPA_CONVERGED 16
#define OGX_PAIR_EPA_DUPLICATE 32
#define OGX_PAIR_EPA_CAP 64
#define OGX_PAIR_EPA_TOUCH 128
#define OGX_PAIR_EPA_TOPOLOGY 256
#define OGX_PAIR_EPA_CAPACITY 512
#define OGX_PAIR_EPA_ESCALATED 1024
#define OGX_PAIR_EPA_CERTIFIED 2048 /* the expansion ran again with FP64 planes and exact
                                     * supports until the FP64 test converged */
#define OGX_PAIR_BAD_INPUT 16384

ogx_status ogx_config_default(ogx_config* cfg);
ogx_status ogx_config_reference(ogx_config* cfg);
const char* ogx_status_string(ogx_status s);
const char* ogx_last_error(void);
/* library version string and the CUDA architecture it was built for */
const char* ogx_version(void);

/* ------------------------------------------------------------------------- */
/* Engine API                                                                 */

/* Pools, graphs and broad-phase objects refer to the context they were created with:
 * destroy them before that context. */
typedef struct ogx_ctx ogx_ctx;
typedef struct ogx_pool ogx_pool;

/* Context on `device` (current device when < 0).  `stream` is a cudaStream_t (NULL:
 * the context creates its own non-blocking stream).  cfg NULL = defaults. */
ogx_status ogx_ctx_create(int device, const ogx_config* cfg, void* stream, ogx_ctx** out);
ogx_status ogx_ctx_destroy(ogx_ctx* ctx);
ogx_status ogx_ctx_set_config(ogx_ctx* ctx, const ogx_config* cfg);
ogx_status ogx_ctx_get_config(const ogx_ctx* ctx, ogx_config* cfg);
ogx_status ogx_ctx_set_stream(ogx_ctx* ctx, void* stream);
void* ogx_ctx_stream(const ogx_ctx* ctx);
ogx_status ogx_ctx_synchronize(ogx_ctx* ctx);

/* Pool of num_bodies polytopes; body b has counts[b] >= 1 points (host array).
 * Device memory: 12 bytes per point plus padding to 4 points per body. */
ogx_status ogx_pool_create(ogx_ctx* ctx, int num_bodies, const int32_t* counts, ogx_pool** out);
ogx_status ogx_pool_destroy(ogx_pool* pool);
int ogx_pool_num_bodies(const ogx_pool* pool);
int64_t ogx_pool_num_points(const ogx_pool* pool);
/* Load all points: xyz interleaved, bodies concatenated in index order (host memory,
 * pinned or pageable).  Asynchronous on the context's stream.  Page-locked sources are
 * read by the packing kernel directly over the host link (keep them unchanged until the
 * stream passes the call, as for any asynchronous copy).  Pageable ones are read by the
 * packing kernel directly too where the device reads pageable memory through the host's
 * page tables (a Grace system), and the call returns once they are packed; elsewhere (or
 * with OGX_UPLOAD_STAGED=1 in the environment) they are staged through the context's
 * pinned buffer. */
ogx_status ogx_pool_upload(ogx_ctx* ctx, ogx_pool* pool, const float* coords);
/* Same from device memory (xyz interleaved, concatenated): a packing kernel. */
ogx_status ogx_pool_load_device(ogx_ctx* ctx, ogx_pool* pool, const float* d_coords);
/* Device pointer of the SoA points and of the per-body {quad offset, count} table
 * (for callers that write the pool with their own kernels). */
ogx_status ogx_pool_device_layout(const ogx_pool* pool, float** d_points, void** d_bodies);

/* GJK over npairs pairs of pool indices (device buffers, asynchronous).
 * d_status may be NULL. */
ogx_status ogx_gjk(ogx_ctx* ctx, const ogx_pool* pool, int npairs, const gkCollisionPair* d_pairs,
                   ogx_simplex_f32* d_simplices, float* d_distances, int32_t* d_status);
/* GJK then EPA on the pairs in contact (fused pipeline; d_normals n*3 floats). */
ogx_status ogx_gjk_epa(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                       const gkCollisionPair* d_pairs, ogx_simplex_f32* d_simplices,
                       float* d_distances, float* d_normals, int32_t* d_status);
/* EPA only, from simplices and distances of an earlier GJK (in/out). */
ogx_status ogx_epa(ogx_ctx* ctx, const ogx_pool* pool, int npairs, const gkCollisionPair* d_pairs,
                   ogx_simplex_f32* d_simplices, float* d_distances, float* d_normals,
                   int32_t* d_status);

/* Kernels launched by the last engine call on this context (for accounting). */
int ogx_ctx_last_launches(const ogx_ctx* ctx);
/* Per-launch timing: when on, each batched call records CUDA events on the context's
 * stream between its launches.  ogx_ctx_kernel_times waits for the last call and
 * fills up to cap (name, milliseconds) entries; returns the number filled. */
ogx_status ogx_ctx_set_timing(ogx_ctx* ctx, int on);
int ogx_ctx_kernel_times(ogx_ctx* ctx, const char** names, float* ms, int cap);
/* Stage timeline of the concurrent (forked) launches, for finding the chain that sets a
 * call's duration: with it on, each call records an event after every bucket's GJK and
 * EPA kernel on that bucket's stream and after the refinement, the late pass, the spill
 * pass, the polish pass and the final join.  ogx_ctx_stage_timeline waits for the last
 * call and fills up to cap (name, ms from the call's start) entries; returns the number
 * filled.  Not recorded while a graph is being captured or with per-kernel timing on. */
ogx_status ogx_ctx_set_stage_timeline(ogx_ctx* ctx, int on);
int ogx_ctx_stage_timeline(ogx_ctx* ctx, const char** names, float* ms, int cap);
/* Work counts of the last call (waits for it): pairs per GJK bucket [0, 7), contacts
 * per EPA bucket [7, 14), EPA faces re-solved in FP64 [14], pairs whose GJK result was
 * refined in FP64 [15], of which continued in FP64 (uncertain FP32 support) [16],
 * contacts whose EPA outgrew the bucket kernels' working set and ran again at full
 * capacity [17], FP64 continuations of pairs with a body above 128 points (one warp
 * each; the others in [16] - [18] run one thread each) [18], contacts that only the
 * FP64 refinement found (certified full-capacity EPA) [19], capacity spills whose
 * expansion the full-capacity pass continued instead of restarting [20] (at most 4096 per
 * call).  cap must be >= 21. */
int ogx_ctx_work_counts(ogx_ctx* ctx, int32_t* counts, int cap);

/* Kernel variant per size bucket (bucket b holds pairs whose larger body has at most
 * 16 * 2^b points, bucket 6 the rest): `lanes` lanes per pair, `blocks` float4 blocks of
 * x, y, z per lane and body kept in registers (0: points re-read from memory).
 * kind 0 = GJK, 1 = EPA. */
ogx_status ogx_ctx_get_kernel_choice(const ogx_ctx* ctx, int kind, int bucket, int* lanes,
                                     int* blocks);
ogx_status ogx_ctx_set_kernel_choice(ogx_ctx* ctx, int kind, int bucket, int lanes, int blocks);
/* Autotuner: times every compiled variant that can serve each bucket on this batch
 * (device buffers; `reps` runs per candidate, kernels one after another, best time
 * kept) and takes the fastest per bucket; since a call runs the buckets concurrently, it
 * then times whole calls with that set and with the context's previous one and keeps
 * the faster, for this context and for contexts created later on the same device.
 * Synchronous. */
ogx_status ogx_autotune(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                        const gkCollisionPair* d_pairs, int reps);

/* Device broad phase (uniform grid): every pair i < j of a pool's bodies whose
 * axis-aligned boxes, each grown by `margin`, overlap - exactly once, sorted by (i, j).
 * The pairs feed the GJK/EPA calls directly (d_pairs).  `cell` is the grid cell size:
 * any positive value gives the same pairs, a cell near the largest box extent the least
 * work; a box may touch at most 64 cells.  Writes min(count, max_pairs) pairs and
 * d_result[0] = count (all overlapping pairs, may exceed max_pairs), d_result[1] = error
 * flags (1: a box beyond 2^20 cells from the origin, 2: a box touching more than 64
 * cells; such bodies get no pairs).  Asynchronous on the context's stream.
 * Replaces the per-frame grid of the reference's visualiser
 * (visualization/integrate_final_gjk.cu:467-570, 916-1002). */
typedef struct ogx_broad ogx_broad;
ogx_status ogx_broad_create(ogx_ctx* ctx, int max_bodies, ogx_broad** out);
ogx_status ogx_broadphase(ogx_broad* broad, const ogx_pool* pool, float cell, float margin,
                          int max_pairs, gkCollisionPair* d_pairs, int* d_result);
ogx_status ogx_broad_destroy(ogx_broad* broad);
/* Candidate pairs with the reference's own broad-phase semantics
 * (visualization/integrate_final_gjk.cu:467-570: insert_objects_kernel /
 * count_pairs_kernel / generate_pairs_kernel): d_spheres[num_bodies] = float4 (x, y, z,
 * bounding radius); each sphere belongs to the grid cell of its centre,
 * floor((p + boundary) / cell) per axis clamped to [0, grid_size); pairs (i, j > i) are
 * the spheres in i's 27 neighbouring cells with fx*fx + fy*fy + fz*fz < (r_i + r_j)^2 in
 * FP32.  The pairs are written sorted by (i, j); d_result[0] = pairs found (may exceed
 * max_pairs: the first max_pairs are written), d_result[1] = 0.  The reference caps the
 * bodies stored per cell and drops the rest in an atomic-dependent order; this mode has
 * no such cap, so the pair sets are equal wherever no reference cell overflows. */
ogx_status ogx_broadphase_spheres(ogx_broad* broad, const float* d_spheres, int num_bodies, float cell,
                                  float boundary, int grid_size, int max_pairs, gkCollisionPair* d_pairs,
                                  int* d_result);

/* GJK then EPA from host memory to host memory in one call, with the transfers
 * overlapped with the kernels: the pool's points (xyz of all bodies, concatenated, as
 * for ogx_pool_upload) and the pairs go up in `chunks` pieces on a copy stream; each
 * piece of the pairs runs as soon as the bodies it references are on the device; its
 * results come back on a second copy stream while later pieces compute.  Returns when
 * every result is in the host arrays (status may be NULL).  Page-locked host arrays
 * let the copies run beside the kernels.  Leaves the pool loaded with xyz. */
ogx_status ogx_gjk_epa_streamed(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs,
                                const gkCollisionPair* pairs, ogx_simplex_f32* simplices,
                                float* distances, float* normals, int32_t* status, int chunks);

/* ogx_gjk_epa_streamed with the caller's pieces: pair range j is
 * [pair_bounds[j], pair_bounds[j + 1]) (nranges + 1 non-decreasing bounds from 0 to
 * npairs, 1 <= nranges <= 64), and up to `lanes` ranges compute side by side
 * (1..8; 0 = the default, 4).  Body range j goes up with pair range j and holds the
 * bodies that pair range j is the first to reference, so pairs listed in body order
 * start computing early.  ogx_gjk_epa_streamed(..., chunks) is this call with
 * `chunks` equal ranges. */
ogx_status ogx_gjk_epa_streamed_ranges(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs,
                                       const gkCollisionPair* pairs, ogx_simplex_f32* simplices,
                                       float* distances, float* normals, int32_t* status,
                                       const int* pair_bounds, int nranges, int lanes);

/* Bodies made of several convex parts (a convex decomposition; parts are the pool's
 * bodies, body B owns parts [first[B], first[B] + count[B])).  Expansion of body pairs
 * into part pairs, as the reference's visualiser does it
 * (visualization/integrate_final_gjk.cu:265-302): body pair p becomes
 * (first[A] + a, first[B] + b) for every a, b, a-major, body pairs in order.
 * d_offsets[num_body_pairs + 1] receives each body pair's first part pair (last entry:
 * the total; only the first max_sub_pairs are written); d_owner (optional) the body pair
 * of each part pair.  The reduction gives per body pair the smallest part-pair distance
 * (closest or most penetrating) and its part-pair index.  Device arrays, asynchronous. */
ogx_status ogx_expand_submesh_pairs(ogx_ctx* ctx, int num_body_pairs,
                                    const gkCollisionPair* d_body_pairs, int num_bodies,
                                    const int32_t* d_first_part, const int32_t* d_part_count,
                                    int max_sub_pairs, gkCollisionPair* d_sub_pairs,
                                    int32_t* d_owner, int32_t* d_offsets);
ogx_status ogx_reduce_submesh_pairs(ogx_ctx* ctx, int num_body_pairs, const int32_t* d_offsets,
                                    int max_sub_pairs, const float* d_sub_distances,
                                    float* d_best_distance, int32_t* d_best_index);

/* Collision response from the results of ogx_gjk_epa (the step after the path; the
 * model of the reference's visualiser, visualization/integrate_final_gjk.cu:572-689):
 * for every pair with distance <= contact_eps, a normal impulse at the witness points
 * with the angular terms of both bodies and restitution (coefficient `restitution` when
 * the approach speed exceeds restitution_threshold, else 0), applied only while the
 * bodies approach, and for penetrating pairs a position correction of baumgarte * depth
 * along the normal, shared by inverse mass.  All impulses come from the input state (a
 * Jacobi step); each body sums its contributions in contact order, so the result is
 * deterministic.  Body arrays are device memory: pos[n][3], quat[n][4] (x, y, z, w,
 * body to world), vel[n][3], ang[n][3] (world frame), inv_mass[n], inv_inertia[n][3]
 * (diagonal, body frame).  Outputs: new vel, ang, pos (device, [n][3]).  Asynchronous on
 * the context's stream (stream-ordered scratch). */
typedef struct ogx_body_state {
  const float* pos;
  const float* quat;
  const float* vel;
  const float* ang;
  const float* inv_mass;
  const float* inv_inertia;
} ogx_body_state;
typedef struct ogx_response_params {
  float contact_eps;            /* default FLT_EPSILON */
  float baumgarte;              /* default 0.2 */
  float restitution;            /* default 0.5 */
  float restitution_threshold;  /* default 1.0 (speed) */
} ogx_response_params;
void ogx_response_params_default(ogx_response_params* params);
ogx_status ogx_contact_response(ogx_ctx* ctx, int num_bodies, const ogx_body_state* state,
                                int npairs, const gkCollisionPair* d_pairs,
                                const float* d_distances, const float* d_normals,
                                const ogx_simplex_f32* d_simplices, const ogx_response_params* params,
                                float* d_vel_out, float* d_ang_out, float* d_pos_out);

/* Timeline of the last ogx_gjk_epa_streamed call made with timing on
 * (ogx_ctx_set_timing): 5 values per chunk, ms from the call's start: end of its body
 * upload, end of its pair upload, start and end of its kernels, end of its download.
 * Returns the number of values (writes at most cap). */
int ogx_ctx_stream_timeline(const ogx_ctx* ctx, float* ms, int cap);

/* CUDA graph of one call: captures the launches of ogx_gjk / ogx_gjk_epa / ogx_epa
 * (mode 1 / 2 / 3) on these buffers once; ogx_graph_launch replays them on the context's
 * stream with one launch.  The buffers' contents may change between launches, their
 * addresses, npairs, the kernel variants and the configuration may not (recreate the
 * graph).  The context must have been created without a caller stream or with a
 * non-legacy one.  A graph must be destroyed before its context. */
typedef struct ogx_graph ogx_graph;
ogx_status ogx_graph_create(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                            const gkCollisionPair* d_pairs, ogx_simplex_f32* d_simplices,
                            float* d_distances, float* d_normals, int32_t* d_status, int mode,
                            ogx_graph** out);
ogx_status ogx_graph_launch(ogx_graph* graph);
/* kernels one replay launches */
int ogx_graph_kernel_launches(const ogx_graph* graph);
ogx_status ogx_graph_destroy(ogx_graph* graph);

/* GJK then EPA that allocates no device memory.  No counterpart in the reference.
 * For callers that must not allocate device memory at query time: loops whose device
 * memory belongs to their own arena, real-time ticks that cannot take allocator
 * latency, plugins whose host forbids them to allocate.  The pool is given by
 * its device arrays in the engine layout (ogx_pool_device_layout, or written by the
 * caller); the caller passes the pairs and all outputs.  The pipeline's work lists live
 * in one static device array of 1,835,264 bytes that every GPU loading this library
 * holds until exit.  At most 16384 pairs per call (OGX_ERR_CAPACITY beyond).  Each call
 * clears the array's counters itself; nothing has to be zeroed by the caller.  All calls
 * share the array, so calls that overlap on the GPU race: serialise them.  The first call on
 * a device looks up the array's address and the launch sizes -- make it before any
 * stream capture.  cfg NULL = defaults; stream = cudaStream_t (NULL: legacy stream). */
ogx_status ogx_gjk_epa_noalloc(const float* d_points, const void* d_bodies, int num_bodies,
                               int npairs, const gkCollisionPair* d_pairs,
                               ogx_simplex_f32* d_simplices, float* d_distances, float* d_normals,
                               int32_t* d_status, const ogx_config* cfg, void* stream);

/* ------------------------------------------------------------------------- */
/* Serving loop.  No counterpart in the reference's library: its per-frame path  */
/* (visualization/integrate_final_gjk.cu:1028-1037) moves every body on the host */
/* and calls the indexed functions synchronously.  A server keeps the bodies on  */
/* the device in their own frame; each transform update writes a world-space     */
/* copy (one of `world_slots` ring buffers, identified by a version); requests   */
/* (the candidate pairs of one tick) are queued and admitted oldest first as     */
/* soon as a slot (stream + buffers for slot_pairs pairs) is free and the pairs  */
/* in flight stay within max_pairs_in_flight; admitted requests run concurrently.*/
/* Warm starts: the first vertex pair of the last simplex of each (i, j) pair is */
/* kept in a device hash table and GJK starts there.                             */

typedef struct ogx_server ogx_server;
typedef struct ogx_server_config {
  int slots;               /* requests on the device at once (one stream each) */
  int slot_pairs;          /* largest request, in pairs */
  int max_pairs_in_flight; /* admission budget over all running requests */
  int world_slots;         /* world-space copies of the pool (transform versions kept) */
  int warm_start;          /* 1: warm-start GJK from the previous simplex of the pair */
  int warm_capacity_log2;  /* warm-start table entries (16 B each) */
  int64_t max_bytes_in_flight; /* admission budget in bytes of device working memory of
                            * the running requests (pairs, results, warm starts and the
                            * pipeline's work lists: ogx_server_admission gives the bytes
                            * per pair); 0: half the device memory free once the server's
                            * buffers are allocated */
  int fused_transform;     /* 1: no world copies; the GJK/EPA kernels apply each body's
                            * pose as they read its points (world point R p + t in FP32,
                            * one fused multiply-add chain per coordinate; support scans
                            * rotate the direction into the body frame instead).  Pair
                            * requests only: broad-phase requests need the world copy. */
} ogx_server_config;

void ogx_server_config_default(ogx_server_config* sc);
/* Bodies in their own frame: counts[num_bodies], local_xyz = concatenated xyz. */
ogx_status ogx_server_create(int device, const ogx_config* cfg, const ogx_server_config* sc,
                             int num_bodies, const int32_t* counts, const float* local_xyz,
                             ogx_server** out);
ogx_status ogx_server_destroy(ogx_server* server);
/* New poses: xf[num_bodies][12] = row-major rotation R (9) then translation t (3); the
 * world point is R p + t evaluated in double and rounded once to float.  Returns the
 * version to submit requests against.  Blocks (at most 10 s, then OGX_ERR_BUSY) while
 * the ring slot it overwrites is still used by a queued or running request.  Several
 * threads may call it at once (each gets its own version); the copy and the upload run
 * without holding the server's lock, so requests keep being admitted meanwhile.  A
 * version becomes valid only when its own call returns: versions handed to concurrent
 * callers are reserved in order but may become valid out of order, and a submit against
 * a version whose call has not returned yet is refused as not resident.  Once
 * ogx_server_destroy has begun, new calls are refused; destroy waits for uploads
 * already under way (at most 10 s, then OGX_ERR_BUSY with the server stopped, not
 * freed: call destroy again). */
ogx_status ogx_server_set_transforms(ogx_server* server, const float* xf, int64_t* version);
/* Queue a request: npairs <= slot_pairs pairs of body indices (copied at once); the
 * results are written to the host arrays (any of them may be NULL) before the request
 * completes, so they must stay valid until ogx_server_wait returns.  Page-locked arrays
 * (cudaMallocHost, cudaHostRegister) receive the results directly from the device;
 * others through the server's pinned staging and one host copy. */
ogx_status ogx_server_submit(ogx_server* server, int64_t version, int npairs,
                             const gkCollisionPair* pairs, ogx_simplex_f32* simplices,
                             float* distances, float* normals, int32_t* status, int64_t* ticket);
/* Queue a broad-phase request: the pairs are every pair of bodies whose boxes (grown by
 * margin) overlap in the version's world copy (ogx_broadphase on the device), then
 * GJK + EPA on them, all on the device.  pairs[max_pairs] receives the pairs (sorted,
 * i < j), count[0] the number found (may exceed max_pairs; the first
 * min(count, max_pairs, slot_pairs) are run), count[1] the broad phase's error flags. */
ogx_status ogx_server_submit_broadphase(ogx_server* server, int64_t version, float cell,
                                        float margin, int max_pairs, gkCollisionPair* pairs,
                                        int32_t* count, ogx_simplex_f32* simplices, float* distances,
                                        float* normals, int32_t* status, int64_t* ticket);
ogx_status ogx_server_poll(ogx_server* server, int64_t ticket, int* done);
/* Wait for a request (timeout_s <= 0: no limit); latency_ms = completion - submission
 * on the host clock.  The ticket is released. */
ogx_status ogx_server_wait(ogx_server* server, int64_t ticket, double timeout_s, double* latency_ms);
/* ogx_server_wait, plus where the latency went (phases_ms[4], may be NULL): [0] queued
 * (submit to admission to a slot), [1] host staging of the pairs before the first copy,
 * [2] device (first copy to results in host memory, CUDA events), [3] the rest (waiting
 * for the version's world copy, launch issue not hidden by the device, completion
 * detection). */
ogx_status ogx_server_wait_phases(ogx_server* server, int64_t ticket, double timeout_s, double* latency_ms,
                                  double* phases_ms);
/* Device layout of the world-space pool of a version (for checks and custom kernels). */
/* The admission budgets of a server: a request is admitted, oldest first, when a slot is
 * free and both the pairs and the device bytes in flight (pairs x bytes_per_pair) stay
 * within their budgets (or nothing else is running); peak_bytes = the most device bytes
 * in flight so far.  Any pointer may be NULL. */
ogx_status ogx_server_admission(ogx_server* server, int64_t* max_pairs, int64_t* max_bytes,
                                int64_t* bytes_per_pair, int64_t* peak_bytes);
ogx_status ogx_server_world_layout(ogx_server* server, int64_t version, float** d_points,
                                   void** d_bodies);

/* ------------------------------------------------------------------------- */
/* Reference-compatible entry points.  Same arguments, meaning and output     */
/* conventions as OpenGJK-GPU's host API; each call returns when its results  */
/* are complete (the reference synchronises the device after every launch).   */
/* n <= 0 returns OGX_OK without work, as the reference returns early.        */

/* compute_minimum_distance (GJK/gpu/openGJK.h:91), GJK::GPU::computeDistances
 * (examples/gpu/example.h:21-25): GJK on pairs (bd1[i], bd2[i]), host buffers. */
ogx_status ogx_compute_minimum_distance(int n, const ogx_polytope_f32* bd1, const ogx_polytope_f32* bd2,
                                        ogx_simplex_f32* simplices, float* distances);
/* computeCollisionInformation(n, ...) (GJK/gpu/openGJK.h:112), GJK::GPU::computeEPA
 * (examples/gpu/example.h:41-46): EPA from GJK simplices/distances (in/out);
 * contact_normals (n*3) may be NULL. */
ogx_status ogx_compute_collision_information(int n, const ogx_polytope_f32* bd1, const ogx_polytope_f32* bd2,
                                             ogx_simplex_f32* simplices, float* distances,
                                             float* contact_normals);
/* compute_gjk_epa (GJK/gpu/openGJK.h:134), GJK::GPU::computeGJKAndEPA
 * (examples/gpu/example.h:62-67). */
ogx_status ogx_compute_gjk_epa(int n, const ogx_polytope_f32* bd1, const ogx_polytope_f32* bd2,
                               ogx_simplex_f32* simplices, float* distances, float* contact_normals);
/* GJK::GPU::computeCollisionInformation as documented in README.md:39-46 (absent from
 * the reference's code): EPA with witnesses also as n*3 arrays, normals nullable. */
ogx_status ogx_compute_collision_information_witnesses(int n, const ogx_polytope_f32* bd1,
                                                       const ogx_polytope_f32* bd2, ogx_simplex_f32* simplices,
                                                       float* distances, float* witness1,
                                                       float* witness2, float* contact_normals);

/* mid-level: allocate_and_copy_device_arrays (GJK/gpu/openGJK.h:212) */
ogx_status ogx_allocate_and_copy_device_arrays(int n, const ogx_polytope_f32* bd1, const ogx_polytope_f32* bd2,
                                               ogx_polytope_f32** d_bd1, ogx_polytope_f32** d_bd2,
                                               float** d_coord1, float** d_coord2,
                                               ogx_simplex_f32** d_simplices, float** d_distances);
/* compute_minimum_distance_device (GJK/gpu/openGJK.h:237): descriptors and coordinates
 * in device memory */
ogx_status ogx_compute_minimum_distance_device(int n, const ogx_polytope_f32* d_bd1,
                                               const ogx_polytope_f32* d_bd2, ogx_simplex_f32* d_simplices,
                                               float* d_distances);
/* compute_epa_device (GJK/gpu/openGJK.h:255) */
ogx_status ogx_compute_epa_device(int n, const ogx_polytope_f32* d_bd1, const ogx_polytope_f32* d_bd2,
                                  ogx_simplex_f32* d_simplices, float* d_distances,
                                  float* d_contact_normals);
/* copy_results_from_device (GJK/gpu/openGJK.h:273) */
ogx_status ogx_copy_results_from_device(int n, const ogx_simplex_f32* d_simplices,
                                        const float* d_distances, ogx_simplex_f32* simplices,
                                        float* distances);
/* free_device_arrays (GJK/gpu/openGJK.h:292) */
ogx_status ogx_free_device_arrays(ogx_polytope_f32* d_bd1, ogx_polytope_f32* d_bd2, float* d_coord1,
                                  float* d_coord2, ogx_simplex_f32* d_simplices, float* d_distances);
/* allocate_epa_device_arrays (GJK/gpu/openGJK.h:155) */
ogx_status ogx_allocate_epa_device_arrays(int n, float** d_witness1, float** d_witness2,
                                          float** d_contact_normals);
/* copy_epa_results_from_device (GJK/gpu/openGJK.h:173) */
ogx_status ogx_copy_epa_results_from_device(int n, const float* d_witness1,
                                            const float* d_witness2,
                                            const float* d_contact_normals, float* witness1,
                                            float* witness2, float* contact_normals);
/* free_epa_device_arrays (GJK/gpu/openGJK.h:194) */
ogx_status ogx_free_epa_device_arrays(float* d_witness1, float* d_witness2,
                                      float* d_contact_normals);

/* indexed: allocate_indexed_device (GJK/gpu/openGJK.h:330) */
ogx_status ogx_allocate_indexed_device(int num_polytopes, int max_pairs,
                                       const ogx_polytope_f32* polytopes, ogx_polytope_f32** d_polytopes,
                                       float** d_coords, gkCollisionPair** d_pairs,
                                       ogx_simplex_f32** d_simplices, float** d_distances,
                                       float** d_contact_normals);
/* free_indexed_device (GJK/gpu/openGJK.h:352) */
ogx_status ogx_free_indexed_device(ogx_polytope_f32* d_polytopes, float* d_coords,
                                   gkCollisionPair* d_pairs, ogx_simplex_f32* d_simplices,
                                   float* d_distances, float* d_contact_normals);
/* upload_pairs_device (GJK/gpu/openGJK.h:368) */
ogx_status ogx_upload_pairs_device(int num_pairs, const gkCollisionPair* pairs,
                                   gkCollisionPair* d_pairs);
/* compute_minimum_distance_indexed (GJK/gpu/openGJK.h:398) */
ogx_status ogx_compute_minimum_distance_indexed(int num_polytopes, int num_pairs,
                                                const ogx_polytope_f32* polytopes,
                                                const gkCollisionPair* pairs,
                                                ogx_simplex_f32* simplices, float* distances);
/* compute_minimum_distance_indexed_device (GJK/gpu/openGJK.h:419) */
ogx_status ogx_compute_minimum_distance_indexed_device(int num_pairs, const ogx_polytope_f32* d_polytopes,
                                                       const gkCollisionPair* d_pairs,
                                                       ogx_simplex_f32* d_simplices, float* d_distances);
/* compute_epa_indexed (GJK/gpu/openGJK.h:473): simplices/distances in/out */
ogx_status ogx_compute_epa_indexed(int num_polytopes, int num_pairs, const ogx_polytope_f32* polytopes,
                                   const gkCollisionPair* pairs, ogx_simplex_f32* simplices,
                                   float* distances, float* contact_normals);
/* compute_epa_indexed_device (GJK/gpu/openGJK.h:450) */
ogx_status ogx_compute_epa_indexed_device(int num_pairs, const ogx_polytope_f32* d_polytopes,
                                          const gkCollisionPair* d_pairs, ogx_simplex_f32* d_simplices,
                                          float* d_distances, float* d_contact_normals);
/* compute_gjk_epa_indexed (GJK/gpu/openGJK.h:497) */
ogx_status ogx_compute_gjk_epa_indexed(int num_polytopes, int num_pairs,
                                       const ogx_polytope_f32* polytopes, const gkCollisionPair* pairs,
                                       ogx_simplex_f32* simplices, float* distances,
                                       float* contact_normals);
/* GJK::GPU::timer() (examples/gpu/example.h:9): GPU milliseconds of the engine pipeline
 * of the calling thread's last reference-compatible call.  The calls above run on an
 * engine context leased for the call (one per concurrent caller, kept for reuse), so calls
 * from several host threads run side by side. */
float ogx_compat_last_gpu_ms(void);

/* The same calls for a caller built with the reference's USE_32BITS off
 * (GJK/common.h:44-60: gkFloat = double, 48-byte gkPolytope, 184-byte gkSimplex).  The
 * coordinates are rounded once to float and the FP32 engine runs on them; the results are
 * widened to double, so they carry that input rounding (a relative 6e-8 per coordinate),
 * not the rounding of an FP64 computation.  Host-buffer calls only: the device-buffer
 * (*_device) functions take the FP32 layouts. */
/* compute_minimum_distance (GJK/gpu/openGJK.h:91), FP64 layout */
ogx_status ogx_compute_minimum_distance_f64(int n, const ogx_polytope_f64* bd1, const ogx_polytope_f64* bd2,
                                            ogx_simplex_f64* simplices, double* distances);
/* computeCollisionInformation(n, ...) (GJK/gpu/openGJK.h:112), FP64 layout */
ogx_status ogx_compute_collision_information_f64(int n, const ogx_polytope_f64* bd1,
                                                 const ogx_polytope_f64* bd2, ogx_simplex_f64* simplices,
                                                 double* distances, double* contact_normals);
/* compute_gjk_epa (GJK/gpu/openGJK.h:134), FP64 layout */
ogx_status ogx_compute_gjk_epa_f64(int n, const ogx_polytope_f64* bd1, const ogx_polytope_f64* bd2,
                                   ogx_simplex_f64* simplices, double* distances, double* contact_normals);
/* GJK::GPU::computeCollisionInformation (README.md:39-46), FP64 layout */
ogx_status ogx_compute_collision_information_witnesses_f64(int n, const ogx_polytope_f64* bd1,
                                                           const ogx_polytope_f64* bd2,
                                                           ogx_simplex_f64* simplices, double* distances,
                                                           double* witness1, double* witness2,
                                                           double* contact_normals);
/* compute_minimum_distance_indexed (GJK/gpu/openGJK.h:398), FP64 layout */
ogx_status ogx_compute_minimum_distance_indexed_f64(int num_polytopes, int num_pairs,
                                                    const ogx_polytope_f64* polytopes,
                                                    const gkCollisionPair* pairs, ogx_simplex_f64* simplices,
                                                    double* distances);
/* compute_epa_indexed (GJK/gpu/openGJK.h:473), FP64 layout */
ogx_status ogx_compute_epa_indexed_f64(int num_polytopes, int num_pairs, const ogx_polytope_f64* polytopes,
                                       const gkCollisionPair* pairs, ogx_simplex_f64* simplices,
                                       double* distances, double* contact_normals);
/* compute_gjk_epa_indexed (GJK/gpu/openGJK.h:497), FP64 layout */
ogx_status ogx_compute_gjk_epa_indexed_f64(int num_polytopes, int num_pairs, const ogx_polytope_f64* polytopes,
                                           const gkCollisionPair* pairs, ogx_simplex_f64* simplices,
                                           double* distances, double* contact_normals);

#ifdef __cplusplus
}
#endif
#endif /* OGX_H_ */
