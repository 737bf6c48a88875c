/*
 * d3d_gb300.h -- C ABI of libd3d_gb300.so, the GB300 (sm_103a) narrow and
 * broad phase for distance3d.
 *
 * Conventions
 * -----------
 * - Every entry point returns an int status: D3D_SUCCESS (0) or a D3D_ERR_*
 *   code; d3d_last_error() returns a message for the calling thread.  No entry
 *   point aborts the process.
 * - Every pointer argument except the d3d_store / options structs themselves
 *   is a DEVICE pointer, caller allocated.  `stream` is a cudaStream_t passed as
 *   void* (NULL = the legacy default stream).  Work is enqueued on that stream;
 *   the call returns without synchronising unless stated otherwise.
 * - Pair results are deterministic: one slot per pair, no atomics in result
 *   slots, the same bits for the same inputs whatever the batch around them.
 * - Collider indices (i1, i2, idx) are device data, so they are checked on
 *   the device: a pair with an index outside [0, n_colliders) gets
 *   D3D_STATUS_BAD_INDEX (NaN results, hit 0) and no record is read for it;
 *   d3d_support and d3d_aabbs write NaN for such an index and
 *   d3d_store_set_poses skips it.  The Python layer also rejects out-of-range
 *   host index arrays before any copy.
 *
 * Each entry point names the distance3d 0.9.0 interface it replaces
 * (path:line inside that project).
 */
#ifndef D3D_GB300_H
#define D3D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define D3D_ABI_VERSION 3

/* return codes */
#define D3D_SUCCESS 0
#define D3D_ERR_INVALID 1   /* bad argument (null pointer, bad size, bad option) */
#define D3D_ERR_CAPACITY 2  /* output or scratch capacity too small */
#define D3D_ERR_CUDA 3      /* a CUDA runtime call failed */

/* collider types (distance3d/colliders.py:109-647) */
#define D3D_SPHERE 0
#define D3D_CAPSULE 1
#define D3D_BOX 2
#define D3D_CYLINDER 3
#define D3D_ELLIPSOID 4
#define D3D_HULL 5          /* ConvexHullVertices */
#define D3D_DISK 6          /* normal = R column 2 (colliders.py:443-497) */
#define D3D_ELLIPSE 7       /* axes = R columns 0 and 1 (colliders.py:500-551) */
#define D3D_CONE 8          /* colliders.py:554-603 */
#define D3D_MESH 9          /* MeshGraph (colliders.py:187-240): vertices in the mesh frame,
                               hill-climbing support over the links block (mesh.py:12-127) */
#define D3D_MARGIN 0x100    /* flag or-ed into a type: the collider wrapped in Margin
                               (colliders.py:606-647), margin = params[3] */

/* per-pair status codes */
#define D3D_STATUS_OK 0
#define D3D_STATUS_CLIPPED 1            /* separation > sqrt(max_distance_squared): dist = DBL_MAX, points NaN
                                           (the reference returns (MAX_FLOAT, None, None, None), _gjk_jolt.py:209-210) */
#define D3D_STATUS_SANITY 2             /* the reference's sanity assertion would fail (_gjk_jolt.py:215-216) */
#define D3D_STATUS_MAX_ITER 3           /* iteration bound reached (the reference loops without bound) */
#define D3D_STATUS_EPA_NOT_CONVERGED 4  /* EPA hit max_iter (epa.py:76-78, success = False) */
#define D3D_STATUS_EPA_FACE_OVERFLOW 5  /* the reference raises AssertionError (epa.py:128) */
#define D3D_STATUS_EPA_DEGENERATE 6     /* every face was removed (the reference raises in np.argmin) */
#define D3D_STATUS_BAD_INDEX 7          /* a collider index of the pair lies outside [0, n_colliders): no record
                                           was read; distances, points and MTVs are NaN, hit flags 0 (the
                                           reference raises IndexError on a bad list index) */

#define D3D_PRECISION_FP64 0   /* plain FP64 drop-in: the reference's arithmetic, bit for bit */
#define D3D_PRECISION_MIXED 1  /* FP32 iterations, FP64 final refinement */

/*
 * Device-resident collider store.  Built by d3d_store_pack from the packed
 * host format (see distance3d_gb300/collider_set.py); all arrays are device
 * memory owned by the caller.
 *   rec64  [n][16] double : R row-major (9), t (3), params (3), margin
 *   rec32  [n][16] float  : the same in FP32
 *   meta   [n][4]  int32  : type (without the margin flag), vertex count,
 *                           vertex offset, 1 if wrapped in Margin else 0
 *   links  [L]     int32  : MeshGraph adjacency blocks (may be NULL without meshes)
 * A disk's R holds column_stack(x, y, normal) with x, y derived from the
 * normal (utils.py:78-122 plane_basis_from_normal) when it is packed or
 * posed, as the reference derives them in every support call.
 * A MeshGraph's vertices (mesh frame) sit in the vertex pool like a hull's;
 * its params are (links offset, start vertex, 0).  Its links block, for nv
 * vertices: the 6 shortcut vertices (argmax x, y, z, argmin x, y, z of the
 * vertices, mesh.py:44-47), then nv + 1 offsets of the neighbour lists
 * (relative to the block), then the neighbour lists in the order the
 * reference iterates them (mesh.py:34-52).  Vertex indices are local to the
 * mesh.
 *   verts64 [V][4] double : hull vertices then 8 vertices per box (xyz, 0)
 *   verts32 [V][4] float  : the same in FP32
 */
typedef struct d3d_store {
    int64_t n_colliders;
    int64_t n_vertices;
    double* rec64;
    float* rec32;
    int32_t* meta;
    double* verts64;
    float* verts32;
    int32_t* links;
    int64_t n_links;
} d3d_store;

typedef struct d3d_gjk_options {
    double tolerance;             /* 1e-10 (_gjk_jolt.py:139) */
    double max_distance_squared;  /* 1e5 */
    double sanity_check;          /* 1e-8 */
    int32_t max_iterations;       /* hard bound on GJK iterations, >= 1 */
    int32_t precision;            /* D3D_PRECISION_* */
} d3d_gjk_options;

typedef struct d3d_epa_options {
    int32_t max_iterations;   /* 64 (epa.py:9) */
    int32_t max_loose_edges;  /* 32 */
    int32_t max_faces;        /* 64 */
    int32_t precision;        /* D3D_PRECISION_FP64 (the reference, bit for bit) or D3D_PRECISION_MIXED
                                 (FP32 polytope search, FP64 refinement of the final face) */
    double epsilon;           /* 1e-8 */
} d3d_epa_options;

int d3d_abi_version(void);
const char* d3d_last_error(void);

/* Diagnostics (no counterpart in the reference): the kernel nodes of a CUDA
 * graph (a cudaGraph_t passed as void*, child graphs included) that launch
 * this library's own kernels (*own) and the CUDA toolkit's CUB kernels the
 * library instantiates (*toolkit), e.g. for a graph captured around
 * d3d_collide: the kernels one replay launches. */
int d3d_graph_kernel_nodes(const void* graph, int64_t* own, int64_t* toolkit);

/* Pack a store.  Input arrays are the packed host format already copied to
 * the device: types[n] (D3D_* or-ed with D3D_MARGIN for a Margin wrapper),
 * poses[n][12], params[n][4] (params[3]: the margin), hull_offset[n] (int64;
 * for a hull or a mesh: its first vertex row;
 * for a box: the row where its 8 derived vertices go, >= n_hull_vertices),
 * hull_count[n]; the caller has copied the n_hull_vertices hull and mesh rows
 * into store->verts64[0 : n_hull_vertices] and the mesh links blocks into
 * store->links.  Box vertices follow geometry.py:138-157
 * (convert_box_to_vertices); FP32 mirrors are rounded from FP64.  Replaces
 * collider construction, colliders.py:109-647. */
int d3d_store_pack(const d3d_store* store, const int32_t* types, const double* poses,
                   const double* params, const int64_t* hull_offset, const int32_t* hull_count,
                   int64_t n_hull_vertices, void* stream);

/* Set the poses of colliders idx[k] to poses[k][12] (R row-major, t) and
 * re-derive box vertices.  Replaces ConvexCollider.update_pose
 * (colliders.py:78-85, 172-176); a hull's pose cannot be set
 * (colliders.py:137-138): D3D_ERR_INVALID is not detected on the device,
 * so callers must not pass hull indices. */
int d3d_store_set_poses(const d3d_store* store, const int32_t* idx, const double* poses,
                        int64_t n, void* stream);

/* Support points out[k] = support of collider idx[k] along dirs[k] (FP64).
 * Replaces ConvexCollider.support_function (colliders.py:54-66). */
int d3d_support(const d3d_store* store, const int32_t* idx, const double* dirs, int64_t n,
                double* out, void* stream);

/* Axis-aligned bounding boxes out[k][3][2] ([axis][min,max]) of colliders
 * idx[k] (idx NULL: colliders 0..n-1).  Replaces ConvexCollider.aabb
 * (colliders.py:88-95) and containment.py:6-148. */
int d3d_aabbs(const d3d_store* store, const int32_t* idx, int64_t n, double* out, void* stream);

/* Batched Jolt GJK distance for pairs (i1[k], i2[k]).  Outputs: dist[n],
 * cp1[n][3], cp2[n][3], simplex[n][4][3] (rows >= n_simplex keep the
 * reference's stale rows; rows never written are 0), n_simplex[n], status[n],
 * iterations[n] (may be NULL).  Replaces gjk.gjk / gjk_distance /
 * gjk_distance_jolt, gjk/_gjk_jolt.py:138-221 (aliases gjk/__init__.py:26-27). */
int d3d_gjk_distance(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                     const d3d_gjk_options* options, double* dist, double* cp1, double* cp2,
                     double* simplex, int8_t* n_simplex, int8_t* status, int32_t* iterations,
                     void* stream);

/* The plain FP64 GJK distance with the reference's MeshGraph vertex caching.
 * The reference's MeshGraph support object starts each hill climb from the
 * vertex its previous call returned and keeps the new answer
 * (MeshHillClimbingSupportFunction.__call__, mesh.py:64-87; the cache starts
 * at the smallest vertex index of the triangles, mesh.py:30), so its results
 * depend on the calls made on that object before.  Here pair k's mesh
 * supports start from mesh_cache[k][0] (collider i1[k]) and mesh_cache[k][1]
 * (collider i2[k]), -1 meaning the mesh's start vertex, chain through the
 * pair's support calls in the reference's order, and leave the last answer
 * in mesh_cache (device int32[n][2], in/out; entries of other colliders
 * pass through).  Passing the cache states the reference's objects hold
 * before a call reproduces that call bit for bit; pairs of one batch run
 * independently, so a collider used by several pairs carries its state from
 * one to the next only across calls.  One thread per pair, input order
 * (no scheduling).  options->precision must be D3D_PRECISION_FP64.  Outputs
 * as d3d_gjk_distance.  Replaces gjk_distance_jolt on MeshGraph colliders
 * (gjk/_gjk_jolt.py:138-221 with colliders.py:187-240). */
int d3d_gjk_distance_cached(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                            const d3d_gjk_options* options, int32_t* mesh_cache, double* dist, double* cp1,
                            double* cp2, double* simplex, int8_t* n_simplex, int8_t* status, int32_t* iterations,
                            void* stream);

/* Batched Jolt GJK intersection test: hit[k] = 1 if the pair intersects.
 * Replaces gjk.gjk_intersection / gjk_intersection_jolt, _gjk_jolt.py:29-135
 * (alias gjk/__init__.py:28). */
int d3d_gjk_intersection(const d3d_store* store, const int32_t* i1, const int32_t* i2,
                         int64_t n, double tolerance, int32_t max_iterations, int8_t* hit,
                         int8_t* status, void* stream);

/* Scratch bytes d3d_epa needs for n pairs. */
size_t d3d_epa_scratch_bytes(int64_t n, const d3d_epa_options* options);

/* Batched EPA on GJK simplices simplex[n][4][3].  Outputs mtv[n][3],
 * status[n], n_faces[n], faces[n][max_faces][4][3] (may be NULL; in the mixed
 * form the FP32 polytope).  `scratch` holds the polytopes
 * (d3d_epa_scratch_bytes).  Replaces epa.epa, epa.py:9-78 (Polytope :81-146,
 * LooseEdges :149-202). */
int d3d_epa(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
            const double* simplex, const d3d_epa_options* options, double* mtv, int8_t* status,
            int32_t* n_faces, double* faces, void* scratch, size_t scratch_bytes, void* stream);

/* EPA that allocates nothing, for callers that may not allocate device memory
 * while they run (a control loop on a fixed memory budget, a plugin whose host
 * application owns every GPU allocation).  It has no counterpart in the
 * reference.  Same arguments and results as d3d_epa, without the scratch.
 * Options of up to 251 iterations whose polytope fits a block's shared memory
 * (the defaults, and 256 faces with 128 loose edges) keep each polytope in
 * shared memory; for other options the polytopes live in a 16 MiB array
 * inside the library, present on every GPU that loads it until the process
 * exits, and the call fails with D3D_ERR_CAPACITY when max_faces /
 * max_loose_edges leave room for fewer than 128 pairs at a time there
 * (12 * max_faces + 6 * max_loose_edges doubles per pair; the defaults with
 * 252 or more iterations take this path, 2,184 polytopes at a time).  The
 * array also holds the work counter.  Every call must be made with the
 * store's device current: the array used is the current device's, and a
 * store on another device is rejected with D3D_ERR_INVALID.  The first call
 * on a device looks up the array's address; make that first call before any
 * stream capture.  All calls share the array: calls whose work overlaps on
 * the GPU race and must be serialised by the caller.  Pairs run in input
 * order (no scheduling sort). */
int d3d_epa_noalloc(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                    const double* simplex, const d3d_epa_options* options, double* mtv, int8_t* status,
                    int32_t* n_faces, double* faces, void* stream);

/* GJK distance then EPA, for a batch whose pair count lives on the device.
 * Replaces the reference's composition gjk() -> epa(simplex) on intersecting
 * pairs (gjk/_gjk_jolt.py:138-221, epa.py:9-78) for a whole batch.  Pairs
 * k < *n_dev of buffers sized `capacity`: GJK outputs as d3d_gjk_distance
 * (precision gjk->precision); then EPA (precision epa->precision) on the
 * pairs with dist == 0 and n_simplex == 4, found on the device.  Pairs without
 * EPA get epa_status -1, NaN mtv and n_faces 0.  No host synchronisation and
 * no allocation (scratch of d3d_collide_scratch_bytes bytes); the launch
 * shapes depend on `capacity` only, so a CUDA graph captured around one call
 * serves any *n_dev <= capacity when replayed. */
size_t d3d_collide_scratch_bytes(int64_t capacity, const d3d_gjk_options* gjk, const d3d_epa_options* epa);
int d3d_collide(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t capacity,
                const int64_t* n_dev, const d3d_gjk_options* gjk, const d3d_epa_options* epa, double* dist,
                double* cp1, double* cp2, double* simplex, int8_t* n_simplex, int8_t* status, int32_t* iterations,
                double* mtv, int8_t* epa_status, int32_t* n_faces, void* scratch, size_t scratch_bytes,
                void* stream);

/* Minkowski portal refinement (MPR).  Replaces mpr.mpr_intersection and
 * mpr.mpr_penetration (mpr.py:21-110).  D3D_PRECISION_FP64 gives the
 * reference's results bit for bit; D3D_PRECISION_MIXED searches the portal
 * in FP32 on the FP32 mirror and evaluates the final portal in FP64 along the
 * FP32 search directions (depth, direction and contact position with the
 * reference's formulas).  hit[k] for pairs
 * (i1[k], i2[k]); with options->penetration also depth[k], dir[k][3] (unit
 * or zero vector: adding depth * dir to the second collider separates them)
 * and pos[k][3] (contact position), NaN where the reference returns None.
 * status[k]: D3D_STATUS_OK, or D3D_STATUS_MAX_ITER after refine_limit portal
 * expansions (the reference's refinement loop has no bound; hit = 0 then).
 * Output pointers depth/dir/pos may be NULL. */
typedef struct d3d_mpr_options {
    double tolerance;        /* 1e-4 (mpr.py:21) */
    int32_t max_iterations;  /* 100: portal discovery and penetration search */
    int32_t refine_limit;    /* 10000: bound on the refinement loop */
    int32_t penetration;     /* 1: mpr_penetration, 0: mpr_intersection */
    int32_t precision;       /* D3D_PRECISION_FP64 or D3D_PRECISION_MIXED */
} d3d_mpr_options;
int d3d_mpr(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n, const d3d_mpr_options* options,
            int8_t* hit, double* depth, double* dir, double* pos, int8_t* status, void* stream);

/* A serial kinematic chain with collision bodies (device pointers).  Link 0
 * is the base; revolute joint j at the fixed transform joint_origin[j] of
 * link j turns link j+1 about the unit axis joint_axis[j]; body b is fixed
 * to link body_link[b] (0..n_joints) at body_origin[b].  Transforms are 12
 * doubles, R row-major then t. */
typedef struct {
    int32_t n_joints;
    int32_t n_bodies;
    const double* joint_axis;    /* [n_joints][3] */
    const double* joint_origin;  /* [n_joints][12] */
    const int32_t* body_link;    /* [n_bodies] */
    const double* body_origin;   /* [n_bodies][12] */
} d3d_chain;
/* Forward kinematics: poses[c][b][12] of every body for joint values
 * q[c][n_joints] of configurations c < n_configs.  Feeds
 * d3d_store_set_poses for batched self-collision checks (the pose updates
 * self_collision.detect relies on, self_collision.py:5-64). */
int d3d_chain_fk(const d3d_chain* chain, const double* q, int64_t n_configs, double* poses, void* stream);

/* Launch parameters of the batch kernels (process-wide, per library load).
 * gjk_block: threads per block of the GJK kernels (64, 128 or 256; the
 * plain FP64 GJK, whose blocks solve their simplices together, runs 128 for
 * 256);
 * gjk_warps_per_sm: resident warps per SM of their persistent grids (0: as
 * many as fit); epa_warps: pairs (warps) per block of the warp EPA (2, 4 or
 * 8); sort_min: batches of at least this many pairs are sorted by collider
 * types before GJK (larger than any batch: never). */
typedef struct {
    int32_t gjk_block;
    int32_t gjk_warps_per_sm;
    int32_t epa_warps;
    int32_t sort_min;
} d3d_tuning;
int d3d_get_tuning(d3d_tuning* out);
int d3d_set_tuning(const d3d_tuning* tuning);
/* Time candidate tunings on the given pairs (GJK distance and EPA, both in
 * options' precisions, on `stream`), set the fastest and return it in *out.
 * Blocks until done. */
int d3d_autotune(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                 const d3d_gjk_options* gjk, const d3d_epa_options* epa, d3d_tuning* out, void* stream);

/* Continuous-batching collision server over one resident store (no
 * counterpart in the reference, which answers one pair per call).  A worker
 * thread batches submitted requests (host pair lists) into up to `slots`
 * d3d_collide batches in flight, each within `capacity` pairs, all within
 * `hbm_budget` bytes of pair slots (0: slots x capacity x 315 B); large
 * requests are split over batches.  `use_graphs` replays one CUDA graph per
 * capacity class.  Results per pair are d3d_collide's; latency runs from
 * submission to the request's results being in host memory.  The store must
 * outlive the server.  `worker_priority` > 0 asks for the worker thread to
 * run under SCHED_FIFO at that priority (1-99), so that other threads on a
 * busy host do not delay its launches and completions; the worker sleeps
 * between passes and never spins.  Where the process may not raise a
 * thread's priority the worker keeps the default policy
 * (d3d_server_stats.worker_realtime says which); 0 leaves it unchanged. */
typedef struct d3d_server d3d_server;
typedef struct {
    int64_t capacity;
    int32_t slots;
    int32_t use_graphs;
    int64_t hbm_budget;
    int32_t worker_priority;
    int32_t reserved; /* 0 */
} d3d_server_options;
/* host output arrays of one request (n pairs), any may be NULL */
typedef struct {
    double* dist;       /* n */
    double* cp1;        /* n x 3 */
    double* cp2;        /* n x 3 */
    double* simplex;    /* n x 4 x 3 */
    int8_t* n_simplex;  /* n */
    int8_t* status;     /* n */
    int32_t* iterations;
    double* mtv;        /* n x 3 */
    int8_t* epa_status; /* n, -1 where no EPA ran */
    int32_t* n_faces;   /* n */
} d3d_pair_results;
int d3d_server_create(const d3d_store* store, const d3d_gjk_options* gjk, const d3d_epa_options* epa,
                      const d3d_server_options* options, d3d_server** out);
void d3d_server_destroy(d3d_server* server);
int d3d_server_submit(d3d_server* server, const int32_t* i1, const int32_t* i2, int64_t n, int64_t* request_id);
int d3d_server_wait(d3d_server* server, int64_t request_id, double timeout_s);
int d3d_server_result(d3d_server* server, int64_t request_id, const d3d_pair_results* out, double* latency_s);
/* Submit n_requests requests at offsets_s[k] seconds from the call (sizes[k]
 * pairs each, concatenated in i1/i2), wait for all, return each one's
 * latency and its wait until its first batch launched (both from its
 * scheduled arrival; wait_s may be NULL) and the span from the call to the
 * last finish; the results are not kept. */
int d3d_server_replay(d3d_server* server, int64_t n_requests, const double* offsets_s, const int64_t* sizes,
                      const int32_t* i1, const int32_t* i2, double* latency_s, double* wait_s, double* span_s);
/* Counters of the worker since the last reset (reset != 0 clears them after
 * reading): batches launched, the longest batch from launch to results in
 * host memory, the longest time the worker took to enqueue one batch
 * (copies, graph launch), and the longest pass of the worker loop (a stall
 * of the host thread).  For telling a slow batch on the device from a
 * stalled host when a latency outlier appears. */
typedef struct {
    int64_t batches;
    double max_batch_s;
    double max_enqueue_s;
    double max_loop_gap_s;
    int32_t worker_realtime; /* 1 if the worker runs under SCHED_FIFO (not reset) */
    int32_t reserved;
} d3d_server_stats;
int d3d_server_stats_read(d3d_server* server, d3d_server_stats* out, int reset);

/* ------------------------------------------------------------------ broad phase
 * A linear BVH over FP64 boxes aabbs[n][3][2] ([axis][min,max]).  The tree
 * lives in a caller buffer of d3d_bvh_bytes(n) bytes (layout private) and
 * refers to `aabbs`, which queries must pass again unchanged.  Pair sets equal
 * the reference's AabbTree / brute-force sets exactly (closed intervals,
 * aabb_tree.py:504-527). */

size_t d3d_bvh_bytes(int64_t n_leaves);

/* Build (stream-ordered).  Replaces AabbTree.insert_aabbs / insert_aabb
 * (aabb_tree.py:31-115, insert_leaf :240-341) and the tree rebuild of
 * BoundingVolumeHierarchy.update_collider_poses (broad_phase.py:144-151). */
int d3d_bvh_build(const double* aabbs, int64_t n, void* tree, size_t tree_bytes, void* stream);

/* Refit a built tree to new boxes aabbs[n][3][2] of the same leaves (same
 * Morton order and topology, boxes of leaves and nodes redone): the pose
 * update of BoundingVolumeHierarchy.update_collider_poses
 * (broad_phase.py:144-151) without the rebuild.  Pair sets stay exact; the
 * tree's pruning degrades only as the leaves move far from their order. */
int d3d_bvh_refit(const double* aabbs, int64_t n, void* tree, size_t tree_bytes, void* stream);

/* Scratch bytes for a query with room for `capacity` pairs. */
size_t d3d_bvh_query_bytes(int64_t capacity);

/* All overlapping leaf pairs (i, j), i < j by input index, ascending, into
 * pairs[capacity][2].  Synchronises the stream once; *n_pairs (host) is the
 * pair count, and when it exceeds capacity the call returns D3D_ERR_CAPACITY
 * so that the caller can retry with a larger buffer.  Replaces
 * AabbTree.overlaps_aabb_tree(self) (aabb_tree.py:121-159, :344-378) as used
 * by BoundingVolumeHierarchy.aabb_overlapping_with_self (broad_phase.py:229-252). */
int d3d_bvh_self_pairs(const double* aabbs, int64_t n, const void* tree, int32_t* pairs, int64_t capacity,
                       int64_t* n_pairs, void* scratch, size_t scratch_bytes, void* stream);

/* All (leaf, query) pairs whose boxes overlap, for query boxes boxes[m][3][2],
 * ascending by leaf then query.  Same capacity protocol as above.  Replaces
 * AabbTree.overlaps_aabb (aabb_tree.py:161-181, query_overlap :381-403) and,
 * with the other tree's boxes as queries, overlaps_aabb_tree(other) /
 * BoundingVolumeHierarchy.aabb_overlapping_with_other_bvh (broad_phase.py:202-227). */
int d3d_bvh_query(const double* aabbs, int64_t n, const void* tree, const double* boxes, int64_t m, int32_t* pairs,
                  int64_t capacity, int64_t* n_pairs, void* scratch, size_t scratch_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* D3D_GB300_H */
