/*
 * fclgpu.h -- C ABI of the GB300 proximity-query library (one GPU, sm_103a).
 *
 * This is the drop-in boundary for FCL 0.7.0's proximity-query hot path.  Plain C:
 * pointers, sizes and int status codes; no C++ or CUDA types cross it except the
 * opaque `stream` argument (a cudaStream_t passed as void*, NULL = legacy default
 * stream).  Every function returns FCLGPU_OK (0) or a negative status; nothing
 * throws.  fclgpu_status_string() names a status.
 *
 * Transforms are 3x4 row-major doubles [R | t] (12 doubles), the rigid part of
 * fcl::Transform3<double> (common/types.h:67-98).  Triangle indices are int32.
 *
 * Reference interfaces replaced (paths inside the FCL repository):
 *   fclgpu_mesh_create      BVHModel<OBBRSS<double>>::beginModel/addSubModel/endModel
 *                           (geometry/bvh/BVH_model-inl.h:207-517), MEAN split
 *   fclgpu_mesh_update*     BVHModel<OBBRSS<double>>::beginUpdateModel/updateVertex/
 *                           endUpdateModel() (BVH_model-inl.h:624-727, 961-1027)
 *   fclgpu_mesh_replace*    BVHModel<OBBRSS<double>>::beginReplaceModel/replaceVertex/
 *                           endReplaceModel(true, true) (BVH_model-inl.h:521-620)
 *   fclgpu_collide_batch*   fcl::collide(...) on BVHModel<OBBRSS> pairs
 *                           (narrowphase/collision.h:55-66, collision-inl.h:79-207)
 *   fclgpu_collide_contacts*  fcl::collide(...) with enable_contact (contact position,
 *                           normal, depth; mesh_collision_traversal_node-inl.h:579-600)
 *   fclgpu_continuous_collide_batch*  fcl::continuousCollide(...) on BVHModel<OBBRSS>
 *                           pairs, naive solver, translation / linear / screw motion
 *                           (narrowphase/continuous_collision-inl.h:134-171, 436-451)
 *   fclgpu_distance_batch*  fcl::distance(...) on BVHModel<OBBRSS> pairs
 *                           (narrowphase/distance.h:51-62, distance-inl.h:71-246)
 *   fclgpu_shape_batch*     fcl::collide / fcl::distance on convex shapes (GJKSolver_indep)
 *   fclgpu_mesh_shape_batch*  fcl::collide / fcl::distance, BVHModel<OBBRSS> x convex shape
 *   fclgpu_broadphase_*     DynamicAABBTreeCollisionManager<double> with the default callbacks
 *                           (broadphase/broadphase_dynamic_AABB_tree-inl.h:727-1009)
 */
#ifndef FCLGPU_H
#define FCLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FCLGPU_API __attribute__((visibility("default")))

/* ---- status codes (FCL returns counts / prints warnings / throws; the C ABI maps
 *      those to codes: collision-inl.h:113-138, BVH_internal.h:61-72,
 *      failed_at_this_configuration.h:65-167) --------------------------------------- */
enum {
  FCLGPU_OK = 0,
  FCLGPU_ERR_INVALID_ARGUMENT = -1,
  FCLGPU_ERR_CUDA = -2,
  FCLGPU_ERR_OUT_OF_MEMORY = -3,
  FCLGPU_ERR_CAPACITY = -4,        /* output buffer too small; required size reported */
  FCLGPU_ERR_EMPTY_MODEL = -5,     /* BVH_ERR_BUILD_EMPTY_MODEL */
  FCLGPU_ERR_STACK_DEPTH = -6,     /* pair of BVHs deeper than the traversal stack */
  FCLGPU_ERR_DEVICE_STATUS = -7,   /* a kernel reported an internal error word */
  FCLGPU_ERR_NOT_INITIALIZED = -8,
  FCLGPU_ERR_UNSUPPORTED = -9,
  FCLGPU_ERR_PENDING = -10,         /* a served request has not finished yet */
  FCLGPU_ERR_INCORRECT_DATA = -11   /* BVH_ERR_INCORRECT_DATA (BVH_internal.h:61-72) */
};

FCLGPU_API const char* fclgpu_status_string(int status);
FCLGPU_API const char* fclgpu_last_error_detail(void);

/* Selects the CUDA device for this process (idempotent). */
FCLGPU_API int fclgpu_init(int device);

/* ---- precision forms ---------------------------------------------------------------
 * FCLGPU_PLAIN_FP64   : every test in FP64 in the reference's operation order.
 * FCLGPU_FP32_RECHECK : FP32 traversal and leaf tests with rigorous forward-error
 *                       bounds; any decision inside its bound is re-decided in FP64
 *                       (reference order, no FMA), so booleans, contact sets and
 *                       traversal statistics equal the FP64 form bit for bit.     */
enum { FCLGPU_PLAIN_FP64 = 0, FCLGPU_FP32_RECHECK = 1 };

/* ---- meshes (BVHModel<OBBRSS<double>>) --------------------------------------------- */
typedef struct fclgpu_mesh_s* fclgpu_mesh;

typedef struct {
  int64_t num_vertices;
  int64_t num_tris;
  int64_t num_nodes;
  int32_t max_depth;       /* root depth 0 */
  int32_t reserved;
  double max_abs_coord;    /* max |vertex coordinate| */
  int64_t device_bytes;    /* HBM held by the device mirror */
} fclgpu_mesh_info;

/* Builds the OBBRSS BVH on the host (FCL's top-down PCA fit, MEAN split) from
 * nv vertices (3 doubles each) and nt triangles (3 int32 each) and uploads a
 * device mirror (FP64 nodes and vertices, packed FP32 nodes and triangles).
 * fclgpu_mesh_create_on_device builds the same tree on the GPU (node for node
 * bit-identical: the same sums in the same order, FCL's node ids) from host arrays;
 * it synchronises `stream`. */
FCLGPU_API int fclgpu_mesh_create(const double* verts, int64_t nv, const int32_t* tris, int64_t nt,
                                  fclgpu_mesh* out);
FCLGPU_API int fclgpu_mesh_create_on_device(const double* verts, int64_t nv, const int32_t* tris, int64_t nt,
                                            fclgpu_mesh* out, void* stream);
FCLGPU_API int fclgpu_mesh_destroy(fclgpu_mesh mesh);
FCLGPU_API int fclgpu_mesh_get_info(fclgpu_mesh mesh, fclgpu_mesh_info* info);
/* Copies the FP64 BVH back to the host: per node 30 doubles (obb.axis row-major 9,
 * obb.To 3, obb.extent 3, rss.axis 9, rss.To 3, rss.l 2, rss.r 1) and first_child
 * (<0: leaf, primitive = -(first_child+1)), in FCL's node order. */
FCLGPU_API int fclgpu_mesh_get_nodes(fclgpu_mesh mesh, double* nodes30, int32_t* first_child);

/* Moves the mesh's vertices and refits its BVH on the device: replaces
 * BVHModel::beginUpdateModel + updateVertex (all vertices, in order) +
 * endUpdateModel(refit = true, bottomup = true) (geometry/bvh/BVH_model-inl.h:624-727,
 * 961-1027).  The tree keeps its shape; each leaf is refitted to its triangle in the
 * previous and the new frame, each internal node is the OBBRSS sum of its children.
 * nv must equal the mesh's vertex count (else FCLGPU_ERR_INCORRECT_DATA, as FCL's
 * endUpdateModel).  The local AABB is not recomputed (FCL does not either).  verts: host
 * (fclgpu_mesh_update) or device (fclgpu_mesh_update_device) pointer, 3 doubles per
 * vertex.  Synchronises the stream. */
FCLGPU_API int fclgpu_mesh_update(fclgpu_mesh mesh, const double* verts, int64_t nv, void* stream);
FCLGPU_API int fclgpu_mesh_update_device(fclgpu_mesh mesh, const double* verts, int64_t nv, void* stream);
/* endUpdateModel(refit, bottomup = true) (BVH_model-inl.h:703-734): refit != 0 is
 * fclgpu_mesh_update; refit = 0 rebuilds the tree on the new vertices on the GPU
 * (buildTree, as fclgpu_mesh_create_on_device) and then refits it bottom-up over both
 * frames, as FCL does.  Synchronises the stream. */
FCLGPU_API int fclgpu_mesh_update_model(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit,
                                        void* stream);
FCLGPU_API int fclgpu_mesh_update_model_device(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit,
                                               void* stream);

/* Replaces the mesh's vertices: BVHModel::beginReplaceModel + replaceVertex (all
 * vertices, in order) + endReplaceModel(refit, bottomup = true) (BVH_model-inl.h:521-620,
 * 961-1027).  FCL drops the previous frame here, so each leaf is refitted to its new
 * triangle alone (fit3 of OBB and RSS), the internal nodes as in fclgpu_mesh_update; a
 * later update uses these vertices as its previous frame.  refit = 0 rebuilds the tree on
 * the new vertices on the GPU (buildTree, BVH_model-inl.h:612-615).  Synchronises the
 * stream. */
FCLGPU_API int fclgpu_mesh_replace(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit,
                                   void* stream);
FCLGPU_API int fclgpu_mesh_replace_device(fclgpu_mesh mesh, const double* verts, int64_t nv,
                                          int32_t refit, void* stream);

/* ---- batched queries ----------------------------------------------------------------
 * A batch is n queries over a table of mesh pairs.  Query i tests meshes
 * (pairs[2*pair_of_query[i]], pairs[2*pair_of_query[i]+1]) at poses tf1[i], tf2[i].
 * pair_of_query == NULL means every query uses pair 0; tf1 == NULL means tf1 = I.
 * "_device" entry points take device pointers for per-query arrays and outputs and
 * are asynchronous on `stream` except where they must read a size back; the plain
 * entry points take host pointers (pinned or pageable) and copy in and out.       */
typedef struct {
  int32_t num_max_contacts;   /* CollisionRequest::num_max_contacts (collision_request.h:58) */
  int32_t precision;          /* FCLGPU_PLAIN_FP64 or FCLGPU_FP32_RECHECK */
  int32_t enable_statistics;  /* fill num_bv_tests / num_leaf_tests */
  int32_t budget;             /* BV tests per work item per round before its frontier is
                                 re-queued (work splitting); 0 = library default */
} fclgpu_collide_request;

/* Outputs of a collide batch.  counts[n] (int32) always.  Contacts (b1,b2 triangle
 * ids, int32 pairs) are written per query in the reference's DFS order, query after
 * query, at offsets[i] (int64, n+1 entries) when `contacts` is non-NULL; if the total
 * exceeds contacts_capacity the call returns FCLGPU_ERR_CAPACITY and *total_contacts
 * holds the size needed.  Optional per-query int64 statistics and FP64-recheck
 * counts (FP32_RECHECK form). */
typedef struct {
  int32_t* counts;
  int64_t* offsets;
  int32_t* contacts;
  int64_t contacts_capacity;
  int64_t* num_bv_tests;
  int64_t* num_leaf_tests;
  int64_t* num_rechecks;
  int64_t total_contacts;     /* written by the call */
} fclgpu_collide_result;

FCLGPU_API int fclgpu_collide_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes,
                                           const int32_t* pairs_host, int32_t num_pairs,
                                           int64_t n, const int32_t* pair_of_query,
                                           const double* tf1, const double* tf2,
                                           const fclgpu_collide_request* req,
                                           fclgpu_collide_result* res, void* stream);
FCLGPU_API int fclgpu_collide_batch(const fclgpu_mesh* meshes, int32_t num_meshes,
                                    const int32_t* pairs_host, int32_t num_pairs, int64_t n,
                                    const int32_t* pair_of_query, const double* tf1,
                                    const double* tf2, const fclgpu_collide_request* req,
                                    fclgpu_collide_result* res, void* stream);

/* Front-list (temporal coherence) collide of BVHModel<OBBRSS> pairs: FCL's
 * collide(node, front_list) with a BVHFrontList (geometry/bvh/detail/BVH_front.h;
 * collision_node-inl.h:72-82; traversal_recurse-inl.h:82-129, 463-521).  Query i's front
 * is front_in[2 * front_in_offsets[i] ..] up to front_in_offsets[i + 1] ((b1, b2) BV node
 * pairs, FCL's node ids), as a previous call returned it; an empty front (or
 * front_in == NULL) starts from the roots.  The call returns the contacts (b1, b2)
 * triangle ids in FCL's order for a front traversal (contacts are kept while fewer than
 * num_max_contacts exist; the traversal does not stop early, and a leaf reached from a
 * front node that overlaps is tested twice, as in FCL) and the query's new front, both
 * per query at int64 offsets (n + 1 entries).  total_contacts and total_front are set;
 * when either exceeds its capacity the call returns FCLGPU_ERR_CAPACITY with counts and
 * both offset arrays filled.  Optional statistics count FCL's BVTesting / leafTesting
 * calls.  front_in and front must not overlap.  "_device": device pointers; plain: host
 * pointers.  Synchronises the stream. */
typedef struct {
  int32_t num_max_contacts;  /* >= 1 */
  int32_t precision;         /* FCLGPU_PLAIN_FP64 or FCLGPU_FP32_RECHECK (same results) */
} fclgpu_front_request;

typedef struct {
  int32_t* counts;           /* n */
  int64_t* contact_offsets;  /* n + 1 */
  int32_t* contacts;         /* 2 x contacts_capacity */
  int64_t contacts_capacity;
  int64_t* front_offsets;    /* n + 1 */
  int32_t* front;            /* 2 x front_capacity */
  int64_t front_capacity;
  int64_t* num_bv_tests;     /* optional, n */
  int64_t* num_leaf_tests;   /* optional, n */
  int64_t total_contacts;    /* written by the call */
  int64_t total_front;       /* written by the call */
} fclgpu_front_result;

FCLGPU_API int fclgpu_collide_front_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes,
                                                 const int32_t* pairs_host, int32_t num_pairs, int64_t n,
                                                 const int32_t* pair_of_query, const double* tf1,
                                                 const double* tf2, const int64_t* front_in_offsets,
                                                 const int32_t* front_in, const fclgpu_front_request* req,
                                                 fclgpu_front_result* res, void* stream);
FCLGPU_API int fclgpu_collide_front_batch(const fclgpu_mesh* meshes, int32_t num_meshes,
                                          const int32_t* pairs_host, int32_t num_pairs, int64_t n,
                                          const int32_t* pair_of_query, const double* tf1, const double* tf2,
                                          const int64_t* front_in_offsets, const int32_t* front_in,
                                          const fclgpu_front_request* req, fclgpu_front_result* res, void* stream);

/* Contacts with their geometry: fcl::collide with CollisionRequest::enable_contact = true
 * on BVHModel<OBBRSS> pairs (mesh_collision_traversal_node-inl.h:579-600;
 * Intersect::intersect_Triangle with contact output, intersect-inl.h:597-617, 800-886).
 * Each intersecting triangle pair, in the reference's DFS order, adds 0, 1 or 2
 * contacts: the deepest points of one triangle below the other's plane (world frame),
 * the world normal (that plane's normal, negated when it is the second triangle's) and
 * the penetration depth, as many as fit under num_max_contacts; the query stops once it
 * holds num_max_contacts contacts.  counts[n] and offsets[n+1] (per query, contacts) are
 * always written; ids (b1, b2: 2 per contact), pos (3 per contact), normal (3 per
 * contact) and depth (1 per contact) when non-NULL, if total_contacts <= capacity
 * (else FCLGPU_ERR_CAPACITY with total_contacts set).  req->precision selects the pair
 * traversal's form; the contact geometry is FP64.  Statistics are not produced here
 * (req->enable_statistics must be 0).  "_device": device pointers, stream-ordered;
 * plain: host pointers.  Synchronises the stream. */
typedef struct {
  int32_t* counts;
  int64_t* offsets;
  int32_t* ids;
  double* pos;
  double* normal;
  double* depth;
  int64_t capacity;
  int64_t total_contacts;     /* written by the call */
} fclgpu_contact_result;

FCLGPU_API int fclgpu_collide_contacts_device(const fclgpu_mesh* meshes, int32_t num_meshes,
                                              const int32_t* pairs_host, int32_t num_pairs,
                                              int64_t n, const int32_t* pair_of_query,
                                              const double* tf1, const double* tf2,
                                              const fclgpu_collide_request* req,
                                              fclgpu_contact_result* res, void* stream);
FCLGPU_API int fclgpu_collide_contacts(const fclgpu_mesh* meshes, int32_t num_meshes,
                                       const int32_t* pairs_host, int32_t num_pairs, int64_t n,
                                       const int32_t* pair_of_query, const double* tf1,
                                       const double* tf2, const fclgpu_collide_request* req,
                                       fclgpu_contact_result* res, void* stream);

/* Continuous collision of mesh pairs: fcl::continuousCollide(o1, tf1_beg, tf1_end, o2,
 * tf2_beg, tf2_end, request, result) (narrowphase/continuous_collision-inl.h:436-451) with
 * the request's default solver CCDC_NAIVE (:134-171) and the motion CCDM_TRANS (default,
 * math/motion/translation_motion-inl.h), CCDM_LINEAR (interp_motion-inl.h, reference point
 * at the origin: FCL's two-transform constructor leaves it unset) or CCDM_SCREW
 * (screw_motion-inl.h): the motion is sampled at
 * n_iter = min(num_max_iterations, ceil(1/toc_err)) times t_i = i/(n_iter-1), each sample is
 * a discrete collide with the default CollisionRequest, and the first colliding t_i is the
 * time of contact (1 and no collision otherwise).  n_iter must be 0 (no sample: no
 * collision) or >= 2 (FCL divides 0 by 0 at n_iter = 1).  The linear and screw motions use
 * sin/cos/tan/atan2, whose device results differ from a host's in the last bits.  Other
 * CCDC_CONSERVATIVE_ADVANCEMENT runs FCL's conservative advancement as its oriented
 * OBBRSS node computes it (conservativeAdvancementMeshOriented with
 * MeshConservativeAdvancementTraversalNodeOBBRSS, conservative_advancement_func_matrix-inl.h
 * :149-218, mesh_conservative_advancement_traversal_node-inl.h:417-747): a discrete collide
 * at the start poses, then distance traversals at the motions' current transforms, each
 * advancing t by the smallest d / (motion bound) over the tested triangle pairs until the
 * step is <= 1e-5 (contact) or t passes 1; num_max_iterations and toc_err are not used, and
 * `iterations` (optional) receives the traversal count per query.  (fcl::continuousCollide's
 * dispatch table reaches the generic node for BVHModel<OBBRSS>, which re-transforms and
 * rebuilds copies of both meshes in the world frame every iteration; the oriented node is
 * FCL's OBBRSS specialisation of the same algorithm.)  The remaining
 * solvers and the spline motion return FCLGPU_ERR_UNSUPPORTED.  tf1_beg/tf1_end may both be NULL (identity).  Outputs per query:
 * is_collide, time_of_contact, and for colliding queries contact_tf1/contact_tf2 (the
 * sampled transforms at the time of contact, 12 doubles each; other entries are left
 * unchanged).  "_device": device pointers, plain: host pointers; both synchronise. */
enum { FCLGPU_CCDM_TRANS = 0, FCLGPU_CCDM_LINEAR = 1, FCLGPU_CCDM_SCREW = 2, FCLGPU_CCDM_SPLINE = 3 };
enum { FCLGPU_CCDC_NAIVE = 0, FCLGPU_CCDC_CONSERVATIVE_ADVANCEMENT = 1, FCLGPU_CCDC_RAY_SHOOTING = 2,
       FCLGPU_CCDC_POLYNOMIAL_SOLVER = 3 };

typedef struct {
  int64_t num_max_iterations; /* ContinuousCollisionRequest::num_max_iterations (10) */
  double toc_err;             /* ::toc_err (1e-4) */
  int32_t motion_type;        /* ::ccd_motion_type (FCLGPU_CCDM_TRANS, _LINEAR or _SCREW) */
  int32_t solver_type;        /* ::ccd_solver_type (FCLGPU_CCDC_NAIVE) */
  int32_t precision;          /* form of the discrete collides */
  int32_t reserved;
} fclgpu_ccd_request;

typedef struct {
  int32_t* is_collide;        /* ContinuousCollisionResult::is_collide */
  double* time_of_contact;    /* ::time_of_contact */
  double* contact_tf1;        /* ::contact_tf1 (3x4 row-major), may be NULL */
  double* contact_tf2;        /* ::contact_tf2, may be NULL */
  int32_t* iterations;        /* conservative advancement: traversals per query, may be NULL */
} fclgpu_ccd_result;

FCLGPU_API int fclgpu_continuous_collide_batch_device(
    const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host, int32_t num_pairs, int64_t n,
    const int32_t* pair_of_query, const double* tf1_beg, const double* tf1_end, const double* tf2_beg,
    const double* tf2_end, const fclgpu_ccd_request* req, fclgpu_ccd_result* res, void* stream);
FCLGPU_API int fclgpu_continuous_collide_batch(
    const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host, int32_t num_pairs, int64_t n,
    const int32_t* pair_of_query, const double* tf1_beg, const double* tf1_end, const double* tf2_beg,
    const double* tf2_end, const fclgpu_ccd_request* req, fclgpu_ccd_result* res, void* stream);

typedef struct {
  int32_t enable_nearest_points;  /* DistanceRequest::enable_nearest_points */
  int32_t precision;
  int32_t enable_statistics;
  int32_t reserved;
} fclgpu_distance_request;

/* min_distance[n] always; ids[2n] (b1,b2) and nearest_points[6n] (world frame, p1 then
 * p2) when given (nearest_points also needs enable_nearest_points); optional margins[n]
 * + within_margin[n] give the tolerance check distance <= margin (int32 0/1).  With
 * FCLGPU_FP32_RECHECK and none of ids, nearest points, margins or statistics, batches
 * of up to 65,536 queries take the distances alone one warp per query (the same
 * values). */
typedef struct {
  double* min_distance;
  int32_t* ids;
  double* nearest_points;
  const double* margins;
  int32_t* within_margin;
  int64_t* num_bv_tests;
  int64_t* num_leaf_tests;
  int64_t* num_rechecks;
} fclgpu_distance_result;

FCLGPU_API int fclgpu_distance_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes,
                                            const int32_t* pairs_host, int32_t num_pairs,
                                            int64_t n, const int32_t* pair_of_query,
                                            const double* tf1, const double* tf2,
                                            const fclgpu_distance_request* req,
                                            fclgpu_distance_result* res, void* stream);
FCLGPU_API int fclgpu_distance_batch(const fclgpu_mesh* meshes, int32_t num_meshes,
                                     const int32_t* pairs_host, int32_t num_pairs, int64_t n,
                                     const int32_t* pair_of_query, const double* tf1,
                                     const double* tf2, const fclgpu_distance_request* req,
                                     fclgpu_distance_result* res, void* stream);

/* Same query and outputs as fclgpu_distance_batch_device (device pointers), but the
 * call allocates no memory: for callers that cannot allocate GPU memory at query time
 * (deadline-bound control loops, processes whose HBM is owned by another allocator).
 * Its scratch is a fixed array inside the library, shared by all calls: at most 64
 * meshes and 256 pairs per call (larger requests return FCLGPU_ERR_INVALID_ARGUMENT),
 * and calls that overlap on the GPU race, so serialise them.  The call waits for its
 * stream before it returns.  The first call on a device looks the array up and should
 * come before any stream capture.  No counterpart in FCL. */
FCLGPU_API int fclgpu_distance_batch_noalloc(const fclgpu_mesh* meshes, int32_t num_meshes,
                                             const int32_t* pairs_host, int32_t num_pairs,
                                             int64_t n, const int32_t* pair_of_query,
                                             const double* tf1, const double* tf2,
                                             const fclgpu_distance_request* req,
                                             fclgpu_distance_result* res, void* stream);

/* Testing aid: the record and work-item capacities the next mesh collide batches start
 * from (0 = automatic; a batch that outgrows them doubles them and runs again), and a
 * traversal stack limit below the compiled one (0 = none; a traversal that needs more
 * reports FCLGPU_ERR_DEVICE_STATUS).  For exercising those two paths.  No counterpart
 * in FCL. */
FCLGPU_API int fclgpu_set_collide_test_limits(int64_t initial_records, int64_t initial_items, int32_t stack_limit);

/* The mesh collide rounds run as one cooperative launch (enable = 1, the default): the
 * grid meets at a device-wide barrier between rounds and the next round's work items
 * come from the device queue, with no host read-back between rounds.  A barrier wait
 * longer than barrier_timeout_ns (default 60 s) makes the launch give up, and the batch
 * runs again one launch per round (enable = 0 always does; results are the same).
 * test_missing_blocks = 1 makes every barrier wait for one block more than the grid
 * has (testing the give-up path).  No counterpart in FCL. */
FCLGPU_API int fclgpu_set_collide_persistent(int32_t enable, int64_t barrier_timeout_ns, int32_t test_missing_blocks);
/* Batches that fell back from the persistent launch since load. */
FCLGPU_API int64_t fclgpu_collide_persistent_fallbacks(void);

/* Number of this library's kernel launches issued since load (for launch accounting). */
FCLGPU_API int64_t fclgpu_kernel_launch_count(void);
/* Device time (ms, CUDA events on the batch's stream) of the traversal kernel of the
 * most recent collide or distance batch.  No counterpart in FCL (profiling hook). */
FCLGPU_API int fclgpu_last_kernel_time(double* ms);
/* Knobs of the collide rounds, chosen by the autotuner (fcl_gb300/api.py
 * autotune_collide): BV tests an item runs per round before its frontier is re-queued
 * (the request's budget overrides it when non-zero), the DFS steps a lane runs between
 * two warp-wide batches of leaf tests, and the register variant of that kernel (0 =
 * unbounded, 1 = 128 registers for a fourth resident block) (FP32 form).  Results do
 * not depend on them.  No counterpart in FCL. */
FCLGPU_API int fclgpu_set_collide_tuning(int32_t budget, int32_t leaf_batch_steps, int32_t variant);
FCLGPU_API int fclgpu_get_collide_tuning(int32_t* budget, int32_t* leaf_batch_steps, int32_t* variant);

/* ---- convex shapes (fcl::Box/Sphere/Capsule/Cylinder/Cone/Convex, geometry/shape/ headers) --
 * GJK/EPA of FCL's own solver (GJKSolver_indep, narrowphase/detail/gjk_solver_indep.h)
 * with its closed-form pairs; replaces fcl::collide / fcl::distance on shape pairs
 * (collision_func_matrix-inl.h:278-311, distance_func_matrix-inl.h:207-226). */
enum {
  FCLGPU_SHAPE_BOX = 0,       /* params: side x, y, z */
  FCLGPU_SHAPE_SPHERE = 1,    /* params: radius */
  FCLGPU_SHAPE_CAPSULE = 2,   /* params: radius, lz */
  FCLGPU_SHAPE_CYLINDER = 3,  /* params: radius, lz */
  FCLGPU_SHAPE_CONE = 4,      /* params: radius, lz */
  FCLGPU_SHAPE_CONVEX = 5     /* vertices [vertex_offset, +vertex_count) of the pool */
};

typedef struct {
  int32_t type;
  int32_t vertex_offset;
  int32_t vertex_count;
  int32_t reserved;
  double params[3];
} fclgpu_shape;

typedef struct fclgpu_shapeset_s* fclgpu_shapeset;

/* Uploads n shapes and the convex vertex pool (nv vertices, 3 doubles each). */
FCLGPU_API int fclgpu_shapeset_create(const fclgpu_shape* shapes, int32_t n, const double* verts, int64_t nv,
                                      fclgpu_shapeset* out);
FCLGPU_API int fclgpu_shapeset_destroy(fclgpu_shapeset set);

/* Per pair i (shapes ia[i], ib[i] at tf1[i], tf2[i]): hit = fcl::collide with contact;
 * when hit, normal / point / depth are the contact (depth is FCL's ContactPoint
 * penetration_depth: positive for closed forms, -epa.depth for GJK/EPA); when not hit,
 * distance and the world-frame witness points p1, p2 are fcl::distance's (-1 if the
 * solver failed).  status[2i] = GJK status, status[2i+1] = EPA status (-1 = not run).
 * hit and distance are required; other outputs may be NULL. */
typedef struct {
  int32_t* hit;
  double* normal;
  double* point;
  double* depth;
  double* distance;
  double* p1;
  double* p2;
  int32_t* status;
} fclgpu_shape_result;

FCLGPU_API int fclgpu_shape_batch_device(fclgpu_shapeset set, int64_t n, const int32_t* ia, const int32_t* ib,
                                         const double* tf1, const double* tf2, fclgpu_shape_result* res,
                                         void* stream);
FCLGPU_API int fclgpu_shape_batch(fclgpu_shapeset set, int64_t n, const int32_t* ia, const int32_t* ib,
                                  const double* tf1, const double* tf2, fclgpu_shape_result* res, void* stream);
/* GJKSolver_indep's parameters (narrowphase/detail/gjk_solver_indep.h: gjk_tolerance,
 * epa_tolerance, gjk_max_iterations, epa_max_iterations).  Process-wide: every later
 * shape-pair, mesh-shape and broadphase call that runs GJK or EPA uses them.  The
 * defaults are the solver's own (2^-45.5, 2^-45.5, 128, 255; gjk_solver_indep-inl.h:
 * 1039-1049); FCL's fcl::collide sets both tolerances to CollisionRequest::gjk_tolerance
 * and fcl::distance the GJK tolerance to DistanceRequest::distance_tolerance (both
 * 1e-6 by default; collision-inl.h:164-170, distance-inl.h:211-215).  NULL restores the
 * defaults.  Tolerances must be positive and finite, iteration caps at least 1. */
typedef struct {
  double gjk_tolerance;
  double epa_tolerance;
  int32_t gjk_max_iterations;
  int32_t epa_max_iterations;
} fclgpu_gjk_solver_params;
FCLGPU_API int fclgpu_set_gjk_solver_params(const fclgpu_gjk_solver_params* params);
FCLGPU_API int fclgpu_get_gjk_solver_params(fclgpu_gjk_solver_params* params);

/* fcl::collide on convex shape pairs with enable_contact = false (GJKSolver_indep):
 * hit[i] = 1 when FCL's ShapeCollisionTraversalNode::leafTesting adds
 * Contact(o1, o2, NONE, NONE) (shape_collision_traversal_node-inl.h:70-136); no contact
 * geometry, no EPA.  Host arrays. */
FCLGPU_API int fclgpu_shape_collide_batch(fclgpu_shapeset set, int64_t n, const int32_t* ia, const int32_t* ib,
                                          const double* tf1, const double* tf2, int32_t* hit, void* stream);
/* Device time (ms) of the most recent shape-pair kernel.  No counterpart in FCL. */
FCLGPU_API int fclgpu_last_shape_kernel_time(double* ms);

/* ---- mesh x convex shape ------------------------------------------------------------
 * fcl::collide / fcl::distance of a BVHModel<OBBRSS> against a convex shape with
 * GJKSolver_indep (narrowphase/detail/collision_func_matrix-inl.h:378-425, 502-523;
 * distance_func_matrix-inl.h BVHShapeDistancer; traversal nodes
 * mesh_shape_collision_traversal_node-inl.h and mesh_shape_distance_traversal_node-inl.h):
 * the shape's OBBRSS is fitted to its bound vertices, the mesh BVH is traversed against
 * it, and the leaves run shapeTriangleIntersect / shapeTriangleDistance (sphere-triangle
 * closed forms, GJK/EPA otherwise).  Results are FCL's FP64 ones: FP32 filters and
 * certified FP32 bounds only skip volumes and triangles that cannot change them, and
 * every deciding test runs in FP64.  Pair i: meshes[mesh_idx[i]] at tf_mesh[i] and
 * shape shape_idx[i] of the set at tf_shape[i].  (fcl::collide(shape, mesh) is the same
 * call: FCL swaps the arguments.) */
enum { FCLGPU_MESH_SHAPE_COLLIDE = 0, FCLGPU_MESH_SHAPE_DISTANCE = 1 };

typedef struct {
  int32_t mode;              /* FCLGPU_MESH_SHAPE_COLLIDE or _DISTANCE */
  int32_t reserved;
  int64_t num_max_contacts;  /* collide: CollisionRequest::num_max_contacts (>= 1) */
} fclgpu_mesh_shape_request;

/* collide: counts[i] = contacts (<= num_max_contacts).  distance: min_distance[i],
 * tri[i] = the mesh triangle of the minimum (DistanceResult b1), nearest_points[6i..6i+5]
 * = the point on the mesh then the point on the shape, in the frames FCL returns them in
 * (world frame from GJK; for a sphere, the sphere point in the sphere's frame and the
 * triangle point in the mesh's frame), -1 if the pair intersects.  Statistics optional. */
typedef struct {
  int32_t* counts;
  double* min_distance;
  int32_t* tri;
  double* nearest_points;
  int64_t* num_bv_tests;
  int64_t* num_leaf_tests;
} fclgpu_mesh_shape_result;

FCLGPU_API int fclgpu_mesh_shape_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes,
                                              int64_t n, const int32_t* mesh_idx, const int32_t* shape_idx,
                                              const double* tf_mesh, const double* tf_shape,
                                              const fclgpu_mesh_shape_request* req, fclgpu_mesh_shape_result* res,
                                              void* stream);
FCLGPU_API int fclgpu_mesh_shape_batch(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes,
                                       int64_t n, const int32_t* mesh_idx, const int32_t* shape_idx,
                                       const double* tf_mesh, const double* tf_shape,
                                       const fclgpu_mesh_shape_request* req, fclgpu_mesh_shape_result* res,
                                       void* stream);

/* Mesh x convex shape collide with the contact list: the mesh triangles that
 * MeshShapeCollisionTraversalNode::leafTesting adds as Contact(mesh, shape, triangle,
 * NONE) (mesh_shape_collision_traversal_node-inl.h:64-102; FCL records the mesh first
 * whichever argument order fcl::collide got, collision-inl.h:124-131), in the order the
 * traversal adds them, at most num_max_contacts per pair.  Pair i's triangles are
 * tris[offsets[i] .. offsets[i+1]); counts[i] = offsets[i+1] - offsets[i].
 * total_contacts is set on return; when it exceeds capacity the call returns
 * FCLGPU_ERR_CAPACITY and tris is left untouched (counts and offsets are filled).
 * With pos, normal and penetration_depth set (all three or none: CollisionRequest::
 * enable_contact) contact k also gets the geometry the leaf records,
 * Contact(mesh, shape, tri, NONE, contactp, -normal, penetration)
 * (mesh_shape_collision_traversal_node-inl.h:233-244): pos[3k..3k+2], normal[3k..3k+2]
 * (world frame) and penetration_depth[k], as shapeTriangleIntersect computes them
 * (sphere: sphereTriangleIntersect, sphere_triangle-inl.h:139-220; other shapes: GJK then
 * EPA, gjk_solver_indep-inl.h:449-505).  The triangle list is the same either way. */
typedef struct {
  int32_t* counts;
  int64_t* offsets;  /* n + 1 entries */
  int32_t* tris;
  int64_t capacity;  /* entries tris can hold */
  int64_t total_contacts;
  double* pos;               /* optional: 3 x capacity */
  double* normal;            /* optional: 3 x capacity */
  double* penetration_depth; /* optional: capacity */
} fclgpu_mesh_shape_contacts_result;

FCLGPU_API int fclgpu_mesh_shape_contacts_device(const fclgpu_mesh* meshes, int32_t num_meshes,
                                                 fclgpu_shapeset shapes, int64_t n, const int32_t* mesh_idx,
                                                 const int32_t* shape_idx, const double* tf_mesh,
                                                 const double* tf_shape, int64_t num_max_contacts,
                                                 fclgpu_mesh_shape_contacts_result* res, void* stream);
FCLGPU_API int fclgpu_mesh_shape_contacts(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes,
                                          int64_t n, const int32_t* mesh_idx, const int32_t* shape_idx,
                                          const double* tf_mesh, const double* tf_shape, int64_t num_max_contacts,
                                          fclgpu_mesh_shape_contacts_result* res, void* stream);

/* ---- broadphase -------------------------------------------------------------------
 * Replaces DynamicAABBTreeCollisionManager<double> (broadphase/
 * broadphase_dynamic_AABB_tree.h:56-157, -inl.h:727-1009) behind
 * BroadPhaseCollisionManager's registerObjects/setup/update and the per-object
 * collide(obj, cdata, DefaultCollisionFunction) / distance(obj, cdata,
 * DefaultDistanceFunction) queries (broadphase_collision_manager.h:65-122,
 * default_broadphase_callbacks.h:88-106, 195-215), batched over many query objects.
 *
 * Geometry is referenced, as CollisionObject's shared_ptr<CollisionGeometry> is
 * (narrowphase/collision_object.h:143-144): the broadphase keeps the shape set and the
 * mesh table it was created with, and scene objects and query objects name a
 * geometry by (kind, index).  World AABBs follow CollisionObject::computeAABB
 * (collision_object-inl.h:116-131) bit for bit.  The device tree is an LBVH rebuilt from
 * Morton codes; its shape differs from FCL's, so the results reported are the ones
 * that do not depend on traversal order (see the result structs). */
enum { FCLGPU_GEOM_SHAPE = 0, FCLGPU_GEOM_MESH = 1 };

typedef struct {
  int32_t kind;   /* FCLGPU_GEOM_SHAPE: index into the shape set; FCLGPU_GEOM_MESH: into meshes[] */
  int32_t index;
} fclgpu_geometry_ref;

typedef struct fclgpu_broadphase_s* fclgpu_broadphase;

/* registerObjects + setup: num_objects scene objects (geometry refs and poses, host
 * arrays).  shapes may be NULL when no shape is referenced; meshes may be NULL when
 * num_meshes is 0.  The shape set and meshes must outlive the broadphase. */
FCLGPU_API int fclgpu_broadphase_create(fclgpu_shapeset shapes, const fclgpu_mesh* meshes, int32_t num_meshes,
                                        const fclgpu_geometry_ref* objects, int32_t num_objects, const double* tf,
                                        fclgpu_broadphase* out);
/* update(): new poses for every scene object (tf: num_objects x 12 doubles, a device
 * pointer when tf_on_device != 0); AABBs are recomputed and the tree rebuilt. */
FCLGPU_API int fclgpu_broadphase_update(fclgpu_broadphase bp, const double* tf, int32_t tf_on_device, void* stream);
FCLGPU_API int fclgpu_broadphase_destroy(fclgpu_broadphase bp);
/* CollisionObject::getAABB() of every scene object: 6 doubles (min, max) each. */
FCLGPU_API int fclgpu_broadphase_get_aabbs(fclgpu_broadphase bp, double* aabb6);

typedef struct {
  int64_t num_max_contacts; /* CollisionRequest::num_max_contacts (>= 1) */
  int32_t precision;        /* mesh-mesh narrowphase form (FCLGPU_PLAIN_FP64 / FCLGPU_FP32_RECHECK) */
  int32_t exhaustive;       /* 1: evaluate every candidate pair; 0: like FCL's callback, stop a
                               query once it has num_max_contacts contacts (shape pairs are
                               evaluated first, then mesh-shape, then mesh-mesh pairs) */
} fclgpu_broadphase_collide_request;

/* Per query q: num_contacts[q] = DefaultCollisionData::result.numContacts() after
 * manager.collide(query, DefaultCollisionFunction), which is min(num_max_contacts,
 * sum over colliding scene objects of their contacts); num_objects[q] = number of
 * scene objects found in collision with the query and first_object[q] = the smallest
 * such object index (-1 if none).  With exhaustive = 1 both cover every object, an
 * extension that does not depend on the order FCL's callback would meet the objects in;
 * with exhaustive = 0 they cover the pairs evaluated before the query stopped.  Outputs
 * may be NULL except num_contacts.  The totals are filled on return. */
typedef struct {
  int64_t* num_contacts;
  int32_t* num_objects;
  int32_t* first_object;
  int64_t total_candidates;  /* (query, object) pairs with overlapping AABBs */
  int64_t total_node_visits; /* tree nodes loaded */
} fclgpu_broadphase_collide_result;

/* queries: nq geometry refs, tf: nq x 12 doubles.  _device: every pointer (queries,
 * tf and the result arrays) is a device pointer; the plain form takes host pointers. */
FCLGPU_API int fclgpu_broadphase_collide_device(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                                const double* tf, const fclgpu_broadphase_collide_request* req,
                                                fclgpu_broadphase_collide_result* res, void* stream);
FCLGPU_API int fclgpu_broadphase_collide(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                         const double* tf, const fclgpu_broadphase_collide_request* req,
                                         fclgpu_broadphase_collide_result* res, void* stream);

typedef struct {
  int32_t enable_nearest_points;
  int32_t precision; /* mesh-mesh narrowphase form */
} fclgpu_broadphase_distance_request;

/* Per query q: min_distance[q] = DefaultDistanceData::result.min_distance after
 * manager.distance(query, DefaultDistanceFunction) for a query in no contact (the
 * minimum over scene objects; ties go to the smaller object index); object[q] = that
 * scene object, ids[2q..2q+1] = its (b1, b2) triangle ids (-1 for shapes),
 * nearest_points[6q..6q+5] = the world-frame witnesses on the object and on the
 * query.  A query in contact reports a value <= 0 (FCL reports the first contact its
 * traversal meets, -1 for shape pairs, 0 for mesh pairs).  DBL_MAX for an empty
 * scene.  Outputs other than min_distance may be NULL. */
typedef struct {
  double* min_distance;
  int32_t* object;
  int32_t* ids;
  double* nearest_points;
  int64_t total_candidates;  /* (query, object) pairs evaluated by the narrowphase */
  int64_t total_node_visits;
} fclgpu_broadphase_distance_result;

FCLGPU_API int fclgpu_broadphase_distance_device(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries,
                                                 int64_t nq, const double* tf,
                                                 const fclgpu_broadphase_distance_request* req,
                                                 fclgpu_broadphase_distance_result* res, void* stream);
FCLGPU_API int fclgpu_broadphase_distance(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                          const double* tf, const fclgpu_broadphase_distance_request* req,
                                          fclgpu_broadphase_distance_result* res, void* stream);
/* Contact lists of broadphase collide queries: the contacts DefaultCollisionFunction
 * records (default_broadphase_callbacks.h:88-106) as Contact(o1, o2, b1, b2), with o1
 * the scene object and o2 the query, as FCL's manager calls the narrowphase
 * (broadphase_dynamic_AABB_tree-inl.h:526-547).  Every (query, scene object) pair
 * whose AABBs overlap is evaluated, each capped at num_max_contacts contacts (a fresh
 * CollisionResult per pair).  Per query the contacts are ordered by scene-object index,
 * and each object's contacts come in the order FCL's narrowphase adds them: (object,
 * -1, -1) for a shape pair, (object, b1, b2) for a mesh pair (b1 the object's
 * triangle, b2 the query's), (object, triangle, -1) for a mesh-shape pair (FCL records
 * the mesh's triangle as b1 whichever is the mesh).  FCL's manager meets the objects in
 * its tree's order and stops at num_max_contacts in all: with num_max_contacts at least
 * the query's total its contact set is this list's; FCL's numContacts() is
 * min(num_max_contacts, counts[q]). */
typedef struct {
  int64_t num_max_contacts;  /* per (query, object) pair, >= 1 */
  int32_t precision;         /* mesh-mesh narrowphase form */
  int32_t reserved;
} fclgpu_broadphase_contacts_request;

/* counts[q] contacts of query q at contacts[3 * offsets[q] ..) as (object, b1, b2)
 * int32 triples; offsets has nq + 1 entries.  capacity = triples contacts can hold;
 * total_contacts is set on return and a larger total returns FCLGPU_ERR_CAPACITY with
 * counts and offsets filled and contacts untouched. */
typedef struct {
  int64_t* counts;
  int64_t* offsets;
  int32_t* contacts;
  int64_t capacity;
  int64_t total_contacts;
  int64_t total_candidates;
  int64_t total_node_visits;
} fclgpu_broadphase_contacts_result;

FCLGPU_API int fclgpu_broadphase_collide_contacts_device(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries,
                                                         int64_t nq, const double* tf,
                                                         const fclgpu_broadphase_contacts_request* req,
                                                         fclgpu_broadphase_contacts_result* res, void* stream);
FCLGPU_API int fclgpu_broadphase_collide_contacts(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries,
                                                  int64_t nq, const double* tf,
                                                  const fclgpu_broadphase_contacts_request* req,
                                                  fclgpu_broadphase_contacts_result* res, void* stream);
/* manager.collide(cdata, DefaultCollisionFunction): the scene against itself
 * (broadphase_dynamic_AABB_tree-inl.h:949-965, selfCollisionRecurse :552-567).  Every
 * unordered pair of scene objects with overlapping AABBs is evaluated once, as
 * Contact(o1, o2, ...) with o1 < o2; the lists are grouped by o2 (counts and offsets
 * have one entry per scene object, segment q holding the pairs (o1 < q, o2 = q) in
 * ascending o1), each triple (o1, b1, b2) with b1 on o1 and b2 on o2. */
FCLGPU_API int fclgpu_broadphase_self_collide_contacts_device(fclgpu_broadphase bp,
                                                              const fclgpu_broadphase_contacts_request* req,
                                                              fclgpu_broadphase_contacts_result* res, void* stream);
FCLGPU_API int fclgpu_broadphase_self_collide_contacts(fclgpu_broadphase bp,
                                                       const fclgpu_broadphase_contacts_request* req,
                                                       fclgpu_broadphase_contacts_result* res, void* stream);
/* manager.distance(cdata, DefaultDistanceFunction): the smallest distance between two
 * scene objects (broadphase_dynamic_AABB_tree-inl.h:968-987 -> selfDistanceRecurse
 * :706-720), evaluated over every unordered pair whose AABB distance is within an
 * upper bound of it.  o1 < o2; b1, b2 their triangle ids (-1 for shapes);
 * nearest_points the world witnesses on o1 then o2 (with enable_nearest_points).  Ties
 * go to the smaller o2, then the smaller o1; FCL reports the first its traversal
 * meets.  A value <= 0 means some pair is in contact (FCL stops there).  DBL_MAX with
 * fewer than two objects.  Host result. */
typedef struct {
  double min_distance;
  int32_t o1, o2;
  int32_t b1, b2;
  double nearest_points[6];
  int64_t total_candidates;
} fclgpu_broadphase_self_distance_result;

FCLGPU_API int fclgpu_broadphase_self_distance(fclgpu_broadphase bp, const fclgpu_broadphase_distance_request* req,
                                               fclgpu_broadphase_self_distance_result* out, void* stream);
/* Wall-clock phases of the broadphase collide (out16[0..7]) and distance (out16[8..15])
 * calls made since the previous read (reading resets them): [0] query setup and
 * candidate passes, [1] shape-shape pairs,
 * [2] mesh-shape pairs, [3] mesh-mesh pairs, [4] reduction (ms); [5] candidate pairs,
 * [6] mesh-shape and [7] mesh-mesh pairs evaluated.  No counterpart in FCL. */
FCLGPU_API int fclgpu_broadphase_last_phase_ms(double* out16);

/* ---- motion-checking request loop --------------------------------------------------
 * No counterpart in FCL: a serving loop over a resident broadphase scene.  A request
 * is a serial robot swept along K waypoints; each link geometry at each waypoint is
 * one broadphase query (manager.collide with num_max_contacts = 1 and, when
 * clearance is on, manager.distance).  The loop runs on its own thread and stream:
 * requests are queued by fclgpu_server_submit from any thread, admitted into the
 * next step while the step's estimated device footprint fits the free-memory budget,
 * and processed in waypoint chunks shared fairly among the admitted requests, so
 * requests arriving while others run join the next launch (continuous batching).
 * A request's result depends only on its own queries. */
typedef struct {
  int32_t num_links;
  const int32_t* joint_axis;                 /* per link: 0 = x, 1 = y, 2 = z of the previous link frame */
  const double* link_offset;                 /* per link: 3 doubles, the link's translation after its joint */
  const fclgpu_geometry_ref* link_geometry;  /* per link: geometry in the scene's registry */
  const double* link_geometry_tf;            /* per link: 12 doubles, geometry pose in the joint frame */
} fclgpu_robot_desc;

typedef struct {
  int64_t max_waypoints_per_step; /* 0 = 4096 */
  int64_t memory_budget_bytes;    /* 0 = half of the free device memory, read at every step */
  int32_t precision;              /* mesh-mesh narrowphase form */
  int32_t compute_clearance;      /* 1 = also report the minimum clearance */
} fclgpu_server_config;

/* A request stops at its first contact (waypoints are checked in order, in chunks):
 * then min_clearance = 0 at (first colliding waypoint, its smallest colliding link).
 * Otherwise min_clearance is the minimum over every waypoint and link of the
 * broadphase distance, with its waypoint, link and scene object. */
typedef struct {
  int32_t first_colliding_waypoint; /* smallest waypoint with any link in collision, -1 if none */
  int32_t clearance_waypoint;       /* argmin of the clearance (ties: smallest waypoint, then link) */
  int32_t clearance_link;
  int32_t clearance_object;         /* -1 for a request in contact */
  double min_clearance;             /* 0 for a request in contact */
  double latency_ms;                /* submit -> result ready */
  double queue_ms;                  /* submit -> first step that included the request */
  int32_t num_steps;                /* loop steps that processed its waypoints */
  int32_t reserved;
} fclgpu_motion_result;

typedef struct {
  int64_t steps;
  int64_t waypoints;
  int64_t queries;
  int64_t candidates;
  double busy_ms;          /* wall time spent in steps */
  int64_t max_step_waypoints;
  double collide_ms;       /* of busy_ms: the broadphase collide calls and their read-back */
  double distance_ms;      /* of busy_ms: the clearance pass (gather, distance, read-back) */
} fclgpu_server_stats;

typedef struct fclgpu_server_s* fclgpu_server;

/* The scene must outlive the server.  The robot description is copied. */
FCLGPU_API int fclgpu_server_create(fclgpu_broadphase scene, const fclgpu_robot_desc* robot,
                                    const fclgpu_server_config* cfg, fclgpu_server* out);
/* Queues a request: base pose (12 doubles) and num_waypoints x num_links joint angles
 * (host arrays, copied).  Thread-safe; returns at once with the request id. */
FCLGPU_API int fclgpu_server_submit(fclgpu_server srv, const double* base_tf, const double* q,
                                    int32_t num_waypoints, int64_t* request_id);
/* Waits up to timeout_ms (< 0: forever) for a request; FCLGPU_OK fills *out and
 * retires the id, FCLGPU_ERR_PENDING means it has not finished. */
FCLGPU_API int fclgpu_server_wait(fclgpu_server srv, int64_t request_id, double timeout_ms,
                                  fclgpu_motion_result* out);
FCLGPU_API int fclgpu_server_get_stats(fclgpu_server srv, fclgpu_server_stats* out);
/* The link-geometry poses the loop computes for one request (num_waypoints x
 * num_links x 12 doubles, host), for checking results against another engine. */
FCLGPU_API int fclgpu_server_link_poses(fclgpu_server srv, const double* base_tf, const double* q,
                                        int32_t num_waypoints, double* out_tf);
/* Stops the loop after its current step.  Unfinished requests are dropped: threads
 * blocked in fclgpu_server_wait on them return FCLGPU_ERR_NOT_INITIALIZED, and this
 * call returns only after every such thread has left fclgpu_server_wait.  No call on
 * the handle may start after destroy has begun. */
FCLGPU_API int fclgpu_server_destroy(fclgpu_server srv);

#ifdef __cplusplus
}
#endif
#endif /* FCLGPU_H */
