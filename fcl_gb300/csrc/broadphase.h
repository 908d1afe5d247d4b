// Device broadphase: a linear BVH (LBVH) over scene-object AABBs, rebuilt on the
// device from Morton codes, queried per query object; plus the record types the
// C ABI layer (capi_broadphase.cu) hands to the kernels (broadphase.cu).
//
// The tree replaces FCL's DynamicAABBTreeCollisionManager tree
// (broadphase/broadphase_dynamic_AABB_tree-inl.h, broadphase/detail/hierarchy_tree-inl.h).
// Its structure differs from FCL's (Morton order instead of median splits), so every
// result it returns is one that does not depend on traversal order: candidate sets,
// contact totals, collision booleans and minimum distances.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fclgpu_types.h"
#include "gjk_epa.cuh"

namespace fclgpu {

enum : int32_t { GEOM_SHAPE = 0, GEOM_MESH = 1 };

// One geometry of the registry the scene and the queries draw from: its kind, index
// (into the shape set or the mesh table) and CollisionGeometry::aabb_local /
// aabb_center / aabb_radius (geometry/collision_geometry.h:104-113).
struct GeomRec {
  int32_t kind;
  int32_t index;
  int32_t pad[2];
  double lo[3], hi[3];
  double center[3];
  double radius;
  double ref[3];  // a point of the geometry (mesh: its first vertex) for distance upper bounds
};

// LBVH internal node: both children's FP32 boxes (rounded outward from the FP64
// object AABBs) and their indices; child >= 0 is an internal node, child < 0 is the
// leaf of scene object ~child.  64 bytes, loaded as four float4.
struct __align__(16) BpNode {
  float lo0[3];
  int32_t c0;
  float hi0[3];
  int32_t c1;
  float lo1[3];
  int32_t pad0;
  float hi1[3];
  int32_t pad1;
};

struct BpSceneView {
  const GeomRec* geoms;
  const DevShape* shapes;
  const double* sverts;
  const DevMesh* meshes;
  int32_t n;         // scene objects
  int32_t root;      // node index, or ~object when n == 1
  const int32_t* gid;
  const double* tf;      // 12 per object
  const double* aabb64;  // 6 per object (min, max), FCL's CollisionObject::getAABB()
  const BpNode* nodes;
  // shape BVs of the scene's objects at their current poses (ShapeBV records), fitted
  // at their first mesh-shape pair after a pose update: bv_ok[o] != 0 once bv_cache[o]
  // holds object o's; both null = no cache
  void* bv_cache = nullptr;
  int32_t* bv_ok = nullptr;
};

// ---------------------------------------------------------------- build ----
// World AABBs (CollisionObject::computeAABB, collision_object-inl.h:116-131) of n
// objects, FP64 (6 per object) and rounded outward to FP32 (6 per object).
cudaError_t launch_world_aabbs(const GeomRec* geoms, int64_t n, const int32_t* gid, const double* tf,
                               double* aabb64, float* aabb32, cudaStream_t s);
// LBVH over n >= 2 leaves.  scratch holds at least bp_build_scratch_bytes(n) bytes.
size_t bp_build_scratch_bytes(int64_t n);
cudaError_t launch_lbvh_build(int32_t n, const float* aabb32, BpNode* nodes, void* scratch, cudaStream_t s);

// ---------------------------------------------------------------- queries ----
struct BpQueryView {
  int64_t nq;
  const int32_t* gid;   // geometry id per query
  const double* tf;     // 12 per query
  const double* aabb64; // 6 per query
  const float* aabb32;  // 6 per query
  // 1: the queries are the scene objects themselves (query q is object q) and only
  // objects of a smaller index are candidates, so each unordered pair is met once
  int32_t self = 0;
};

enum : uint32_t { BP_ERR_STACK = 1u, BP_ERR_REF = 2u };

// Geometry refs (kind, index) of nq queries -> registry ids (shapes first, then meshes);
// an out-of-range ref sets BP_ERR_REF.
cudaError_t launch_bp_query_gids(const int2* refs, int64_t nq, int32_t ns, int32_t nm, int32_t* gid,
                                 unsigned* status, cudaStream_t s);

// Candidate pass: scene objects whose FP64 AABB overlaps the query's (exactly the
// pairs FCL's collisionRecurse hands to its callback).  counts_only: write counts[q];
// else write (query, object) pairs at offsets[q].
cudaError_t launch_bp_overlap(const BpSceneView& S, const BpQueryView& Q, int32_t* counts, const int64_t* offsets,
                              int2* pairs, int64_t* node_visits, unsigned* status, cudaStream_t s);
// Distance upper bound per query: min over visited objects of |p_obj - p_query| for
// one point of each geometry, visiting nearest-first with pruning by the FP32 lower
// bound.  Then the candidate pass: objects whose FP64 AABB distance is below it.
cudaError_t launch_bp_dist_bound(const BpSceneView& S, const BpQueryView& Q, double* ub, unsigned* status,
                                 cudaStream_t s);
cudaError_t launch_bp_dist_candidates(const BpSceneView& S, const BpQueryView& Q, const double* ub, int32_t* counts,
                                      const int64_t* offsets, int2* pairs, int64_t* node_visits, unsigned* status,
                                      cudaStream_t s);

// Narrowphase of candidate pairs.  kind[i] = 0 shape-shape, 1 mesh-mesh, 2 mixed.
cudaError_t launch_bp_classify(const BpSceneView& S, const BpQueryView& Q, const int2* pairs, int64_t n,
                               int32_t* kind, cudaStream_t s);
// Shape-shape pairs (kind 0) in place: collide -> hit[i]; distance -> dist/points.
cudaError_t launch_bp_shape_narrow(const BpSceneView& S, const BpQueryView& Q, const int2* pairs, int64_t n,
                                   const int32_t* kind, int mode, int32_t* hit, double* dist, double* pts,
                                   cudaStream_t s);
// Gathers of the mesh-mesh pairs (kind 1): per listed pair, the mesh-pair index
// (scene mesh * nm + query mesh) and both transforms.
cudaError_t launch_bp_gather_mesh(const BpSceneView& S, const BpQueryView& Q, const int2* pairs,
                                  const int64_t* list, int64_t nlist, int32_t nm, int32_t* pair_index, double* tf1,
                                  double* tf2, cudaStream_t s);
// Candidates of one kind; with qdone, only those whose query is not yet done.
cudaError_t launch_bp_list(const int32_t* kind, int64_t n, int32_t want, const int2* pairs, const int32_t* qdone,
                           int64_t* list, unsigned long long* count, cudaStream_t s);
// qdone[q] = 1 when the contacts found so far for query q reach max_contacts.
cudaError_t launch_bp_query_done(int64_t nq, const int64_t* offsets, const int32_t* hit, int64_t max_contacts,
                                 int32_t* qdone, cudaStream_t s);
// Mixed pairs (kind 2): FCL calls BVH-shape with the mesh first whichever object is
// the mesh (collision-inl.h:100-111, distance-inl.h:117-126); gather (mesh, shape)
// indices and poses in that order.
// bv_src (optional): per pair, the shape's BV source (query q -> q, scene object o ->
// nq + o), with need[src] = 1 set for every source used.
cudaError_t launch_bp_gather_mixed(const BpSceneView& S, const BpQueryView& Q, const int2* pairs,
                                   const int64_t* list, int64_t nlist, int32_t* mesh_idx, int32_t* shape_idx,
                                   double* tfm, double* tfs, int32_t* bv_src, int32_t* need, int32_t* query_of,
                                   cudaStream_t s);
// The shape BV (computeBV<OBBRSS> in the world frame) of every needed source into
// table (ShapeBV records of mesh_shape.cuh): a shape at one pose is fitted once however
// many mesh-shape pairs it is in.
cudaError_t launch_bp_shape_bvs(const BpSceneView& S, const BpQueryView& Q, const int32_t* need, void* table,
                                cudaStream_t s);
cudaError_t launch_bp_scatter_mixed_dist(const int64_t* list, int64_t nlist, const double* d, const int32_t* tri,
                                         const double* pts, double* dist, int32_t* b12, double* outpts,
                                         cudaStream_t s);
// Scatter mesh results back to candidate slots.
cudaError_t launch_bp_scatter_hits(const int64_t* list, int64_t nlist, const int32_t* counts, int32_t* hit,
                                   cudaStream_t s);
cudaError_t launch_bp_scatter_dist(const int64_t* list, int64_t nlist, const double* d, const int32_t* ids,
                                   const double* pts, double* dist, int32_t* b12, double* outpts, cudaStream_t s);

// Contact lists.  perm: each query's candidate slots sorted by scene-object index.
cudaError_t launch_bp_sort_segments(int64_t nq, const int64_t* offsets, const int2* pairs, int64_t* perm,
                                    cudaStream_t s);
// index[list[k]] = k for the nlist slots of one pair kind
cudaError_t launch_bp_inverse_index(const int64_t* list, int64_t nlist, int32_t* index, cudaStream_t s);
// ccount[j] = contacts of slot perm[j] (hit)
cudaError_t launch_bp_gather_counts(const int64_t* perm, int64_t total, const int32_t* hit, int32_t* ccount,
                                    cudaStream_t s);
// per query: counts[q] and offsets[q] of its contacts from the scanned per-slot counts
cudaError_t launch_bp_query_contacts(int64_t nq, const int64_t* offsets, const int64_t* coff, int64_t* counts,
                                     int64_t* out_offsets, cudaStream_t s);
// (object, b1, b2) triples of every slot in perm order at coff[j]: shape pairs
// (object, -1, -1); mesh-mesh pairs the (b1, b2) list of their collide; mesh-shape
// pairs (object, triangle, -1)
cudaError_t launch_bp_fill_contacts(const int64_t* perm, int64_t total, const int2* pairs, const int32_t* kind,
                                    const int32_t* hit, const int64_t* coff, const int32_t* mm_index,
                                    const int64_t* mm_off, const int32_t* mm_contacts, const int32_t* ms_index,
                                    const int64_t* ms_off, const int32_t* ms_tris, int32_t* out, cudaStream_t s);

// Per-query reductions over the candidate segments [offsets[q], offsets[q+1]).
cudaError_t launch_bp_reduce_collide(int64_t nq, const int64_t* offsets, const int2* pairs, const int32_t* hit,
                                     int64_t max_contacts, int64_t* num_contacts, int32_t* num_objects,
                                     int32_t* first_object, cudaStream_t s);
cudaError_t launch_bp_reduce_distance(int64_t nq, const int64_t* offsets, const int2* pairs, const double* dist,
                                      const int32_t* b12, const double* pts, double* min_distance, int32_t* object,
                                      int32_t* ids, double* nearest, cudaStream_t s);

}  // namespace fclgpu
