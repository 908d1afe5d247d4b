// FP64 CPU oracle for the broadphase: CollisionObject world AABBs, the
// DynamicAABBTreeCollisionManager tree and its query recursions with FCL's default
// callbacks, and the brute-force manager they are checked against.
//
// TEST INFRASTRUCTURE ONLY (see oracle_math.h).  Every function cites the FCL 0.7.0
// source it restates (paths relative to the FCL repository).
#pragma once
#include <cstdint>
#include <vector>
#include "oracle_gjk.h"
#include "oracle_mesh.h"
#include "oracle_meshshape.h"

namespace oracle {

// math/bv/AABB.h:52-60 (min_, max_); AABB-inl.h:52-57 default = empty box
struct AABB {
  V3 mn, mx;
};

// A collision geometry as the broadphase sees it: a convex shape or a
// BVHModel<OBBRSS> mesh, with CollisionGeometry::aabb_local / aabb_center /
// aabb_radius (collision_geometry.h:104-113) filled by compute_local_aabb.
struct BpGeom {
  int kind = 0;  // 0 = shape, 1 = mesh
  Shape shape;
  const Mesh* mesh = nullptr;
  AABB local;
  V3 center;
  double radius = 0;
};

// Shape::computeLocalAABB (box-inl.h:80-88, sphere-inl.h:62-69, capsule-inl.h:64-72,
// cylinder-inl.h:64-72, cone-inl.h:64-72, convex-inl.h:86-96) and
// BVHModel::computeLocalAABB (BVH_model-inl.h:1080-1100).
void compute_local_aabb(BpGeom& g);
// CollisionObject::computeAABB (collision_object-inl.h:116-131).
AABB compute_aabb(const BpGeom& g, const Tf& tf);
bool aabb_overlap(const AABB& a, const AABB& b);     // AABB-inl.h:98-107
double aabb_distance(const AABB& a, const AABB& b);  // AABB-inl.h:292-315

struct BpObject {
  const BpGeom* geom;
  Tf tf;
  AABB aabb;
};

// HierarchyTree<AABB> as DynamicAABBTreeCollisionManager::registerObjects builds it
// (broadphase_dynamic_AABB_tree-inl.h:746-776 -> hierarchy_tree-inl.h:70-90 init_0,
// 424-459 topdown_0, 344-377 bottomup; bu_threshold = 2, topdown_level = 0).
struct DynTree {
  struct Node {
    AABB bv;
    int child[2];
    int obj;  // scene object index at a leaf, -1 inside
  };
  std::vector<Node> nodes;
  int root = -1;
  void build(const std::vector<AABB>& leaf_bv);
};

// DefaultCollisionData / DefaultDistanceData results (default_broadphase_callbacks.h).
struct BpCollideOut {
  int64_t num_contacts = 0;
  std::vector<int> hit_objects;  // scene objects whose narrowphase reported contact, in callback order
  int64_t narrow_calls = 0;
};
struct BpDistanceOut {
  double min_distance;
  int object = -1;  // scene object that set min_distance
  int b1 = -1, b2 = -1;
  V3 p1, p2;
  int64_t narrow_calls = 0;
};

// manager.collide(query, &data, DefaultCollisionFunction) with
// data.request.num_max_contacts = max_contacts: tree recursion
// (broadphase_dynamic_AABB_tree-inl.h:526-547, 894-917) or the naive manager's loop
// (broadphase_bruteforce-inl.h:110-119).  Both pass (scene object, query) to the
// narrowphase in the tree manager's order.
void bp_collide(const std::vector<BpObject>& scene, const DynTree* tree, const BpObject& query,
                int64_t max_contacts, BpCollideOut& out);
// manager.distance(query, &data, DefaultDistanceFunction): tree recursion
// (broadphase_dynamic_AABB_tree-inl.h:658-701, 920-944) or the naive loop
// (broadphase_bruteforce-inl.h:123-136).
void bp_distance(const std::vector<BpObject>& scene, const DynTree* tree, const BpObject& query,
                 BpDistanceOut& out);

// The contact lists of the GPU broadphase contacts call: every scene object whose
// AABB overlaps the query, in index order, collide(object, query) with a fresh
// CollisionResult capped at max_per_pair; triples (object, b1, b2) appended to out.
void bp_collide_lists(const std::vector<BpObject>& scene, const BpObject& query, int64_t max_per_pair,
                      std::vector<int>& out);

// NaiveCollisionManager::collide(cdata, DefaultCollisionFunction)
// (broadphase_bruteforce-inl.h:140-157): pairs (i < j) with overlapping AABBs in list
// order, one CollisionResult capped at max_contacts; returns its numContacts().
int64_t bp_self_collide_naive(const std::vector<BpObject>& scene, int64_t max_contacts);

// The self-collision lists of the GPU call: for each o2, the objects o1 < o2 with
// overlapping AABBs in ascending order, collide(o1, o2) with a fresh result capped at
// max_per_pair; counts per o2 and (o1, b1, b2) triples.
void bp_self_collide_lists(const std::vector<BpObject>& scene, int64_t max_per_pair, std::vector<int64_t>& counts,
                           std::vector<int>& out);

// NaiveCollisionManager::distance(cdata, DefaultDistanceFunction)
// (broadphase_bruteforce-inl.h:161-177): the first smallest distance over pairs
// (i < j) in list order, pruned by AABB distance; stops at a distance <= 0.
struct BpSelfDistanceOut {
  double min_distance = 0;
  int o1 = -1, o2 = -1, b1 = -1, b2 = -1;
  V3 p1, p2;
};
void bp_self_distance_naive(const std::vector<BpObject>& scene, BpSelfDistanceOut& out);

}  // namespace oracle
