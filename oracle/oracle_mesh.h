// FP64 CPU oracle for the BVHModel<OBBRSS> mesh path: BVH build, OBB/RSS bounding
// volume tests, triangle leaf tests and the two traversals.
//
// TEST INFRASTRUCTURE ONLY (see oracle_math.h).  Every function cites the FCL 0.7.0
// source it restates (paths relative to the FCL repository).
#pragma once
#include <vector>
#include <cstdint>
#include "oracle_math.h"

namespace oracle {

// math/bv/OBB.h:62-68
struct OBB {
  M3 axis;
  V3 To;
  V3 extent;
};
// math/bv/RSS.h:70-82
struct RSS {
  M3 axis;
  V3 To;
  double l[2];
  double r;
};
// geometry/bvh/BV_node.h:51-74, BV_node_base.h:50-76
struct Node {
  OBB obb;
  RSS rss;
  int first_child;  // <0: leaf, primitive = -(first_child+1)
  int first_primitive;
  int num_primitives;
};

struct Tri {
  int v[3];
};

struct Mesh {
  std::vector<V3> verts;
  std::vector<Tri> tris;
  std::vector<Node> nodes;
  std::vector<unsigned> prim_idx;
};

// --- BVH build (geometry/bvh/BVH_model-inl.h:450-517, 833-938) -------------------
void build_bvh(Mesh& m);

// --- point-set fits and bottom-up refit (oracle_refit.cpp) ---------------------------
void covariance_points(const V3* ps, int n, M3& M);
void extent_center_points(const V3* ps, int n, const M3& axis, V3& center, V3& extent, std::vector<V3>* P);
void fit_points_obbrss(const V3* ps, int n, OBB& obb, RSS& rss);  // fit<OBBRSS>, n >= 4
OBB obb_merge(const OBB& a, const OBB& b);                           // OBB::operator+
RSS rss_merge(const RSS& self, const RSS& other);                    // RSS::operator+
// beginUpdateModel, updateVertex x nv, endUpdateModel(refit = true, bottomup = true)
void update_refit_bottomup(Mesh& m, const std::vector<V3>& new_verts);
// beginReplaceModel, replaceVertex x nv, endReplaceModel(refit = true, bottomup = true)
void replace_refit_bottomup(Mesh& m, const std::vector<V3>& new_verts);
void fit3_obbrss(const V3 ps[3], OBB& obb, RSS& rss);                // fit<OBBRSS>, n = 3

// --- point-set RSS fit for three points (math/bv/utility-inl.h:208-230) ----------
void rss_fit3(const V3 ps[3], RSS& bv);

// --- bounding-volume tests ----------------------------------------------------------
bool obb_disjoint(const M3& B, const V3& T, const V3& a, const V3& b);          // OBB-inl.h:398-523
bool obb_overlap(const M3& R0, const V3& T0, const OBB& b1, const OBB& b2);      // OBB-inl.h:383-395
double rect_distance(const M3& Rab, const V3& Tab, const double a[2], const double b[2],
                     V3* P, V3* Q);                                              // RSS-inl.h:512-1224
double rss_distance(const M3& R0, const V3& T0, const RSS& b1, const RSS& b2,
                    V3* P, V3* Q);                                               // RSS-inl.h:1956-1974
double rss_member_distance(const RSS& a, const RSS& b);                         // RSS-inl.h:432-446
inline double obb_size(const OBB& b) { return sqnorm(b.extent); }               // OBB-inl.h:205-209

// --- leaf tests -----------------------------------------------------------------------
bool tri_intersect(const V3& P1, const V3& P2, const V3& P3, const V3& Q1, const V3& Q2,
                   const V3& Q3, const M3& R, const V3& T);                      // intersect-inl.h:597-617,727-798
double tri_distance(const V3 T1[3], const V3 T2[3], V3& P, V3& Q);             // triangle_distance-inl.h:170-394

// --- queries ----------------------------------------------------------------------
struct CollideStats {
  int64_t num_bv_tests = 0;
  int64_t num_leaf_tests = 0;
};

// fcl::collide for BVHModel<OBBRSS> x BVHModel<OBBRSS> with enable_contact=false.
// Contacts are appended in the reference's DFS order as (b1, b2) triangle ids.
size_t collide_mesh(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2,
                    size_t num_max_contacts, std::vector<int>& contacts, CollideStats* st);

// collide(node, front_list) with a BVHFrontList (collision_node-inl.h:72-82,
// traversal_recurse-inl.h:82-129, 463-521): front holds the (b1, b2) list in and out;
// an empty list starts from the roots.  Contacts are kept while fewer than
// num_max_contacts exist; the traversal does not stop early.
size_t collide_mesh_front(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2, size_t num_max_contacts,
                          std::vector<int>& front, std::vector<int>& contacts, CollideStats* st);

// fcl::collide with enable_contact = true: each intersecting triangle pair adds 0..2
// contacts with position and normal in the world frame and the penetration depth
// (mesh_collision_traversal_node-inl.h:579-600, intersect-inl.h:800-886).
struct ContactOut {
  int b1, b2;
  V3 pos, normal;
  double depth;
};
size_t collide_mesh_contacts(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2,
                             size_t num_max_contacts, std::vector<ContactOut>& out, CollideStats* st);
// the contact part of intersect_Triangle on P and Qm (Q moved into P's frame)
int tri_contact_info(const V3 P[3], const V3 Qm[3], V3 cp[2], V3& normal, double& depth);

// fcl::continuousCollide with the naive solver and the translation (0), linear (1) or
// screw (2) motion; toc = time of
// contact (1 without collision), ca / cb = the sampled transforms at that time.
// continuousCollide with CCDC_CONSERVATIVE_ADVANCEMENT on BVHModel<OBBRSS> pairs, as
// FCL's oriented OBBRSS node computes it (conservativeAdvancementMeshOriented with
// MeshConservativeAdvancementTraversalNodeOBBRSS, conservative_advancement_func_matrix-inl.h
// :149-218, mesh_conservative_advancement_traversal_node-inl.h:417-747): a discrete collide
// at the start; then repeated distance traversals under the current relative transform,
// each giving delta_t = min over tested triangle pairs of d / (motion bound along the
// pair's direction), advancing t by delta_t until delta_t <= 1e-5 (contact) or t > 1.
bool continuous_collide_ca(const Mesh& m1, const Tf& a0, const Tf& a1, const Mesh& m2, const Tf& b0, const Tf& b1,
                           int motion, double& toc, Tf& ca, Tf& cb, int64_t* iterations);

bool continuous_collide_naive(const Mesh& m1, const Tf& a0, const Tf& a1, const Mesh& m2, const Tf& b0,
                              const Tf& b1, size_t num_max_iterations, double toc_err, int motion, double& toc,
                              Tf& ca, Tf& cb);

struct DistanceOut {
  double min_distance;
  int b1, b2;
  V3 p1, p2;  // world frame (postprocess maps by tf1)
};
// fcl::distance for BVHModel<OBBRSS> pairs with rel_err = abs_err = 0.
double distance_mesh(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2,
                     bool nearest_points, DistanceOut& out, CollideStats* st);

// --- fit helpers shared with the mesh-shape oracle ---------------------------------
void eigen_old(const M3& m, V3& dout, M3& vout);                            // math/geometry-inl.h:477-558
void axis_from_eigen(const M3& eigenV, const V3& eigenS, M3& axis);          // math/geometry-inl.h:294-318
void rss_from_projected(const std::vector<V3>& P, const M3& axis, V3& origin, double l[2],
                        double& r);                                          // math/geometry-inl.h:709-990

}  // namespace oracle
