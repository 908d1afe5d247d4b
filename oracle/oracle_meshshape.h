// FP64 CPU oracle for BVHModel<OBBRSS> x convex shape: fcl::collide and fcl::distance
// with GJKSolver_indep.  TEST INFRASTRUCTURE ONLY (see oracle_math.h).  Every function
// cites the FCL 0.7.0 source it restates (paths relative to the FCL repository).
#pragma once
#include <vector>

#include "oracle_gjk.h"
#include "oracle_mesh.h"

namespace oracle {

// Shape::getBoundVertices (box-inl.h:121-138, sphere-inl.h:95-120,
// capsule-inl.h:107-160, cylinder-inl.h:101-126, cone-inl.h:108-128,
// convex-inl.h:252-262)
std::vector<V3> bound_vertices(const Shape& s, const Tf& tf);

// computeBV<OBBRSS>(shape, tf): the generic ComputeBVImpl (geometry/shape/utility-inl.h:
// 123-133) fits the bound vertices (math/bv/utility-inl.h:516-520 -> OBB fitn :133-145,
// RSS fitn :247-260).
void shape_obbrss(const Shape& s, const Tf& tf, OBB& obb, RSS& rss);

// detail::sphereTriangleIntersect (primitive_shape_algorithm/sphere_triangle-inl.h),
// triangle already in the world frame.
// With the optional outputs: contact point, normal and depth as the function reports
// them (contact_points, normal_, penetration_depth).
bool sphere_triangle_intersect(double radius, const V3& center, const V3& P1, const V3& P2, const V3& P3,
                               V3* contact_point = nullptr, V3* normal_out = nullptr, double* depth = nullptr);

// The contact MeshShapeCollisionTraversalNode::leafTesting adds with enable_contact
// (mesh_shape_collision_traversal_node-inl.h:91-103): shapeTriangleIntersect with its
// contact outputs (gjk_solver_indep-inl.h:449-548; sphere: sphereTriangleIntersect),
// recorded as Contact(..., contactp, -normal, penetration).  pos, normal, depth are those
// recorded values; false when the pair does not intersect.
bool shape_triangle_contact(const Shape& s, const Tf& tfs, const V3& P1, const V3& P2, const V3& P3, const Tf& tfm,
                            V3& pos, V3& normal, double& depth);

// Project<S>::projectLine / projectTriangle with an explicit point
// (math/detail/project-inl.h:54-136).
ProjectResult project_line_p(const V3& a, const V3& b, const V3& p);
ProjectResult project_triangle_p(const V3& a, const V3& b, const V3& c, const V3& p);

// GJKSolver_indep::shapeTriangleIntersect (gjk_solver_indep-inl.h:449-548): the
// triangle P1..P3 is in the frame of tfm.
bool shape_triangle_intersect(const Shape& s, const Tf& tfs, const V3& P1, const V3& P2, const V3& P3,
                              const Tf& tfm);
// GJKSolver_indep::shapeTriangleDistance (gjk_solver_indep-inl.h:946-1040).  ps is the
// point on the shape, pt the point on the triangle, in the frames FCL returns them in
// (world frame for GJK; for a sphere: ps in the sphere's frame, pt in tfm's frame).
// Returns false (d = -1) when the pair intersects.
bool shape_triangle_distance(const Shape& s, const Tf& tfs, const V3& P1, const V3& P2, const V3& P3,
                             const Tf& tfm, double& d, V3& ps, V3& pt);

// fcl::collide(mesh, shape) for BVHModel<OBBRSS>: orientedBVHShapeCollide
// (collision_func_matrix-inl.h:378-425) over MeshShapeCollisionTraversalNodeOBBRSS
// (mesh_shape_collision_traversal_node-inl.h:191-265, 351-375, 377-406) and
// collisionRecurse (traversal_recurse-inl.h:82-129).  Returns the contacts added,
// at most max_contacts; their triangle ids go to tris when given.
size_t collide_mesh_shape(const Mesh& m, const Tf& tfm, const Shape& s, const Tf& tfs, size_t max_contacts,
                          std::vector<int>* tris, CollideStats* st);

// fcl::distance(mesh, shape): MeshShapeDistanceTraversalNodeOBBRSS
// (mesh_shape_distance_traversal_node-inl.h:164-226, 345-455), distanceRecurse
// (traversal_recurse-inl.h:257-316).  out.b1 = triangle id, out.b2 = -1, out.p1 on the
// mesh, out.p2 on the shape (frames as shape_triangle_distance).
double distance_mesh_shape(const Mesh& m, const Tf& tfm, const Shape& s, const Tf& tfs, DistanceOut& out,
                           CollideStats* st);

}  // namespace oracle
