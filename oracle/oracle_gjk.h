// FP64 CPU oracle for convex shape pairs: FCL's own GJK/EPA (GST_INDEP solver) and
// the closed-form pairs its dispatch prefers.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <vector>

#include "oracle_math.h"

namespace oracle {

// geometry/shape/*.h (Box side, Sphere radius, Capsule/Cylinder/Cone radius + lz,
// Convex vertex list)
enum ShapeType { SH_BOX = 0, SH_SPHERE = 1, SH_CAPSULE = 2, SH_CYLINDER = 3, SH_CONE = 4, SH_CONVEX = 5,
                 SH_TRIANGLE = 6 /* TriangleP: verts[0..2], used by the mesh-shape leaves */ };

struct Shape {
  int type;
  double p[3];             // box: side[3]; sphere: radius; capsule/cylinder/cone: radius, lz
  const V3* verts = nullptr;  // convex
  int nverts = 0;
};

struct ShapeResult {
  bool collide;
  V3 normal, point;  // contact (only when collide)
  double depth;      // penetration depth (>= 0) when collide
  double distance;   // when not colliding (GJK / closed form), -1 when that failed
  V3 p1, p2;         // world-frame witness points when not colliding
  int gjk_status, epa_status;
};

// fcl::collide + fcl::distance for one convex pair with GJKSolver_indep.
void shape_pair(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r);
// The two halves of shape_pair: the intersect dispatch (gjk_solver_indep-inl.h:182-200;
// fills normal/point/depth/statuses when it returns true) and the distance dispatch
// (gjk_solver_indep-inl.h:686-708; distance -1 when the pair intersects).
// enable_contact = false is collide() without contact information: it only changes
// the box-box answer in the case the reference's clipping keeps no point
// (box_box-inl.h:747, 775), which collides without contacts and so collide() with
// contacts reports no contact.
bool shape_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r,
                     bool enable_contact = true);
void shape_distance(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r);

// Pure GJK/EPA without closed-form dispatch (used to check the device solver).
bool gjk_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, V3* normal, V3* point,
                   double* depth, int* gjk_status, int* epa_status);
bool gjk_distance(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, double* dist, V3* p1, V3* p2,
                  int* gjk_status);

// Simplex projections (math/detail/project-inl.h:183-320), exposed for the
// known-answer tests of test_fcl_simple.cpp.
struct ProjectResult {
  double parameterization[4] = {0, 0, 0, 0};
  double sqr_distance = -1;
  unsigned encode = 0;
};
ProjectResult project_line(const V3& a, const V3& b);
ProjectResult project_triangle(const V3& a, const V3& b, const V3& c);
ProjectResult project_tetra(const V3& a, const V3& b, const V3& c, const V3& d);

// The GJKSolver_indep parameters every later GJK / EPA uses (process-wide; defaults
// 2^-45.5, 2^-45.5, 128, 255 as gjk_solver_indep-inl.h:1039-1049).
void set_solver_params(double gjk_tolerance, double epa_tolerance, size_t gjk_max_iterations,
                       size_t epa_max_iterations);

}  // namespace oracle
