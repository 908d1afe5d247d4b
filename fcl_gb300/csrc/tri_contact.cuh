// Contact information of an intersecting triangle pair, FP64 in the reference's
// operation order (CollisionRequest::enable_contact = true):
//
//   Intersect::intersect_Triangle(P1, P2, P3, Q1, Q2, Q3, R, T, contacts, ...)
//     (narrowphase/detail/traversal/collision/intersect-inl.h:597-617, 800-844): the
//     second triangle is moved into the first one's frame (R Q + T); each triangle gets
//     its plane (buildTrianglePlane, :1040-1053); the deepest points of each triangle
//     below the other's plane are found (computeDeepestPoints, :848-886); the side
//     whose deepest point is shallower gives the contact points (at most two), the
//     normal (the first triangle's plane normal, or the negated normal of the second)
//     and the penetration depth.
//   meshCollisionOrientedNodeLeafTesting (mesh_collision_traversal_node-inl.h:579-600)
//     then maps the points and the normal to the world by tf1.
//
// A triangle whose edge cross product is zero has no plane; FCL's caller then reads an
// unset normal and offset.  Here such a triangle gets the zero plane (normal 0,
// offset 0), in the oracle as on the device.
#pragma once
#include <float.h>

#include "geom.cuh"

namespace fclgpu {

constexpr double kContactEps = 1e-5;       // Intersect<S>::getEpsilon() (intersect-inl.h:1117-1120)
constexpr double kDeepestTie = 1e-6;       // computeDeepestPoints' tie band (intersect-inl.h:870)

// buildTrianglePlane: n = normalized((b - a) x (c - a)), t = n . a
FCLG_HD void tri_plane(const V3<double>& a, const V3<double>& b, const V3<double>& c, V3<double>& n, double& t) {
  const V3<double> m = cross(b - a, c - a);
  const double sq = sqnorm(m);
  if (sq > 0) {
    const double l = sqrt(sq);
    n = v3<double>(m.x / l, m.y / l, m.z / l);
    t = dot(n, a);
  } else {
    n = v3<double>(0.0, 0.0, 0.0);
    t = 0.0;
  }
}

// computeDeepestPoints over the three points of a triangle: depth = max of
// -(n . p - t); the points within 1e-6 of the running maximum are kept in visiting
// order; none are kept when the deepest point lies above the plane by more than eps or
// when no point lies on the plane and all lie on one side of it.
FCLG_HD void deepest_points(const V3<double> p[3], const V3<double>& n, double t, double& depth,
                            V3<double> out[3], int& nout) {
  double max_depth = -DBL_MAX;
  int k = 0, npos = 0, nneg = 0, nzero = 0;
  for (int i = 0; i < 3; ++i) {
    const double dist = -(dot(n, p[i]) - t);
    if (dist > kContactEps)
      ++npos;
    else if (dist < -kContactEps)
      ++nneg;
    else
      ++nzero;
    if (dist > max_depth) {
      max_depth = dist;
      k = 1;
      out[0] = p[i];
    } else if (dist + kDeepestTie >= max_depth) {
      out[k++] = p[i];
    }
  }
  if (max_depth < -kContactEps) k = 0;
  if (nzero == 0 && (nneg == 0 || npos == 0)) k = 0;
  depth = max_depth;
  nout = k;
}

// P: triangle of model 1; Qm: triangle of model 2 already moved into model 1's frame.
// Returns the number of contacts (0, 1 or 2); pts, normal and depth in model 1's frame.
FCLG_HD int tri_contact(const V3<double> P[3], const V3<double> Qm[3], V3<double> pts[2], V3<double>& normal,
                        double& depth) {
  V3<double> n1, n2;
  double t1, t2;
  tri_plane(P[0], P[1], P[2], n1, t1);
  tri_plane(Qm[0], Qm[1], Qm[2], n2, t2);
  V3<double> d1[3], d2[3];
  int k1, k2;
  double pd1, pd2;
  deepest_points(Qm, n1, t1, pd2, d2, k2);
  deepest_points(P, n2, t2, pd1, d1, k1);
  int k;
  if (pd1 > pd2) {
    k = k2 < 2 ? k2 : 2;
    for (int i = 0; i < k; ++i) pts[i] = d2[i];
    normal = n1;
    depth = pd2;
  } else {
    k = k1 < 2 ? k1 : 2;
    for (int i = 0; i < k; ++i) pts[i] = d1[i];
    normal = v3<double>(-n2.x, -n2.y, -n2.z);
    depth = pd1;
  }
  return k;
}

// The leaf's contact in world coordinates: triangles p1 of A and p2 of B at the query's
// relative transform (R, T); tf1 (3x4 row-major) maps model 1's frame to the world.
struct TriContact {
  int n;
  double pos[2][3];
  double normal[3];
  double depth;
};

FCLG_HD void tri_contact_world(const V3<double> P[3], const V3<double> Q[3], const M3<double>& R,
                               const V3<double>& T, const double* tf1, TriContact& c) {
  V3<double> Qm[3];
  for (int k = 0; k < 3; ++k) Qm[k] = mulv(R, Q[k]) + T;
  V3<double> pts[2], nrm;
  double depth;
  c.n = tri_contact(P, Qm, pts, nrm, depth);
  M3<double> R1;
  V3<double> t1;
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) R1(r, q) = tf1[4 * r + q];
  t1 = v3<double>(tf1[3], tf1[7], tf1[11]);
  for (int i = 0; i < 2; ++i) {
    const V3<double> w = i < c.n ? mulv(R1, pts[i]) + t1 : v3<double>(0.0, 0.0, 0.0);
    c.pos[i][0] = w.x;
    c.pos[i][1] = w.y;
    c.pos[i][2] = w.z;
  }
  const V3<double> nw = mulv(R1, nrm);
  c.normal[0] = nw.x;
  c.normal[1] = nw.y;
  c.normal[2] = nw.z;
  c.depth = depth;
}

}  // namespace fclgpu
